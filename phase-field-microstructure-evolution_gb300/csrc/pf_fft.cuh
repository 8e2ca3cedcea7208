// Shared-memory FFT building blocks for the sm_103a phase-field step.
//
// These replace the FFTs that the reference obtains from P3DFFT/FFTW through
// f_trans (src/f_trans.f90:11, forward R2C) and inv_trans
// (src/inv_trans.f90:10, inverse C2R).  A line of length L = N1*N2 is
// transformed in place by a two-pass "four-step" algorithm:
//
//   pass A (per column n1 < N1):  V = DFT_N2(x[n1 + N1*n2]),  x[n1+N1*k2] = V[k2]*W_L^(n1*k2)
//   pass B (per row    k2 < N2):  x[k1+N1*k2] = DFT_N1(x[n1+N1*k2])[k1]
//
// so that after the forward transform position p = k1 + N1*k2 holds the
// coefficient of frequency k = k2 + N2*k1 ("digit-transposed" order).  The
// inverse runs the same passes backwards (B then A, conjugate twiddles) and
// takes that order back to natural order.  The spectral update in between is
// pointwise, so no reordering pass is ever needed.
//
// Each DFT of size <= 20 lives in registers (17 as a direct DFT); in shared memory every run of N1
// consecutive elements is followed by one pad slot and the line pitch is odd,
// which makes pass A, pass B and line-to-line transposes free of bank
// conflicts for 8-byte complex elements.
#pragma once
#include <cuda_runtime.h>

namespace pf {

// The in-register DFTs and complex helpers compile for the host as well, so
// that tests can check them against a reference DFT on the CPU.
#define PF_HD __host__ __device__ __forceinline__

// complex add and subtract: one packed FP32-pair instruction each on the device
PF_HD float2 cadd(float2 a, float2 b) {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
  return __fadd2_rn(a, b);
#else
  return make_float2(a.x + b.x, a.y + b.y);
#endif
}
PF_HD float2 csub(float2 a, float2 b) {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
  return __ffma2_rn(b, make_float2(-1.f, -1.f), a);
#else
  return make_float2(a.x - b.x, a.y - b.y);
#endif
}
PF_HD float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
PF_HD float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
// a * b
PF_HD float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// a * conj(b)
PF_HD float2 cmulc(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.y, b.x, -a.x * b.y));
}
// -i * a
PF_HD float2 cmul_mi(float2 a) { return make_float2(a.y, -a.x); }
// +i * a
PF_HD float2 cmul_pi(float2 a) { return make_float2(-a.y, a.x); }

// ---------------------------------------------------------------------------
// Exact twiddle constants for the in-register DFTs (W_R^j = e^{-2 pi i j / R})
// ---------------------------------------------------------------------------
#define PF_C16_1 0.92387953251128675613f  // cos(pi/8)
#define PF_S16_1 0.38268343236508977173f  // sin(pi/8)
#define PF_SQRT1_2 0.70710678118654752440f
#define PF_SQRT3_2 0.86602540378443864676f
// cos(2 pi j / 20), j = 1..4 (the radix-5 stages)
#define PF_C20_1 0.95105651629515357212f  // cos(pi/10)
#define PF_C20_2 0.80901699437494742410f  // cos(pi/5)
#define PF_C20_3 0.58778525229247312917f  // cos(3 pi/10)
#define PF_C20_4 0.30901699437494742410f  // cos(2 pi/5)

// cos and sin of 2 pi m / 17, m = 1..8 (the prime-17 DFT)
#define PF_C17_1 0.932472229404355804573f
#define PF_C17_2 0.739008917220659115925f
#define PF_C17_3 0.445738355776538267396f
#define PF_C17_4 0.0922683594633019952397f
#define PF_C17_5 -0.273662990072082863539f
#define PF_C17_6 -0.602634636379256389179f
#define PF_C17_7 -0.850217135729614152134f
#define PF_C17_8 -0.982973099683901778282f
#define PF_S17_1 0.361241666187152948745f
#define PF_S17_2 0.673695643646557211713f
#define PF_S17_3 0.895163291355062322067f
#define PF_S17_4 0.995734176295034521871f
#define PF_S17_5 0.961825643172819070409f
#define PF_S17_6 0.798017227280239503333f
#define PF_S17_7 0.526432162877355800245f
#define PF_S17_8 0.183749517816570331574f

// W_R^j for R in {2,3,4,5,6,8,10,12,16,20} (forward sign), j in [0, R)
template <int R>
PF_HD float2 wconst(int j);

template <>
PF_HD float2 wconst<16>(int j) {
  // angles j * 22.5 degrees, clockwise
  const float c[16] = {1.f, PF_C16_1, PF_SQRT1_2, PF_S16_1, 0.f, -PF_S16_1, -PF_SQRT1_2, -PF_C16_1,
                       -1.f, -PF_C16_1, -PF_SQRT1_2, -PF_S16_1, 0.f, PF_S16_1, PF_SQRT1_2, PF_C16_1};
  return make_float2(c[j & 15], -c[(j + 12) & 15]);
}
template <>
PF_HD float2 wconst<8>(int j) { return wconst<16>(2 * j); }
template <>
PF_HD float2 wconst<4>(int j) { return wconst<16>(4 * j); }
template <>
PF_HD float2 wconst<12>(int j) {
  // angles j * 30 degrees, clockwise
  const float c[12] = {1.f, PF_SQRT3_2, 0.5f, 0.f, -0.5f, -PF_SQRT3_2, -1.f, -PF_SQRT3_2, -0.5f, 0.f, 0.5f, PF_SQRT3_2};
  return make_float2(c[j % 12], -c[(j + 9) % 12]);
}
template <>
PF_HD float2 wconst<6>(int j) { return wconst<12>(2 * j); }
template <>
PF_HD float2 wconst<20>(int j) {
  // angles j * 18 degrees, clockwise
  const float c[20] = {1.f,       PF_C20_1,  PF_C20_2,  PF_C20_3,  PF_C20_4,  0.f,       -PF_C20_4,
                       -PF_C20_3, -PF_C20_2, -PF_C20_1, -1.f,      -PF_C20_1, -PF_C20_2, -PF_C20_3,
                       -PF_C20_4, 0.f,       PF_C20_4,  PF_C20_3,  PF_C20_2,  PF_C20_1};
  return make_float2(c[j % 20], -c[(j + 15) % 20]);
}
template <>
PF_HD float2 wconst<10>(int j) { return wconst<20>(2 * j); }
template <>
PF_HD float2 wconst<5>(int j) { return wconst<20>(4 * j); }
template <>
PF_HD float2 wconst<3>(int j) { return wconst<12>(4 * j); }

// ---------------------------------------------------------------------------
// In-register forward DFTs, natural order in and out
// ---------------------------------------------------------------------------
template <int R>
struct Dft;
template <int R>
PF_HD void dft_inv(float2* v);

template <>
struct Dft<1> {
  PF_HD static void fwd(float2*) {}
};

template <>
struct Dft<2> {
  PF_HD static void fwd(float2* v) {
    float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  }
};

template <>
struct Dft<3> {
  PF_HD static void fwd(float2* v) {
    float2 a = v[0];
    float2 t1 = cadd(v[1], v[2]);
    float2 t2 = csub(v[1], v[2]);
    float2 m = make_float2(fmaf(-0.5f, t1.x, a.x), fmaf(-0.5f, t1.y, a.y));
    float2 s = cscale(t2, PF_SQRT3_2);
    v[0] = cadd(a, t1);
    v[1] = cadd(m, cmul_mi(s));
    v[2] = cadd(m, cmul_pi(s));
  }
};

template <>
struct Dft<4> {
  // INV: +i instead of -i in the odd outputs; (v1 - v3) times -i (or +i) is
  // formed directly in swapped order, so the butterflies stay packed pairs.
  template <bool INV>
  PF_HD static void run(float2* v) {
    const float2 t0 = cadd(v[0], v[2]);
    const float2 t1 = csub(v[0], v[2]);
    const float2 t2 = cadd(v[1], v[3]);
    const float2 t3 = INV ? make_float2(v[3].y - v[1].y, v[1].x - v[3].x)   // +i (v1 - v3)
                          : make_float2(v[1].y - v[3].y, v[3].x - v[1].x);  // -i (v1 - v3)
    v[0] = cadd(t0, t2);
    v[2] = csub(t0, t2);
    v[1] = cadd(t1, t3);
    v[3] = csub(t1, t3);
  }
  PF_HD static void fwd(float2* v) { run<false>(v); }
};

// Radix 5 from the pairs x1 +- x4, x2 +- x3:
//   X0 = x0 + t1 + t2,  X1,4 = x0 + c1 t1 + c2 t2 -+ i (s1 d1 + s2 d2),
//   X2,3 = x0 + c2 t1 + c1 t2 -+ i (s2 d1 - s1 d2),
// with t1 = x1 + x4, t2 = x2 + x3, d1 = x1 - x4, d2 = x2 - x3,
// c1 = cos(2 pi/5), c2 = cos(4 pi/5), s1 = sin(2 pi/5), s2 = sin(4 pi/5).
template <>
struct Dft<5> {
  PF_HD static void fwd(float2* v) {
    const float c1 = PF_C20_4, c2 = -PF_C20_2, s1 = PF_C20_1, s2 = PF_C20_3;
    const float2 x0 = v[0];
    const float2 t1 = cadd(v[1], v[4]), d1 = csub(v[1], v[4]);
    const float2 t2 = cadd(v[2], v[3]), d2 = csub(v[2], v[3]);
    const float2 a1 = make_float2(fmaf(c2, t2.x, fmaf(c1, t1.x, x0.x)), fmaf(c2, t2.y, fmaf(c1, t1.y, x0.y)));
    const float2 a2 = make_float2(fmaf(c1, t2.x, fmaf(c2, t1.x, x0.x)), fmaf(c1, t2.y, fmaf(c2, t1.y, x0.y)));
    const float2 b1 = make_float2(fmaf(s2, d2.x, s1 * d1.x), fmaf(s2, d2.y, s1 * d1.y));
    const float2 b2 = make_float2(fmaf(-s1, d2.x, s2 * d1.x), fmaf(-s1, d2.y, s2 * d1.y));
    v[0] = cadd(x0, cadd(t1, t2));
    v[1] = cadd(a1, cmul_mi(b1));
    v[4] = cadd(a1, cmul_pi(b1));
    v[2] = cadd(a2, cmul_mi(b2));
    v[3] = cadd(a2, cmul_pi(b2));
  }
};

// Prime 17 as a direct DFT on the symmetric pairs t_j = x_j + x_{17-j},
// d_j = x_j - x_{17-j} (j = 1..8): with theta = 2 pi jk / 17,
//   X_k      = x0 + sum_j cos(theta) t_j - i sum_j sin(theta) d_j,
//   X_{17-k} = x0 + sum_j cos(theta) t_j + i sum_j sin(theta) d_j   (k = 1..8).
template <>
struct Dft<17> {
  PF_HD static void fwd(float2* v) {
    const float C[9] = {1.f, PF_C17_1, PF_C17_2, PF_C17_3, PF_C17_4, PF_C17_5, PF_C17_6, PF_C17_7, PF_C17_8};
    const float S[9] = {0.f, PF_S17_1, PF_S17_2, PF_S17_3, PF_S17_4, PF_S17_5, PF_S17_6, PF_S17_7, PF_S17_8};
    float2 t[9], d[9], out[17];
    const float2 x0 = v[0];
    float2 sum = x0;
#pragma unroll
    for (int j = 1; j <= 8; ++j) {
      t[j] = cadd(v[j], v[17 - j]);
      d[j] = csub(v[j], v[17 - j]);
      sum = cadd(sum, t[j]);
    }
#pragma unroll
    for (int k = 1; k <= 8; ++k) {
      float2 a = x0, b = make_float2(0.f, 0.f);
#pragma unroll
      for (int j = 1; j <= 8; ++j) {
        const int m = (j * k) % 17;
        const int mm = m <= 8 ? m : 17 - m;
        const float sn = m <= 8 ? S[mm] : -S[mm];
        a = make_float2(fmaf(C[mm], t[j].x, a.x), fmaf(C[mm], t[j].y, a.y));
        b = make_float2(fmaf(sn, d[j].x, b.x), fmaf(sn, d[j].y, b.y));
      }
      out[k] = make_float2(a.x + b.y, a.y - b.x);
      out[17 - k] = make_float2(a.x - b.y, a.y + b.x);
    }
    v[0] = sum;
#pragma unroll
    for (int k = 1; k < 17; ++k) v[k] = out[k];
  }
};

// Composite R = R1*R2 in registers: x[n1 + R1*n2] -> X[k2 + R2*k1]
template <int R1, int R2>
struct DftComposite {
  static constexpr int R = R1 * R2;
  template <bool INV>
  PF_HD static void run(float2* v) {
    float2 t[R];
#pragma unroll
    for (int n1 = 0; n1 < R1; ++n1) {
      float2 c[R2];
#pragma unroll
      for (int n2 = 0; n2 < R2; ++n2) c[n2] = v[n1 + R1 * n2];
      if constexpr (INV) dft_inv<R2>(c);
      else Dft<R2>::fwd(c);
#pragma unroll
      for (int k2 = 0; k2 < R2; ++k2) {
        float2 w = wconst<R>(n1 * k2);
        t[n1 + R1 * k2] = (n1 * k2 == 0) ? c[k2] : (INV ? cmulc(c[k2], w) : cmul(c[k2], w));
      }
    }
#pragma unroll
    for (int k2 = 0; k2 < R2; ++k2) {
      float2 r[R1];
#pragma unroll
      for (int n1 = 0; n1 < R1; ++n1) r[n1] = t[n1 + R1 * k2];
      if constexpr (INV) dft_inv<R1>(r);
      else Dft<R1>::fwd(r);
#pragma unroll
      for (int k1 = 0; k1 < R1; ++k1) v[k2 + R2 * k1] = r[k1];
    }
  }
  PF_HD static void fwd(float2* v) { run<false>(v); }
};

template <>
struct Dft<6> {
  PF_HD static void fwd(float2* v) { DftComposite<2, 3>::fwd(v); }
};
template <>
struct Dft<8> {
  template <bool INV>
  PF_HD static void run(float2* v) { DftComposite<2, 4>::template run<INV>(v); }
  PF_HD static void fwd(float2* v) { run<false>(v); }
};
template <>
struct Dft<12> {
  PF_HD static void fwd(float2* v) { DftComposite<4, 3>::fwd(v); }
};
template <>
struct Dft<16> {
  template <bool INV>
  PF_HD static void run(float2* v) { DftComposite<4, 4>::template run<INV>(v); }
  PF_HD static void fwd(float2* v) { run<false>(v); }
};
template <>
struct Dft<10> {
  PF_HD static void fwd(float2* v) { DftComposite<2, 5>::fwd(v); }
};
template <>
struct Dft<20> {
  PF_HD static void fwd(float2* v) { DftComposite<4, 5>::fwd(v); }
};

// Inverse (unnormalised, e^{+2 pi i jk/R}): sizes built from radix 4 run
// their butterflies with +i directly; the others as conj(DFT(conj(x))).
template <int R>
struct HasRun {
  static constexpr bool value = (R == 4) || (R == 8) || (R == 16);
};
template <int R>
PF_HD void dft_inv(float2* v) {
  if constexpr (HasRun<R>::value) {
    Dft<R>::template run<true>(v);
  } else {
#pragma unroll
    for (int i = 0; i < R; ++i) v[i].y = -v[i].y;
    Dft<R>::fwd(v);
#pragma unroll
    for (int i = 0; i < R; ++i) v[i].y = -v[i].y;
  }
}

// ---------------------------------------------------------------------------
// Line plans
// ---------------------------------------------------------------------------
template <int L>
struct Plan;
// (N1 = contiguous run length of pass B, N2 = stride count of pass A)
template <> struct Plan<4>   { static constexpr int N1 = 2,  N2 = 2; };
template <> struct Plan<8>   { static constexpr int N1 = 4,  N2 = 2; };
template <> struct Plan<12>  { static constexpr int N1 = 4,  N2 = 3; };
template <> struct Plan<16>  { static constexpr int N1 = 4,  N2 = 4; };
template <> struct Plan<24>  { static constexpr int N1 = 8,  N2 = 3; };
template <> struct Plan<32>  { static constexpr int N1 = 8,  N2 = 4; };
template <> struct Plan<40>  { static constexpr int N1 = 8,  N2 = 5; };
template <> struct Plan<48>  { static constexpr int N1 = 8,  N2 = 6; };
template <> struct Plan<51>  { static constexpr int N1 = 3,  N2 = 17; };
template <> struct Plan<64>  { static constexpr int N1 = 8,  N2 = 8; };
template <> struct Plan<80>  { static constexpr int N1 = 16, N2 = 5; };
template <> struct Plan<96>  { static constexpr int N1 = 8,  N2 = 12; };
template <> struct Plan<100> { static constexpr int N1 = 10, N2 = 10; };
template <> struct Plan<102> { static constexpr int N1 = 6,  N2 = 17; };
template <> struct Plan<128> { static constexpr int N1 = 16, N2 = 8; };
template <> struct Plan<160> { static constexpr int N1 = 16, N2 = 10; };
template <> struct Plan<192> { static constexpr int N1 = 16, N2 = 12; };
template <> struct Plan<200> { static constexpr int N1 = 20, N2 = 10; };
template <> struct Plan<256> { static constexpr int N1 = 16, N2 = 16; };

// Line<L>: the plan's factorization; Line<L, A, B> any other L = A * B.
template <int L, int A = Plan<L>::N1, int B = Plan<L>::N2>
struct Line {
  static constexpr int LEN = L;
  static constexpr int N1 = A;
  static constexpr int N2 = B;
  static_assert(N1 * N2 == L, "bad plan");
  // padded storage: one pad slot after every run of N1, odd line pitch
  static constexpr int RAW = N2 * (N1 + 1);
  static constexpr int PITCH = (RAW % 2 == 1) ? RAW : RAW + 1;
  PF_HD static int phys(int j) { return j + j / N1; }
  // frequency held at (natural) position p after a forward transform
  PF_HD static int freq_of_pos(int p) { return p / N1 + N2 * (p % N1); }
  PF_HD static int pos_of_freq(int k) { return k / N2 + N1 * (k % N2); }
};

// ---------------------------------------------------------------------------
// Single passes (no barrier inside), over `nb` (1 or 2) buffers of `nl` lines
// each: line l of buffer b starts at (b ? b1 : b0) + l*pitch.
// ---------------------------------------------------------------------------
template <int L>
__device__ __forceinline__ void pass_a_fwd(float2* b0, float2* b1, int nb, int nl, int pitch, const float2* __restrict__ tw) {
  constexpr int N1 = Line<L>::N1, N2 = Line<L>::N2;
  const int tot = nb * nl * N1;
  for (int it = threadIdx.x; it < tot; it += blockDim.x) {
    const int n1 = it % N1, r = it / N1, l = r % nl, b = r / nl;
    float2* p = (b ? b1 : b0) + l * pitch + n1;
    float2 v[N2];
#pragma unroll
    for (int n2 = 0; n2 < N2; ++n2) v[n2] = p[n2 * (N1 + 1)];
    Dft<N2>::fwd(v);
#pragma unroll
    for (int k2 = 1; k2 < N2; ++k2) v[k2] = cmul(v[k2], __ldg(tw + n1 * k2));
#pragma unroll
    for (int k2 = 0; k2 < N2; ++k2) p[k2 * (N1 + 1)] = v[k2];
  }
}

template <int L, bool INV>
__device__ __forceinline__ void pass_b(float2* b0, float2* b1, int nb, int nl, int pitch) {
  constexpr int N1 = Line<L>::N1, N2 = Line<L>::N2;
  const int tot = nb * nl * N2;
  for (int it = threadIdx.x; it < tot; it += blockDim.x) {
    const int k2 = it % N2, r = it / N2, l = r % nl, b = r / nl;
    float2* p = (b ? b1 : b0) + l * pitch + k2 * (N1 + 1);
    float2 u[N1];
#pragma unroll
    for (int n1 = 0; n1 < N1; ++n1) u[n1] = p[n1];
    if (INV) dft_inv<N1>(u); else Dft<N1>::fwd(u);
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) p[k1] = u[k1];
  }
}

template <int L>
__device__ __forceinline__ void pass_a_inv(float2* b0, float2* b1, int nb, int nl, int pitch, const float2* __restrict__ tw) {
  constexpr int N1 = Line<L>::N1, N2 = Line<L>::N2;
  const int tot = nb * nl * N1;
  for (int it = threadIdx.x; it < tot; it += blockDim.x) {
    const int n1 = it % N1, r = it / N1, l = r % nl, b = r / nl;
    float2* p = (b ? b1 : b0) + l * pitch + n1;
    float2 v[N2];
    v[0] = p[0];
#pragma unroll
    for (int k2 = 1; k2 < N2; ++k2) v[k2] = cmulc(p[k2 * (N1 + 1)], __ldg(tw + n1 * k2));
    dft_inv<N2>(v);
#pragma unroll
    for (int n2 = 0; n2 < N2; ++n2) p[n2 * (N1 + 1)] = v[n2];
  }
}

// Forward transform of `nlines` lines of length L stored at buf + l*pitch
// (phys() layout inside each line).  tw = W_L^j, j in [0, L), from a table.
// Must be called by all threads of the block; ends with __syncthreads().
template <int L>
__device__ __forceinline__ void fft_fwd_lines(float2* buf, int nlines, int pitch, const float2* __restrict__ tw) {
  using Ln = Line<L>;
  constexpr int N1 = Ln::N1, N2 = Ln::N2;
  for (int it = threadIdx.x; it < nlines * N1; it += blockDim.x) {
    const int l = it / N1, n1 = it - l * N1;
    float2* p = buf + l * pitch + n1;
    float2 v[N2];
#pragma unroll
    for (int n2 = 0; n2 < N2; ++n2) v[n2] = p[n2 * (N1 + 1)];
    Dft<N2>::fwd(v);
#pragma unroll
    for (int k2 = 1; k2 < N2; ++k2) v[k2] = cmul(v[k2], __ldg(tw + n1 * k2));
#pragma unroll
    for (int k2 = 0; k2 < N2; ++k2) p[k2 * (N1 + 1)] = v[k2];
  }
  __syncthreads();
  for (int it = threadIdx.x; it < nlines * N2; it += blockDim.x) {
    const int l = it / N2, k2 = it - l * N2;
    float2* p = buf + l * pitch + k2 * (N1 + 1);
    float2 u[N1];
#pragma unroll
    for (int n1 = 0; n1 < N1; ++n1) u[n1] = p[n1];
    Dft<N1>::fwd(u);
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) p[k1] = u[k1];
  }
  __syncthreads();
}

// Inverse (unnormalised) transform: digit-transposed in, natural out.
template <int L>
__device__ __forceinline__ void fft_inv_lines(float2* buf, int nlines, int pitch, const float2* __restrict__ tw) {
  using Ln = Line<L>;
  constexpr int N1 = Ln::N1, N2 = Ln::N2;
  for (int it = threadIdx.x; it < nlines * N2; it += blockDim.x) {
    const int l = it / N2, k2 = it - l * N2;
    float2* p = buf + l * pitch + k2 * (N1 + 1);
    float2 u[N1];
#pragma unroll
    for (int n1 = 0; n1 < N1; ++n1) u[n1] = p[n1];
    dft_inv<N1>(u);
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) p[k1] = u[k1];
  }
  __syncthreads();
  for (int it = threadIdx.x; it < nlines * N1; it += blockDim.x) {
    const int l = it / N1, n1 = it - l * N1;
    float2* p = buf + l * pitch + n1;
    float2 v[N2];
    v[0] = p[0];
#pragma unroll
    for (int k2 = 1; k2 < N2; ++k2) v[k2] = cmulc(p[k2 * (N1 + 1)], __ldg(tw + n1 * k2));
    dft_inv<N2>(v);
#pragma unroll
    for (int n2 = 0; n2 < N2; ++n2) p[n2 * (N1 + 1)] = v[n2];
  }
  __syncthreads();
}

}  // namespace pf
