// Fused FP32 kernels of the semi-implicit spectral step (sm_103a).
//
// State of one run, for every field f (the var order parameters, then the
// concentration c):
//   Sk[f][kx][ypos][zpos]  u_hat in k-space (normalised like f_trans,
//                          src/f_trans.f90:12), y/z in digit-transposed order;
//   Sm[f][kx][z][y]        the same field in "mixed" space: its x half
//                          spectrum (1/Nx) sum_x u e^{-2 pi i kx x/Nx} with y, z
//                          in real space (what the x pass needs).
// The reference keeps phi/con in real space and takes a full 3-D R2C per
// field and use (src/f_trans.f90:11-12, 7*var+9 transforms per step); here one
// step is two passes over the fields:
//
//   x pass  (x_pass_kernel, one CTA per WY y-rows at one z, all fields):
//       Sm --C2R_x--> phi, c --bulk terms (src/var_diff.f90:685-898)-->
//       dF/dphi_i, dF/dc (, mobility) --R2C_x/Nx--> D
//   yz pass (yz_kernel, one CTA cluster per (field, kx) plane):
//       D --DFT_yz--> D_hat;  u_hat += m1 u_hat + m2 D_hat  (pointwise);
//       u_hat --IDFT_yz--> Sm
//
// In exact arithmetic the pointwise update is the reference's
//   u_hat_new = (u_hat - L dt D_hat) / (1 - L kappa dt K2)                (AC, :1020-1024)
//   c_hat_new = (c_hat + D_mean K2 dt mu_hat) / (1 + D_mean dt kappa_c K4)  (CH, :976-983)
// written as an increment so that the state never takes an FP32 round trip
// through an FFT.  The variable-mobility term dt G J'_hat / (...) of :976-983 is
// added by a second x/yz pass pair (xj pass + yz_kernel in C2 mode).
#pragma once
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "pf_fft.cuh"

namespace cg = cooperative_groups;

namespace pf {

// Per-block diagnostic partials of the x pass (floats; the sums as
// compensated hi + lo pairs): part_x[(par * XQ_COUNT + q) * nblk_x + block],
// par = Shape::par, the step's parity: the record of one step reads its
// partials while the next step's x pass writes the other set.
enum XDiag {
  XQ_FETA_H = 0, XQ_FETA_L, XQ_FCH_H, XQ_FCH_L, XQ_MASS_H, XQ_MASS_L,
  XQ_CMIN, XQ_CMAX, XQ_PHIMIN, XQ_PHIPMAX, XQ_BAD, XQ_COUNT
};
// room reserved per (z, y) row for the x partials of both parities (doubles'
// worth, any variant)
constexpr int XD_COUNT = 12;
static_assert(2 * XQ_COUNT * 4 <= XD_COUNT * 8, "x partials must fit the reserved room");
// Per-step diagnostic record layout (doubles)
enum DiagRec {
  DR_STEP = 0, DR_FINT, DR_FETA, DR_FCH, DR_CMIN, DR_CMAX, DR_PHIMIN, DR_PHIPMAX, DR_MASS, DR_NONFINITE, DR_COUNT
};

enum Mobility { MOB_CONST = 0, MOB_REF_VAR = 1, MOB_C1MC = 2 };

// Device-side description of one run (all runs of a launch share one shape)
struct RunParams {
  float2* Sk;      // [nF][Kx] planes of the k-space state (digit-transposed y, z positions; the
                   // order inside a plane belongs to the yz-pass variant that runs the batch)
  float2* Sm;      // [nF][Kx][Nz][Ny] state in mixed space (x spectrum, real-space y, z)
  float2* D;       // [nF][Kx][Nz][Ny] x-spectra of dF/dphi_i and dF/dc
  float* mob;      // [Nz][Ny][Nx] mobility minus D_mean (variable mobility only)
  float2* J;       // [Kx][Nz][Ny] CH flux scratch (variable mobility only)
  float* part_x;   // [2][XQ_COUNT][nblk_x]: per step parity
  float* part_yz;  // [2][2][nblk_yz]: per step parity, hi and lo of each yz CTA's weighted f_int sum
  double* diag;    // [ring][DR_COUNT]
  int* counter;    // step counter (device)
  unsigned* err;     // bit 0: a TMA tile of the x pass never arrived (the step's record is flagged)
  const void* tmap_sm;  // TMA tensor map over Sm [nF][Kx][Nz][Ny] (x pass TMA variant), global memory
  float* fin;      // [nF][Nz][Ny][Nx] real fields for import/export
  float L, kappa_phi, kappa_c, dt, D_L, D_gb, sigma1, sigma2, am, ap, c0m, c0p;
  int mobility;
  int V;           // number of order parameters
  int ring;        // diag ring length
  int pad;
};

// Per-shape tables (FP64-derived, stored as float)
struct Shape {
  int Nx, Ny, Nz, Kx;
  const float2* twM;  // W_{Nx/2}^j, j < Nx/2
  const float2* twN;  // W_{Nx}^j,   j < Nx
  const float2* twY;  // W_{Ny}^j
  const float2* twZ;  // W_{Nz}^j
  const float* qx2; const float* qy2; const float* qz2;  // q_d^2 (kf_sq)
  const float* qx4; const float* qy4; const float* qz4;  // q_d^4 (kf_4)
  const float* qnx; const float* qny; const float* qnz;  // Nyquist-zeroed q_d (kf / i)
  int nblk_x;   // blocks of the x pass per run
  int nblk_yz;  // blocks of the yz pass per run
  int plane0;   // first (field, kx) plane of a yz-pass launch (a launch may cover a subset)
  // L2 prefetch distance in CTAs of the yz variants that prefetch: the CTAs
  // resident at once, so that CTA b fetches into L2 what CTA b + pref (which
  // starts about when b ends) will read; 0: none
  int pref_yz;
  int par;  // parity of the step: which set of diagnostic partials its passes write and its record reads
};

// ---------------------------------------------------------------------------
// Compensated sums for the mass of c (src/var_diff.f90:1076-1102).  A thread
// keeps its running sum as an unevaluated FP32 pair hi + lo updated with
// Knuth's error-free TwoSum (s + e == a + b exactly), warps combine the pairs
// the same way, and from there on the sum is FP64 with Neumaier's
// compensation (KSum) across warps, blocks and the final record.  FP64
// arithmetic is scarce on this part, so only the per-warp and later stages
// use it.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
struct FF {
  float hi, lo;
  __device__ __forceinline__ void add(float v) {
    float s, e;
    two_sum(hi, v, s, e);
    hi = s;
    lo = __fadd_rn(lo, e);
  }
  __device__ __forceinline__ void add(const FF& o) {
    float s, e;
    two_sum(hi, o.hi, s, e);
    hi = s;
    lo = __fadd_rn(__fadd_rn(lo, o.lo), e);
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};
__device__ __forceinline__ FF ff(float hi, float lo = 0.f) {
  FF x;
  x.hi = hi;
  x.lo = lo;
  return x;
}
// sum of the pairs of a warp (every lane gets a sum of all 32)
__device__ __forceinline__ FF warp_sum_ff(FF x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x.add(ff(__shfl_xor_sync(0xffffffffu, x.hi, o), __shfl_xor_sync(0xffffffffu, x.lo, o)));
  return x;
}
// compensated FP64 sum (Kahan-Babuska-Neumaier, the error of each addition
// taken exactly by TwoSum): value() = s + c
struct KSum {
  double s = 0.0, c = 0.0;
  __device__ __forceinline__ void add(double v) {
    const double t = __dadd_rn(s, v);
    const double bb = __dsub_rn(t, s);
    c = __dadd_rn(c, __dadd_rn(__dsub_rn(s, __dsub_rn(t, bb)), __dsub_rn(v, bb)));
    s = t;
  }
  __device__ __forceinline__ void add(const KSum& o) {
    add(o.s);
    c = __dadd_rn(c, o.c);
  }
  __device__ __forceinline__ double value() const { return __dadd_rn(s, c); }
};

__device__ __forceinline__ float warp_min(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// ---------------------------------------------------------------------------
// x-direction half spectrum <-> interleaved real line (M = Nx/2 complex).
// With z[m] = x[2m] + i x[2m+1] and Z = DFT_M(z):
//   X[k] = (Z[k] + conj Z[M-k])/2 - (i/2) W_N^k (Z[k] - conj Z[M-k]),
//   X[0] = Re Z0 + Im Z0,  X[M] = Re Z0 - Im Z0;
// the inverse builds Z'[k] = (X[k] + conj X[M-k]) + i conj(W_N^k) (X[k] - conj X[M-k])
// so that IDFT_M(Z') = N z.  Frequencies k and M-k always sit in mirrored
// runs of the four-step layout, so one thread owns both halves of every pair.
// ---------------------------------------------------------------------------
// inverse pre-processing of the pair (k, M-k), 0 < k < M.  With
// s = x_k + conj(x_m), d = x_k - conj(x_m):
//   z_k = s + i d conj(w_k),   z_m = conj(s) + i (-conj(d)) conj(w_m);
// the rotated products are formed directly in their final component order so
// that the sums are packed FP32-pair instructions.
__device__ __forceinline__ void pre_pair(float2 xk, float2 xm, float2 wk, float2 wm, float2& zk, float2& zm) {
  const float2 s = __ffma2_rn(xm, make_float2(1.f, -1.f), xk);
  const float2 d = __ffma2_rn(xm, make_float2(-1.f, 1.f), xk);
  const float2 ie = make_float2(fmaf(d.x, wk.y, -d.y * wk.x), fmaf(d.x, wk.x, d.y * wk.y));     // i d conj(wk)
  const float2 ie2 = make_float2(fmaf(-d.y, wm.x, -d.x * wm.y), fmaf(-d.x, wm.x, d.y * wm.y));  // i (-conj d) conj(wm)
  zk = __fadd2_rn(s, ie);
  zm = __ffma2_rn(s, make_float2(1.f, -1.f), ie2);
}
// forward post-processing of the pair (k, M-k), 0 < k < M, scaled by h = scale/2:
//   x_k = h (s - i d w_k),   x_m = h (conj(s) - i (-conj(d)) w_m),
// s = z_k + conj(z_m), d = z_k - conj(z_m).
__device__ __forceinline__ void post_pair(float2 zk, float2 zm, float2 wk, float2 wm, float h, float2& xk, float2& xm) {
  const float2 hh = make_float2(h, h);
  const float2 s = __ffma2_rn(zm, make_float2(1.f, -1.f), zk);
  const float2 d = __ffma2_rn(zm, make_float2(-1.f, 1.f), zk);
  const float2 mie = make_float2(fmaf(d.x, wk.y, d.y * wk.x), fmaf(-d.x, wk.x, d.y * wk.y));    // -i d wk
  const float2 mie2 = make_float2(fmaf(-d.x, wm.y, d.y * wm.x), fmaf(d.x, wm.x, d.y * wm.y));   // -i (-conj d) wm
  xk = __fmul2_rn(__fadd2_rn(s, mie), hh);
  xm = __fmul2_rn(__ffma2_rn(s, make_float2(1.f, -1.f), mie2), hh);
}

// Factorization of the x pass's lines (M = Nx/2 complex points): the plan's,
// except M = 128 as 8 x 16.  With runs of 8 the largest per-thread state of
// the x pass is one DFT_16 instead of a pair of them: 80 registers a thread
// at Nx = 256 instead of 128 with spills (the same speed at 33 fields).
template <int M>
struct XPlan {
  static constexpr int N1 = Plan<M>::N1, N2 = Plan<M>::N2;
};
template <>
struct XPlan<128> {
  static constexpr int N1 = 8, N2 = 16;
};
template <int M>
using XLine = Line<M, XPlan<M>::N1, XPlan<M>::N2>;

// A twiddle of the x pass: from a copy of the table in shared memory (TWS),
// else from the global table through the read-only path.
template <bool TWS>
__device__ __forceinline__ float2 ldtw(const float2* p) {
  if constexpr (TWS) return *p;
  else return __ldg(p);
}

// pass A over a runtime number of lines (pitch P, T threads).  A warp takes 32
// consecutive lines at one column n1: with an odd pitch those 32 accesses hit
// distinct bank pairs.
template <int L, int P, int T, bool INV, bool TWS = false>
__device__ __forceinline__ void passA_rt(float2* buf, int NL, const float2* __restrict__ tw) {
  constexpr int N1 = XLine<L>::N1, N2 = XLine<L>::N2;
  const int nlb = (NL + 31) >> 5;  // groups of 32 lines
  const int items = nlb * 32 * N1;
  for (int it = threadIdx.x; it < items; it += T) {
    const int lo = it & 31, rest = it >> 5;
    const int n1 = rest % N1, l = (rest / N1) * 32 + lo;
    if (l >= NL) continue;
    float2* p = buf + l * P + n1;
    float2 v[N2];
    if (!INV) {
#pragma unroll
      for (int n2 = 0; n2 < N2; ++n2) v[n2] = p[n2 * (N1 + 1)];
      Dft<N2>::fwd(v);
#pragma unroll
      for (int k2 = 1; k2 < N2; ++k2) v[k2] = cmul(v[k2], ldtw<TWS>(tw + n1 * k2));
    } else {
      v[0] = p[0];
#pragma unroll
      for (int k2 = 1; k2 < N2; ++k2) v[k2] = cmulc(p[k2 * (N1 + 1)], ldtw<TWS>(tw + n1 * k2));
      dft_inv<N2>(v);
    }
#pragma unroll
    for (int k = 0; k < N2; ++k) p[k * (N1 + 1)] = v[k];
  }
}

// Where element kx of a line's half spectrum is read from:
//   SPEC_GLOBAL  src + kx * stride in read-only global memory;
//   SPEC_SMEM    src + kx * stride in shared memory (a staging buffer);
//   SPEC_INPLACE the line itself, kx at run kx % N2, element kx / N2 of the
//                run (x_spec_slot), and kx = M in the pad slot after run 0.
// In place, the inputs of a run pair are exactly the slots its outputs go
// to, so every item reads its inputs into registers and overwrites them.
enum SpecSrc { SPEC_GLOBAL = 0, SPEC_SMEM = 1, SPEC_INPLACE = 2 };

template <int M>
__device__ __forceinline__ int x_spec_slot(int kx) {
  constexpr int N1 = XLine<M>::N1, N2 = XLine<M>::N2;
  return kx == M ? N1 : (N1 + 1) * (kx % N2) + kx / N2;
}

template <int SRC, int M>
__device__ __forceinline__ float2 ld_spec(const float2* src, size_t stride, int kx) {
  if constexpr (SRC == SPEC_INPLACE) return src[x_spec_slot<M>(kx)];
  else if constexpr (SRC == SPEC_SMEM) return src[(size_t)kx * stride];
  else return __ldg(src + (size_t)kx * stride);
}

// Run pair of item group q of a line (x_inv_runs / x_fwd_runs), q < N2/2 + 1:
// the pairs (pr, N2 - pr), 0 < pr < N2/2, first, then the single runs 0 and
// (N2 even) N2/2.  A pair item costs two DFT_N1, a single one, so with the
// pairs handed out first the last round of items holds only single runs
// (132 lines at N2 = 8 and 512 threads: 3 rounds of DFT_N1 instead of 4).
template <int M>
__device__ __forceinline__ int x_run_pair(int q) {
  constexpr int N2 = XLine<M>::N2, NPR = (N2 - 1) / 2;
  return q < NPR ? q + 1 : (q == NPR ? 0 : N2 / 2);
}

// Inverse x transform, first half: read the half spectrum of line (f, yy)
// for the run pair `pr` (from where SRC says), pre-process, inverse DFT_N1 of
// each run, store the runs (pass B' output) into the padded line.
template <int M, int SRC = SPEC_GLOBAL, bool TWS = false>
__device__ __forceinline__ void x_inv_runs(const float2* src, size_t plane, float2* line, int pr,
                                           const float2* __restrict__ twN) {  // src may be line (in place)
  constexpr int N1 = XLine<M>::N1, N2 = XLine<M>::N2;
  if (pr > 0 && 2 * pr < N2) {
    const int ra = pr, rb = N2 - pr;
    float2 a[N1], b[N1];
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) {
      a[k1] = ld_spec<SRC, M>(src, plane, ra + N2 * k1);
      b[k1] = ld_spec<SRC, M>(src, plane, rb + N2 * k1);
    }
    float2 za[N1], zb[N1];
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) {
      const int k = ra + N2 * k1;
      pre_pair(a[k1], b[N1 - 1 - k1], ldtw<TWS>(twN + k), ldtw<TWS>(twN + M - k), za[k1], zb[N1 - 1 - k1]);
    }
    dft_inv<N1>(za);
    dft_inv<N1>(zb);
#pragma unroll
    for (int n1 = 0; n1 < N1; ++n1) {
      line[n1 + (N1 + 1) * ra] = za[n1];
      line[n1 + (N1 + 1) * rb] = zb[n1];
    }
  } else if (pr == 0) {
    float2 a[N1];
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) a[k1] = ld_spec<SRC, M>(src, plane, N2 * k1);
    const float2 xM = ld_spec<SRC, M>(src, plane, M);
    float2 z[N1];
    z[0] = make_float2(a[0].x + xM.x, a[0].x - xM.x);
#pragma unroll
    for (int k1 = 1; k1 <= N1 / 2; ++k1) {
      const int k = N2 * k1;
      float2 zk, zm;
      pre_pair(a[k1], a[N1 - k1], ldtw<TWS>(twN + k), ldtw<TWS>(twN + M - k), zk, zm);
      z[k1] = zk;
      if (k1 != N1 - k1) z[N1 - k1] = zm;
    }
    dft_inv<N1>(z);
#pragma unroll
    for (int n1 = 0; n1 < N1; ++n1) line[n1] = z[n1];
  } else {  // pr == N2/2: the run pairs with itself, element k1 with N1-1-k1
    const int ra = N2 / 2;
    float2 a[N1];
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) a[k1] = ld_spec<SRC, M>(src, plane, ra + N2 * k1);
    float2 z[N1];
#pragma unroll
    for (int k1 = 0; k1 < N1 / 2; ++k1) {
      const int k = ra + N2 * k1;
      pre_pair(a[k1], a[N1 - 1 - k1], ldtw<TWS>(twN + k), ldtw<TWS>(twN + M - k), z[k1], z[N1 - 1 - k1]);
    }
    dft_inv<N1>(z);
#pragma unroll
    for (int n1 = 0; n1 < N1; ++n1) line[n1 + (N1 + 1) * ra] = z[n1];
  }
}

// Forward x transform, last half: forward DFT_N1 of the run pair `pr` (pass
// B), post-process, store the half spectrum (scaled) to global.
template <int M, bool TWS = false>
__device__ __forceinline__ void x_fwd_runs(float2* __restrict__ dst, size_t plane, const float2* line, int pr,
                                           float scale, const float2* __restrict__ twN) {
  constexpr int N1 = XLine<M>::N1, N2 = XLine<M>::N2;
  const float h = 0.5f * scale;
  if (pr > 0 && 2 * pr < N2) {
    const int ra = pr, rb = N2 - pr;
    float2 za[N1], zb[N1];
#pragma unroll
    for (int n1 = 0; n1 < N1; ++n1) {
      za[n1] = line[n1 + (N1 + 1) * ra];
      zb[n1] = line[n1 + (N1 + 1) * rb];
    }
    Dft<N1>::fwd(za);
    Dft<N1>::fwd(zb);
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) {
      const int k = ra + N2 * k1;
      float2 xk, xm;
      post_pair(za[k1], zb[N1 - 1 - k1], ldtw<TWS>(twN + k), ldtw<TWS>(twN + M - k), h, xk, xm);
      dst[(size_t)k * plane] = xk;
      dst[(size_t)(M - k) * plane] = xm;
    }
  } else if (pr == 0) {
    float2 z[N1];
#pragma unroll
    for (int n1 = 0; n1 < N1; ++n1) z[n1] = line[n1];
    Dft<N1>::fwd(z);
    dst[0] = make_float2((z[0].x + z[0].y) * scale, 0.f);
    dst[(size_t)M * plane] = make_float2((z[0].x - z[0].y) * scale, 0.f);
#pragma unroll
    for (int k1 = 1; k1 <= N1 / 2; ++k1) {
      const int k = N2 * k1;
      float2 xk, xm;
      post_pair(z[k1], z[N1 - k1], ldtw<TWS>(twN + k), ldtw<TWS>(twN + M - k), h, xk, xm);
      dst[(size_t)k * plane] = xk;
      if (k1 != N1 - k1) dst[(size_t)(M - k) * plane] = xm;
    }
  } else {
    const int ra = N2 / 2;
    float2 z[N1];
#pragma unroll
    for (int n1 = 0; n1 < N1; ++n1) z[n1] = line[n1 + (N1 + 1) * ra];
    Dft<N1>::fwd(z);
#pragma unroll
    for (int k1 = 0; k1 < N1 / 2; ++k1) {
      const int k = ra + N2 * k1;
      float2 xk, xm;
      post_pair(z[k1], z[N1 - 1 - k1], ldtw<TWS>(twN + k), ldtw<TWS>(twN + M - k), h, xk, xm);
      dst[(size_t)k * plane] = xk;
      dst[(size_t)(M - k) * plane] = xm;
    }
  }
}

// ---------------------------------------------------------------------------
// Bulk terms (src/var_diff.f90:685-898) on the interleaved real lines of all
// fields.
// ---------------------------------------------------------------------------
struct BulkAcc {
  float feta, fch;  // per-thread partial sums over a few cells (FP64 from the warp level up)
  FF mass;          // compensated (exact) per-thread sum of c
  float cmin, cmax, phimin, phipmax;
  int nonfinite;
  __device__ __forceinline__ void init() {
    feta = 0.f; fch = 0.f; mass.hi = 0.f; mass.lo = 0.f;
    cmin = 1.0f; cmax = 0.0f; phimin = 1.0f; phipmax = 0.0f;  // reference start values (:1076-1079)
    nonfinite = 0;
  }
};

// Bulk terms of the two cells x = 2m, 2m+1 held in one float2 slot of every
// field line.  Pass 1 forms the per-cell aggregates, pass 2 overwrites each
// phi slot with dF/dphi_i; dF/dc and the mobility are returned.
template <int PM, int WY>
__device__ __forceinline__ void bulk_slot(float2* smem, int yy, int slot, const RunParams& rp, float2& dfdc,
                                          float2& mob, BulkAcc& acc) {
  const int V = rp.V;
  const float sg1 = rp.sigma1, sg2 = rp.sigma2;
  float2* base = smem + yy * PM + slot;
  constexpr int FS = WY * PM;  // stride between fields
  // pass 1: S2 = sum phi^2, Smat = sum_{i<V-1} phi^2, S4, N4, f_eta pair
  // sum, both cells of the slot at once in packed FP32 pairs
  float2 pre = make_float2(0.f, 0.f), n4v = make_float2(0.f, 0.f), prs = make_float2(0.f, 0.f);
#pragma unroll 4
  for (int f = 0; f < V - 1; ++f) {
    const float2 p = base[f * FS];
    const float2 a = __fmul2_rn(p, p);
    prs = __ffma2_rn(a, pre, prs);
    pre = __fadd2_rn(pre, a);
    n4v = __ffma2_rn(a, a, n4v);
  }
  const float pre0 = pre.x, pre1 = pre.y, n40 = n4v.x, n41 = n4v.y, pr0 = prs.x, pr1 = prs.y;
  const float2 pP = base[(V - 1) * FS];
  const float2 cc = base[V * FS];
  float2 out_df[2];
  float t4a[2], t4p[2], invm[2], rP4[2];
  float Smat[2], gP[2];
  // per-cell scalar work (two cells)
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const float pp = q ? pP.y : pP.x;
    const float c = q ? cc.y : cc.x;
    const float pre = q ? pre1 : pre0;
    const float n4 = q ? n41 : n40;
    const float pairs = q ? pr1 : pr0;
    const float pp2 = pp * pp;
    const float S2 = pre + pp2;
    const float S4 = n4 + pp2 * pp2;
    // h = N4/S4 and the term4 ratios (phi^3/S4)(phiP^4/S4).  Below S4 = 1e-30
    // (|phi| < ~1e-8) FP32 would lose them: rescale phi by 1/max|phi|.  All-zero
    // cells give 0/0 in the reference; here h = 0 and term4 = 0.
    float invS4, n4n, sc, im = 1.f;
    float mabs = 0.f;
    if (S4 < 1e-30f) {  // rare: max |phi| of the cell for the rescaled branch
      mabs = fabsf(pp);
      for (int f = 0; f < V - 1; ++f) {
        const float2 p = base[f * FS];
        mabs = fmaxf(mabs, fabsf(q ? p.y : p.x));
      }
    }
    if (S4 >= 1e-30f) {
      invS4 = 1.f / S4;
      n4n = n4 * invS4;
      sc = 4.f;
    } else if (mabs > 0.f) {
      im = 1.f / mabs;
      float s4 = 0.f, nn = 0.f;
      for (int f = 0; f < V - 1; ++f) {
        const float2 p = base[f * FS];
        const float x = (q ? p.y : p.x) * im;
        nn = fmaf(x * x, x * x, nn);
      }
      const float xq = pp * im;
      s4 = nn + (xq * xq) * (xq * xq);
      invS4 = 1.f / s4;
      n4n = nn * invS4;
      sc = 4.f * im;
    } else {
      invS4 = 0.f;
      n4n = 0.f;
      sc = 0.f;
    }
    const float h = n4n;  // phi_mat (:741)
    const float dcm = c - rp.c0m, dcp = c - rp.c0p;
    const float fm = rp.am * dcm * dcm, fp = rp.ap * dcp * dcp;
    const float dfm = fm - fp;
    acc.fch += h * fm + (1.f - h) * fp;
    const float dc = 2.f * h * rp.am * dcm + 2.f * (1.f - h) * rp.ap * dcp;
    acc.feta += -0.5f * S2 + 0.25f * S4 + sg1 * pairs + sg2 * pp2 * pre;
    acc.mass.add(c);
    acc.cmin = fminf(acc.cmin, c);
    acc.cmax = fmaxf(acc.cmax, c);
    acc.phimin = fminf(acc.phimin, S2);
    acc.phipmax = fmaxf(acc.phipmax, pp);
    float mb;
    if (rp.mobility == MOB_REF_VAR) mb = 2.f * (1.f - S2) * rp.D_gb;
    else if (rp.mobility == MOB_C1MC) mb = rp.D_L * c * (1.f - c);
    else mb = 0.f;
    const float qP = pp * im;
    const float qP2 = qP * qP;
    rP4[q] = qP2 * qP2 * invS4;           // phiP^4 / S4
    t4a[q] = sc * invS4 * rP4[q] * dfm;   // term4_i = t4a * q_i^3         (i < V-1)
    t4p[q] = -sc * (qP * qP2 * invS4) * n4n * dfm;  // term4_P                 (:829-835)
    invm[q] = im;
    Smat[q] = pre;
    gP[q] = sg2 * pp2;
    out_df[q] = make_float2(dc, mb);
  }
  dfdc = make_float2(out_df[0].x, out_df[1].x);
  mob = make_float2(out_df[0].y, out_df[1].y);
  // pass 2: dF/dphi_i = phi^3 - phi + 2 phi Gamma_i + term4_i   (:782-857)
  // with Gamma_i = sigma1 (Smat - phi_i^2) + sigma2 phiP^2 and term4_i =
  // t4a q_i^3, q_i = phi_i / max|phi| (the rescaled branch) or phi_i.
  float dsum = dfdc.x + dfdc.y;
  if (invm[0] == 1.f && invm[1] == 1.f) {
    // packed over the slot's two cells:
    //   dF = phi (2 sigma1 (Smat - phi^2) + phi^2 (1 + t4a) + 2 gP - 1)
    const float2 two_s1 = make_float2(2.f * sg1, 2.f * sg1), m1 = make_float2(-1.f, -1.f);
    const float2 opt4 = make_float2(1.f + t4a[0], 1.f + t4a[1]);
    const float2 cterm = make_float2(fmaf(2.f, gP[0], -1.f), fmaf(2.f, gP[1], -1.f));
    const float2 sm = make_float2(Smat[0], Smat[1]);
    float2 ds = make_float2(0.f, 0.f);
#pragma unroll 4
    for (int f = 0; f < V - 1; ++f) {
      const float2 p = base[f * FS];
      const float2 p2 = __fmul2_rn(p, p);
      const float2 sd = __ffma2_rn(p2, m1, sm);                              // Smat - phi^2
      const float2 h = __ffma2_rn(sd, two_s1, __ffma2_rn(p2, opt4, cterm));
      const float2 d = __fmul2_rn(p, h);
      ds = __fadd2_rn(ds, d);
      base[f * FS] = d;
    }
    dsum += ds.x + ds.y;
  } else {
    for (int f = 0; f < V - 1; ++f) {
      float2 p = base[f * FS];
      const float g0 = fmaf(sg1, Smat[0] - p.x * p.x, gP[0]);
      const float g1 = fmaf(sg1, Smat[1] - p.y * p.y, gP[1]);
      const float q0 = p.x * invm[0], q1 = p.y * invm[1];
      const float d0 = fmaf(p.x, p.x * p.x, -p.x) + 2.f * p.x * g0 + t4a[0] * (q0 * q0 * q0);
      const float d1 = fmaf(p.y, p.y * p.y, -p.y) + 2.f * p.y * g1 + t4a[1] * (q1 * q1 * q1);
      dsum += d0 + d1;
      base[f * FS] = make_float2(d0, d1);
    }
  }
  {
    const float g0 = sg2 * Smat[0], g1 = sg2 * Smat[1];
    const float d0 = fmaf(pP.x, pP.x * pP.x, -pP.x) + 2.f * pP.x * g0 + t4p[0];
    const float d1 = fmaf(pP.y, pP.y * pP.y, -pP.y) + 2.f * pP.y * g1 + t4p[1];
    dsum += d0 + d1;
    base[(V - 1) * FS] = make_float2(d0, d1);
  }
  acc.nonfinite += !isfinite(dsum);  // any NaN/Inf term makes the sum non-finite
}

// Block reduction of the x pass's diagnostics into the block's partials
// part_x[(par * XQ_COUNT + q) * nblk_x + blk] (all threads of the block call it).  Sums travel as
// compensated FP32 pairs: FP64 arithmetic is scarce on this part, and a
// serial FP64 chain at the end of every block held its shared memory (and
// the next block) back.
template <int T>
__device__ __forceinline__ void store_block_diag(const BulkAcc& acc, const RunParams& rp, const Shape& sh, int blk) {
  static_assert(T % 32 == 0 && T <= 1024, "whole warps");
  constexpr int NW = T / 32;
  __shared__ float red_s[6][NW];  // hi, lo of f_eta, f_ch, mass per warp
  __shared__ float red_m[4][NW];
  __shared__ int red_i[NW];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const FF s0 = warp_sum_ff(ff(acc.feta)), s1 = warp_sum_ff(ff(acc.fch)), s2 = warp_sum_ff(acc.mass);
  const float m0 = warp_min(acc.cmin), m1 = warp_max(acc.cmax), m2 = warp_min(acc.phimin), m3 = warp_max(acc.phipmax);
  const int nb = __reduce_add_sync(0xffffffffu, acc.nonfinite);
  if (lane == 0) {
    red_s[0][wid] = s0.hi; red_s[1][wid] = s0.lo; red_s[2][wid] = s1.hi; red_s[3][wid] = s1.lo;
    red_s[4][wid] = s2.hi; red_s[5][wid] = s2.lo;
    red_m[0][wid] = m0; red_m[1][wid] = m1; red_m[2][wid] = m2; red_m[3][wid] = m3;
    red_i[wid] = nb;
  }
  __syncthreads();
  if (wid == 0) {  // the warps' values, one per lane (the reference's start values as identities)
    const bool in = lane < NW;
    const FF a0 = warp_sum_ff(in ? ff(red_s[0][lane], red_s[1][lane]) : ff(0.f));
    const FF a1 = warp_sum_ff(in ? ff(red_s[2][lane], red_s[3][lane]) : ff(0.f));
    const FF a2 = warp_sum_ff(in ? ff(red_s[4][lane], red_s[5][lane]) : ff(0.f));
    const float b0 = warp_min(in ? red_m[0][lane] : 1.f), b1 = warp_max(in ? red_m[1][lane] : 0.f);
    const float b2 = warp_min(in ? red_m[2][lane] : 1.f), b3 = warp_max(in ? red_m[3][lane] : 0.f);
    const int nn = __reduce_add_sync(0xffffffffu, in ? red_i[lane] : 0);
    if (lane == 0) {
      const int nbk = sh.nblk_x;
      float* p = rp.part_x + (size_t)sh.par * XQ_COUNT * nbk + blk;
      p[XQ_FETA_H * nbk] = a0.hi; p[XQ_FETA_L * nbk] = a0.lo;
      p[XQ_FCH_H * nbk] = a1.hi;  p[XQ_FCH_L * nbk] = a1.lo;
      p[XQ_MASS_H * nbk] = a2.hi; p[XQ_MASS_L * nbk] = a2.lo;
      p[XQ_CMIN * nbk] = b0;
      p[XQ_CMAX * nbk] = b1;
      p[XQ_PHIMIN * nbk] = b2;
      p[XQ_PHIPMAX * nbk] = b3;
      p[XQ_BAD * nbk] = (float)nn;
    }
  }
}

// Bulk terms of one tile (WY rows of every field in shared memory), one
// float2 slot (two cells) per item.  Consecutive lanes take consecutive
// physical slots of the padded lines and the pad slots stay idle, so that the
// 16 slots of a half warp always fall in distinct bank pairs (a walk over the
// logical cells would span 17 slots and put its first and last in one pair).
template <int NX, int WY, int T, bool PHYS = true>
__device__ __forceinline__ void bulk_tile(float2* smem, const RunParams& rp, const Shape& sh, int z, int y0,
                                          BulkAcc& acc) {
  constexpr int M = NX / 2;
  using LM = XLine<M>;
  constexpr int PM = LM::PITCH, N1 = LM::N1;
  if constexpr (!PHYS) {  // walk over the logical cells (a half warp spans N1 + 1 slots per N1 cells)
    for (int it = threadIdx.x; it < WY * M; it += T) {
      const int m = it % M, yy = it / M;
      const int slot = LM::phys(m);
      float2 dfdc, mob;
      bulk_slot<PM, WY>(smem, yy, slot, rp, dfdc, mob, acc);
      smem[(rp.V * WY + yy) * PM + slot] = dfdc;
      if (rp.mobility != MOB_CONST)
        *reinterpret_cast<float2*>(rp.mob + ((size_t)z * sh.Ny + y0 + yy) * NX + 2 * m) = mob;
    }
  } else {
    for (int it = threadIdx.x; it < WY * PM; it += T) {
      const int yy = it / PM, ps = it - yy * PM;
      const int q = ps / (N1 + 1), r = ps - q * (N1 + 1);
      if (r == N1 || ps >= LM::RAW) continue;  // pad slot
      const int m = q * N1 + r;
      float2 dfdc, mob;
      bulk_slot<PM, WY>(smem, yy, ps, rp, dfdc, mob, acc);
      smem[(rp.V * WY + yy) * PM + ps] = dfdc;
      if (rp.mobility != MOB_CONST)
        *reinterpret_cast<float2*>(rp.mob + ((size_t)z * sh.Ny + y0 + yy) * NX + 2 * m) = mob;
    }
  }
}

// ---------------------------------------------------------------------------
// TMA (cp.async.bulk.tensor) and mbarrier helpers.  Tensor maps live in
// global memory (one per run, written by the host before the launch); every
// copy is a plain tile load from this GPU's own memory (no multicast).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"((uint32_t)__cvta_generic_to_shared(bar)), "r"(count)
               : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
                   (uint32_t)__cvta_generic_to_shared(bar)),
               "r"(bytes)
               : "memory");
}
// Wait for the phase of the given parity to complete, for at most about one
// second of the global timer: false if it never completed.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(bar);
  uint64_t t0;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  for (;;) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    uint64_t t1;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
    if (t1 - t0 > 1000000000ull) return false;
  }
}
// 4-D tile load of the box at coordinates (c0 innermost .. c3) into dst,
// completing on bar.  c0 * element size must be a multiple of 16 bytes.
__device__ __forceinline__ void tma_load_4d(void* dst, const void* tmap, int c0, int c1, int c2, int c3,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
      "l"(tmap), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"((uint32_t)__cvta_generic_to_shared(bar))
      : "memory");
}

// ---------------------------------------------------------------------------
// x pass.  MODE_BULK: S -> D (+ mob, diagnostics).  MODE_XJ: J~ -> J~' with the
// variable-mobility multiply (:947-965).  MODE_IMPORT: real fields -> S.
// MODE_EXPORT: S -> real fields.
// ---------------------------------------------------------------------------
enum XMode { MODE_BULK = 0, MODE_XJ = 1, MODE_IMPORT = 2, MODE_EXPORT = 3 };

__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;" ::: "memory");
}
// Prefetch [p, p + bytes) into L2 (cp.async.bulk.prefetch): no registers, no
// completion to wait for.  p 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void prefetch_l2(const void* p, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}
// Prefetch [p, p + bytes) into L2 in chunks of at most 4 KB, one per lane of
// the calling warp.
__device__ __forceinline__ void prefetch_l2_warp(const void* p, size_t bytes, int lane) {
  constexpr size_t CH = 4096;
  for (size_t o = (size_t)lane * CH; o < bytes; o += 32 * CH)
    prefetch_l2(static_cast<const char*>(p) + o, (unsigned)(bytes - o < CH ? bytes - o : CH));
}

// ASYNC: the tile's half spectra are copied into the line buffer by cp.async
// (all of them in flight at once, no registers held) in the in-place slot
// order, and the inverse transform then runs in place; otherwise each item
// loads its own inputs from global memory.
template <int NX, int WY, int T, int MODE, bool PHYS = true, bool ASYNC = false>
__global__ void __launch_bounds__(T) x_pass_kernel(const RunParams* __restrict__ runs, const Shape sh) {
  constexpr int M = NX / 2;
  using LM = XLine<M>;
  constexpr int PM = LM::PITCH;
  constexpr int NP = LM::N2 / 2 + 1;  // run pairs per line
  // run pairs (pr, N2 - pr) for 0 < pr < N2/2, run 0 alone, and for even N2
  // the run N2/2 paired with itself (x_inv_runs / x_fwd_runs)
  extern __shared__ float2 smem[];
  // The twiddle tables W_NX^j and W_M^j, read by every run and pass-A item:
  // copied to shared memory from Nx = 96 up.  There a CTA's tile of every
  // field leaves room for one or two CTAs per SM, so the extra registers the
  // compiler then spends on early twiddle loads cost no occupancy (x pass
  // 0.129 -> 0.124 ms at 128^3 x 16, 2.67 -> 2.59 ms at 256^3 x 32); the
  // small grids' tiles fit more CTAs than those registers would.
  constexpr bool TWS = NX >= 96;
  __shared__ float2 stwN[TWS ? NX : 1], stwM[TWS ? M : 1];
  if constexpr (TWS) {
    for (int j = threadIdx.x; j < NX; j += T) stwN[j] = __ldg(sh.twN + j);
    for (int j = threadIdx.x; j < M; j += T) stwM[j] = __ldg(sh.twM + j);
    __syncthreads();
  }
  const float2* twN = TWS ? stwN : sh.twN;
  const float2* twM = TWS ? stwM : sh.twM;
  const RunParams& rp = runs[blockIdx.y];
  const int nF = (MODE == MODE_XJ) ? 1 : rp.V + 1;
  const int ny_tiles = sh.Ny / WY;
  const int z = blockIdx.x / ny_tiles;
  const int y0 = (blockIdx.x - z * ny_tiles) * WY;
  const size_t plane = (size_t)sh.Nz * sh.Ny;
  const size_t fstride = (size_t)sh.Kx * plane;
  const size_t row_off = (size_t)z * sh.Ny + y0;
  const float2* __restrict__ src = (MODE == MODE_XJ) ? rp.J : rp.Sm;

  if (MODE == MODE_IMPORT) {
    // real rows -> interleaved lines (natural order)
    for (int it = threadIdx.x; it < nF * WY * M; it += T) {
      const int m = it % M, r = it / M, yy = r % WY, f = r / WY;
      const float2 v = *reinterpret_cast<const float2*>(rp.fin + (((size_t)f * sh.Nz + z) * sh.Ny + y0 + yy) * NX + 2 * m);
      smem[(f * WY + yy) * PM + LM::phys(m)] = v;
    }
  } else {
    // 1. inverse x transform: global half spectrum -> pre-processing -> pass B'
    // a warp covers consecutive (y row, field) lines at one run pair: the
    // global reads are y-contiguous and the line offsets hit distinct banks
    if constexpr (ASYNC) {
      constexpr int KX = M + 1;
      // consecutive threads copy consecutive rows of one (field, kx): 64-byte
      // runs of global memory, destination lines PM apart (distinct banks)
      for (int it = threadIdx.x; it < nF * KX * WY; it += T) {
        const int yy = it % WY, r = it / WY, kx = r % KX, f = r / KX;
        cp_async8(smem + (f * WY + yy) * PM + x_spec_slot<M>(kx),
                  src + f * fstride + (size_t)kx * plane + row_off + yy);
      }
      cp_async_wait_all();
      __syncthreads();
      for (int it = threadIdx.x; it < nF * WY * NP; it += T) {
        const int l = it % (nF * WY), pr = x_run_pair<M>(it / (nF * WY));
        x_inv_runs<M, SPEC_INPLACE, TWS>(smem + l * PM, 0, smem + l * PM, pr, twN);
      }
    } else {
      for (int it = threadIdx.x; it < nF * WY * NP; it += T) {
        const int l = it % (nF * WY), pr = x_run_pair<M>(it / (nF * WY));
        const int f = l / WY, yy = l - f * WY;
        x_inv_runs<M, SPEC_GLOBAL, TWS>(src + f * fstride + row_off + yy, plane, smem + l * PM, pr, twN);
      }
    }
    __syncthreads();
    passA_rt<M, PM, T, true, TWS>(smem, nF * WY, twM);
  }
  __syncthreads();

  if (MODE == MODE_EXPORT) {
    for (int it = threadIdx.x; it < nF * WY * M; it += T) {
      const int m = it % M, r = it / M, yy = r % WY, f = r / WY;
      *reinterpret_cast<float2*>(rp.fin + (((size_t)f * sh.Nz + z) * sh.Ny + y0 + yy) * NX + 2 * m) =
          smem[(f * WY + yy) * PM + LM::phys(m)];
    }
    return;
  }

  BulkAcc acc;
  acc.init();

  if (MODE == MODE_BULK) {
    // 2. bulk terms, two cells per slot
    bulk_tile<NX, WY, T, PHYS>(smem, rp, sh, z, y0, acc);
    __syncthreads();
  } else if (MODE == MODE_XJ) {
    for (int it = threadIdx.x; it < WY * M; it += T) {
      const int m = it % M, yy = it / M;
      const int slot = LM::phys(m);
      const float2 mb = *reinterpret_cast<const float2*>(rp.mob + ((size_t)z * sh.Ny + y0 + yy) * NX + 2 * m);
      float2 v = smem[yy * PM + slot];
      v.x *= mb.x;
      v.y *= mb.y;
      smem[yy * PM + slot] = v;
    }
    __syncthreads();
  }

  // 3. forward x transform: pass A, then pass B + post-processing -> global
  passA_rt<M, PM, T, false, TWS>(smem, nF * WY, twM);
  __syncthreads();
  float2* __restrict__ dst = (MODE == MODE_BULK) ? rp.D : (MODE == MODE_XJ ? rp.J : rp.Sm);
  const float scale = 1.0f / (float)NX;
  for (int it = threadIdx.x; it < nF * WY * NP; it += T) {
    const int l = it % (nF * WY), pr = x_run_pair<M>(it / (nF * WY));
    const int f = l / WY, yy = l - f * WY;
    x_fwd_runs<M, TWS>(dst + f * fstride + row_off + yy, plane, smem + l * PM, pr, scale, twN);
  }

  if (MODE != MODE_BULK) return;

  // 6. diagnostics: block reduction into per-block partials
  store_block_diag<T>(acc, rp, sh, blockIdx.x);
}


// ---------------------------------------------------------------------------
// x pass (bulk mode) with TMA-staged loads, persistent over tiles.
//
// MINB CTAs per SM (the grid holds as many as are resident at once) walk the
// tiles (WY rows at one z, all fields) tile = blockIdx.x, blockIdx.x +
// gridDim.x, ...  The mixed-space half spectra
// of a tile arrive by TMA -- one box {WY rows, 1 z, Kx, 1 field} per field of
// the run's tensor map over Sm [nF][Kx][Nz][Ny] -- into a staging buffer
// [field][kx][row]; as soon as the inverse x transform has consumed them,
// one thread issues the next tile's boxes, which land while the CTA runs the
// rest of this tile (inverse pass A, bulk terms, forward transform, stores of
// D and diagnostics).  The HBM latency that stalls the plain kernel's loads
// thus overlaps the previous tile's arithmetic.  Results are identical to the
// plain kernel's (same arithmetic, same per-tile partials).
// ---------------------------------------------------------------------------
template <int NX, int WY>
struct XTMA {
  static constexpr int M = NX / 2, KX = M + 1, PM = XLine<M>::PITCH;
  // staging of one field, a multiple of 128 bytes so that every TMA
  // destination starts on a 128-byte boundary
  static constexpr int FSTRIDE = ((KX * WY * 8 + 127) / 128) * 16;  // float2 elements
  static constexpr size_t stage_bytes(int nF) { return (size_t)nF * FSTRIDE * 8; }
  static constexpr size_t smem(int nF) { return stage_bytes(nF) + (size_t)nF * WY * PM * 8 + 16; }
};

template <int NX, int WY, int T, int MINB = 1>
__global__ void __launch_bounds__(T, MINB) x_pass_tma_kernel(const RunParams* __restrict__ runs, const Shape sh) {
  using G = XTMA<NX, WY>;
  constexpr int M = G::M, KX = G::KX, PM = G::PM;
  using LM = XLine<M>;
  constexpr int NP = LM::N2 / 2 + 1;
  extern __shared__ __align__(128) unsigned char xsm[];
  const RunParams& rp = runs[blockIdx.y];
  const int nF = rp.V + 1;
  float2* stage = reinterpret_cast<float2*>(xsm);  // [nF][KX][WY], field stride FSTRIDE
  float2* smem = reinterpret_cast<float2*>(xsm + G::stage_bytes(nF));  // lines [nF * WY][PM]
  uint64_t* bar = reinterpret_cast<uint64_t*>(xsm + G::stage_bytes(nF) + (size_t)nF * WY * PM * 8);
  const int ny_tiles = sh.Ny / WY;
  const int ntiles = sh.Nz * ny_tiles;
  const unsigned tile_bytes = (unsigned)(nF * KX * WY * 8);
  const size_t plane = (size_t)sh.Nz * sh.Ny;
  const size_t fstride = (size_t)sh.Kx * plane;
  if (threadIdx.x == 0) mbar_init(bar, 1);
  __syncthreads();
  auto issue = [&](int t) {
    const int zt = t / ny_tiles, yt = (t - zt * ny_tiles) * WY;
    mbar_expect_tx(bar, tile_bytes);
    for (int f = 0; f < nF; ++f) tma_load_4d(stage + (size_t)f * G::FSTRIDE, rp.tmap_sm, yt, zt, 0, f, bar);
  };
  int tile = blockIdx.x;
  if (threadIdx.x == 0 && tile < ntiles) issue(tile);
  unsigned parity = 0;
  for (; tile < ntiles; tile += gridDim.x) {
    const int z = tile / ny_tiles;
    const int y0 = (tile - z * ny_tiles) * WY;
    const size_t row_off = (size_t)z * sh.Ny + y0;
    const bool ok = mbar_wait(bar, parity);
    if (!__syncthreads_and(ok)) {  // the tile never arrived: flag the step and stop
      if (threadIdx.x == 0) atomicOr(rp.err, 1u);
      return;
    }
    parity ^= 1u;
    // 1. inverse x transform from the staged half spectra (element kx of row yy at [kx][yy])
    for (int it = threadIdx.x; it < nF * WY * NP; it += T) {
      const int l = it % (nF * WY), pr = x_run_pair<M>(it / (nF * WY));
      const int f = l / WY, yy = l - f * WY;
      x_inv_runs<M, SPEC_SMEM>(stage + (size_t)f * G::FSTRIDE + yy, WY, smem + l * PM, pr, sh.twN);
    }
    __syncthreads();
    if (threadIdx.x == 0 && tile + (int)gridDim.x < ntiles) issue(tile + gridDim.x);  // staging is free again
    passA_rt<M, PM, T, true>(smem, nF * WY, sh.twM);
    __syncthreads();
    // 2. bulk terms
    BulkAcc acc;
    acc.init();
    bulk_tile<NX, WY, T>(smem, rp, sh, z, y0, acc);
    __syncthreads();
    // 3. forward x transform -> D
    passA_rt<M, PM, T, false>(smem, nF * WY, sh.twM);
    __syncthreads();
    const float scale = 1.0f / (float)NX;
    for (int it = threadIdx.x; it < nF * WY * NP; it += T) {
      const int l = it % (nF * WY), pr = x_run_pair<M>(it / (nF * WY));
      const int f = l / WY, yy = l - f * WY;
      x_fwd_runs<M>(rp.D + f * fstride + row_off + yy, plane, smem + l * PM, pr, scale, sh.twN);
    }
    // 4. diagnostics of the tile (its block partials; ends with a barrier, so
    //    the lines are free for the next tile afterwards)
    store_block_diag<T>(acc, rp, sh, tile);
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// yz pass.  The state of every field is kept in full k-space,
//     Sk[f][kx][ypos][zpos] = u_hat (normalised like f_trans, src/f_trans.f90:12),
// in the digit-transposed position order of the y and z transforms, and is
// updated pointwise there (exact increment, no FFT round trip of the state).
// Per (field, kx) plane the yz pass
//   * transforms D~ (the x pass output, mixed space) forward over y and z,
//   * forms u_hat_new = u_hat + m1 u_hat + m2 D_hat (semi-implicit update),
//   * transforms u_hat_new back over z and y to the mixed-space field the next
//     x pass reads (Sm).
// A cluster of C CTAs shares a plane: CTA r holds z rows [r*NZ/C, ...) for
// the y transforms ("A layout") and y positions [r*NY/C, ...) for the z
// transforms ("B layout"); the layouts are exchanged through distributed
// shared memory.  All loops have compile-time trip counts.
// ---------------------------------------------------------------------------
template <int NY, int NZ, int C>
struct YZ {
  static constexpr int LA = NZ / C;  // z rows per CTA (A layout)
  static constexpr int LB = NY / C;  // y positions per CTA (B layout)
  static constexpr int PY = Line<NY>::PITCH;
  static constexpr int PZ = Line<NZ>::PITCH;
  static constexpr int UA = LA * PY;
  static constexpr int UB = LB * PZ;
  static constexpr size_t SMEM = (size_t)(UA + UB) * sizeof(float2);
  // in-place variant: the A and B layouts share one buffer
  static constexpr size_t SMEM_INPL = (size_t)(UA > UB ? UA : UB) * sizeof(float2);
  static_assert(NZ % C == 0 && NY % C == 0, "cluster must divide the plane");
};

enum YZMode { YZ_MAIN = 0, YZ_C2 = 1, YZ_IMPORT = 2 };

// ---------------------------------------------------------------------------
// Pointwise semi-implicit update of one k-point, shared by both yz kernels.
// The reference's forms (var_diff.f90 lines cited at the call sites)
//   AC: u += (-L dt kappa q^2 u - L dt D) / (1 + L dt kappa q^2)
//   CH: c += (-D dt kappa_c K4 c - D dt q^2 mu) / (1 + D dt kappa_c K4)
// are evaluated as u' = u - (t u + b D) / (1 + t), t = a Q, Q = q^2 (AC) or
// K4 (CH), with the 1/(NY NZ) normalisation of the transform folded into b.
// The increment is formed first and added to u, as in the reference: the
// rounding of the (fast, about 2 ulp) reciprocal then scales only the
// increment, so low modes, whose factor is close to 1, do not drift by a
// fixed relative bias per step.  The kz factors come from a shared-memory
// table {qz^2, qz^4, qn_z, qn_z^2} staged once per CTA.
// ---------------------------------------------------------------------------
template <int NZ, int T>
__device__ __forceinline__ void stage_kz(float4* qt, const Shape& sh) {
  for (int k = threadIdx.x; k < NZ; k += T) {
    const float n = __ldg(sh.qnz + k);
    qt[k] = make_float4(__ldg(sh.qz2 + k), __ldg(sh.qz4 + k), n, n * n);
  }
}

struct KPlane {
  float qx2, qx4, qnx;
  float a;    // t = a Q
  float b;    // coefficient of the driving term, normalisation included
  float nrm;  // 1 / (NY NZ)
  float kc;   // kappa_c
  __device__ __forceinline__ KPlane(const RunParams& rp, const Shape& sh, int kx, int mode, bool is_c, float nrm_) {
    qx2 = sh.qx2[kx];
    qx4 = sh.qx4[kx];
    qnx = sh.qnx[kx];
    nrm = nrm_;
    kc = rp.kappa_c;
    if (mode == YZ_MAIN && !is_c) {
      a = rp.L * rp.dt * rp.kappa_phi;
      b = rp.L * rp.dt * nrm_;
    } else {
      a = rp.D_L * rp.dt * rp.kappa_c;
      b = (mode == YZ_MAIN ? rp.D_L * rp.dt : rp.dt) * nrm_;
    }
  }
};

// the kx + ky parts of the k-point factors of one y position
struct KRow {
  float q2, q4, n2, g, k3;
  __device__ __forceinline__ KRow(const KPlane& P, const Shape& sh, int ky) {
    const float qy2 = __ldg(sh.qy2 + ky), qy4 = __ldg(sh.qy4 + ky), qny = __ldg(sh.qny + ky);
    q2 = P.qx2 + qy2;
    q4 = P.qx4 + qy4;
    n2 = fmaf(P.qnx, P.qnx, qny * qny);
    g = P.qnx + qny;
    k3 = fmaf(P.qnx, P.qx2, qny * qy2);
  }
};

// u: the k-space state (in: old, out: new); d: the unnormalised transform of
// the driving term (MAIN: dF/dphi or mu; C2: J'), on return J_hat where the
// c plane of a variable-mobility run hands it to the inverse transform.
template <int MODE>
__device__ __forceinline__ void kpoint(const KPlane& P, const KRow& R, const float4 z, const bool is_c, const bool var_c,
                                       float2& u, float2& d, float& fint) {
  if (MODE == YZ_IMPORT) {
    u = make_float2(d.x * P.nrm, d.y * P.nrm);
    return;
  }
  const float2 uu = u;
  const float q2 = R.q2 + z.x;
  if (MODE == YZ_MAIN) {
    // f_int by Parseval: |kf|^2 |u_hat|^2
    fint = fmaf(R.n2 + z.w, fmaf(uu.x, uu.x, uu.y * uu.y), fint);
    if (!is_c) {
      // AC (:1015-1024)
      const float t = P.a * q2;
      const float inv = __fdividef(1.0f, 1.0f + t);
      const float ix = fmaf(t, uu.x, P.b * d.x), iy = fmaf(t, uu.y, P.b * d.y);
      u = make_float2(fmaf(-ix, inv, uu.x), fmaf(-iy, inv, uu.y));
    } else {
      // CH (:976-983), K2 = -q^2
      const float t = P.a * (R.q4 + z.y);
      const float inv = __fdividef(1.0f, 1.0f + t);
      const float bq = P.b * q2;
      const float ix = fmaf(t, uu.x, bq * d.x), iy = fmaf(t, uu.y, bq * d.y);
      u = make_float2(fmaf(-ix, inv, uu.x), fmaf(-iy, inv, uu.y));
      if (var_c) {
        // J_hat = G mu_hat - kappa_c c_hat K3 (:932-935), G = i g, K3 = -i (qn . q^2)
        const float gn = (R.g + z.z) * P.nrm;
        const float kk = P.kc * fmaf(z.z, z.x, R.k3);
        d = cmul_pi(make_float2(fmaf(gn, d.x, kk * uu.x), fmaf(gn, d.y, kk * uu.y)));
      }
    }
  } else {
    // C2: c += dt G J'_hat / (1 + D dt kappa_c K4)  (:976)
    const float sg = __fdividef(P.b * (R.g + z.z), fmaf(P.a, R.q4 + z.y, 1.0f));
    u = cadd(uu, cmul_pi(make_float2(d.x * sg, d.y * sg)));
  }
}

// ---------------------------------------------------------------------------
// The step's record (src/var_diff.f90:1058-1118): one CTA per run reduces the
// x-pass partials and the yz pass's f_int partials in a fixed order (the same
// bits whichever other runs share the launch), writes the record into the
// ring and advances the step counter.  Sums are compensated FP32 pairs up to
// the warp totals; the mass is then summed over the warps in FP64 with
// compensation (KSum).  A separate launch, not the last CTA of the yz pass:
// the fence a CTA needs before announcing its partial holds that CTA (and the
// SM's next one) until all of its stores have drained.
// ---------------------------------------------------------------------------
template <int T>
__global__ void __launch_bounds__(T) record_kernel(const RunParams* __restrict__ runs, const Shape sh) {
  static_assert(T % 32 == 0 && T <= 1024, "whole warps");
  constexpr int NW = T / 32;
  __shared__ float sd[10][NW];  // hi, lo of f_eta, f_ch, mass, f_int (order parameters), f_int (c)
  __shared__ float sf[4][NW];
  __shared__ int si[NW];
  const RunParams& rp = runs[blockIdx.x];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int nb = sh.nblk_x;
  const float* __restrict__ px = rp.part_x + (size_t)sh.par * XQ_COUNT * sh.nblk_x;
  FF eta = ff(0.f), ch = ff(0.f), mass = ff(0.f), fphi = ff(0.f), fc = ff(0.f);
  float cmin = 1.f, cmax = 0.f, pmin = 1.f, ppmax = 0.f;  // reference start values (:1076-1079)
  int bad = 0;
  for (int i = t; i < nb; i += T) {
    eta.add(ff(__ldcg(px + XQ_FETA_H * nb + i), __ldcg(px + XQ_FETA_L * nb + i)));
    ch.add(ff(__ldcg(px + XQ_FCH_H * nb + i), __ldcg(px + XQ_FCH_L * nb + i)));
    mass.add(ff(__ldcg(px + XQ_MASS_H * nb + i), __ldcg(px + XQ_MASS_L * nb + i)));
    cmin = fminf(cmin, __ldcg(px + XQ_CMIN * nb + i));
    cmax = fmaxf(cmax, __ldcg(px + XQ_CMAX * nb + i));
    pmin = fminf(pmin, __ldcg(px + XQ_PHIMIN * nb + i));
    ppmax = fmaxf(ppmax, __ldcg(px + XQ_PHIPMAX * nb + i));
    bad += (int)__ldcg(px + XQ_BAD * nb + i);
  }
  // f_int partials: the last nblk_yz / nF slots belong to the c planes
  const int nyz = sh.nblk_yz, cstart = nyz - nyz / (rp.V + 1);
  const float* __restrict__ pyz = rp.part_yz + (size_t)sh.par * 2 * nyz;
  for (int i = t; i < nyz; i += T) {
    const FF v = ff(__ldcg(pyz + i), __ldcg(pyz + nyz + i));
    if (i < cstart) fphi.add(v);
    else fc.add(v);
  }
  eta = warp_sum_ff(eta); ch = warp_sum_ff(ch); mass = warp_sum_ff(mass);
  fphi = warp_sum_ff(fphi); fc = warp_sum_ff(fc);
  cmin = warp_min(cmin); cmax = warp_max(cmax); pmin = warp_min(pmin); ppmax = warp_max(ppmax);
  bad = __reduce_add_sync(0xffffffffu, bad);
  if (lane == 0) {
    sd[0][w] = eta.hi; sd[1][w] = eta.lo; sd[2][w] = ch.hi; sd[3][w] = ch.lo; sd[4][w] = mass.hi; sd[5][w] = mass.lo;
    sd[6][w] = fphi.hi; sd[7][w] = fphi.lo; sd[8][w] = fc.hi; sd[9][w] = fc.lo;
    sf[0][w] = cmin; sf[1][w] = cmax; sf[2][w] = pmin; sf[3][w] = ppmax;
    si[w] = bad;
  }
  __syncthreads();
  if (w == 0) {
    const bool in = lane < NW;
    const FF e = warp_sum_ff(in ? ff(sd[0][lane], sd[1][lane]) : ff(0.f));
    const FF c = warp_sum_ff(in ? ff(sd[2][lane], sd[3][lane]) : ff(0.f));
    const FF a = warp_sum_ff(in ? ff(sd[6][lane], sd[7][lane]) : ff(0.f));
    const FF b = warp_sum_ff(in ? ff(sd[8][lane], sd[9][lane]) : ff(0.f));
    // mass: the warps' compensated sums in FP64, combined with compensation
    KSum m;
    if (in) m.add(ff(sd[4][lane], sd[5][lane]).value());
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      KSum other;
      other.s = __shfl_xor_sync(0xffffffffu, m.s, o);
      other.c = __shfl_xor_sync(0xffffffffu, m.c, o);
      m.add(other);
    }
    const float m0 = warp_min(in ? sf[0][lane] : 1.f), m1 = warp_max(in ? sf[1][lane] : 0.f);
    const float m2 = warp_min(in ? sf[2][lane] : 1.f), m3 = warp_max(in ? sf[3][lane] : 0.f);
    const int nbad = __reduce_add_sync(0xffffffffu, in ? si[lane] : 0);
    if (lane == 0) {
      const int step = *rp.counter;
      double* d = rp.diag + (size_t)(step % rp.ring) * DR_COUNT;
      const double n3 = (double)sh.Nx * sh.Ny * sh.Nz;
      d[DR_STEP] = step + 1;
      d[DR_FINT] = 0.5 * n3 * ((double)rp.kappa_phi * a.value() + (double)rp.kappa_c * b.value());
      d[DR_FETA] = e.value();
      d[DR_FCH] = c.value();
      d[DR_CMIN] = m0;
      d[DR_CMAX] = m1;
      d[DR_PHIMIN] = m2;
      d[DR_PHIPMAX] = m3;
      d[DR_MASS] = m.value();
      d[DR_NONFINITE] = nbad + (*rp.err ? 1e9 : 0.0);  // a failed TMA wait flags every later step
      *rp.counter = step + 1;
    }
  }
}

// Store this CTA's f_int partial -- w times the sum of the per-thread FP32
// sums of |kf|^2 |u_hat|^2 (w = 2 for the kx planes that stand for their
// conjugates, else 1) -- as a compensated pair in slot `slot`.
template <int T>
__device__ __forceinline__ void yz_finish(const RunParams& rp, const Shape& sh, float fint, float w, size_t slot) {
  constexpr int NW = T / 32;
  __shared__ float red[2][NW];
  const FF v = warp_sum_ff(ff(fint * w));
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    red[0][wid] = v.hi;
    red[1][wid] = v.lo;
  }
  __syncthreads();
  if (wid == 0) {
    const FF s = warp_sum_ff(lane < NW ? ff(red[0][lane], red[1][lane]) : ff(0.f));
    if (lane == 0) {
      float* pyz = rp.part_yz + (size_t)sh.par * 2 * sh.nblk_yz;
      pyz[slot] = s.hi;
      pyz[sh.nblk_yz + slot] = s.lo;
    }
  }
}

template <int C>
__device__ __forceinline__ void cluster_barrier() {
  if constexpr (C == 1) {
    __syncthreads();
  } else {
    cg::this_cluster().sync();
  }
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ uint32_t map_rank(uint32_t a, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}
template <int C>
__device__ __forceinline__ float2 ld_peer(uint32_t a) {
  float2 v;
  if constexpr (C == 1) {
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(a));
  } else {
    asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(a));
  }
  return v;
}

// B[yl][phys_z(z)] <- A_{owner(z)}[z % LA][phys_y(r*LB + yl)], consecutive
// threads read consecutive y positions of one peer row.
template <int NY, int NZ, int C, int T>
__device__ __forceinline__ void exch_AB(float2* __restrict__ B, uint32_t A_base, int r) {
  using G = YZ<NY, NZ, C>;
  constexpr int TOTAL = G::LB * NZ;
  static_assert(T % G::LB == 0, "threads must cover whole rows");
  constexpr int S = T / G::LB;  // z step per iteration
  constexpr int ITER = (TOTAL + T - 1) / T;
  const int yl = threadIdx.x % G::LB;
  const int z0 = threadIdx.x / G::LB;
  const uint32_t src_off = (uint32_t)(Line<NY>::phys(r * G::LB + yl)) * 8u;
  constexpr int K = 8;
#pragma unroll
  for (int j0 = 0; j0 < ITER; j0 += K) {
    float2 v[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int z = z0 + (j0 + k) * S;
      if (j0 + k < ITER && z < NZ) {
        const int owner = z / G::LA, zl = z - owner * G::LA;
        const uint32_t a = A_base + (uint32_t)(zl * G::PY) * 8u + src_off;
        v[k] = ld_peer<C>(C == 1 ? a : map_rank(a, owner));
      }
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int z = z0 + (j0 + k) * S;
      if (j0 + k < ITER && z < NZ) B[yl * G::PZ + Line<NZ>::phys(z)] = v[k];
    }
  }
}

// A[zl][phys_y(y)] <- B_{owner(y)}[y % LB][phys_z(r*LA + zl)], consecutive
// threads read consecutive z positions of one peer line.
template <int NY, int NZ, int C, int T>
__device__ __forceinline__ void exch_BA(float2* __restrict__ A, uint32_t B_base, int r) {
  using G = YZ<NY, NZ, C>;
  constexpr int TOTAL = G::LA * NY;
  static_assert(T % G::LA == 0, "threads must cover whole lines");
  constexpr int S = T / G::LA;
  constexpr int ITER = (TOTAL + T - 1) / T;
  const int zl = threadIdx.x % G::LA;
  const int y0 = threadIdx.x / G::LA;
  const uint32_t src_off = (uint32_t)(Line<NZ>::phys(r * G::LA + zl)) * 8u;
  constexpr int K = 8;
#pragma unroll
  for (int j0 = 0; j0 < ITER; j0 += K) {
    float2 v[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int y = y0 + (j0 + k) * S;
      if (j0 + k < ITER && y < NY) {
        const int owner = y / G::LB, yl = y - owner * G::LB;
        const uint32_t a = B_base + (uint32_t)(yl * G::PZ) * 8u + src_off;
        v[k] = ld_peer<C>(C == 1 ? a : map_rank(a, owner));
      }
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int y = y0 + (j0 + k) * S;
      if (j0 + k < ITER && y < NY) A[zl * G::PY + Line<NY>::phys(y)] = v[k];
    }
  }
}

// In-place exchanges: every thread first reads all the elements it will own
// in the new layout from the cluster's old layouts (into registers), the
// cluster waits until every CTA has read everything it needs, and then each
// CTA overwrites its own buffer with the new layout.  One buffer per CTA
// instead of two, so a quarter of a 256 x 256 plane (140 KB) fits one CTA.
template <int NY, int NZ, int C, int T>
__device__ __forceinline__ void exch_AB_inpl(float2* __restrict__ buf, uint32_t A_base, int r) {
  using G = YZ<NY, NZ, C>;
  constexpr int TOTAL = G::LB * NZ;
  static_assert(T % G::LB == 0 && TOTAL % T == 0, "threads must cover whole rows");
  constexpr int S = T / G::LB;
  constexpr int ITER = TOTAL / T;
  const int yl = threadIdx.x % G::LB;
  const int z0 = threadIdx.x / G::LB;
  const uint32_t src_off = (uint32_t)(Line<NY>::phys(r * G::LB + yl)) * 8u;
  float2 v[ITER];
#pragma unroll
  for (int k = 0; k < ITER; ++k) {
    const int z = z0 + k * S;
    const int owner = z / G::LA, zl = z - owner * G::LA;
    v[k] = ld_peer<C>(map_rank(A_base + (uint32_t)(zl * G::PY) * 8u + src_off, owner));
  }
  cluster_barrier<C>();  // every CTA holds its new layout in registers
#pragma unroll
  for (int k = 0; k < ITER; ++k) buf[yl * G::PZ + Line<NZ>::phys(z0 + k * S)] = v[k];
  __syncthreads();
}

template <int NY, int NZ, int C, int T>
__device__ __forceinline__ void exch_BA_inpl(float2* __restrict__ buf, uint32_t B_base, int r) {
  using G = YZ<NY, NZ, C>;
  constexpr int TOTAL = G::LA * NY;
  static_assert(T % G::LA == 0 && TOTAL % T == 0, "threads must cover whole lines");
  constexpr int S = T / G::LA;
  constexpr int ITER = TOTAL / T;
  const int zl = threadIdx.x % G::LA;
  const int y0 = threadIdx.x / G::LA;
  const uint32_t src_off = (uint32_t)(Line<NZ>::phys(r * G::LA + zl)) * 8u;
  float2 v[ITER];
#pragma unroll
  for (int k = 0; k < ITER; ++k) {
    const int y = y0 + k * S;
    const int owner = y / G::LB, yl = y - owner * G::LB;
    v[k] = ld_peer<C>(map_rank(B_base + (uint32_t)(yl * G::PZ) * 8u + src_off, owner));
  }
  cluster_barrier<C>();  // no CTA reads a peer's buffer after this point
#pragma unroll
  for (int k = 0; k < ITER; ++k) buf[zl * G::PY + Line<NY>::phys(y0 + k * S)] = v[k];
  __syncthreads();
}

// pass A (forward or inverse) over NL lines of length L, pitch P, T threads
template <int L, int NL, int P, int T, bool INV>
__device__ __forceinline__ void passA(float2* buf, const float2* __restrict__ tw) {
  constexpr int N1 = Line<L>::N1, N2 = Line<L>::N2;
  static_assert(T % N1 == 0, "threads must be a multiple of N1");
  const int n1 = threadIdx.x % N1;
  float2 w[N2];
#pragma unroll
  for (int k2 = 1; k2 < N2; ++k2) w[k2] = __ldg(tw + n1 * k2);
  constexpr int ITEMS = NL * N1, ITER = (ITEMS + T - 1) / T;
#pragma unroll
  for (int j = 0; j < ITER; ++j) {
    const int it = threadIdx.x + j * T;
    if (ITEMS % T != 0 && it >= ITEMS) break;
    const int l = it / N1;
    float2* p = buf + l * P + n1;
    float2 v[N2];
    if (!INV) {
#pragma unroll
      for (int n2 = 0; n2 < N2; ++n2) v[n2] = p[n2 * (N1 + 1)];
      Dft<N2>::fwd(v);
#pragma unroll
      for (int k2 = 1; k2 < N2; ++k2) v[k2] = cmul(v[k2], w[k2]);
    } else {
      v[0] = p[0];
#pragma unroll
      for (int k2 = 1; k2 < N2; ++k2) v[k2] = cmulc(p[k2 * (N1 + 1)], w[k2]);
      dft_inv<N2>(v);
    }
#pragma unroll
    for (int k = 0; k < N2; ++k) p[k * (N1 + 1)] = v[k];
  }
}

template <int L, int NL, int P, int T, bool INV>
__device__ __forceinline__ void passB(float2* buf) {
  constexpr int N1 = Line<L>::N1, N2 = Line<L>::N2;
  constexpr int ITEMS = NL * N2, ITER = (ITEMS + T - 1) / T;
#pragma unroll
  for (int j = 0; j < ITER; ++j) {
    const int it = threadIdx.x + j * T;
    if (ITEMS % T != 0 && it >= ITEMS) break;
    const int l = it / N2, k2 = it - l * N2;  // k2 is fixed per thread when N2 divides T
    float2* p = buf + l * P + k2 * (N1 + 1);
    float2 u[N1];
#pragma unroll
    for (int n1 = 0; n1 < N1; ++n1) u[n1] = p[n1];
    if (INV) dft_inv<N1>(u); else Dft<N1>::fwd(u);
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) p[k1] = u[k1];
  }
}

// PREF (main mode): before its k-space update the CTA prefetches into L2 the
// D~ rows and k-space block that CTA blockIdx.x + sh.pref_yz (a multiple of C:
// the same cluster rank, about one generation of resident CTAs later) reads.
template <int NY, int NZ, int C, int T, int MODE, bool INPL = false, bool PREF = false>
__global__ void __launch_bounds__(T) yz_kernel(const RunParams* __restrict__ runs, const Shape sh) {
  using G = YZ<NY, NZ, C>;
  using LY = Line<NY>;
  using LZ = Line<NZ>;
  constexpr int N1y = LY::N1, N2y = LY::N2, N1z = LZ::N1, N2z = LZ::N2;
  static_assert(T % N1y == 0 && T % N2z == 0, "thread count");
  extern __shared__ float2 smem[];
  __shared__ float4 qzt[NZ];  // kz factors of the k-space update
  stage_kz<NZ, T>(qzt, sh);   // read after the barriers of the forward passes
  float2* UA = smem;
  float2* UB = INPL ? smem : smem + G::UA;  // in place: both layouts in one buffer
  const RunParams& rp = runs[blockIdx.y];
  const int r = (C == 1) ? 0 : (int)(blockIdx.x % C);
  const int p = sh.plane0 + (int)(blockIdx.x / C);
  const int Kx = sh.Kx;
  const int f = (MODE == YZ_C2) ? rp.V : p / Kx;
  const int kx = p - (p / Kx) * Kx;
  const size_t plane_elems = (size_t)NZ * NY;
  const size_t fstride = (size_t)Kx * plane_elems;
  const size_t poff = f * fstride + kx * plane_elems;
  const bool is_c = (f == rp.V);
  const bool var_c = (MODE == YZ_MAIN) && is_c && rp.mobility != MOB_CONST;
  const int z0 = r * G::LA;

  // 1. forward y transform of the mixed-space input rows z0..z0+LA
  //    (MAIN/IMPORT: D~ or S~; C2: J~'), first pass straight from global
  {
    const float2* src = (MODE == YZ_MAIN) ? rp.D + poff : (MODE == YZ_C2 ? rp.J + kx * plane_elems : rp.Sm + poff);
    const int n1 = threadIdx.x % N1y;
    float2 w[N2y];
#pragma unroll
    for (int k2 = 1; k2 < N2y; ++k2) w[k2] = __ldg(sh.twY + n1 * k2);
    constexpr int ITEMS = G::LA * N1y, ITER = (ITEMS + T - 1) / T;
#pragma unroll
    for (int j = 0; j < ITER; ++j) {
      const int it = threadIdx.x + j * T;
      if (ITEMS % T != 0 && it >= ITEMS) break;
      const int zl = it / N1y;
      const float2* s = src + (size_t)(z0 + zl) * NY + n1;
      float2 v[N2y];
#pragma unroll
      for (int n2 = 0; n2 < N2y; ++n2) v[n2] = __ldg(s + n2 * N1y);
      Dft<N2y>::fwd(v);
      float2* d = UA + zl * G::PY + n1;
      d[0] = v[0];
#pragma unroll
      for (int k2 = 1; k2 < N2y; ++k2) d[k2 * (N1y + 1)] = cmul(v[k2], w[k2]);
    }
  }
  __syncthreads();
  passB<NY, G::LA, G::PY, T, false>(UA);
  cluster_barrier<C>();
  if constexpr (INPL) exch_AB_inpl<NY, NZ, C, T>(UB, smem_addr(UA), r);
  else exch_AB<NY, NZ, C, T>(UB, smem_addr(UA), r);
  __syncthreads();
  passA<NZ, G::LB, G::PZ, T, false>(UB, sh.twZ);
  __syncthreads();
  if constexpr (PREF && MODE == YZ_MAIN) {
    const int b2 = (int)blockIdx.x + sh.pref_yz;
    if (sh.pref_yz > 0 && b2 < (int)gridDim.x && threadIdx.x < 64) {
      const int p2 = sh.plane0 + b2 / C, f2 = p2 / Kx, kx2 = p2 - f2 * Kx, r2 = b2 % C;
      const size_t poff2 = f2 * fstride + kx2 * plane_elems;
      const int lane = threadIdx.x & 31;
      if (threadIdx.x < 32) {
        prefetch_l2_warp(rp.D + poff2 + (size_t)r2 * G::LA * NY, (size_t)G::LA * NY * 8, lane);
      } else {
        for (int k1 = lane; k1 < N1z; k1 += 32)
          prefetch_l2(rp.Sk + poff2 + (size_t)k1 * NY * N2z + (size_t)r2 * G::LB * N2z, G::LB * N2z * 8);
      }
    }
  }

  // 2. last forward z pass, pointwise k-space update, first inverse z pass,
  //    fused per run of N1z positions
  const KPlane P(rp, sh, kx, MODE, is_c, 1.0f / (float)(NY * NZ));
  const float wkx = (kx == 0 || 2 * kx == sh.Nx) ? 1.0f : 2.0f;
  float fint = 0.f;
  {
    const int k2 = threadIdx.x % N2z;
    constexpr int ITEMS = G::LB * N2z, ITER = (ITEMS + T - 1) / T;
#pragma unroll 1
    for (int j = 0; j < ITER; ++j) {
      const int it = threadIdx.x + j * T;
      if (ITEMS % T != 0 && it >= ITEMS) break;
      const int yl = it / N2z;
      const int ypos = r * G::LB + yl;
      const KRow R(P, sh, LY::freq_of_pos(ypos));
      float2* pb = UB + yl * G::PZ + k2 * (N1z + 1);
      // k-space state of this plane in [k1][y position][k2] order: for every
      // k1 a warp reads and writes consecutive (y position, k2) (coalesced)
      float2* gk = rp.Sk + poff + (size_t)ypos * N2z + k2;
      constexpr size_t SK1 = (size_t)NY * N2z;  // stride of k1
      float2 d[N1z], u[N1z];
#pragma unroll
      for (int k1 = 0; k1 < N1z; ++k1) d[k1] = pb[k1];
      Dft<N1z>::fwd(d);
      if (MODE != YZ_IMPORT) {
#pragma unroll
        for (int k1 = 0; k1 < N1z; ++k1) u[k1] = gk[k1 * SK1];
      }
#pragma unroll
      for (int k1 = 0; k1 < N1z; ++k1) kpoint<MODE>(P, R, qzt[k2 + N2z * k1], is_c, var_c, u[k1], d[k1], fint);
#pragma unroll
      for (int k1 = 0; k1 < N1z; ++k1) gk[k1 * SK1] = u[k1];
      if (MODE != YZ_IMPORT) {
        if (var_c) {
          dft_inv<N1z>(d);
#pragma unroll
          for (int k1 = 0; k1 < N1z; ++k1) pb[k1] = d[k1];
        } else {
          dft_inv<N1z>(u);
#pragma unroll
          for (int k1 = 0; k1 < N1z; ++k1) pb[k1] = u[k1];
        }
      }
    }
  }
  if (MODE == YZ_IMPORT) {
    cluster_barrier<C>();  // peers may still read this CTA's A buffer
    return;
  }
  __syncthreads();
  passA<NZ, G::LB, G::PZ, T, true>(UB, sh.twZ);
  cluster_barrier<C>();
  if constexpr (INPL) {
    exch_BA_inpl<NY, NZ, C, T>(UA, smem_addr(UB), r);  // ends after the last peer read
  } else {
    exch_BA<NY, NZ, C, T>(UA, smem_addr(UB), r);
    cluster_barrier<C>();  // no CTA reads a peer's buffers after this point
  }
  passB<NY, G::LA, G::PY, T, true>(UA);
  __syncthreads();

  // 3. last inverse y pass straight to the mixed-space output
  //    (u~ for the next x pass, or J~ for the variable-mobility chain)
  {
    const bool real_plane = (kx == 0) || (2 * kx == sh.Nx);  // the x-DFT of real data is real there
    float2* dst = var_c ? rp.J + kx * plane_elems : rp.Sm + poff;
    const int n1 = threadIdx.x % N1y;
    float2 w[N2y];
#pragma unroll
    for (int k2 = 1; k2 < N2y; ++k2) w[k2] = __ldg(sh.twY + n1 * k2);
    constexpr int ITEMS = G::LA * N1y, ITER = (ITEMS + T - 1) / T;
#pragma unroll
    for (int j = 0; j < ITER; ++j) {
      const int it = threadIdx.x + j * T;
      if (ITEMS % T != 0 && it >= ITEMS) break;
      const int zl = it / N1y;
      const float2* s = UA + zl * G::PY + n1;
      float2 v[N2y];
      v[0] = s[0];
#pragma unroll
      for (int k2 = 1; k2 < N2y; ++k2) v[k2] = cmulc(s[k2 * (N1y + 1)], w[k2]);
      dft_inv<N2y>(v);
      float2* o = dst + (size_t)(z0 + zl) * NY + n1;
#pragma unroll
      for (int n2 = 0; n2 < N2y; ++n2) {
        float2 x = v[n2];
        if (real_plane && !var_c) x.y = 0.f;
        o[n2 * N1y] = x;
      }
    }
  }

  if (MODE == YZ_MAIN) {
    // f_int partial (:609-678 by Parseval): 0.5 kappa N^3 w |kf|^2 |u_hat|^2
    yz_finish<T>(rp, sh, fint, wkx, (size_t)sh.plane0 * C + blockIdx.x);
  }
}

// ---------------------------------------------------------------------------
// Single-CTA yz pass for planes that fit one CTA's shared memory: the plane
// stays in one buffer U[z][phys_y(y)] (row pitch PY, odd); y transforms run
// along rows, z transforms down columns (consecutive threads take consecutive
// y positions, so column accesses are conflict-free).  No re-layout, no
// cluster.  Same k-space position order as the cluster kernel.
// ---------------------------------------------------------------------------
// Row pitch: the odd line pitch, or (RAWP) the unpadded run layout
// N2 (N1 + 1).  yz1 reads columns with lanes along y, so only its row passes
// see the pitch: a warp covers two rows (first/last y pass) or 32/N2 rows of
// N2 runs (pass B); with N2 (N1 + 1) = 8 (mod 16) float2 the rows of a half
// warp fall in disjoint bank pairs (128 x 128: no conflicts, against one
// extra wavefront in four at the odd pitch).
template <int NY, int NZ, bool RAWP = false>
struct YZ1 {
  static constexpr int PY = RAWP ? Line<NY>::RAW : Line<NY>::PITCH;
  static constexpr size_t SMEM = (size_t)NZ * PY * sizeof(float2);
};

// column pass A (forward or inverse) over the NY y positions
template <int NY, int NZ, int T, bool INV, bool RAWP, bool TWS = false>
__device__ __forceinline__ void colA(float2* U, const float2* __restrict__ tw) {
  constexpr int N1 = Line<NZ>::N1, N2 = Line<NZ>::N2, PY = YZ1<NY, NZ, RAWP>::PY;
  constexpr int ITEMS = NY * N1, ITER = (ITEMS + T - 1) / T;
#pragma unroll 1
  for (int j = 0; j < ITER; ++j) {
    const int it = threadIdx.x + j * T;
    if (ITEMS % T != 0 && it >= ITEMS) break;
    const int yp = it % NY, n1 = it / NY;
    float2* p = U + n1 * PY + Line<NY>::phys(yp);
    float2 v[N2];
    if (!INV) {
#pragma unroll
      for (int n2 = 0; n2 < N2; ++n2) v[n2] = p[n2 * N1 * PY];
      Dft<N2>::fwd(v);
#pragma unroll
      for (int k2 = 1; k2 < N2; ++k2) v[k2] = cmul(v[k2], ldtw<TWS>(tw + n1 * k2));
    } else {
      v[0] = p[0];
#pragma unroll
      for (int k2 = 1; k2 < N2; ++k2) v[k2] = cmulc(p[k2 * N1 * PY], ldtw<TWS>(tw + n1 * k2));
      dft_inv<N2>(v);
    }
#pragma unroll
    for (int k = 0; k < N2; ++k) p[k * N1 * PY] = v[k];
  }
}

template <int NY, int NZ, int T, int MODE, bool RAWP = false>
__global__ void __launch_bounds__(T) yz1_kernel(const RunParams* __restrict__ runs, const Shape sh) {
  using LY = Line<NY>;
  using LZ = Line<NZ>;
  constexpr int N1y = LY::N1, N2y = LY::N2, N1z = LZ::N1, N2z = LZ::N2;
  constexpr int PY = YZ1<NY, NZ, RAWP>::PY;
  static_assert(T % 32 == 0, "whole warps");
  extern __shared__ float2 U[];
  __shared__ float4 qzt[NZ];  // kz factors of the k-space update
  stage_kz<NZ, T>(qzt, sh);   // read after the barriers of the forward passes
  // the z twiddles of the column passes in shared memory from 128 x 128 planes
  // up (one CTA per SM there: the registers of early loads cost no occupancy)
  constexpr bool TWS = NY >= 128;
  __shared__ float2 stwZ[TWS ? NZ : 1];
  if constexpr (TWS)
    for (int j = threadIdx.x; j < NZ; j += T) stwZ[j] = __ldg(sh.twZ + j);  // read after the first barrier
  const float2* twZ = TWS ? stwZ : sh.twZ;
  const RunParams& rp = runs[blockIdx.y];
  const int p = sh.plane0 + (int)blockIdx.x;
  const int Kx = sh.Kx;
  const int f = (MODE == YZ_C2) ? rp.V : p / Kx;
  const int kx = p - (p / Kx) * Kx;
  const size_t plane_elems = (size_t)NZ * NY;
  const size_t poff = ((size_t)f * Kx + kx) * plane_elems;
  const bool is_c = (f == rp.V);
  const bool var_c = (MODE == YZ_MAIN) && is_c && rp.mobility != MOB_CONST;

  // 1. forward y transform of all NZ rows, first pass straight from global
  {
    const float2* src = (MODE == YZ_MAIN) ? rp.D + poff : (MODE == YZ_C2 ? rp.J + kx * plane_elems : rp.Sm + poff);
    // twiddles: preloaded when every iteration of a thread has the same n1
    constexpr bool FIXED = (T % N1y) == 0;
    float2 wt[N2y];
    if constexpr (FIXED) {
#pragma unroll
      for (int k2 = 1; k2 < N2y; ++k2) wt[k2] = __ldg(sh.twY + (threadIdx.x % N1y) * k2);
    }
    constexpr int ITEMS = NZ * N1y, ITER = (ITEMS + T - 1) / T;
#pragma unroll 4
    for (int j = 0; j < ITER; ++j) {
      const int it = threadIdx.x + j * T;
      if (ITEMS % T != 0 && it >= ITEMS) break;
      const int z = it / N1y, n1 = it - z * N1y;
      const float2* s = src + (size_t)z * NY + n1;
      float2 v[N2y];
#pragma unroll
      for (int n2 = 0; n2 < N2y; ++n2) v[n2] = __ldg(s + n2 * N1y);
      Dft<N2y>::fwd(v);
      float2* d = U + z * PY + n1;
      d[0] = v[0];
#pragma unroll
      for (int k2 = 1; k2 < N2y; ++k2) d[k2 * (N1y + 1)] = cmul(v[k2], FIXED ? wt[k2] : __ldg(sh.twY + n1 * k2));
    }
  }
  __syncthreads();
  passB<NY, NZ, PY, T, false>(U);
  __syncthreads();
  colA<NY, NZ, T, false, RAWP, TWS>(U, twZ);
  __syncthreads();
  // 2. last forward z pass, pointwise k-space update, first inverse z pass
  const KPlane P(rp, sh, kx, MODE, is_c, 1.0f / (float)(NY * NZ));
  const float wkx = (kx == 0 || 2 * kx == sh.Nx) ? 1.0f : 2.0f;
  float fint = 0.f;
  {
    constexpr int ITEMS = NY * N2z, ITER = (ITEMS + T - 1) / T;
#pragma unroll 1
    for (int j = 0; j < ITER; ++j) {
      const int it = threadIdx.x + j * T;
      if (ITEMS % T != 0 && it >= ITEMS) break;
      const int yp = it % NY, k2 = it / NY;
      const KRow R(P, sh, LY::freq_of_pos(yp));
      float2* pc = U + (k2 * N1z) * PY + LY::phys(yp);
      // k-space state of this plane in [k1][k2][y position] order: for every
      // k1 a warp reads and writes 32 consecutive y positions (coalesced)
      float2* gk = rp.Sk + poff + it;  // it == k2 NY + yp
      constexpr size_t SK1 = (size_t)N2z * NY;  // stride of k1
      float2 d[N1z], u[N1z];
      if (MODE != YZ_IMPORT) {
#pragma unroll
        for (int k1 = 0; k1 < N1z; ++k1) u[k1] = gk[k1 * SK1];
      }
#pragma unroll
      for (int k1 = 0; k1 < N1z; ++k1) d[k1] = pc[k1 * PY];
      Dft<N1z>::fwd(d);
#pragma unroll
      for (int k1 = 0; k1 < N1z; ++k1) kpoint<MODE>(P, R, qzt[k2 + N2z * k1], is_c, var_c, u[k1], d[k1], fint);
#pragma unroll
      for (int k1 = 0; k1 < N1z; ++k1) gk[k1 * SK1] = u[k1];
      if (MODE != YZ_IMPORT) {
        if (var_c) {
          dft_inv<N1z>(d);
#pragma unroll
          for (int k1 = 0; k1 < N1z; ++k1) pc[k1 * PY] = d[k1];
        } else {
          dft_inv<N1z>(u);
#pragma unroll
          for (int k1 = 0; k1 < N1z; ++k1) pc[k1 * PY] = u[k1];
        }
      }
    }
  }
  if (MODE == YZ_IMPORT) return;
  __syncthreads();
  colA<NY, NZ, T, true, RAWP, TWS>(U, twZ);
  __syncthreads();
  passB<NY, NZ, PY, T, true>(U);
  __syncthreads();

  // 3. last inverse y pass straight to the mixed-space output
  {
    const bool real_plane = (kx == 0) || (2 * kx == sh.Nx);  // the x-DFT of real data is real there
    float2* dst = var_c ? rp.J + kx * plane_elems : rp.Sm + poff;
    constexpr bool FIXED = (T % N1y) == 0;
    float2 wt[N2y];
    if constexpr (FIXED) {
#pragma unroll
      for (int k2 = 1; k2 < N2y; ++k2) wt[k2] = __ldg(sh.twY + (threadIdx.x % N1y) * k2);
    }
    constexpr int ITEMS = NZ * N1y, ITER = (ITEMS + T - 1) / T;
#pragma unroll 4
    for (int j = 0; j < ITER; ++j) {
      const int it = threadIdx.x + j * T;
      if (ITEMS % T != 0 && it >= ITEMS) break;
      const int z = it / N1y, n1 = it - z * N1y;
      const float2* sp = U + z * PY + n1;
      float2 v[N2y];
      v[0] = sp[0];
#pragma unroll
      for (int k2 = 1; k2 < N2y; ++k2) v[k2] = cmulc(sp[k2 * (N1y + 1)], FIXED ? wt[k2] : __ldg(sh.twY + n1 * k2));
      dft_inv<N2y>(v);
      float2* o = dst + (size_t)z * NY + n1;
#pragma unroll
      for (int n2 = 0; n2 < N2y; ++n2) {
        float2 x = v[n2];
        if (real_plane && !var_c) x.y = 0.f;
        o[n2 * N1y] = x;
      }
    }
  }

  if (MODE == YZ_MAIN) {
    yz_finish<T>(rp, sh, fint, wkx, (size_t)p);
  }
}

// ---------------------------------------------------------------------------
// x pass (bulk mode) split over a cluster of two CTAs.
//
// With many order parameters the one-CTA x pass holds (P+1) field rows and
// fits one CTA per SM.  Here the two CTAs of a cluster take the same WY rows
// and about half of the fields each (rank 0: fields [0, h), rank 1: [h, P+1),
// h = ceil((P+1)/2); rank 1 owns phi_P and c), so twice as many CTAs fit an
// SM.  The cross-field terms need per-cell sums over all fields: each CTA
// forms partial sums over its own fields (sum phi^2, sum phi^4, pair sum,
// max |phi|), the pair reads the other's partials through distributed shared
// memory (pairs = pairs_0 + pairs_1 + pre_0 pre_1), and both derive the same
// per-cell scalars; rank 1 also writes dF/dc, the mobility and the
// diagnostics.  Cells whose sum of phi^4 is below 1e-30 take the rescaled
// branch of bulk_slot with a second exchange (sum of (phi/max|phi|)^4).
// HBM traffic is that of the one-CTA pass.
// ---------------------------------------------------------------------------
template <int NX, int WY>
struct XCL {
  static constexpr int M = NX / 2;
  static constexpr int PM = XLine<M>::PITCH;
  static constexpr int S = WY * M;  // float2 slots (two cells each) per CTA
  static constexpr int NA = 7;      // per-slot arrays: pre, n4, pairs, mabs (partials), nn (partial), phiP, c
  static constexpr size_t smem(int nF) { return ((size_t)((nF + 1) / 2) * WY * PM + (size_t)NA * S) * sizeof(float2); }
};

struct CellOut {
  float t4a, t4p, invm, dc, mb;
  int bad;
};

// per-cell scalars of bulk_slot from the full aggregates of one cell
__device__ __forceinline__ CellOut cell_terms(float pp, float c, float pre, float n4, float pairs, float mabs, float nn,
                                              const RunParams& rp, BulkAcc& acc) {
  const float pp2 = pp * pp;
  const float S2 = pre + pp2;
  const float S4 = n4 + pp2 * pp2;
  float invS4, n4n, sc, im = 1.f;
  if (S4 >= 1e-30f) {
    invS4 = 1.f / S4;
    n4n = n4 * invS4;
    sc = 4.f;
  } else if (mabs > 0.f) {
    im = 1.f / mabs;
    const float xq = pp * im;
    const float s4 = nn + (xq * xq) * (xq * xq);
    invS4 = 1.f / s4;
    n4n = nn * invS4;
    sc = 4.f * im;
  } else {
    invS4 = 0.f;
    n4n = 0.f;
    sc = 0.f;
  }
  const float h = n4n;
  const float dcm = c - rp.c0m, dcp = c - rp.c0p;
  const float fm = rp.am * dcm * dcm, fp = rp.ap * dcp * dcp;
  const float dfm = fm - fp;
  acc.fch += h * fm + (1.f - h) * fp;
  CellOut o;
  o.dc = 2.f * h * rp.am * dcm + 2.f * (1.f - h) * rp.ap * dcp;
  acc.feta += -0.5f * S2 + 0.25f * S4 + rp.sigma1 * pairs + rp.sigma2 * pp2 * pre;
  acc.mass.add(c);
  acc.cmin = fminf(acc.cmin, c);
  acc.cmax = fmaxf(acc.cmax, c);
  acc.phimin = fminf(acc.phimin, S2);
  acc.phipmax = fmaxf(acc.phipmax, pp);
  if (rp.mobility == MOB_REF_VAR) o.mb = 2.f * (1.f - S2) * rp.D_gb;
  else if (rp.mobility == MOB_C1MC) o.mb = rp.D_L * c * (1.f - c);
  else o.mb = 0.f;
  const float qP = pp * im;
  const float qP2 = qP * qP;
  const float rP4 = qP2 * qP2 * invS4;
  o.t4a = sc * invS4 * rP4 * dfm;
  o.t4p = -sc * (qP * qP2 * invS4) * n4n * dfm;
  o.invm = im;
  o.bad = !isfinite(S4 + S2 + pairs + o.dc + o.t4a + o.t4p);
  return o;
}

template <int NX, int WY, int T>
__global__ void __launch_bounds__(T) x_pass_cl_kernel(const RunParams* __restrict__ runs, const Shape sh) {
  using G = XCL<NX, WY>;
  constexpr int M = G::M, PM = G::PM, S = G::S;
  using LM = XLine<M>;
  constexpr int NP = LM::N2 / 2 + 1;
  enum { A_PRE = 0, A_N4, A_PAIRS, A_MABS, A_NN, A_PP, A_C };
  extern __shared__ float2 smem[];
  const RunParams& rp = runs[blockIdx.y];
  const int V = rp.V, nF = V + 1, h = (nF + 1) / 2;
  const int rank = (int)(blockIdx.x & 1), peer = rank ^ 1, bp = (int)(blockIdx.x >> 1);
  const int fbase = rank ? h : 0, nloc = rank ? nF - h : h;
  const int ny_tiles = sh.Ny / WY;
  const int z = bp / ny_tiles;
  const int y0 = (bp - z * ny_tiles) * WY;
  const size_t plane = (size_t)sh.Nz * sh.Ny;
  const size_t fstride = (size_t)sh.Kx * plane;
  const size_t row_off = (size_t)z * sh.Ny + y0;
  float2* lines = smem;                          // nloc * WY lines
  float2* A = smem + (size_t)h * WY * PM;        // the same offset in both CTAs
  const uint32_t peer_A = map_rank(smem_addr(A), peer);
  const uint32_t peer_lines = map_rank(smem_addr(lines), peer);

  // 1. inverse x transform of the local fields
  for (int it = threadIdx.x; it < nloc * WY * NP; it += T) {
    const int l = it % (nloc * WY), pr = x_run_pair<M>(it / (nloc * WY));
    const int fl = l / WY, yy = l - fl * WY;
    x_inv_runs<M>(rp.Sm + (fbase + fl) * fstride + row_off + yy, plane, lines + l * PM, pr, sh.twN);
  }
  __syncthreads();
  passA_rt<M, PM, T, true>(lines, nloc * WY, sh.twM);
  __syncthreads();

  // 2. partial sums over the local matrix fields (f < V-1), in field order
  const int fend = min(fbase + nloc, V - 1);
  for (int it = threadIdx.x; it < S; it += T) {
    const int m = it % M, yy = it / M;
    const float2* base = lines + yy * PM + LM::phys(m);
    float pre0 = 0.f, pre1 = 0.f, n40 = 0.f, n41 = 0.f, pr0 = 0.f, pr1 = 0.f, ma0 = 0.f, ma1 = 0.f;
    for (int f = fbase; f < fend; ++f) {
      const float2 p = base[(f - fbase) * WY * PM];
      const float a0 = p.x * p.x, a1 = p.y * p.y;
      pr0 = fmaf(a0, pre0, pr0);
      pr1 = fmaf(a1, pre1, pr1);
      pre0 += a0;
      pre1 += a1;
      n40 = fmaf(a0, a0, n40);
      n41 = fmaf(a1, a1, n41);
      ma0 = fmaxf(ma0, fabsf(p.x));
      ma1 = fmaxf(ma1, fabsf(p.y));
    }
    A[A_PRE * S + it] = make_float2(pre0, pre1);
    A[A_N4 * S + it] = make_float2(n40, n41);
    A[A_PAIRS * S + it] = make_float2(pr0, pr1);
    A[A_MABS * S + it] = make_float2(ma0, ma1);
  }
  cluster_barrier<2>();

  // full sums (rank 0's part first in both CTAs: both get the same bits)
  auto totals = [&](int it, float2& pre, float2& n4, float2& pairs, float2& mabs) {
    float2 a[4], b[4];  // rank 0's and rank 1's partials
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float2 own = A[k * S + it];
      const float2 oth = ld_peer<2>(peer_A + (uint32_t)((k * S + it) * 8));
      a[k] = rank ? oth : own;
      b[k] = rank ? own : oth;
    }
    pre = make_float2(a[0].x + b[0].x, a[0].y + b[0].y);
    n4 = make_float2(a[1].x + b[1].x, a[1].y + b[1].y);
    pairs = make_float2(fmaf(a[0].x, b[0].x, a[2].x + b[2].x), fmaf(a[0].y, b[0].y, a[2].y + b[2].y));
    mabs = make_float2(fmaxf(a[3].x, b[3].x), fmaxf(a[3].y, b[3].y));
  };

  // 3. phi_P and c from rank 1; the rescaled sum where a cell needs it
  for (int it = threadIdx.x; it < S; it += T) {
    const int m = it % M, yy = it / M;
    const int off_p = ((V - 1 - h) * WY + yy) * PM + LM::phys(m);  // in rank 1's lines
    const int off_c = ((V - h) * WY + yy) * PM + LM::phys(m);
    float2 pP, cc;
    if (rank) {
      pP = lines[off_p];
      cc = lines[off_c];
    } else {
      pP = ld_peer<2>(peer_lines + (uint32_t)(off_p * 8));
      cc = ld_peer<2>(peer_lines + (uint32_t)(off_c * 8));
    }
    A[A_PP * S + it] = pP;
    A[A_C * S + it] = cc;
    float2 pre, n4, pairs, mabs;
    totals(it, pre, n4, pairs, mabs);
    float nn[2] = {0.f, 0.f};
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const float pp = q ? pP.y : pP.x;
      const float S4 = (q ? n4.y : n4.x) + (pp * pp) * (pp * pp);
      const float ma = fmaxf(q ? mabs.y : mabs.x, fabsf(pp));
      if (S4 < 1e-30f && ma > 0.f) {
        const float im = 1.f / ma;
        const float2* base = lines + yy * PM + LM::phys(m);
        for (int f = fbase; f < fend; ++f) {
          const float2 p = base[(f - fbase) * WY * PM];
          const float x = (q ? p.y : p.x) * im;
          nn[q] = fmaf(x * x, x * x, nn[q]);
        }
      }
    }
    A[A_NN * S + it] = make_float2(nn[0], nn[1]);
  }
  cluster_barrier<2>();

  // 4. per-cell scalars and dF of the local fields, in place
  BulkAcc acc;
  acc.init();
  const float sg1 = rp.sigma1, sg2 = rp.sigma2;
  for (int it = threadIdx.x; it < S; it += T) {
    const int m = it % M, yy = it / M;
    float2 pre, n4, pairs, mabs;
    totals(it, pre, n4, pairs, mabs);
    const float2 pP = A[A_PP * S + it], cc = A[A_C * S + it];
    const float2 own_nn = A[A_NN * S + it];
    const float2 oth_nn = ld_peer<2>(peer_A + (uint32_t)((A_NN * S + it) * 8));
    const float2 nn0 = rank ? oth_nn : own_nn, nn1 = rank ? own_nn : oth_nn;
    CellOut o[2];
    o[0] = cell_terms(pP.x, cc.x, pre.x, n4.x, pairs.x, fmaxf(mabs.x, fabsf(pP.x)), nn0.x + nn1.x, rp, acc);
    o[1] = cell_terms(pP.y, cc.y, pre.y, n4.y, pairs.y, fmaxf(mabs.y, fabsf(pP.y)), nn0.y + nn1.y, rp, acc);
    float2* base = lines + yy * PM + LM::phys(m);
    for (int f = fbase; f < fbase + nloc; ++f) {
      float2& slot = base[(f - fbase) * WY * PM];
      float2 d;
      if (f < V - 1) {
        const float2 p = slot;
        const float g0 = fmaf(sg1, pre.x - p.x * p.x, sg2 * (pP.x * pP.x));
        const float g1 = fmaf(sg1, pre.y - p.y * p.y, sg2 * (pP.y * pP.y));
        const float q0 = p.x * o[0].invm, q1 = p.y * o[1].invm;
        d.x = fmaf(p.x, p.x * p.x, -p.x) + 2.f * p.x * g0 + o[0].t4a * (q0 * q0 * q0);
        d.y = fmaf(p.y, p.y * p.y, -p.y) + 2.f * p.y * g1 + o[1].t4a * (q1 * q1 * q1);
      } else if (f == V - 1) {
        d.x = fmaf(pP.x, pP.x * pP.x, -pP.x) + 2.f * pP.x * (sg2 * pre.x) + o[0].t4p;
        d.y = fmaf(pP.y, pP.y * pP.y, -pP.y) + 2.f * pP.y * (sg2 * pre.y) + o[1].t4p;
      } else {
        d = make_float2(o[0].dc, o[1].dc);
      }
      slot = d;
    }
    if (rank && rp.mobility != MOB_CONST)
      *reinterpret_cast<float2*>(rp.mob + ((size_t)z * sh.Ny + y0 + yy) * NX + 2 * m) = make_float2(o[0].mb, o[1].mb);
    acc.nonfinite += o[0].bad | o[1].bad;
  }
  cluster_barrier<2>();  // no distributed-shared-memory access after this point

  // 5. forward x transform of the local fields -> D
  passA_rt<M, PM, T, false>(lines, nloc * WY, sh.twM);
  __syncthreads();
  const float scale = 1.0f / (float)NX;
  for (int it = threadIdx.x; it < nloc * WY * NP; it += T) {
    const int l = it % (nloc * WY), pr = x_run_pair<M>(it / (nloc * WY));
    const int fl = l / WY, yy = l - fl * WY;
    x_fwd_runs<M>(rp.D + (fbase + fl) * fstride + row_off + yy, plane, lines + l * PM, pr, scale, sh.twN);
  }
  if (!rank) return;

  // 6. diagnostics (rank 1): block reduction into the pair's partials
  store_block_diag<T>(acc, rp, sh, bp);
}

}  // namespace pf
