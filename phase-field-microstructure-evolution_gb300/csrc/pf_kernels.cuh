// Fused FP32 kernels of the semi-implicit spectral step (sm_103a).
//
// State of one run ("mixed" representation): for every field f (the var order
// parameters, then the concentration c) the x-direction half spectrum
//     S[f][kx][z][y] = (1/Nx) sum_x u_f(x,y,z) e^{-2 pi i kx x / Nx},  kx = 0..Nx/2
// (float2, y fastest).  The reference keeps phi/con in real space and takes a
// full 3-D R2C per field (src/f_trans.f90:11-12); here the x transform of the
// state is kept, so one step costs exactly two passes over the fields:
//
//   x pass  (x_pass_kernel, one CTA per WY y-rows at one z, all fields):
//       S --C2R_x--> phi, c --bulk terms (src/var_diff.f90:685-898)-->
//       dF/dphi_i, dF/dc (, mobility) --R2C_x/Nx--> D
//   yz pass (yz_kernel, one CTA cluster per (field, kx) plane):
//       DFT_yz(S), DFT_yz(D) --semi-implicit increment--> IDFT_yz --> S += increment
//
// The update is applied as an increment, delta_hat = m1 * u_hat + m2 * D_hat,
// so that the O(1) state never takes an FP32 round trip through the FFT; only
// the small increment does.  In exact arithmetic
//   u_hat + delta_hat = (u_hat - L dt D_hat) / (1 - L kappa dt K2)      (AC, :1020-1024)
//   c_hat + delta_hat = (c_hat + D_mean K2 dt mu_hat) / (1 + D_mean dt kappa_c K4)   (CH, :976-983)
// with the variable-mobility term dt G J'_hat / (...) of :976-983 added by a
// second x/yz pass pair (xj pass + yz_kernel in C2 mode).
#pragma once
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "pf_fft.cuh"

namespace cg = cooperative_groups;

namespace pf {

// Number of per-block diagnostic partials written by the x pass.
enum XDiag { XD_FETA = 0, XD_FCH, XD_MASS, XD_CMIN, XD_CMAX, XD_PHIMIN, XD_PHIPMAX, XD_NONFINITE, XD_COUNT };
// Per-step diagnostic record layout (doubles)
enum DiagRec {
  DR_STEP = 0, DR_FINT, DR_FETA, DR_FCH, DR_CMIN, DR_CMAX, DR_PHIMIN, DR_PHIPMAX, DR_MASS, DR_NONFINITE, DR_COUNT
};

enum Mobility { MOB_CONST = 0, MOB_REF_VAR = 1, MOB_C1MC = 2 };

// Device-side description of one run (all runs of a launch share one shape)
struct RunParams {
  float2* S;       // [nF][Kx][Nz][Ny] state
  float2* D;       // [nF][Kx][Nz][Ny] x-spectra of dF/dphi_i and dF/dc
  float* mob;      // [Nz][Ny][Nx] mobility minus D_mean (variable mobility only)
  float2* J;       // [Kx][Nz][Ny] CH flux scratch (variable mobility only)
  float2* A;       // [Kx][Nz][Ny] constant-mobility part of the c increment (idem)
  double* part_x;  // [XD_COUNT][nblk_x]
  double* part_yz; // [nblk_yz]
  double* diag;    // [ring][DR_COUNT]
  int* counter;    // step counter (device)
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
};

// ---------------------------------------------------------------------------
// Block reductions
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
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
// x-direction half-spectrum <-> interleaved real line (length M = Nx/2 complex)
// ---------------------------------------------------------------------------
// C2R pre-processing of the pair (k, M-k) into digit-transposed positions.
// X = normalised half spectrum; output Z' such that IDFT_M(Z')[m] = x[2m] + i x[2m+1].
template <int M>
__device__ __forceinline__ void c2r_pre(float2* line, int k, float2 Xk, float2 Xmk, const float2* __restrict__ twN) {
  using LM = Line<M>;
  if (k == 0) {
    line[LM::phys(LM::pos_of_freq(0))] = make_float2(Xk.x + Xmk.x, Xk.x - Xmk.x);
    return;
  }
  {
    const float2 w = __ldg(twN + k);
    const float2 b = cconj(Xmk);
    const float2 s = cadd(Xk, b), d = csub(Xk, b);
    line[LM::phys(LM::pos_of_freq(k))] = cadd(s, cmul_pi(cmulc(d, w)));
  }
  if (2 * k != M) {
    const float2 w = __ldg(twN + (M - k));
    const float2 b = cconj(Xk);
    const float2 s = cadd(Xmk, b), d = csub(Xmk, b);
    line[LM::phys(LM::pos_of_freq(M - k))] = cadd(s, cmul_pi(cmulc(d, w)));
  }
}

// R2C post-processing: from Z = DFT_M(x[2m] + i x[2m+1]) (digit-transposed) to
// X[k], X[M-k] scaled by `scale` (X[0] and X[M] are real).
template <int M>
__device__ __forceinline__ void r2c_post(const float2* line, int k, float scale, const float2* __restrict__ twN,
                                         float2& Xk, float2& Xmk) {
  using LM = Line<M>;
  if (k == 0) {
    const float2 z0 = line[LM::phys(LM::pos_of_freq(0))];
    Xk = make_float2((z0.x + z0.y) * scale, 0.f);
    Xmk = make_float2((z0.x - z0.y) * scale, 0.f);
    return;
  }
  const float2 zk = line[LM::phys(LM::pos_of_freq(k))];
  const float2 zm = line[LM::phys(LM::pos_of_freq(M - k))];
  const float h = 0.5f * scale;
  {
    const float2 b = cconj(zm);
    const float2 s = cadd(zk, b), d = csub(zk, b);
    const float2 t = cmul_mi(cmul(d, __ldg(twN + k)));
    Xk = cscale(cadd(s, t), h);
  }
  {
    const float2 b = cconj(zk);
    const float2 s = cadd(zm, b), d = csub(zm, b);
    const float2 t = cmul_mi(cmul(d, __ldg(twN + (M - k))));
    Xmk = cscale(cadd(s, t), h);
  }
}

// ---------------------------------------------------------------------------
// Bulk terms of one cell (src/var_diff.f90:685-898), reading/writing the
// interleaved real lines of all fields.  `sel` picks the x (0) or y (1)
// component of the float2 slot, i.e. cell x = 2m + sel.
// ---------------------------------------------------------------------------
struct BulkAcc {
  double feta, fch, mass;
  float cmin, cmax, phimin, phipmax;
  int nonfinite;
};

__device__ __forceinline__ float get_c(const float2& v, int sel) { return sel ? v.y : v.x; }
__device__ __forceinline__ void set_c(float2& v, int sel, float a) {
  if (sel) v.y = a; else v.x = a;
}

template <int PM, int WY>
__device__ __forceinline__ void bulk_cell(float2* smem, int yy, int slot, int sel, const RunParams& rp,
                                          float& dfdc_out, float& mob_out, BulkAcc& acc) {
  const int V = rp.V;
  const float sg1 = rp.sigma1, sg2 = rp.sigma2;
  // pass 1: aggregates.  S2 = sum phi^2, Smat = sum_{i<V-1} phi^2,
  // S4 = sum phi^4, N4 = sum_{i<V-1} phi^4, prefix pair sum for f_eta.
  float S2 = 0.f, Smat = 0.f, S4 = 0.f, N4 = 0.f, pairs = 0.f, pre = 0.f, mabs = 0.f;
  for (int f = 0; f < V - 1; ++f) {
    const float p = get_c(smem[(f * WY + yy) * PM + slot], sel);
    const float p2 = p * p;
    pairs = fmaf(p2, pre, pairs);
    pre += p2;
    N4 = fmaf(p2, p2, N4);
    mabs = fmaxf(mabs, fabsf(p));
  }
  const float pP = get_c(smem[((V - 1) * WY + yy) * PM + slot], sel);
  const float pP2 = pP * pP;
  Smat = pre;
  S2 = pre + pP2;
  S4 = N4 + pP2 * pP2;
  mabs = fmaxf(mabs, fabsf(pP));
  const float c = get_c(smem[(V * WY + yy) * PM + slot], sel);

  // h = N4/S4 and the term4 ratios.  S4 below 1e-30 (|phi| < ~1e-8) would lose
  // precision or underflow in FP32: recompute with phi scaled by 1/max|phi|.
  // All-zero cells give 0/0 in the reference; here they get h = 0, term4 = 0.
  float invS4, n4n, scale_t4;  // term4 factors use (phi^3/S4)*(phiP^4/S4)
  bool scaled = false;
  float inv_m = 1.f;
  if (S4 >= 1e-30f) {
    invS4 = 1.f / S4;
    n4n = N4 * invS4;
    scale_t4 = 4.f;
  } else if (mabs > 0.f) {
    scaled = true;
    inv_m = 1.f / mabs;
    float s4 = 0.f, n4 = 0.f;
    for (int f = 0; f < V - 1; ++f) {
      const float p = get_c(smem[(f * WY + yy) * PM + slot], sel) * inv_m;
      const float p2 = p * p;
      n4 = fmaf(p2, p2, n4);
    }
    const float q = pP * inv_m;
    s4 = n4 + (q * q) * (q * q);
    invS4 = 1.f / s4;
    n4n = n4 * invS4;
    scale_t4 = 4.f * inv_m;
  } else {
    invS4 = 0.f;
    n4n = 0.f;
    scale_t4 = 0.f;
  }
  const float h = n4n;  // phi_mat (:741)
  const float dcm = c - rp.c0m, dcp = c - rp.c0p;
  const float fm = rp.am * dcm * dcm, fp = rp.ap * dcp * dcp;
  const float dfm = fm - fp;
  acc.fch += (double)(h * fm + (1.f - h) * fp);
  dfdc_out = 2.f * h * rp.am * dcm + 2.f * (1.f - h) * rp.ap * dcp;
  acc.feta += (double)(-0.5f * S2 + 0.25f * S4 + sg1 * pairs + sg2 * pP2 * Smat);
  acc.mass += (double)c;
  acc.cmin = fminf(acc.cmin, c);
  acc.cmax = fmaxf(acc.cmax, c);
  acc.phimin = fminf(acc.phimin, S2);
  acc.phipmax = fmaxf(acc.phipmax, pP);
  if (rp.mobility == MOB_REF_VAR) mob_out = 2.f * (1.f - S2) * rp.D_gb;
  else if (rp.mobility == MOB_C1MC) mob_out = rp.D_L * c * (1.f - c);
  else mob_out = 0.f;

  // pass 2: dF/dphi_i = phi^3 - phi + 2 phi Gamma_i + term4_i   (:782-857)
  const float qP = scaled ? pP * inv_m : pP;
  const float qP2 = qP * qP;
  const float rP4 = qP2 * qP2 * invS4;  // phiP^4 / S4 (scaled consistently)
  const float gP = sg2 * pP2;
  int bad = 0;
  for (int f = 0; f < V - 1; ++f) {
    float2& slotv = smem[(f * WY + yy) * PM + slot];
    const float p = get_c(slotv, sel);
    const float gam = fmaf(sg1, Smat - p * p, gP);
    const float q = scaled ? p * inv_m : p;
    const float t4 = scale_t4 * (q * q * q * invS4) * rP4 * dfm;
    const float d = fmaf(p, p * p, -p) + 2.f * p * gam + t4;
    bad |= !isfinite(d);
    set_c(slotv, sel, d);
  }
  {
    float2& slotv = smem[((V - 1) * WY + yy) * PM + slot];
    const float gam = sg2 * Smat;
    const float t4 = -scale_t4 * (qP * qP2 * invS4) * n4n * dfm;
    const float d = fmaf(pP, pP2, -pP) + 2.f * pP * gam + t4;
    bad |= !isfinite(d);
    set_c(slotv, sel, d);
  }
  bad |= !isfinite(dfdc_out);
  acc.nonfinite += bad;
}

// ---------------------------------------------------------------------------
// x pass.  MODE_BULK: S -> D (+ mob, diagnostics).  MODE_XJ: J~ -> J~' with the
// variable-mobility multiply (:947-965).  MODE_IMPORT: real fields -> S.
// MODE_EXPORT: S -> real fields.
// ---------------------------------------------------------------------------
enum XMode { MODE_BULK = 0, MODE_XJ = 1, MODE_IMPORT = 2, MODE_EXPORT = 3 };

template <int NX, int WY, int MODE>
__global__ void __launch_bounds__(256) x_pass_kernel(const RunParams* __restrict__ runs, const Shape sh) {
  constexpr int M = NX / 2;
  using LM = Line<M>;
  constexpr int PM = LM::PITCH;
  constexpr int NPAIR = M / 2 + 1;
  extern __shared__ float2 smem[];
  const RunParams& rp = runs[blockIdx.y];
  const int nF = (MODE == MODE_XJ) ? 1 : rp.V + 1;
  const int ny_tiles = sh.Ny / WY;
  const int z = blockIdx.x / ny_tiles;
  const int y0 = (blockIdx.x - z * ny_tiles) * WY;
  const size_t plane = (size_t)sh.Nz * sh.Ny;
  const size_t fstride = (size_t)sh.Kx * plane;
  const size_t row_off = (size_t)z * sh.Ny + y0;
  const float2* __restrict__ src = (MODE == MODE_XJ) ? rp.J : rp.S;

  if (MODE == MODE_IMPORT) {
    // real rows -> interleaved lines (natural order)
    for (int it = threadIdx.x; it < nF * WY * M; it += blockDim.x) {
      const int m = it % M, r = it / M, yy = r % WY, f = r / WY;
      const float2 v = *reinterpret_cast<const float2*>(rp.fin + (((size_t)f * sh.Nz + z) * sh.Ny + y0 + yy) * NX + 2 * m);
      smem[(f * WY + yy) * PM + LM::phys(m)] = v;
    }
    __syncthreads();
  } else {
    // 1. load the half-spectrum rows, C2R pre-processing
    for (int it = threadIdx.x; it < nF * WY * NPAIR; it += blockDim.x) {
      const int yy = it % WY, r = it / WY, k = r % NPAIR, f = r / NPAIR;
      const float2* sf = src + f * fstride + row_off + yy;
      const float2 xk = sf[(size_t)k * plane];
      const float2 xm = sf[(size_t)(M - k) * plane];
      c2r_pre<M>(smem + (f * WY + yy) * PM, k, xk, xm, sh.twN);
    }
    __syncthreads();
    // 2. inverse x transform -> interleaved real values (natural order)
    fft_inv_lines<M>(smem, nF * WY, PM, sh.twM);
  }

  if (MODE == MODE_EXPORT) {
    for (int it = threadIdx.x; it < nF * WY * M; it += blockDim.x) {
      const int m = it % M, r = it / M, yy = r % WY, f = r / WY;
      *reinterpret_cast<float2*>(rp.fin + (((size_t)f * sh.Nz + z) * sh.Ny + y0 + yy) * NX + 2 * m) =
          smem[(f * WY + yy) * PM + LM::phys(m)];
    }
    return;
  }

  BulkAcc acc;
  acc.feta = 0.0; acc.fch = 0.0; acc.mass = 0.0;
  acc.cmin = 1.0f; acc.cmax = 0.0f; acc.phimin = 1.0f; acc.phipmax = 0.0f;  // reference start values
  acc.nonfinite = 0;

  if (MODE == MODE_BULK) {
    // 3. bulk terms, two cells per slot
    for (int it = threadIdx.x; it < WY * M; it += blockDim.x) {
      const int m = it % M, yy = it / M;
      const int slot = LM::phys(m);
      float dfdc0, dfdc1, mob0, mob1;
      bulk_cell<PM, WY>(smem, yy, slot, 0, rp, dfdc0, mob0, acc);
      bulk_cell<PM, WY>(smem, yy, slot, 1, rp, dfdc1, mob1, acc);
      smem[(rp.V * WY + yy) * PM + slot] = make_float2(dfdc0, dfdc1);
      if (rp.mobility != MOB_CONST)
        *reinterpret_cast<float2*>(rp.mob + ((size_t)z * sh.Ny + y0 + yy) * NX + 2 * m) = make_float2(mob0, mob1);
    }
    __syncthreads();
  } else if (MODE == MODE_XJ) {
    for (int it = threadIdx.x; it < WY * M; it += blockDim.x) {
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

  // 4. forward x transform and 5. R2C post-processing, scaled by 1/Nx
  fft_fwd_lines<M>(smem, nF * WY, PM, sh.twM);
  float2* __restrict__ dst = (MODE == MODE_BULK) ? rp.D : (MODE == MODE_XJ ? rp.J : rp.S);
  const float scale = 1.0f / (float)NX;
  for (int it = threadIdx.x; it < nF * WY * NPAIR; it += blockDim.x) {
    const int yy = it % WY, r = it / WY, k = r % NPAIR, f = r / NPAIR;
    float2 xk, xm;
    r2c_post<M>(smem + (f * WY + yy) * PM, k, scale, sh.twN, xk, xm);
    float2* df = dst + f * fstride + row_off + yy;
    df[(size_t)k * plane] = xk;
    if (2 * k != M) df[(size_t)(M - k) * plane] = xm;
  }

  if (MODE != MODE_BULK) return;

  // 6. diagnostics: block reduction into per-block partials
  __shared__ double red_d[3][8];
  __shared__ float red_f[4][8];
  __shared__ int red_i[8];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  double s0 = warp_sum(acc.feta), s1 = warp_sum(acc.fch), s2 = warp_sum(acc.mass);
  float m0 = warp_min(acc.cmin), m1 = warp_max(acc.cmax), m2 = warp_min(acc.phimin), m3 = warp_max(acc.phipmax);
  int nb = __reduce_add_sync(0xffffffffu, acc.nonfinite);
  if (lane == 0) {
    red_d[0][wid] = s0; red_d[1][wid] = s1; red_d[2][wid] = s2;
    red_f[0][wid] = m0; red_f[1][wid] = m1; red_f[2][wid] = m2; red_f[3][wid] = m3;
    red_i[wid] = nb;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = blockDim.x >> 5;
    double a0 = 0, a1 = 0, a2 = 0;
    float b0 = red_f[0][0], b1 = red_f[1][0], b2 = red_f[2][0], b3 = red_f[3][0];
    int nn = 0;
    for (int w = 0; w < nw; ++w) {
      a0 += red_d[0][w]; a1 += red_d[1][w]; a2 += red_d[2][w];
      b0 = fminf(b0, red_f[0][w]); b1 = fmaxf(b1, red_f[1][w]);
      b2 = fminf(b2, red_f[2][w]); b3 = fmaxf(b3, red_f[3][w]);
      nn += red_i[w];
    }
    const int nbk = sh.nblk_x;
    double* p = rp.part_x + blockIdx.x;
    p[XD_FETA * nbk] = a0;
    p[XD_FCH * nbk] = a1;
    p[XD_MASS * nbk] = a2;
    p[XD_CMIN * nbk] = b0;
    p[XD_CMAX * nbk] = b1;
    p[XD_PHIMIN * nbk] = b2;
    p[XD_PHIPMAX * nbk] = b3;
    p[XD_NONFINITE * nbk] = nn;
  }
}

// ---------------------------------------------------------------------------
// yz pass: 2-D DFT over (y, z) of one kx plane, the spectral update, inverse.
// A cluster of C CTAs shares one plane: CTA r holds z rows [r*NZ/C, ...) for the
// y transforms ("A layout", lines along y) and y positions [r*NY/C, ...) for
// the z transforms ("B layout", lines along z); the two layouts are exchanged
// through distributed shared memory.
// ---------------------------------------------------------------------------
template <int NY, int NZ, int C>
struct YZ {
  static constexpr int LA = NZ / C;
  static constexpr int LB = NY / C;
  static constexpr int PY = Line<NY>::PITCH;
  static constexpr int PZ = Line<NZ>::PITCH;
  static constexpr int UA = LA * PY;
  static constexpr int UB = LB * PZ;
  static constexpr int U = (UA > UB ? UA : UB);
  static constexpr size_t SMEM = 3 * (size_t)U * sizeof(float2);
  static_assert(NZ % C == 0 && NY % C == 0, "cluster must divide the plane");
};

enum YZMode { YZ_MAIN = 0, YZ_C2 = 1 };

template <int C>
__device__ __forceinline__ void cluster_barrier() {
  if constexpr (C == 1) {
    __syncthreads();
  } else {
    cg::this_cluster().sync();
  }
}

// B[yl][phys_z(z)] <- A_{owner(z)}[z % LA][phys_y(r*LB + yl)]
template <int NY, int NZ, int C>
__device__ __forceinline__ void exch_AB(float2* __restrict__ dstB, float2* const* srcA, int r) {
  using G = YZ<NY, NZ, C>;
  constexpr int TOTAL = G::LB * NZ;
  constexpr int K = 4;
  for (int base = threadIdx.x; base < TOTAL; base += blockDim.x * K) {
    float2 v[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int i = base + k * blockDim.x;
      if (i < TOTAL) {
        const int yl = i % G::LB, z = i / G::LB;
        const int owner = z / G::LA, zl = z - owner * G::LA;
        v[k] = srcA[owner][zl * G::PY + Line<NY>::phys(r * G::LB + yl)];
      }
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int i = base + k * blockDim.x;
      if (i < TOTAL) {
        const int yl = i % G::LB, z = i / G::LB;
        dstB[yl * G::PZ + Line<NZ>::phys(z)] = v[k];
      }
    }
  }
}

// A[zl][phys_y(y)] <- B_{owner(y)}[y % LB][phys_z(r*LA + zl)]
template <int NY, int NZ, int C>
__device__ __forceinline__ void exch_BA(float2* __restrict__ dstA, float2* const* srcB, int r) {
  using G = YZ<NY, NZ, C>;
  constexpr int TOTAL = G::LA * NY;
  constexpr int K = 4;
  for (int base = threadIdx.x; base < TOTAL; base += blockDim.x * K) {
    float2 v[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int i = base + k * blockDim.x;
      if (i < TOTAL) {
        const int zl = i % G::LA, y = i / G::LA;
        const int owner = y / G::LB, yl = y - owner * G::LB;
        v[k] = srcB[owner][yl * G::PZ + Line<NZ>::phys(r * G::LA + zl)];
      }
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int i = base + k * blockDim.x;
      if (i < TOTAL) {
        const int zl = i % G::LA, y = i / G::LA;
        dstA[zl * G::PY + Line<NY>::phys(y)] = v[k];
      }
    }
  }
}

// global rows z in [z0, z0+LA) of a plane -> A layout
template <int NY, int NZ, int C>
__device__ __forceinline__ void load_rows(float2* __restrict__ dstA, const float2* __restrict__ plane, int z0) {
  using G = YZ<NY, NZ, C>;
  constexpr int TOTAL = G::LA * NY / 2;
  constexpr int K = 4;
  for (int base = threadIdx.x; base < TOTAL; base += blockDim.x * K) {
    float4 v[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int i = base + k * blockDim.x;
      if (i < TOTAL) {
        const int y2 = i % (NY / 2), zl = i / (NY / 2);
        v[k] = __ldg(reinterpret_cast<const float4*>(plane + (size_t)(z0 + zl) * NY) + y2);
      }
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int i = base + k * blockDim.x;
      if (i < TOTAL) {
        const int y2 = i % (NY / 2), zl = i / (NY / 2);
        float2* d = dstA + zl * G::PY + Line<NY>::phys(2 * y2);
        d[0] = make_float2(v[k].x, v[k].y);
        d[1] = make_float2(v[k].z, v[k].w);  // 2*y2 and 2*y2+1 share a run (N1 even)
      }
    }
  }
}

template <int NY, int NZ, int C, int MODE>
__global__ void __launch_bounds__(512) yz_kernel(const RunParams* __restrict__ runs, const Shape sh) {
  using G = YZ<NY, NZ, C>;
  extern __shared__ float2 smem[];
  __shared__ float2* rU[3][C > 0 ? C : 1];
  __shared__ double red[16];
  float2* U0 = smem;
  float2* U1 = smem + G::U;
  float2* U2 = smem + 2 * G::U;
  const RunParams& rp = runs[blockIdx.y];
  const int r = (C == 1) ? 0 : (int)(blockIdx.x % C);
  const int p = blockIdx.x / C;
  const int Kx = sh.Kx;
  const int f = (MODE == YZ_C2) ? rp.V : p / Kx;
  const int kx = p - (p / Kx) * Kx;
  const size_t plane_elems = (size_t)NZ * NY;
  const size_t fstride = (size_t)Kx * plane_elems;
  const bool is_c = (f == rp.V);
  const bool var_c = is_c && rp.mobility != MOB_CONST;  // variable-mobility c plane
  const int z0 = r * G::LA;

  if (threadIdx.x < C) {
    if constexpr (C == 1) {
      rU[0][0] = U0; rU[1][0] = U1; rU[2][0] = U2;
    } else {
      cg::cluster_group cl = cg::this_cluster();
      rU[0][threadIdx.x] = cl.map_shared_rank(U0, threadIdx.x);
      rU[1][threadIdx.x] = cl.map_shared_rank(U1, threadIdx.x);
      rU[2][threadIdx.x] = cl.map_shared_rank(U2, threadIdx.x);
    }
  }

  // 1. load rows (A layout): u -> U1, D -> U2   (C2 mode: J~' -> U1)
  if (MODE == YZ_MAIN) {
    load_rows<NY, NZ, C>(U1, rp.S + f * fstride + kx * plane_elems, z0);
    load_rows<NY, NZ, C>(U2, rp.D + f * fstride + kx * plane_elems, z0);
  } else {
    load_rows<NY, NZ, C>(U1, rp.J + kx * plane_elems, z0);
  }
  __syncthreads();
  // 2. y transforms
  fft_fwd_lines<NY>(U1, G::LA, G::PY, sh.twY);
  if (MODE == YZ_MAIN) fft_fwd_lines<NY>(U2, G::LA, G::PY, sh.twY);
  cluster_barrier<C>();
  // 3. A -> B exchanges: u -> U0, D -> U1
  exch_AB<NY, NZ, C>(U0, rU[1], r);
  if (MODE == YZ_MAIN) {
    cluster_barrier<C>();
    exch_AB<NY, NZ, C>(U1, rU[2], r);
  }
  __syncthreads();
  // 4. z transforms
  fft_fwd_lines<NZ>(U0, G::LB, G::PZ, sh.twZ);
  if (MODE == YZ_MAIN) fft_fwd_lines<NZ>(U1, G::LB, G::PZ, sh.twZ);

  // 5. spectral update at every (ky, kz) held by this CTA
  const float inv_nyz = 1.0f / (float)(NY * NZ);
  const float qx2 = sh.qx2[kx], qx4 = sh.qx4[kx], qnx = sh.qnx[kx];
  const float wkx = (kx == 0 || 2 * kx == sh.Nx) ? 1.0f : 2.0f;
  float fint = 0.f;
  for (int it = threadIdx.x; it < G::LB * NZ; it += blockDim.x) {
    const int zp = it % NZ, yl = it / NZ;
    const int ky = Line<NY>::freq_of_pos(r * G::LB + yl);
    const int kz = Line<NZ>::freq_of_pos(zp);
    const int a = yl * G::PZ + Line<NZ>::phys(zp);
    const float q2 = qx2 + __ldg(sh.qy2 + ky) + __ldg(sh.qz2 + kz);
    const float qn_y = __ldg(sh.qny + ky), qn_z = __ldg(sh.qnz + kz);
    if (MODE == YZ_MAIN) {
      const float2 u = U0[a];
      const float2 d = U1[a];
      const float kn2 = qnx * qnx + qn_y * qn_y + qn_z * qn_z;
      fint = fmaf(kn2, u.x * u.x + u.y * u.y, fint);
      if (!is_c) {
        // AC, :1015-1024.  den = 1 + L kappa dt q^2
        const float lk = rp.L * rp.dt;
        const float den = fmaf(lk * rp.kappa_phi, q2, 1.0f);
        const float inv = inv_nyz / den;
        const float m1 = -lk * rp.kappa_phi * q2 * inv;
        const float m2 = -lk * inv;
        U0[a] = make_float2(fmaf(m1, u.x, m2 * d.x), fmaf(m1, u.y, m2 * d.y));
      } else {
        // CH, :976-983.  den = 1 + D dt kappa_c K4,  K2 = -q^2
        const float q4 = qx4 + __ldg(sh.qy4 + ky) + __ldg(sh.qz4 + kz);
        const float dd = rp.D_L * rp.dt;
        const float den = fmaf(dd * rp.kappa_c, q4, 1.0f);
        const float inv = inv_nyz / den;
        const float m1 = -dd * rp.kappa_c * q4 * inv;
        const float m2 = -dd * q2 * inv;
        U0[a] = make_float2(fmaf(m1, u.x, m2 * d.x), fmaf(m1, u.y, m2 * d.y));
        if (var_c) {
          // J_hat = G mu_hat - kappa_c c_hat K3 (:932-935), G = i*g, K3 = i*k3
          const float g = qnx + qn_y + qn_z;
          const float k3 = -(qnx * qx2 + qn_y * __ldg(sh.qy2 + ky) + qn_z * __ldg(sh.qz2 + kz));
          // i*(g*d - kappa_c*k3*u) * inv_nyz
          const float2 t = make_float2((g * d.x - rp.kappa_c * k3 * u.x) * inv_nyz,
                                       (g * d.y - rp.kappa_c * k3 * u.y) * inv_nyz);
          U1[a] = cmul_pi(t);
        }
      }
    } else {
      // C2: increment dt G J'_hat / den_c  (:976)
      const float2 jp = U0[a];
      const float q4 = qx4 + __ldg(sh.qy4 + ky) + __ldg(sh.qz4 + kz);
      const float dd = rp.D_L * rp.dt;
      const float den = fmaf(dd * rp.kappa_c, q4, 1.0f);
      const float g = qnx + qn_y + qn_z;
      const float s = rp.dt * g * inv_nyz / den;
      U0[a] = cmul_pi(make_float2(jp.x * s, jp.y * s));
    }
  }
  __syncthreads();
  // 6. inverse z transforms
  fft_inv_lines<NZ>(U0, G::LB, G::PZ, sh.twZ);
  if (MODE == YZ_MAIN && var_c) fft_inv_lines<NZ>(U1, G::LB, G::PZ, sh.twZ);
  cluster_barrier<C>();
  // 7. B -> A exchanges: increment -> U2 (, J_hat -> U0)
  exch_BA<NY, NZ, C>(U2, rU[0], r);
  if (MODE == YZ_MAIN && var_c) {
    cluster_barrier<C>();
    exch_BA<NY, NZ, C>(U0, rU[1], r);
  }
  cluster_barrier<C>();  // no CTA reads a peer's buffers after this point
  // 8. inverse y transforms
  fft_inv_lines<NY>(U2, G::LA, G::PY, sh.twY);
  if (MODE == YZ_MAIN && var_c) fft_inv_lines<NY>(U0, G::LA, G::PY, sh.twY);

  // 9. epilogue
  const bool real_plane = (kx == 0) || (2 * kx == sh.Nx);  // x-DFT of real data is real here
  constexpr int TOT = G::LA * NY / 2;
  if (MODE == YZ_MAIN && var_c) {
    float2* Ag = rp.A + kx * plane_elems;
    float2* Jg = rp.J + kx * plane_elems;
    for (int i = threadIdx.x; i < TOT; i += blockDim.x) {
      const int y2 = i % (NY / 2), zl = i / (NY / 2);
      const int s = zl * G::PY + Line<NY>::phys(2 * y2);
      const size_t g = (size_t)(z0 + zl) * NY + 2 * y2;
      const float2 a0 = U2[s], a1 = U2[s + 1];
      const float2 j0 = U0[s], j1 = U0[s + 1];
      *reinterpret_cast<float4*>(Ag + g) = make_float4(a0.x, a0.y, a1.x, a1.y);
      *reinterpret_cast<float4*>(Jg + g) = make_float4(j0.x, j0.y, j1.x, j1.y);
    }
  } else {
    float2* Sg = rp.S + f * fstride + kx * plane_elems;
    const float2* Ag = (MODE == YZ_C2) ? rp.A + kx * plane_elems : nullptr;
    constexpr int K = 4;
    for (int base = threadIdx.x; base < TOT; base += blockDim.x * K) {
      float4 sv[K], av[K];
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const int i = base + k * blockDim.x;
        if (i < TOT) {
          const int y2 = i % (NY / 2), zl = i / (NY / 2);
          const size_t g = (size_t)(z0 + zl) * NY + 2 * y2;
          sv[k] = *reinterpret_cast<const float4*>(Sg + g);
          if (MODE == YZ_C2) av[k] = *reinterpret_cast<const float4*>(Ag + g);
        }
      }
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const int i = base + k * blockDim.x;
        if (i < TOT) {
          const int y2 = i % (NY / 2), zl = i / (NY / 2);
          const size_t g = (size_t)(z0 + zl) * NY + 2 * y2;
          const int s = zl * G::PY + Line<NY>::phys(2 * y2);
          const float2 d0 = U2[s], d1 = U2[s + 1];
          float4 o = make_float4(sv[k].x + d0.x, sv[k].y + d0.y, sv[k].z + d1.x, sv[k].w + d1.y);
          if (MODE == YZ_C2) { o.x += av[k].x; o.y += av[k].y; o.z += av[k].z; o.w += av[k].w; }
          if (real_plane) { o.y = 0.f; o.w = 0.f; }
          *reinterpret_cast<float4*>(Sg + g) = o;
        }
      }
    }
  }

  if (MODE == YZ_MAIN) {
    // f_int partial (:609-678 by Parseval): 0.5 kappa N^3 w |kf|^2 |u_hat|^2
    double v = warp_sum((double)fint);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) red[wid] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
      const double kap = is_c ? rp.kappa_c : rp.kappa_phi;
      const double n3 = (double)sh.Nx * NY * NZ;
      const double nyz = (double)NY * NZ;
      rp.part_yz[blockIdx.x] = s * wkx * 0.5 * kap * n3 / (nyz * nyz);
    }
  }
}

}  // namespace pf
