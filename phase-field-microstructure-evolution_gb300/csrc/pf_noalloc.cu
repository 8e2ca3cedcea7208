// pf_diag_fields_noalloc: the diagnostics of the x pass (f_eta, f_ch, mass and
// the statistics c_min, c_max, phi_min, phi_P_max of src/var_diff.f90:685-759,
// :1076-1102) for fields a caller already holds in device memory, with no
// device allocation at all.
//
// Who needs it: hosts that may not call cudaMalloc -- for example a Fortran or
// C driver whose device memory is owned by another runtime's pool allocator,
// code running inside a region where allocation is forbidden (a memory-capped
// service process, a callback of another library), or a caller that wants a
// fixed, up-front device footprint.  pf_create/pf_step allocate their
// buffers; this entry point instead keeps its scratch (the per-block partial
// sums and the final record) in a file-scope __device__ array that exists on
// every GPU that loads the library, from load until process exit.
//
// Contract (also in include/pfgpu.h):
//  * fields: float [var+1][nz][ny][nx] in device memory, phi_1..phi_var then c;
//  * at most PF_NOALLOC_MAX_CELLS cells (larger grids are rejected);
//  * every call looks the scratch address up in the caller's current context
//    (cudaGetSymbolAddress allocates nothing), so a host that switches
//    contexts itself still gets that context's copy of the array;
//  * the call copies its result to the host and waits for it, so it may not be
//    made on a stream that is being captured into a graph (rejected);
//  * every call shares the scratch: calls that overlap on the GPU (two streams
//    or two host threads at once) race.  Each call writes every partial it
//    reads, so nothing has to be cleared between calls.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>

#include "../../include/pfgpu.h"
#include "pf_internal.h"

namespace pf {
namespace {

constexpr int kThreads = 256;
constexpr int kCellsPerThread = 8;
constexpr int kMaxBlocks = (PF_NOALLOC_MAX_CELLS + kThreads * kCellsPerThread - 1) / (kThreads * kCellsPerThread);
constexpr int kQ = 8;  // partials per block: f_eta, f_ch, mass, nonfinite, c_min, c_max, phi_min, phi_P_max

// kMaxBlocks * kQ doubles (512 KiB) of partials + one record, per device.
__device__ __align__(256) double g_noalloc_scratch[kMaxBlocks * kQ + 16];

struct Coef {
  float am, ap, c0m, c0p, sigma1, sigma2;
};

__device__ __forceinline__ float warp_sum_f32(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__global__ void __launch_bounds__(kThreads) noalloc_cells_kernel(const float* __restrict__ fld, int V, size_t ncell,
                                                                 Coef k, double* __restrict__ part) {
  float feta = 0.f, fch = 0.f;
  FF mass{0.f, 0.f};  // compensated sum of c
  float cmin = 1.f, cmax = 0.f, pmin = 1.f, ppmax = 0.f;  // reference start values
  int bad = 0;
  for (size_t i = blockIdx.x * (size_t)kThreads + threadIdx.x; i < ncell; i += (size_t)gridDim.x * kThreads) {
    float pre = 0.f, n4 = 0.f, pairs = 0.f, mabs = 0.f;
    bool fin = true;  // every value of the cell finite (tested value by value)
    for (int f = 0; f < V - 1; ++f) {
      const float p = fld[(size_t)f * ncell + i];
      const float a = p * p;
      pairs = fmaf(a, pre, pairs);
      pre += a;
      n4 = fmaf(a, a, n4);
      mabs = fmaxf(mabs, fabsf(p));
      fin = fin && isfinite(p);
    }
    const float pp = fld[(size_t)(V - 1) * ncell + i];
    const float c = fld[(size_t)V * ncell + i];
    fin = fin && isfinite(pp) && isfinite(c);
    mabs = fmaxf(mabs, fabsf(pp));
    const float pp2 = pp * pp, S2 = pre + pp2, S4 = n4 + pp2 * pp2;
    // h = N4/S4, rescaled by 1/max|phi| below S4 = 1e-30 as in the x pass
    float h;
    if (S4 >= 1e-30f) {
      h = n4 / S4;
    } else if (mabs > 0.f) {
      const float im = 1.f / mabs;
      float nn = 0.f;
      for (int f = 0; f < V - 1; ++f) {
        const float x = fld[(size_t)f * ncell + i] * im;
        nn = fmaf(x * x, x * x, nn);
      }
      const float xq = pp * im;
      h = nn / (nn + (xq * xq) * (xq * xq));
    } else {
      h = 0.f;
    }
    const float dcm = c - k.c0m, dcp = c - k.c0p;
    fch += h * k.am * dcm * dcm + (1.f - h) * k.ap * dcp * dcp;
    feta += -0.5f * S2 + 0.25f * S4 + k.sigma1 * pairs + k.sigma2 * pp2 * pre;
    mass.add(c);
    cmin = fminf(cmin, c);
    cmax = fmaxf(cmax, c);
    pmin = fminf(pmin, S2);
    ppmax = fmaxf(ppmax, pp);
    bad += !fin;
  }
  __shared__ double sd[4][kThreads / 32];
  __shared__ float sf[4][kThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const double s0 = warp_sum_f32(feta), s1 = warp_sum_f32(fch), s2 = warp_sum_ff(mass).value();
  const double s3 = (double)__reduce_add_sync(0xffffffffu, bad);
  const float m0 = warp_min(cmin), m1 = warp_max(cmax), m2 = warp_min(pmin), m3 = warp_max(ppmax);
  if (lane == 0) {
    sd[0][w] = s0; sd[1][w] = s1; sd[2][w] = s2; sd[3][w] = s3;
    sf[0][w] = m0; sf[1][w] = m1; sf[2][w] = m2; sf[3][w] = m3;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a[4] = {0, 0, 0, 0};
    KSum am;
    float m[4] = {1.f, 0.f, 1.f, 0.f};
    for (int q = 0; q < kThreads / 32; ++q) {
      a[0] += sd[0][q]; a[1] += sd[1][q]; a[3] += sd[3][q];
      am.add(sd[2][q]);
      m[0] = fminf(m[0], sf[0][q]); m[1] = fmaxf(m[1], sf[1][q]);
      m[2] = fminf(m[2], sf[2][q]); m[3] = fmaxf(m[3], sf[3][q]);
    }
    a[2] = am.value();
    double* o = part + (size_t)blockIdx.x * kQ;
    o[0] = a[0]; o[1] = a[1]; o[2] = a[2]; o[3] = a[3];
    o[4] = m[0]; o[5] = m[1]; o[6] = m[2]; o[7] = m[3];
  }
}

// one block: fixed-order sums of the block partials into the record slot
// (the mass with compensation)
__global__ void __launch_bounds__(kThreads) noalloc_final_kernel(const double* __restrict__ part, int nblocks,
                                                                 double* __restrict__ rec) {
  __shared__ double sd[5][kThreads];
  __shared__ double sm[4][kThreads];
  const int t = threadIdx.x;
  double a[3] = {0, 0, 0}, m[4] = {1.0, 0.0, 1.0, 0.0};
  KSum mass;
  for (int b = t; b < nblocks; b += kThreads) {
    const double* o = part + (size_t)b * kQ;
    a[0] += o[0]; a[1] += o[1]; a[2] += o[3];
    mass.add(o[2]);
    m[0] = fmin(m[0], o[4]); m[1] = fmax(m[1], o[5]); m[2] = fmin(m[2], o[6]); m[3] = fmax(m[3], o[7]);
  }
  sd[0][t] = a[0]; sd[1][t] = a[1]; sd[2][t] = a[2]; sd[3][t] = mass.s; sd[4][t] = mass.c;
  for (int j = 0; j < 4; ++j) sm[j][t] = m[j];
  __syncthreads();
  for (int s = kThreads / 2; s > 0; s >>= 1) {
    if (t < s) {
      for (int j = 0; j < 3; ++j) sd[j][t] += sd[j][t + s];
      KSum x, y;
      x.s = sd[3][t]; x.c = sd[4][t];
      y.s = sd[3][t + s]; y.c = sd[4][t + s];
      x.add(y);
      sd[3][t] = x.s; sd[4][t] = x.c;
      sm[0][t] = fmin(sm[0][t], sm[0][t + s]); sm[1][t] = fmax(sm[1][t], sm[1][t + s]);
      sm[2][t] = fmin(sm[2][t], sm[2][t + s]); sm[3][t] = fmax(sm[3][t], sm[3][t + s]);
    }
    __syncthreads();
  }
  if (t == 0) {
    KSum x;
    x.s = sd[3][0]; x.c = sd[4][0];
    rec[0] = sd[0][0]; rec[1] = sd[1][0]; rec[2] = x.value(); rec[3] = sd[2][0];
    for (int j = 0; j < 4; ++j) rec[4 + j] = sm[j][0];
  }
}

// Device address of the scratch array in the calling thread's current
// context.  Looked up on every call: it allocates nothing and is cheap, and a
// host that makes its own contexts current gets the right copy each time.
int scratch_in_current_context(double** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p) {
    set_error(std::string("pf_diag_fields_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    return PF_ECUDA;
  }
  *out = static_cast<double*>(p);
  return PF_OK;
}

}  // namespace
}  // namespace pf

extern "C" int pf_diag_fields_noalloc(const pf_config* cfg, const float* d_fields, pf_diag* out, void* stream) {
  using namespace pf;
  if (!cfg || !d_fields || !out) {
    set_error("pf_diag_fields_noalloc: null argument");
    return PF_EINVAL;
  }
  if (cfg->nx < 1 || cfg->ny < 1 || cfg->nz < 1 || cfg->var < 1) {
    set_error("pf_diag_fields_noalloc: bad grid or var");
    return PF_EINVAL;
  }
  const double cells = (double)cfg->nx * cfg->ny * cfg->nz;
  if (cells > (double)PF_NOALLOC_MAX_CELLS) {
    char buf[160];
    snprintf(buf, sizeof buf, "pf_diag_fields_noalloc: %d x %d x %d cells exceed the limit of %d (scratch is fixed)",
             cfg->nx, cfg->ny, cfg->nz, PF_NOALLOC_MAX_CELLS);
    set_error(buf);
    return PF_EINVAL;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // the call waits for its result on the host: never on a capturing stream
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaError_t ce = cudaStreamIsCapturing(s, &cap);
  if (ce != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
    cudaGetLastError();
    set_error("pf_diag_fields_noalloc: the stream is being captured (or its capture state is unknown); "
              "this call copies its result to the host and may not be captured");
    return PF_EINVAL;
  }
  double* scratch = nullptr;
  int rc = scratch_in_current_context(&scratch);
  if (rc) return rc;
  const size_t ncell = (size_t)cells;
  const int nblocks = (int)std::min<size_t>((size_t)kMaxBlocks, (ncell + kThreads - 1) / kThreads);
  Coef k{(float)cfg->am, (float)cfg->ap, (float)cfg->con_0_mat, (float)cfg->con_0_ppt, (float)cfg->sigma_1,
         (float)cfg->sigma_2};
  double* rec = scratch + (size_t)kMaxBlocks * kQ;
  noalloc_cells_kernel<<<nblocks, kThreads, 0, s>>>(d_fields, cfg->var, ncell, k, scratch);
  noalloc_final_kernel<<<1, kThreads, 0, s>>>(scratch, nblocks, rec);
  double h[8];
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, rec, sizeof h, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    set_error(std::string("pf_diag_fields_noalloc: ") + cudaGetErrorString(e));
    return PF_ECUDA;
  }
  out->step = 0;
  out->nonfinite = (int)h[3];  // cells with a non-finite value
  out->f_int = NAN;  // needs the spectral transform: not computed here
  out->f_eta = h[0];
  out->f_ch = h[1];
  out->e_tot = NAN;
  out->mass = h[2];  // compensated sum
  out->c_min = h[4];
  out->c_max = h[5];
  out->phi_min = h[6];
  out->phi_P_max = h[7];
  return out->nonfinite ? PF_ENONFINITE : PF_OK;
}
