// Voxel analysis of the post-processor paraview.x (src/paraview.f90) on the GPU.
//
// Per voxel (src/paraview.f90:189-244), in FP64 with the reference's order
// of operations (no contraction into FMA, so results are bit-identical to a
// plain loop):
//   phi_sq   = sum_{i=1..var} phi_i^2
//   var_num  = the last i with phi_i > 0.8 (0 if none)
//   phi_3    = phi_3 (the index 3 is fixed in the reference, whatever var is)
//   boundary = 1 if more than one phi_i > threshold, else 0
// and two counts: boundary voxels, and boundary voxels with phi_var > threshold.
// |grad phi_3| (src/paraview.f90:380-429): central differences / 2 on the
// interior cells 2..N-1 of every axis, 0 on the outer layer.
//
// One HBM pass each (the classification reads var+1 values and writes up to
// four per voxel; the gradient reads phi_3 with its six neighbours through L1
// and L2 and writes one value), grid-stride loops over 152 SMs x 8 blocks,
// counts reduced per block and added once per block (integers: the result
// does not depend on the order).
#include <cuda_runtime.h>

#include <cstdio>
#include <string>

#include "../../include/pfgpu.h"
#include "pf_internal.h"
#include "pf_plain64.h"

namespace pf {
namespace {

constexpr int kThreads = 256;

// Source fields: value of field f at cell i is base[f * fstride + i * cstride].
template <typename T>
struct Src {
  const T* phi;
  const T* con;
  size_t fstride, cstride;
  __device__ __forceinline__ double at(int f, size_t i) const { return (double)phi[f * fstride + i * cstride]; }
};

template <typename T>
__global__ void __launch_bounds__(kThreads) classify_kernel(Src<T> s, int V, size_t n, double thr, double* phi_sq,
                                                            int* var_num, double* phi3, double* boundary,
                                                            double* con_out, unsigned long long* counts) {
  unsigned nb = 0, np = 0;
  for (size_t i = blockIdx.x * (size_t)kThreads + threadIdx.x; i < n; i += (size_t)gridDim.x * kThreads) {
    double sq = 0.0;
    int vmax = 0, above = 0;
    for (int f = 0; f < V; ++f) {
      const double p = s.at(f, i);
      sq = __dadd_rn(sq, __dmul_rn(p, p));
      if (p > 0.8) vmax = f + 1;
      above += p > thr;
    }
    const bool b = above > 1;
    nb += b;
    np += b && s.at(V - 1, i) > thr;
    if (phi_sq) phi_sq[i] = sq;
    if (var_num) var_num[i] = vmax;
    if (phi3) phi3[i] = s.at(2, i);
    if (boundary) boundary[i] = b ? 1.0 : 0.0;
    if (con_out) con_out[i] = (double)s.con[i];  // c is contiguous in both layouts
  }
  nb = __reduce_add_sync(0xffffffffu, nb);
  np = __reduce_add_sync(0xffffffffu, np);
  __shared__ unsigned sb[kThreads / 32], sp[kThreads / 32];
  if ((threadIdx.x & 31) == 0) {
    sb[threadIdx.x >> 5] = nb;
    sp[threadIdx.x >> 5] = np;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long tb = 0, tp = 0;
    for (int w = 0; w < kThreads / 32; ++w) {
      tb += sb[w];
      tp += sp[w];
    }
    if (tb) atomicAdd(&counts[0], tb);
    if (tp) atomicAdd(&counts[1], tp);
  }
}

template <typename T>
__global__ void __launch_bounds__(kThreads) grad3_kernel(Src<T> s, int Nx, int Ny, int Nz, double* grad) {
  const size_t n = (size_t)Nx * Ny * Nz;
  const size_t sx = 1, sy = (size_t)Nx, sz = (size_t)Nx * Ny;
  for (size_t i = blockIdx.x * (size_t)kThreads + threadIdx.x; i < n; i += (size_t)gridDim.x * kThreads) {
    const int x = (int)(i % Nx), y = (int)((i / Nx) % Ny), z = (int)(i / sz);
    double g = 0.0;
    if (x > 0 && x < Nx - 1 && y > 0 && y < Ny - 1 && z > 0 && z < Nz - 1) {
      const double gx = __ddiv_rn(__dsub_rn(s.at(2, i + sx), s.at(2, i - sx)), 2.0);
      const double gy = __ddiv_rn(__dsub_rn(s.at(2, i + sy), s.at(2, i - sy)), 2.0);
      const double gz = __ddiv_rn(__dsub_rn(s.at(2, i + sz), s.at(2, i - sz)), 2.0);
      g = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(gx, gx), __dmul_rn(gy, gy)), __dmul_rn(gz, gz)));
    }
    grad[i] = g;
  }
}

int grid_for(size_t n) {
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t want = (n + kThreads - 1) / kThreads;
  return (int)std::min<size_t>(want, (size_t)sms * 8);
}

// Device outputs of one analysis; any host pointer may be NULL.
struct Outs {
  double *phi_sq, *phi_3, *grad, *boundary, *con;
  int* var_num;
};

#define AN_CUDA(call)                                                                  \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess) {                                                           \
      set_error(std::string("analysis: ") + #call + ": " + cudaGetErrorString(e_));   \
      rc = PF_ECUDA;                                                                   \
      goto done;                                                                       \
    }                                                                                  \
  } while (0)

template <typename T>
int analyze(const Src<T>& src, int Nx, int Ny, int Nz, int V, double thr, cudaStream_t st, const pf_analysis_out* ho,
            pf_voxel_counts* counts) {
  const size_t n = (size_t)Nx * Ny * Nz;
  int rc = PF_OK;
  Outs d{};
  unsigned long long* dcnt = nullptr;
  unsigned long long hc[2] = {0, 0};
  const int grid = grid_for(n);
  AN_CUDA(cudaMalloc(&dcnt, 2 * sizeof(unsigned long long)));
  AN_CUDA(cudaMemsetAsync(dcnt, 0, 2 * sizeof(unsigned long long), st));
  if (ho && ho->phi_sq) AN_CUDA(cudaMalloc(&d.phi_sq, n * sizeof(double)));
  if (ho && ho->var_num) AN_CUDA(cudaMalloc(&d.var_num, n * sizeof(int)));
  if (ho && ho->phi_3) AN_CUDA(cudaMalloc(&d.phi_3, n * sizeof(double)));
  if (ho && ho->grad_phi_3) AN_CUDA(cudaMalloc(&d.grad, n * sizeof(double)));
  if (ho && ho->boundary) AN_CUDA(cudaMalloc(&d.boundary, n * sizeof(double)));
  if (ho && ho->con) AN_CUDA(cudaMalloc(&d.con, n * sizeof(double)));
  classify_kernel<T><<<grid, kThreads, 0, st>>>(src, V, n, thr, d.phi_sq, d.var_num, d.phi_3, d.boundary, d.con,
                                                dcnt);
  AN_CUDA(cudaGetLastError());
  if (d.grad) {
    grad3_kernel<T><<<grid, kThreads, 0, st>>>(src, Nx, Ny, Nz, d.grad);
    AN_CUDA(cudaGetLastError());
  }
  AN_CUDA(cudaMemcpyAsync(hc, dcnt, sizeof hc, cudaMemcpyDeviceToHost, st));
  if (d.phi_sq) AN_CUDA(cudaMemcpyAsync(ho->phi_sq, d.phi_sq, n * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (d.var_num) AN_CUDA(cudaMemcpyAsync(ho->var_num, d.var_num, n * sizeof(int), cudaMemcpyDeviceToHost, st));
  if (d.phi_3) AN_CUDA(cudaMemcpyAsync(ho->phi_3, d.phi_3, n * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (d.grad) AN_CUDA(cudaMemcpyAsync(ho->grad_phi_3, d.grad, n * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (d.boundary) AN_CUDA(cudaMemcpyAsync(ho->boundary, d.boundary, n * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (d.con) AN_CUDA(cudaMemcpyAsync(ho->con, d.con, n * sizeof(double), cudaMemcpyDeviceToHost, st));
  AN_CUDA(cudaStreamSynchronize(st));
  counts->boundary_voxels = (long long)hc[0];
  counts->precipitate_voxels = (long long)hc[1];
  counts->precipitate_fraction = hc[0] ? (double)hc[1] / (double)hc[0] : 0.0;
done:
  cudaFree(dcnt);
  cudaFree(d.phi_sq);
  cudaFree(d.var_num);
  cudaFree(d.phi_3);
  cudaFree(d.grad);
  cudaFree(d.boundary);
  cudaFree(d.con);
  return rc;
}

int check_args(const pf_config* c, pf_voxel_counts* counts) {
  if (!c || !counts) {
    set_error("analysis: null argument");
    return PF_EINVAL;
  }
  if (c->nx < 1 || c->ny < 1 || c->nz < 1 || c->var < 3) {
    set_error("analysis: needs a grid and var >= 3 (phi_3 is analysed)");
    return PF_EINVAL;
  }
  return PF_OK;
}

}  // namespace
}  // namespace pf

extern "C" int pf_analyze_fields(const pf_config* cfg, const double* phi_aos, const double* con, double threshold,
                                 const pf_analysis_out* out, pf_voxel_counts* counts) {
  using namespace pf;
  int rc = check_args(cfg, counts);
  if (rc) return rc;
  if (!phi_aos || !con) {
    set_error("analysis: null field");
    return PF_EINVAL;
  }
  const size_t n = (size_t)cfg->nx * cfg->ny * cfg->nz;
  const int V = cfg->var;
  double *dphi = nullptr, *dcon = nullptr;
  cudaStream_t st = nullptr;
  {
    cudaError_t e = cudaSetDevice(cfg->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&dphi, n * V * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&dcon, n * sizeof(double));
    if (e == cudaSuccess) e = cudaMemcpyAsync(dphi, phi_aos, n * V * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dcon, con, n * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) {
      set_error(std::string("analysis: ") + cudaGetErrorString(e));
      rc = e == cudaErrorMemoryAllocation ? PF_ENOMEM : PF_ECUDA;
    }
  }
  if (!rc) {
    Src<double> s{dphi, dcon, 1, (size_t)V};
    rc = analyze(s, cfg->nx, cfg->ny, cfg->nz, V, threshold, st, out, counts);
  }
  cudaFree(dphi);
  cudaFree(dcon);
  if (st) cudaStreamDestroy(st);
  return rc;
}

// In-situ analysis of a run's resident fields (no host copy of the fields).
extern "C" int pf_analyze_run(pf_run* run, double threshold, const pf_analysis_out* out, pf_voxel_counts* counts) {
  using namespace pf;
  DeviceFields f{};
  int rc = run_device_fields(run, &f);
  if (rc) return rc;
  pf_config c{};
  c.nx = f.nx; c.ny = f.ny; c.nz = f.nz; c.var = f.var; c.device = f.device;
  rc = check_args(&c, counts);
  if (rc) return rc;
  if (f.is_double) {
    Src<double> s{(const double*)f.phi, (const double*)f.con, f.fstride, f.cstride};
    return analyze(s, f.nx, f.ny, f.nz, f.var, threshold, (cudaStream_t)f.stream, out, counts);
  }
  Src<float> s{(const float*)f.phi, (const float*)f.con, f.fstride, f.cstride};
  return analyze(s, f.nx, f.ny, f.nz, f.var, threshold, (cudaStream_t)f.stream, out, counts);
}
