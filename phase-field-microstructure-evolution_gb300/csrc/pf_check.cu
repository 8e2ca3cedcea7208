// pf_check_fp64: the error of the fused FP32 path against the plain FP64 GPU
// path for one run -- the same start stepped nsteps times on both, the fields
// compared on the device.  The FP64 path (cuFFT and one kernel per phase of
// src/var_diff.f90:556-1050) is held to the FP64 CPU oracle at 1e-10 by the
// tests, so this is the run's error against an FP64 oracle of the reference's
// algorithm, reported as max-abs and L2 differences relative to the FP64
// fields' max-abs and L2 norms, for the order parameters together and for c.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/pfgpu.h"
#include "pf_internal.h"
#include "pf_plain64.h"

namespace pf {
namespace {

constexpr int kCmpThreads = 256;
constexpr int kCmpBlocks = 1024;
constexpr int kCmpQ = 8;  // per block: max|d|, max|r|, sum d^2, sum r^2 for phi, then for c

__device__ __forceinline__ double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double s = 0;
  if (threadIdx.x == 0)
    for (int i = 0; i < kCmpThreads / 32; ++i) s += sh[i];
  return s;
}
__device__ __forceinline__ double block_max(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double s = 0;
  if (threadIdx.x == 0)
    for (int i = 0; i < kCmpThreads / 32; ++i) s = fmax(s, sh[i]);
  return s;
}

// a: the fused path's FP32 fields, b: the FP64 path's; order parameters
// [field][cell] with field strides afs / bfs, c at a_con / b_con
__global__ void __launch_bounds__(kCmpThreads) compare_kernel(const float* __restrict__ a_phi,
                                                              const float* __restrict__ a_con, size_t afs,
                                                              const double* __restrict__ b_phi,
                                                              const double* __restrict__ b_con, size_t bfs, int V,
                                                              size_t ncell, double* __restrict__ part) {
  __shared__ double sh[kCmpThreads / 32];
  double q[kCmpQ] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int f = 0; f <= V; ++f) {
    const int o = f < V ? 0 : 4;
    const float* a = f < V ? a_phi + (size_t)f * afs : a_con;
    const double* b = f < V ? b_phi + (size_t)f * bfs : b_con;
    for (size_t i = blockIdx.x * (size_t)kCmpThreads + threadIdx.x; i < ncell; i += (size_t)gridDim.x * kCmpThreads) {
      const double r = b[i];
      const double d = (double)a[i] - r;
      q[o] = fmax(q[o], fabs(d));
      q[o + 1] = fmax(q[o + 1], fabs(r));
      q[o + 2] += d * d;
      q[o + 3] += r * r;
    }
  }
  for (int k = 0; k < kCmpQ; ++k) {
    const double v = (k % 4 < 2) ? block_max(q[k], sh) : block_sum(q[k], sh);
    if (threadIdx.x == 0) part[(size_t)blockIdx.x * kCmpQ + k] = v;
  }
}

}  // namespace
}  // namespace pf

using namespace pf;

extern "C" int pf_check_fp64(const pf_config* cfg, const double* phi_aos, const double* con, int nsteps,
                             pf_error_report* out) {
  if (!cfg || !phi_aos || !con || !out || nsteps < 0) {
    set_error("pf_check_fp64: bad arguments");
    return PF_EINVAL;
  }
  pf_config c32 = *cfg, c64 = *cfg;
  c32.precision = PF_FP32_FUSED;
  c64.precision = PF_FP64_PLAIN;
  pf_run *r32 = nullptr, *r64 = nullptr;
  double* dpart = nullptr;
  int rc = pf_create(&c32, &r32);
  if (rc == PF_OK) rc = pf_create(&c64, &r64);
  if (rc == PF_OK) rc = pf_set_fields(r32, phi_aos, con);
  if (rc == PF_OK) rc = pf_set_fields(r64, phi_aos, con);
  if (rc == PF_OK && nsteps > 0) rc = pf_step(r32, nsteps, nullptr);
  if (rc == PF_OK && nsteps > 0) rc = pf_step(r64, nsteps, nullptr);
  DeviceFields fa{}, fb{};
  if (rc == PF_OK) rc = run_device_fields(r32, &fa);
  if (rc == PF_OK) rc = run_device_fields(r64, &fb);
  if (rc == PF_OK) {
    const size_t ncell = (size_t)cfg->nx * cfg->ny * cfg->nz;
    cudaError_t e = cudaSetDevice(cfg->device);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();  // both paths' fields in place
    if (e == cudaSuccess) e = cudaMalloc(&dpart, (size_t)kCmpBlocks * kCmpQ * sizeof(double));
    if (e == cudaSuccess && (fa.is_double || !fb.is_double || fa.cstride != 1 || fb.cstride != 1))
      e = cudaErrorInvalidValue;  // not the two layouts this comparison reads
    if (e == cudaSuccess) {
      compare_kernel<<<kCmpBlocks, kCmpThreads>>>((const float*)fa.phi, (const float*)fa.con, fa.fstride,
                                                  (const double*)fb.phi, (const double*)fb.con, fb.fstride, cfg->var,
                                                  ncell, dpart);
      e = cudaGetLastError();
    }
    std::vector<double> h((size_t)kCmpBlocks * kCmpQ);
    if (e == cudaSuccess) e = cudaMemcpy(h.data(), dpart, h.size() * sizeof(double), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
      set_error(std::string("pf_check_fp64: ") + cudaGetErrorString(e));
      rc = PF_ECUDA;
    } else {
      double q[kCmpQ] = {0, 0, 0, 0, 0, 0, 0, 0};
      for (int bk = 0; bk < kCmpBlocks; ++bk)
        for (int k = 0; k < kCmpQ; ++k) {
          const double v = h[(size_t)bk * kCmpQ + k];
          q[k] = (k % 4 < 2) ? std::max(q[k], v) : q[k] + v;
        }
      out->steps = nsteps;
      out->phi_max_abs_rel = q[0] / std::max(q[1], 1e-300);
      out->phi_l2_rel = std::sqrt(q[2] / std::max(q[3], 1e-300));
      out->c_max_abs_rel = q[4] / std::max(q[5], 1e-300);
      out->c_l2_rel = std::sqrt(q[6] / std::max(q[7], 1e-300));
    }
  }
  if (dpart) cudaFree(dpart);
  const std::string keep = pf_last_error();
  if (r32) pf_destroy(r32);
  if (r64) pf_destroy(r64);
  if (rc != PF_OK) set_error(keep);
  return rc;
}
