// Host-side declarations shared by the kernel translation units and the API.
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "pf_kernels.cuh"

namespace pf {

typedef void (*KernelFn)(const RunParams*, const Shape);

struct XKernels {
  KernelFn bulk, xj, imp, exp;
  int wy;  // y rows per CTA
};

struct YZKernels {
  KernelFn main, c2, imp;  // modes YZ_MAIN, YZ_C2, YZ_IMPORT
  int cluster;   // CTAs per plane
  int threads;   // threads per CTA
  size_t smem;   // dynamic shared memory per CTA
};

// implemented in pf_x.cu / pf_yz_*.cu
bool get_x_kernels(int nx, XKernels* out);
bool get_yz_kernels_small(int ny, int nz, YZKernels* out);
bool get_yz_kernels_128(int ny, int nz, YZKernels* out);
bool get_yz_kernels_256(int ny, int nz, YZKernels* out);

inline bool get_yz_kernels(int ny, int nz, YZKernels* out) {
  return get_yz_kernels_small(ny, nz, out) || get_yz_kernels_128(ny, nz, out) ||
         get_yz_kernels_256(ny, nz, out);
}

// x-pass shared memory for nF fields
template <int NX>
constexpr size_t x_smem_bytes(int nF, int wy) {
  return (size_t)nF * wy * Line<NX / 2>::PITCH * sizeof(float2);
}

void set_error(const std::string& msg);

}  // namespace pf
