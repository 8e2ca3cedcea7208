// Host-side declarations shared by the kernel translation units and the API.
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "pf_kernels.cuh"

namespace pf {

typedef void (*KernelFn)(const RunParams*, const Shape);

// One compiled variant of the x pass (all four modes) ...
struct XKernels {
  KernelFn bulk, xj, imp, exp;
  int wy;       // y rows per CTA
  int threads;  // threads per CTA
  int cl = 0;   // 2: the bulk kernel runs as clusters of two CTAs sharing the fields (x_pass_cl_kernel)
  int tma = 0;  // > 0: the bulk kernel is the persistent TMA-staged x_pass_tma_kernel, at most this many CTAs per SM
  size_t (*bulk_smem)(int nF) = nullptr;  // its dynamic shared memory (cluster and TMA variants)
  const char* tag = "";  // how the tile is loaded and walked, for reports
};

// ... and of the yz pass (all three modes).
struct YZKernels {
  KernelFn main, c2, imp;  // modes YZ_MAIN, YZ_C2, YZ_IMPORT
  int cluster;   // CTAs per plane
  int threads;   // threads per CTA
  size_t smem;   // dynamic shared memory per CTA
  int inpl = 0;  // 1: the cluster exchanges the plane in place (one buffer per CTA)
  int pref = 0;  // 1: the main kernel prefetches the next generation's planes into L2 (Shape::pref_yz)
};

// Variant lists: each translation unit appends the variants it compiled for a
// shape to `out` (room for kMaxVariants entries) and returns the new count.  The first variant of a shape is its
// default; the run-creation autotuner times the others.
constexpr int kMaxVariants = 20;
int x_variants_a(int nx, XKernels* out, int n);
int x_variants_r5(int nx, XKernels* out, int n);
int yz_variants_small(int ny, int nz, YZKernels* out, int n);
int yz_variants_128a(int ny, int nz, YZKernels* out, int n);
int yz_variants_128b(int ny, int nz, YZKernels* out, int n);
int yz_variants_256a(int ny, int nz, YZKernels* out, int n);
int yz_variants_256b(int ny, int nz, YZKernels* out, int n);
int yz_variants_r5(int ny, int nz, YZKernels* out, int n);

inline int get_x_variants(int nx, XKernels* out) { return x_variants_r5(nx, out, x_variants_a(nx, out, 0)); }
inline int get_yz_variants(int ny, int nz, YZKernels* out) {
  int n = 0;
  n = yz_variants_small(ny, nz, out, n);
  n = yz_variants_128a(ny, nz, out, n);
  n = yz_variants_128b(ny, nz, out, n);
  n = yz_variants_256a(ny, nz, out, n);
  n = yz_variants_256b(ny, nz, out, n);
  n = yz_variants_r5(ny, nz, out, n);
  return n;
}
// default (first) variant of a shape; `out` receives one entry
inline bool get_x_kernels(int nx, XKernels* out) {
  XKernels v[kMaxVariants];
  if (get_x_variants(nx, v) == 0) return false;
  *out = v[0];
  return true;
}
inline bool get_yz_kernels(int ny, int nz, YZKernels* out) {
  YZKernels v[kMaxVariants];
  if (get_yz_variants(ny, nz, v) == 0) return false;
  *out = v[0];
  return true;
}

// x-pass shared memory for nF fields
template <int NX>
constexpr size_t x_smem_bytes(int nF, int wy) {
  return (size_t)nF * wy * XLine<NX / 2>::PITCH * sizeof(float2);
}

void set_error(const std::string& msg);

}  // namespace pf
