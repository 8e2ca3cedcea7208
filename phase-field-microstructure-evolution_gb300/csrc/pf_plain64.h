// Plain FP64 GPU path: cuFFT D2Z/Z2D plus one simple kernel per phase of the
// reference loop body, following its 7*var+9 transforms per step.  It is the
// comparator for the fused FP32 path and an FP64 GPU cross-check of the CPU
// oracle; it is not the performance path.
#pragma once
#include "../../include/pfgpu.h"

namespace pf {
// A run's real-space fields on its device: field f of cell i is
// phi[f * fstride + i * cstride] (float or double), c contiguous; valid on
// `stream` until the run is stepped or destroyed.
struct DeviceFields {
  const void* phi;
  const void* con;
  int is_double;
  size_t fstride, cstride;
  int nx, ny, nz, var, device;
  void* stream;
};
// for either precision path (the fused path first transforms its spectral
// state into its float staging buffer)
int run_device_fields(pf_run* run, DeviceFields* out);

struct Plain64;
int plain64_device_fields(Plain64* p, DeviceFields* out);
int plain64_validate(const pf_config* c);
int plain64_create(const pf_config* c, Plain64** out);
int plain64_set_fields(Plain64* p, const double* phi_aos, const double* con);
int plain64_step(Plain64* p, int nsteps, pf_diag* diag);
int plain64_get_fields(Plain64* p, double* phi_aos, double* con);
void plain64_destroy(Plain64* p);
}  // namespace pf
