// Instantiations of the x pass for the rest of the reference's weak-scaling
// grids (inputs/config.yaml:71-106): 80, 160 and 200 (x lines of M = Nx/2 =
// 40, 80, 100 complex points, plans 8 x 5, 16 x 5, 10 x 10) and 102 (M = 51,
// plan 3 x 17).  The first variant of a size is its default; the autotuner
// picks among them.
#include "pf_internal.h"

namespace pf {

template <int NX, int WY, int T>
static int add(XKernels* out, int n) {
  if (n >= kMaxVariants) return n;
  XKernels& k = out[n];
  k.bulk = x_pass_kernel<NX, WY, T, MODE_BULK>;
  k.xj = x_pass_kernel<NX, WY, T, MODE_XJ>;
  k.imp = x_pass_kernel<NX, WY, T, MODE_IMPORT>;
  k.exp = x_pass_kernel<NX, WY, T, MODE_EXPORT>;
  k.wy = WY;
  k.threads = T;
  k.cl = 0;
  k.tma = 0;
  k.bulk_smem = nullptr;
  return n + 1;
}

template <int NX, int WY>
static size_t cl_smem(int nF) {
  return XCL<NX, WY>::smem(nF);
}

template <int NX, int WY, int T>
static int addcl(XKernels* out, int n) {
  if (n >= kMaxVariants) return n;
  n = add<NX, WY, T>(out, n);
  XKernels& k = out[n - 1];
  k.bulk = x_pass_cl_kernel<NX, WY, T>;
  k.cl = 2;
  k.bulk_smem = cl_smem<NX, WY>;
  return n;
}

int x_variants_r5(int nx, XKernels* out, int n) {
  switch (nx) {
    case 80: n = add<80, 8, 256>(out, n); n = add<80, 4, 256>(out, n); n = add<80, 16, 256>(out, n); break;
    case 160:
      n = add<160, 4, 256>(out, n); n = add<160, 8, 256>(out, n); n = add<160, 4, 512>(out, n);
      n = addcl<160, 4, 256>(out, n);
      break;
    case 200:
      n = add<200, 4, 256>(out, n); n = add<200, 8, 256>(out, n); n = add<200, 2, 256>(out, n);
      n = addcl<200, 4, 256>(out, n);
      break;
    case 102: n = add<102, 6, 256>(out, n); n = add<102, 2, 256>(out, n); n = add<102, 3, 256>(out, n); break;
    default: break;
  }
  return n;
}

}  // namespace pf
