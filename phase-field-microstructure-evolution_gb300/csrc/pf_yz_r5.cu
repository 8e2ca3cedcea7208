// yz-pass instantiations for the rest of the reference's weak-scaling grids:
// 80^2, 160^2, 200^2 planes (lines of 16 x 5, 16 x 10 and 20 x 10) and 102^2
// (lines of 6 x 17).  80^2, 102^2 and 160^2 planes fit one CTA (54, 97 and
// 219 KB); 200^2 planes are shared by clusters of 5 (135 KB per CTA) or 10
// CTAs (67 KB, a non-portable cluster size), whose thread counts are multiples
// of both run lengths of a line and of the warp size.
#include "pf_internal.h"

namespace pf {

template <int NY, int NZ, int C, int T>
static int add(YZKernels* out, int n) {
  if (n >= kMaxVariants) return n;
  YZKernels& k = out[n];
  k.main = yz_kernel<NY, NZ, C, T, YZ_MAIN>;
  k.c2 = yz_kernel<NY, NZ, C, T, YZ_C2>;
  k.imp = yz_kernel<NY, NZ, C, T, YZ_IMPORT>;
  k.cluster = C;
  k.threads = T;
  k.smem = YZ<NY, NZ, C>::SMEM;
  return n + 1;
}

template <int NY, int NZ, int T>
static int add1(YZKernels* out, int n) {
  if (n >= kMaxVariants) return n;
  YZKernels& k = out[n];
  k.main = yz1_kernel<NY, NZ, T, YZ_MAIN>;
  k.c2 = yz1_kernel<NY, NZ, T, YZ_C2>;
  k.imp = yz1_kernel<NY, NZ, T, YZ_IMPORT>;
  k.cluster = 1;
  k.threads = T;
  k.smem = YZ1<NY, NZ>::SMEM;
  return n + 1;
}

int yz_variants_r5(int ny, int nz, YZKernels* out, int n) {
  if (ny == 80 && nz == 80) { n = add1<80, 80, 320>(out, n); n = add1<80, 80, 160>(out, n); }
  if (ny == 160 && nz == 160) { n = add1<160, 160, 480>(out, n); n = add1<160, 160, 320>(out, n); n = add<160, 160, 4, 320>(out, n); }
  if (ny == 102 && nz == 102) { n = add1<102, 102, 384>(out, n); n = add1<102, 102, 256>(out, n); }
  if (ny == 200 && nz == 200) { n = add<200, 200, 5, 320>(out, n); n = add<200, 200, 10, 320>(out, n); }
  return n;
}

}  // namespace pf
