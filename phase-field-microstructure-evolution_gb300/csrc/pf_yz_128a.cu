// yz-pass instantiations: 128 x 128 planes -- one CTA per plane (136-140 KB
// of shared memory, no re-layout) and clusters of 4 CTAs.
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

template <int NY, int NZ, int T, bool RAWP = false>
static int add1(YZKernels* out, int n) {
  if (n >= kMaxVariants) return n;
  YZKernels& k = out[n];
  k.main = yz1_kernel<NY, NZ, T, YZ_MAIN, RAWP>;
  k.c2 = yz1_kernel<NY, NZ, T, YZ_C2, RAWP>;
  k.imp = yz1_kernel<NY, NZ, T, YZ_IMPORT, RAWP>;
  k.cluster = 1;
  k.threads = T;
  k.smem = YZ1<NY, NZ, RAWP>::SMEM;
  return n + 1;
}

int yz_variants_128a(int ny, int nz, YZKernels* out, int n) {
  if (ny == 128 && nz == 128) {
    n = add1<128, 128, 512, true>(out, n);  // unpadded row pitch: no bank conflicts in the row passes
    n = add1<128, 128, 512>(out, n);
    n = add1<128, 128, 1024>(out, n);
    n = add<128, 128, 4, 256>(out, n);
  }
  return n;
}

}  // namespace pf
