// yz-pass instantiations: 128 x 128 planes, clusters of 2 and 8 CTAs, and the
// one-CTA kernel that prefetches the next generation's planes into L2.
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

// one CTA per plane, unpadded row pitch, L2 prefetch of the planes CTA
// blockIdx.x + Shape::pref_yz reads
template <int NY, int NZ, int T>
static int add1pref(YZKernels* out, int n) {
  if (n >= kMaxVariants) return n;
  YZKernels& k = out[n];
  k.main = yz1_kernel<NY, NZ, T, YZ_MAIN, true, true>;
  k.c2 = yz1_kernel<NY, NZ, T, YZ_C2, true>;
  k.imp = yz1_kernel<NY, NZ, T, YZ_IMPORT, true>;
  k.cluster = 1;
  k.threads = T;
  k.smem = YZ1<NY, NZ, true>::SMEM;
  k.pref = 1;
  return n + 1;
}

int yz_variants_128b(int ny, int nz, YZKernels* out, int n) {
  if (ny == 128 && nz == 128) {
    n = add<128, 128, 2, 512>(out, n);
    n = add<128, 128, 8, 128>(out, n);
    n = add1pref<128, 128, 512>(out, n);
  }
  return n;
}

}  // namespace pf
