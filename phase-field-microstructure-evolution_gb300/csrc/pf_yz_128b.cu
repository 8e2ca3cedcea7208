// yz-pass instantiations: 128 x 128 planes, clusters of 2 and 8 CTAs.
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

int yz_variants_128b(int ny, int nz, YZKernels* out, int n) {
  if (ny == 128 && nz == 128) {
    n = add<128, 128, 2, 512>(out, n);
    n = add<128, 128, 8, 128>(out, n);
  }
  return n;
}

}  // namespace pf
