// yz-pass instantiations: 128 x 128 planes, clusters of 2 and 8 CTAs, and the
// one-CTA kernel with its k-space values staged in shared memory.
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

// one CTA per plane, unpadded row pitch, k-space values of the update staged
// by cp.async behind the plane
template <int NY, int NZ, int T>
static int add1stg(YZKernels* out, int n) {
  if (n >= kMaxVariants) return n;
  YZKernels& k = out[n];
  k.main = yz1_kernel<NY, NZ, T, YZ_MAIN, true, true>;
  k.c2 = yz1_kernel<NY, NZ, T, YZ_C2, true, true>;
  k.imp = yz1_kernel<NY, NZ, T, YZ_IMPORT, true, true>;
  k.cluster = 1;
  k.threads = T;
  k.smem = YZ1<NY, NZ, true>::template smem_staged<T>();
  k.stg = 1;
  return n + 1;
}

int yz_variants_128b(int ny, int nz, YZKernels* out, int n) {
  if (ny == 128 && nz == 128) {
    n = add<128, 128, 2, 512>(out, n);
    n = add<128, 128, 8, 128>(out, n);
    n = add1stg<128, 128, 512>(out, n);
  }
  return n;
}

}  // namespace pf
