// yz-pass instantiations: 256 x 256 planes, clusters of 16 CTAs (non-portable
// size), and in-place clusters of 4 that prefetch the next generation's planes
// into L2.
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

// in-place exchange, L2 prefetch of what CTA blockIdx.x + Shape::pref_yz reads
template <int NY, int NZ, int C, int T>
static int addpref(YZKernels* out, int n) {
  if (n >= kMaxVariants) return n;
  YZKernels& k = out[n];
  k.main = yz_kernel<NY, NZ, C, T, YZ_MAIN, true, true>;
  k.c2 = yz_kernel<NY, NZ, C, T, YZ_C2, true>;
  k.imp = yz_kernel<NY, NZ, C, T, YZ_IMPORT, true>;
  k.cluster = C;
  k.threads = T;
  k.smem = YZ<NY, NZ, C>::SMEM_INPL;
  k.inpl = 1;
  k.pref = 1;
  return n + 1;
}

int yz_variants_256b(int ny, int nz, YZKernels* out, int n) {
  if (ny == 256 && nz == 256) {
    n = add<256, 256, 16, 256>(out, n);
    n = addpref<256, 256, 4, 512>(out, n);
  }
  return n;
}

}  // namespace pf
