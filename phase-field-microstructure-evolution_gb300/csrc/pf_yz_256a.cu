// yz-pass instantiations: 256 x 256 planes, clusters of 8 CTAs, and clusters
// of 4 or 8 CTAs that exchange the plane's layouts in place (one buffer each).
#include "pf_internal.h"

namespace pf {

template <int NY, int NZ, int C, int T, bool INPL = false>
static int add(YZKernels* out, int n) {
  if (n >= kMaxVariants) return n;
  YZKernels& k = out[n];
  k.main = yz_kernel<NY, NZ, C, T, YZ_MAIN, INPL>;
  k.c2 = yz_kernel<NY, NZ, C, T, YZ_C2, INPL>;
  k.imp = yz_kernel<NY, NZ, C, T, YZ_IMPORT, INPL>;
  k.cluster = C;
  k.threads = T;
  k.smem = INPL ? YZ<NY, NZ, C>::SMEM_INPL : YZ<NY, NZ, C>::SMEM;
  k.inpl = INPL ? 1 : 0;
  return n + 1;
}

int yz_variants_256a(int ny, int nz, YZKernels* out, int n) {
  if (ny == 256 && nz == 256) {
    n = add<256, 256, 8, 512>(out, n);
    n = add<256, 256, 8, 256>(out, n);
    n = add<256, 256, 4, 512, true>(out, n);
    n = add<256, 256, 8, 256, true>(out, n);
  }
  return n;
}

}  // namespace pf
