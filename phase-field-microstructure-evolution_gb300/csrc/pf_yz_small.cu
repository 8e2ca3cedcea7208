// yz-pass instantiations: planes up to 64 x 64 -- single-CTA in-place planes
// (add1) and cluster variants (add: cluster size C, threads T).
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

int yz_variants_small(int ny, int nz, YZKernels* out, int n) {
  if (ny == 16 && nz == 16) { n = add1<16, 16, 128>(out, n); n = add<16, 16, 1, 128>(out, n); }
  if (ny == 32 && nz == 32) {
    n = add1<32, 32, 256>(out, n);
    n = add1<32, 32, 128>(out, n);
    n = add<32, 32, 1, 256>(out, n);
  }
  if (ny == 16 && nz == 32) { n = add1<16, 32, 256>(out, n); n = add<16, 32, 1, 256>(out, n); }
  if (ny == 32 && nz == 16) { n = add1<32, 16, 256>(out, n); n = add<32, 16, 1, 256>(out, n); }
  if (ny == 32 && nz == 64) { n = add1<32, 64, 256>(out, n); n = add<32, 64, 2, 256>(out, n); }
  if (ny == 64 && nz == 32) { n = add1<64, 32, 256>(out, n); n = add<64, 32, 2, 256>(out, n); }
  if (ny == 64 && nz == 64) {
    n = add1<64, 64, 256>(out, n);
    n = add1<64, 64, 128>(out, n);
    n = add1<64, 64, 512>(out, n);
    n = add<64, 64, 2, 256>(out, n);
    n = add1<64, 64, 256, true>(out, n);  // unpadded row pitch
  }
  if (ny == 96 && nz == 96) {  // the reference's own grid (inputs/config.yaml, inputs/input.txt)
    n = add1<96, 96, 384>(out, n);
    n = add1<96, 96, 192>(out, n);
    n = add1<96, 96, 768>(out, n);
    n = add1<96, 96, 384, true>(out, n);  // unpadded row pitch
  }
  return n;
}

}  // namespace pf
