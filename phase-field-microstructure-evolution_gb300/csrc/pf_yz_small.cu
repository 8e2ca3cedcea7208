// yz-pass instantiations for planes up to 64 x 64.
#include "pf_internal.h"

namespace pf {

template <int NY, int NZ, int C, int T>
static void fill(YZKernels* k) {
  k->main = yz_kernel<NY, NZ, C, T, YZ_MAIN>;
  k->c2 = yz_kernel<NY, NZ, C, T, YZ_C2>;
  k->imp = yz_kernel<NY, NZ, C, T, YZ_IMPORT>;
  k->cluster = C;
  k->threads = T;
  k->smem = YZ<NY, NZ, C>::SMEM;
}

bool get_yz_kernels_small(int ny, int nz, YZKernels* out) {
  if (ny == 16 && nz == 16) { fill<16, 16, 1, 128>(out); return true; }
  if (ny == 32 && nz == 32) { fill<32, 32, 1, 256>(out); return true; }
  if (ny == 16 && nz == 32) { fill<16, 32, 1, 256>(out); return true; }
  if (ny == 32 && nz == 16) { fill<32, 16, 1, 256>(out); return true; }
  if (ny == 32 && nz == 64) { fill<32, 64, 2, 256>(out); return true; }
  if (ny == 64 && nz == 32) { fill<64, 32, 2, 256>(out); return true; }
  if (ny == 64 && nz == 64) { fill<64, 64, 2, 256>(out); return true; }
  return false;
}

}  // namespace pf
