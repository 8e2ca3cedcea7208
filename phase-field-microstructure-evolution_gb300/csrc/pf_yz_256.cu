// yz-pass instantiation for 256 x 256 planes: clusters of 8 CTAs (32 z rows / 32 y positions each), 140 KB of shared
// memory per CTA.
#include "pf_internal.h"

namespace pf {

bool get_yz_kernels_256(int ny, int nz, YZKernels* out) {
  if (ny == 256 && nz == 256) {
    out->main = yz_kernel<256, 256, 8, 512, YZ_MAIN>;
    out->c2 = yz_kernel<256, 256, 8, 512, YZ_C2>;
    out->imp = yz_kernel<256, 256, 8, 512, YZ_IMPORT>;
    out->cluster = 8;
    out->threads = 512;
    out->smem = YZ<256, 256, 8>::SMEM;
    return true;
  }
  return false;
}

}  // namespace pf
