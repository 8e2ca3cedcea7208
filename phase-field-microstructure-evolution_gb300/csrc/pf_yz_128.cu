// yz-pass instantiation for 128 x 128 planes: clusters of 4 CTAs (32 z rows / 32 y positions each), 70 KB of shared
// memory per CTA.
#include "pf_internal.h"

namespace pf {

bool get_yz_kernels_128(int ny, int nz, YZKernels* out) {
  if (ny == 128 && nz == 128) {
    out->main = yz_kernel<128, 128, 4, 256, YZ_MAIN>;
    out->c2 = yz_kernel<128, 128, 4, 256, YZ_C2>;
    out->imp = yz_kernel<128, 128, 4, 256, YZ_IMPORT>;
    out->cluster = 4;
    out->threads = 256;
    out->smem = YZ<128, 128, 4>::SMEM;
    return true;
  }
  return false;
}

}  // namespace pf
