// Instantiations of the x pass (fused bulk kernel and x-direction transforms)
// for the supported Nx.  y rows per CTA (WY) are chosen so that a CTA has
// 128-256 two-cell work items and global rows are read in >= 32-byte runs.
#include "pf_internal.h"

namespace pf {

template <int NX, int WY>
static void fill(XKernels* k) {
  k->bulk = x_pass_kernel<NX, WY, 256, MODE_BULK>;
  k->xj = x_pass_kernel<NX, WY, 256, MODE_XJ>;
  k->imp = x_pass_kernel<NX, WY, 256, MODE_IMPORT>;
  k->exp = x_pass_kernel<NX, WY, 256, MODE_EXPORT>;
  k->wy = WY;
}

bool get_x_kernels(int nx, XKernels* out) {
  switch (nx) {
    case 16: fill<16, 16>(out); return true;
    case 32: fill<32, 16>(out); return true;
    case 64: fill<64, 8>(out); return true;
    case 128: fill<128, 8>(out); return true;
    case 256: fill<256, 4>(out); return true;
    default: return false;
  }
}

}  // namespace pf
