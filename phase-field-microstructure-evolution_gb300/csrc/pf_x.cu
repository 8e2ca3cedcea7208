// Instantiations of the x pass (fused bulk kernel and x-direction transforms)
// for the supported Nx: several (rows per CTA, threads per CTA) variants per
// size; the first one is the default, the autotuner picks among them.
#include "pf_internal.h"

namespace pf {

template <int NX, int WY, int T>
static int add(XKernels* out, int n) {
  if (n >= kMaxVariants) return n;
  XKernels& k = out[n];
  k.bulk = x_pass_kernel<NX, WY, T, MODE_BULK>;
  k.xj = x_pass_kernel<NX, WY, T, MODE_XJ>;
  k.imp = x_pass_kernel<NX, WY, T, MODE_IMPORT>;
  k.exp = x_pass_kernel<NX, WY, T, MODE_EXPORT>;
  k.wy = WY;
  k.threads = T;
  k.cl = 0;
  k.tma = 0;
  k.bulk_smem = nullptr;
  k.tag = "";
  return n + 1;
}

template <int NX, int WY>
static size_t cl_smem(int nF) {
  return XCL<NX, WY>::smem(nF);
}

template <int NX, int WY>
static size_t tma_smem(int nF) {
  return XTMA<NX, WY>::smem(nF);
}

// bulk pass as the persistent TMA-staged kernel, at most MINB CTAs per SM;
// the other modes use the plain kernel
template <int NX, int WY, int T, int MINB = 1>
static int addtma(XKernels* out, int n) {
  if (n >= kMaxVariants) return n;
  n = add<NX, WY, T>(out, n);
  XKernels& k = out[n - 1];
  k.bulk = x_pass_tma_kernel<NX, WY, T, MINB>;
  k.tma = MINB;
  k.bulk_smem = tma_smem<NX, WY>;
  return n;
}

// every mode with the tile's spectra copied in by cp.async and transformed in
// place (PHYS: the bulk walk over physical slots)
template <int NX, int WY, int T, bool PHYS = false>
static int addas(XKernels* out, int n) {
  if (n >= kMaxVariants) return n;
  XKernels& k = out[n];
  k.bulk = x_pass_kernel<NX, WY, T, MODE_BULK, PHYS, true>;
  k.xj = x_pass_kernel<NX, WY, T, MODE_XJ, PHYS, true>;
  k.imp = x_pass_kernel<NX, WY, T, MODE_IMPORT>;
  k.exp = x_pass_kernel<NX, WY, T, MODE_EXPORT, PHYS, true>;
  k.wy = WY;
  k.threads = T;
  k.cl = 0;
  k.tma = 0;
  k.bulk_smem = nullptr;
  k.tag = PHYS ? ",async" : ",async,logical";
  return n + 1;
}

// bulk pass walking the logical cells (for comparison with the physical-slot walk)
template <int NX, int WY, int T>
static int addlog(XKernels* out, int n) {
  if (n >= kMaxVariants) return n;
  n = add<NX, WY, T>(out, n);
  out[n - 1].bulk = x_pass_kernel<NX, WY, T, MODE_BULK, false>;
  out[n - 1].tag = ",logical";
  return n;
}

// bulk pass split over two-CTA clusters; the other modes use the one-CTA kernel
template <int NX, int WY, int T>
static int addcl(XKernels* out, int n) {
  if (n >= kMaxVariants) return n;
  n = add<NX, WY, T>(out, n);
  XKernels& k = out[n - 1];
  k.bulk = x_pass_cl_kernel<NX, WY, T>;
  k.cl = 2;
  k.bulk_smem = cl_smem<NX, WY>;
  return n;
}

int x_variants_a(int nx, XKernels* out, int n) {
  switch (nx) {
    case 16: n = add<16, 16, 256>(out, n); break;
    case 32: n = add<32, 16, 256>(out, n); n = add<32, 8, 128>(out, n); break;
    case 64:
      n = add<64, 8, 256>(out, n); n = add<64, 16, 256>(out, n); n = add<64, 4, 128>(out, n);
      n = addcl<64, 8, 256>(out, n);
      n = addtma<64, 8, 512>(out, n);
      break;
    case 96:  // 512-thread CTAs keep 16 warps per SM when many fields leave room for one CTA only
      n = add<96, 8, 256>(out, n); n = add<96, 4, 256>(out, n); n = add<96, 16, 256>(out, n);
      n = add<96, 4, 512>(out, n); n = add<96, 8, 512>(out, n);
      n = addcl<96, 4, 256>(out, n); n = addcl<96, 8, 256>(out, n);
      break;
    case 128:
      n = add<128, 8, 256>(out, n);
      n = add<128, 4, 256>(out, n);
      n = add<128, 4, 128>(out, n);
      n = add<128, 16, 256>(out, n);
      n = add<128, 4, 512>(out, n);
      n = addcl<128, 4, 256>(out, n); n = addcl<128, 8, 256>(out, n);
      n = addtma<128, 8, 512>(out, n); n = addtma<128, 8, 256>(out, n);
      n = addlog<128, 8, 256>(out, n);
      n = addtma<128, 4, 256, 3>(out, n); n = addtma<128, 4, 384, 2>(out, n);
      n = addas<128, 8, 256>(out, n); n = addas<128, 8, 256, true>(out, n); n = addas<128, 4, 256>(out, n);
      // many rows for the one-field xj pass (its bulk mode does not fit: never chosen for the bulk pass)
      n = add<128, 32, 256>(out, n);
      break;
    case 256:
      n = add<256, 4, 256>(out, n); n = add<256, 2, 256>(out, n); n = add<256, 4, 512>(out, n);
      n = addcl<256, 4, 256>(out, n); n = addcl<256, 4, 512>(out, n);
      n = addtma<256, 4, 512>(out, n); n = addtma<256, 2, 512>(out, n);
      n = addas<256, 4, 512>(out, n); n = addas<256, 2, 256>(out, n);
      n = addcl<256, 8, 512>(out, n);  // fields split over two CTAs: 8-row (64-byte) tiles at 33 fields
      n = add<256, 1, 256>(out, n);  // one row per tile: up to 196 fields
      break;
    default: break;
  }
  return n;
}

}  // namespace pf
