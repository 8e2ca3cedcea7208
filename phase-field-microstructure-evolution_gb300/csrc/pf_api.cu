// C ABI of libpfgpu.so (include/pfgpu.h): run/batch management, FP64 table
// construction, CUDA-graph step driver and host<->device field transfer for
// the fused FP32 path.  The FP64 plain path and the Fortran shims live in
// pf_plain64.cu, the host-side RNG in pf_host.cpp.
#include <cuda.h>  // CUtensorMap and its enums (the encoder is fetched through the runtime)
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/pfgpu.h"
#include "pf_internal.h"
#include "pf_plain64.h"

namespace pf {

static thread_local std::string g_err;

void set_error(const std::string& msg) { g_err = msg; }

static int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define PF_CUDA(call)                                                                            \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess) return fail(PF_ECUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                                       __FILE__, __LINE__);                                      \
  } while (0)

// Fortran-order host fields (REAL*8) <-> float SoA staging [f][z][y][x]
__global__ void aos_to_soa_kernel(const double* __restrict__ phi, const double* __restrict__ con, float* __restrict__ fin,
                                  int V, size_t ncell) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= ncell) return;
  for (int f = 0; f < V; ++f) fin[(size_t)f * ncell + i] = (float)phi[i * V + f];
  fin[(size_t)V * ncell + i] = (float)con[i];
}
__global__ void soa_to_aos_kernel(const float* __restrict__ fin, double* __restrict__ phi, double* __restrict__ con,
                                  int V, size_t ncell) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= ncell) return;
  for (int f = 0; f < V; ++f) phi[i * V + f] = (double)fin[(size_t)f * ncell + i];
  con[i] = (double)fin[(size_t)V * ncell + i];
}

// ---------------------------------------------------------------------------
// FP64 tables
// ---------------------------------------------------------------------------
static void twiddles(int L, std::vector<float2>& out) {
  out.resize(L);
  const double pi = std::atan(1.0) * 4.0;
  for (int j = 0; j < L; ++j) {
    // FP64 cos/sin of the angle, rounded once to FP32
    const double a = 2.0 * pi * (double)j / (double)L;
    out[j] = make_float2((float)std::cos(a), (float)(-std::sin(a)));
  }
}

// src/k_space.f90:13-59: m' = m (m <= n/2) else m - n; q = m' * (2 pi / n);
// kf = i q but 0 where 2m = n; kf_sq = -q^2; kf_4 = q^4.
static void axis_tables(int n, int count, std::vector<float>& q2, std::vector<float>& q4, std::vector<float>& qn) {
  const double pi = std::atan(1.0) * 4.0;
  const double unit = 2.0 * pi / (double)n;
  q2.resize(count); q4.resize(count); qn.resize(count);
  for (int m = 0; m < count; ++m) {
    const int mp = (m <= n / 2) ? m : m - n;
    const double q = (double)mp * unit;
    q2[m] = (float)(q * q);
    q4[m] = (float)(q * q * q * q);
    qn[m] = (2 * m == n) ? 0.0f : (float)q;
  }
}

struct DevTables {
  void* base = nullptr;
  Shape sh;
};

static int build_tables(int Nx, int Ny, int Nz, DevTables& t) {
  std::vector<float2> twM, twN, twY, twZ;
  twiddles(Nx / 2, twM);
  twiddles(Nx, twN);
  twiddles(Ny, twY);
  twiddles(Nz, twZ);
  std::vector<float> a[9];
  const int Kx = Nx / 2 + 1;
  axis_tables(Nx, Kx, a[0], a[3], a[6]);
  axis_tables(Ny, Ny, a[1], a[4], a[7]);
  axis_tables(Nz, Nz, a[2], a[5], a[8]);
  size_t bytes = 0;
  auto align = [](size_t b) { return (b + 255) & ~(size_t)255; };
  size_t off_tw[4], off_a[9];
  const std::vector<float2>* tws[4] = {&twM, &twN, &twY, &twZ};
  for (int i = 0; i < 4; ++i) { off_tw[i] = bytes; bytes = align(bytes + tws[i]->size() * sizeof(float2)); }
  for (int i = 0; i < 9; ++i) { off_a[i] = bytes; bytes = align(bytes + a[i].size() * sizeof(float)); }
  std::vector<char> host(bytes, 0);
  for (int i = 0; i < 4; ++i) memcpy(host.data() + off_tw[i], tws[i]->data(), tws[i]->size() * sizeof(float2));
  for (int i = 0; i < 9; ++i) memcpy(host.data() + off_a[i], a[i].data(), a[i].size() * sizeof(float));
  PF_CUDA(cudaMalloc(&t.base, bytes));
  PF_CUDA(cudaMemcpy(t.base, host.data(), bytes, cudaMemcpyHostToDevice));
  char* b = (char*)t.base;
  Shape& s = t.sh;
  s.Nx = Nx; s.Ny = Ny; s.Nz = Nz; s.Kx = Kx;
  s.plane0 = 0;
  s.pref_yz = 0;
  s.par = 0;
  s.twM = (const float2*)(b + off_tw[0]);
  s.twN = (const float2*)(b + off_tw[1]);
  s.twY = (const float2*)(b + off_tw[2]);
  s.twZ = (const float2*)(b + off_tw[3]);
  s.qx2 = (const float*)(b + off_a[0]); s.qy2 = (const float*)(b + off_a[1]); s.qz2 = (const float*)(b + off_a[2]);
  s.qx4 = (const float*)(b + off_a[3]); s.qy4 = (const float*)(b + off_a[4]); s.qz4 = (const float*)(b + off_a[5]);
  s.qnx = (const float*)(b + off_a[6]); s.qny = (const float*)(b + off_a[7]); s.qnz = (const float*)(b + off_a[8]);
  return PF_OK;
}

static size_t x_smem(int nx, int nF, int wy) {
  int pitch;
  switch (nx) {
    case 16: pitch = XLine<8>::PITCH; break;
    case 32: pitch = XLine<16>::PITCH; break;
    case 64: pitch = XLine<32>::PITCH; break;
    case 96: pitch = XLine<48>::PITCH; break;
    case 128: pitch = XLine<64>::PITCH; break;
    case 256: pitch = XLine<128>::PITCH; break;
    case 80: pitch = XLine<40>::PITCH; break;
    case 160: pitch = XLine<80>::PITCH; break;
    case 200: pitch = XLine<100>::PITCH; break;
    case 102: pitch = XLine<51>::PITCH; break;
    default: return 0;
  }
  return (size_t)nF * wy * pitch * sizeof(float2);
}

static const size_t kMaxSmem = 227 * 1024;

// Static shared memory of the one-CTA x-pass kernels beside the dynamic line
// buffer: the twiddle tables (Nx + Nx/2 float2, from Nx = 96 up) and the
// diagnostics reduction's arrays (under 1 KB).  Both count against kMaxSmem.
static size_t x_static_smem(int nx) { return (nx >= 96 ? (size_t)(nx + nx / 2) * sizeof(float2) : 0) + 1024; }

// cuTensorMapEncodeTiled through the runtime's driver entry points (no link
// against the driver library).
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    else
      cudaGetLastError();
  });
  return fn;
}

// Tensor map over a run's mixed-space state Sm [nF][Kx][Nz][Ny] (8-byte
// complex elements) with box {wy rows, 1 z, Kx, 1 field}: one TMA copy brings
// the half spectra of wy rows of one field at one z.
static int encode_sm_map(void* Sm, int Ny, int Nz, int Kx, int nF, int wy, CUtensorMap* out) {
  const PFN_cuTensorMapEncodeTiled_v12000 fn = tensor_map_encoder();
  if (!fn) return fail(PF_ECUDA, "cuTensorMapEncodeTiled is not available from the driver");
  const cuuint64_t dims[4] = {(cuuint64_t)Ny, (cuuint64_t)Nz, (cuuint64_t)Kx, (cuuint64_t)nF};
  const cuuint64_t strides[3] = {(cuuint64_t)Ny * 8, (cuuint64_t)Ny * Nz * 8, (cuuint64_t)Kx * Ny * Nz * 8};
  const cuuint32_t box[4] = {(cuuint32_t)wy, 1, (cuuint32_t)Kx, 1};
  const cuuint32_t es[4] = {1, 1, 1, 1};
  const CUresult r = fn(out, CU_TENSOR_MAP_DATA_TYPE_UINT64, 4, Sm, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(PF_ECUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return PF_OK;
}
// order parameters per run; the x pass must also fit (var+1) field lines of
// its rows in shared memory (checked below)
static const int kMaxVar = 255;

static int validate(const pf_config* c) {
  if (!c) return fail(PF_EINVAL, "null config");
  XKernels xv[kMaxVariants];
  YZKernels yk;
  const int nxv = get_x_variants(c->nx, xv);
  if (nxv == 0) return fail(PF_EINVAL, "Nx=%d not supported (16, 32, 64, 80, 96, 102, 128, 160, 200, 256)", c->nx);
  if (!get_yz_kernels(c->ny, c->nz, &yk))
    return fail(PF_EINVAL, "(Ny, Nz)=(%d, %d) not supported by the fused FP32 path", c->ny, c->nz);
  if (c->var < 1 || c->var > kMaxVar) return fail(PF_EINVAL, "var=%d outside [1, %d]", c->var, kMaxVar);
  bool fits = false;
  for (int i = 0; i < nxv; ++i)
    fits = fits || (c->ny % xv[i].wy == 0 && x_smem(c->nx, c->var + 1, xv[i].wy) + x_static_smem(c->nx) <= kMaxSmem);
  if (!fits) return fail(PF_EINVAL, "var=%d with Nx=%d, Ny=%d does not fit the x pass", c->var, c->nx, c->ny);
  if (c->mobility != PF_MOB_REFERENCE && c->mobility != PF_MOB_C1MC)
    return fail(PF_EINVAL, "unknown mobility form %d", c->mobility);
  if (!std::isfinite(c->t_step)) return fail(PF_EINVAL, "t_step not finite");
  return PF_OK;
}

static int mob_mode(const pf_config* c) {
  if (c->mobility == PF_MOB_C1MC) return MOB_C1MC;
  return c->D_gb == 0.0 ? MOB_CONST : MOB_REF_VAR;
}

}  // namespace pf

using namespace pf;

// ---------------------------------------------------------------------------
// Batch = one or more same-shape runs stepped by one set of launches
// ---------------------------------------------------------------------------
struct pf_batch {
  int nruns = 0;
  int device = 0;
  int Nx = 0, Ny = 0, Nz = 0, V = 0, nF = 0, Kx = 0;
  int mob = MOB_CONST;
  DevTables tab;
  XKernels xk{};
  XKernels xjk{};              // variant of the xj pass (one field: its best rows per CTA differ)
  YZKernels yk{};
  size_t smem_x = 0, smem_xj = 0, smem_bulk = 0;
  std::vector<RunParams> hrp;
  std::vector<CUtensorMap> tmaps;  // host copies of the runs' tensor maps (TMA x pass)
  RunParams* drp = nullptr;
  void* mem = nullptr;         // all per-run buffers
  float* fin = nullptr;        // float staging [nF][Nz][Ny][Nx]
  double* dstage = nullptr;    // double staging for one run's AoS fields
  int ring = 0;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t gexec = nullptr;   // one step
  cudaGraphExec_t gexec_k = nullptr; // kGraphSteps steps, each step's record beside the next step's x pass
  cudaStream_t side = nullptr;        // second branch of the captured step (concentration chain)
  cudaStream_t copy = nullptr;        // record copies of completed steps (never waits for later steps)
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_c = nullptr;
  cudaStream_t rec = nullptr;         // the step records of the multi-step graph
  cudaEvent_t ev_yz = nullptr, ev_rec[2] = {nullptr, nullptr};
  int prio_hi = 0;                    // greatest stream priority of the device
  int nsm = 0;                        // multiprocessors of the device (persistent TMA x pass)
  int tma_occ = 1;                    // resident CTAs per SM of the chosen TMA x pass
  std::vector<double> hdiag;
  std::vector<int> steps_done;
  std::string variant;  // chosen kernel variants, for reports
};

struct pf_run {
  int precision = PF_FP32_FUSED;
  pf_batch* b = nullptr;
  pf::Plain64* p64 = nullptr;
};

// One cluster launch of a yz-pass kernel over `planes` (field, kx) planes,
// from plane `plane0` on, of `nruns` runs starting at `runs`; `prio` != 0
// gives the launch that scheduling priority.
static int launch_yz(pf_batch* b, KernelFn fn, int planes, const RunParams* runs, int nruns, cudaStream_t s,
                     int plane0 = 0, int prio = 0) {
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute at[2];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = b->yk.cluster;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  at[1].id = cudaLaunchAttributePriority;
  at[1].val.priority = prio;
  cfg.gridDim = dim3(b->yk.cluster * planes, nruns);
  cfg.blockDim = dim3(b->yk.threads);
  cfg.dynamicSmemBytes = b->yk.smem;
  cfg.stream = s;
  cfg.attrs = at;
  cfg.numAttrs = prio ? 2 : 1;
  Shape sh = b->tab.sh;
  sh.plane0 = plane0;
  PF_CUDA(cudaLaunchKernelEx(&cfg, fn, runs, sh));
  return PF_OK;
}

// The xj pass with an optional scheduling priority.
static int launch_xj(pf_batch* b, cudaStream_t s, int prio = 0) {
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributePriority;
  at[0].val.priority = prio;
  cfg.gridDim = dim3(b->Nz * (b->Ny / b->xjk.wy), b->nruns);
  cfg.blockDim = dim3(b->xjk.threads);
  cfg.dynamicSmemBytes = b->smem_xj;
  cfg.stream = s;
  cfg.attrs = at;
  cfg.numAttrs = prio ? 1 : 0;
  PF_CUDA(cudaLaunchKernelEx(&cfg, b->xjk.xj, (const RunParams*)b->drp, b->tab.sh));
  return PF_OK;
}

// The bulk x pass (one CTA per WY rows, or two-CTA clusters sharing the fields).
static int launch_x_bulk(pf_batch* b, cudaStream_t s) {
  const int R = b->nruns;
  const unsigned nblk = (unsigned)(b->Nz * (b->Ny / b->xk.wy));
  if (b->xk.tma) {  // persistent: as many CTAs as are resident at once, over all runs
    const unsigned g = (unsigned)std::max(1, std::min((int)nblk, b->nsm * b->tma_occ / R));
    b->xk.bulk<<<dim3(g, R), b->xk.threads, b->smem_bulk, s>>>(b->drp, b->tab.sh);
    PF_CUDA(cudaGetLastError());
    return PF_OK;
  }
  if (!b->xk.cl) {
    b->xk.bulk<<<dim3(nblk, R), b->xk.threads, b->smem_bulk, s>>>(b->drp, b->tab.sh);
    PF_CUDA(cudaGetLastError());
    return PF_OK;
  }
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = b->xk.cl;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(b->xk.cl * nblk, R);
  cfg.blockDim = dim3(b->xk.threads);
  cfg.dynamicSmemBytes = b->smem_bulk;
  cfg.stream = s;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  PF_CUDA(cudaLaunchKernelEx(&cfg, b->xk.bulk, (const RunParams*)b->drp, b->tab.sh));
  return PF_OK;
}

// One step on stream s.  With `branch` (the captured graph) and variable
// mobility, the concentration field's chain -- its yz planes, the xj pass and
// the yz C2 pass, which the order-parameter planes do not need -- runs on a
// second branch at high priority beside the order-parameter planes, so that
// its small launches fill SMs as the big launch drains; the record of the
// step follows the order-parameter planes once the c planes' f_int partials
// are in, beside the rest of the concentration chain.
static constexpr int kRecordThreads = 1024;
static int launch_record(pf_batch* b, cudaStream_t s) {
  record_kernel<kRecordThreads><<<b->nruns, kRecordThreads, 0, s>>>(b->drp, b->tab.sh);
  PF_CUDA(cudaGetLastError());
  return PF_OK;
}

static int enqueue_step(pf_batch* b, cudaStream_t s, bool branch = false) {
  const int R = b->nruns;
  {
    const int rc0 = launch_x_bulk(b, s);
    if (rc0) return rc0;
  }
  const bool var = b->mob != MOB_CONST;
  if (branch && var && b->side) {
    const int pc = b->V * b->Kx;  // first plane of the c field
    PF_CUDA(cudaEventRecord(b->ev_fork, s));
    PF_CUDA(cudaStreamWaitEvent(b->side, b->ev_fork, 0));
    int rc = launch_yz(b, b->yk.main, b->Kx, b->drp, R, b->side, pc, b->prio_hi);
    if (rc) return rc;
    PF_CUDA(cudaEventRecord(b->ev_c, b->side));
    rc = launch_xj(b, b->side, b->prio_hi);
    if (rc) return rc;
    rc = launch_yz(b, b->yk.c2, b->Kx, b->drp, R, b->side, 0, b->prio_hi);
    if (rc) return rc;
    PF_CUDA(cudaEventRecord(b->ev_join, b->side));
    rc = launch_yz(b, b->yk.main, pc, b->drp, R, s);
    if (rc) return rc;
    PF_CUDA(cudaStreamWaitEvent(s, b->ev_c, 0));
    rc = launch_record(b, s);
    if (rc) return rc;
    PF_CUDA(cudaStreamWaitEvent(s, b->ev_join, 0));
    return PF_OK;
  }
  int rc = launch_yz(b, b->yk.main, b->nF * b->Kx, b->drp, R, s);
  if (rc) return rc;
  if (var) {
    rc = launch_xj(b, s);
    if (rc) return rc;
    rc = launch_yz(b, b->yk.c2, b->Kx, b->drp, R, s);
    if (rc) return rc;
  }
  return launch_record(b, s);
}

// Steps captured together in the multi-step graph.
static constexpr int kGraphSteps = 4;

// K steps for the multi-step graph.  Every step runs as in enqueue_step, but
// its record goes to the record stream, where it runs beside the next step's
// x pass instead of ahead of it.  Steps alternate the two sets of diagnostic
// partials (Shape::par); a step waits for the record of the step two before
// it, the last reader of its set.  The graph ends after its last record.
static int enqueue_steps_overlapped(pf_batch* b, cudaStream_t s, int K, bool branch) {
  const int R = b->nruns;
  const bool var = b->mob != MOB_CONST;
  const bool two = branch && var && b->side;
  struct ParityReset {  // later launches outside the graph use the first set
    Shape& sh;
    ~ParityReset() { sh.par = 0; }
  } reset{b->tab.sh};
  int rc = PF_OK;
  for (int k = 0; k < K && rc == PF_OK; ++k) {
    const int par = k & 1;
    b->tab.sh.par = par;
    if (k >= 2) PF_CUDA(cudaStreamWaitEvent(s, b->ev_rec[par], 0));
    rc = launch_x_bulk(b, s);
    if (rc) break;
    if (two) {
      const int pc = b->V * b->Kx;  // first plane of the c field
      PF_CUDA(cudaEventRecord(b->ev_fork, s));
      PF_CUDA(cudaStreamWaitEvent(b->side, b->ev_fork, 0));
      rc = launch_yz(b, b->yk.main, b->Kx, b->drp, R, b->side, pc, b->prio_hi);
      if (rc) break;
      PF_CUDA(cudaEventRecord(b->ev_c, b->side));
      rc = launch_xj(b, b->side, b->prio_hi);
      if (rc) break;
      rc = launch_yz(b, b->yk.c2, b->Kx, b->drp, R, b->side, 0, b->prio_hi);
      if (rc) break;
      PF_CUDA(cudaEventRecord(b->ev_join, b->side));
      rc = launch_yz(b, b->yk.main, pc, b->drp, R, s);
      if (rc) break;
      PF_CUDA(cudaEventRecord(b->ev_yz, s));
      PF_CUDA(cudaStreamWaitEvent(b->rec, b->ev_yz, 0));
      PF_CUDA(cudaStreamWaitEvent(b->rec, b->ev_c, 0));
      rc = launch_record(b, b->rec);
      if (rc) break;
      PF_CUDA(cudaEventRecord(b->ev_rec[par], b->rec));
      PF_CUDA(cudaStreamWaitEvent(s, b->ev_join, 0));  // this step's c field before the next x pass
    } else {
      rc = launch_yz(b, b->yk.main, b->nF * b->Kx, b->drp, R, s);
      if (rc) break;
      PF_CUDA(cudaEventRecord(b->ev_yz, s));  // the record needs the yz partials only
      PF_CUDA(cudaStreamWaitEvent(b->rec, b->ev_yz, 0));
      rc = launch_record(b, b->rec);
      if (rc) break;
      PF_CUDA(cudaEventRecord(b->ev_rec[par], b->rec));
      if (var) {
        rc = launch_xj(b, s);
        if (rc) break;
        rc = launch_yz(b, b->yk.c2, b->Kx, b->drp, R, s);
      }
    }
  }
  if (rc) return rc;
  PF_CUDA(cudaStreamWaitEvent(s, b->ev_rec[(K - 1) & 1], 0));
  return PF_OK;
}

// n steps on the batch's stream: multi-step graphs, then single steps.
static int launch_steps(pf_batch* b, int n) {
  for (; b->gexec_k && n >= kGraphSteps; n -= kGraphSteps) PF_CUDA(cudaGraphLaunch(b->gexec_k, b->stream));
  for (; n > 0; --n) PF_CUDA(cudaGraphLaunch(b->gexec, b->stream));
  return PF_OK;
}

// ---------------------------------------------------------------------------
// Autotuner: time every compiled variant of the x and yz passes on this batch
// (whole steps, three interleaved rounds, on a synthetic non-zero state) and
// keep the fastest.  The choice is cached per (shape, var, mobility, device)
// for the life of the process, so every batch of a shape runs the same
// kernels.  PFGPU_AUTOTUNE=0 keeps the default variants; PFGPU_X_VARIANT /
// PFGPU_YZ_VARIANT force one.
// ---------------------------------------------------------------------------
__global__ void fill_kernel(float* p, size_t n, float v0, float v1) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) p[i] = (i & 1) ? v1 : v0;
}

static std::mutex g_tune_mu;
static std::map<std::string, std::tuple<int, int, int>> g_tune_cache;  // x, yz, xj variant

// Clusters of a yz-pass variant resident on the device at once (0: it cannot
// be scheduled).
static int yz_clusters(pf_batch* b, const YZKernels& k) {
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = k.cluster;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(k.cluster * b->nF * b->Kx, 1);
  cfg.blockDim = dim3(k.threads);
  cfg.dynamicSmemBytes = k.smem;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int ncl = 0;
  const cudaError_t e = cudaOccupancyMaxActiveClusters(&ncl, (const void*)k.main, &cfg);
  cudaGetLastError();
  return e == cudaSuccess ? ncl : 0;
}

static bool yz_ok(pf_batch* b, const YZKernels& k) {
  if (k.smem > kMaxSmem) return false;
  for (KernelFn f : {k.main, k.c2, k.imp}) {
    if (cudaFuncSetAttribute((const void*)f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k.smem) != cudaSuccess)
      return false;
    if (k.cluster > 8 &&
        cudaFuncSetAttribute((const void*)f, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)
      return false;
  }
  return yz_clusters(b, k) >= 1;
}

// Dynamic shared memory a kernel may use is a per-function setting shared by
// every batch in the process: only ever raise it, so that a batch of fewer
// fields never lowers it under a live batch of the same grid with more fields.
static std::mutex g_attr_mu;
static std::map<std::pair<int, const void*>, int> g_attr_smem;
static bool raise_smem(const void* fn, size_t bytes) {
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(g_attr_mu);
  int& cur = g_attr_smem[std::make_pair(dev, fn)];
  if ((int)bytes <= cur) return true;
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  cur = (int)bytes;
  return true;
}

static bool x_ok(pf_batch* b, const XKernels& k) {
  if (b->Ny % k.wy != 0) return false;
  const size_t sm = x_smem(b->Nx, b->nF, k.wy);
  if (sm + x_static_smem(b->Nx) > kMaxSmem) return false;
  if (k.tma) {  // persistent TMA bulk kernel: staging + lines must fit one CTA; inner TMA box of 16-byte multiples
    const size_t sb = k.bulk_smem(b->nF);
    CUtensorMap probe;
    if (sb > kMaxSmem || (k.wy * 8) % 16 != 0 || b->Kx > 256 ||
        encode_sm_map(b->hrp[0].Sm, b->Ny, b->Nz, b->Kx, b->nF, k.wy, &probe) != PF_OK ||
        !raise_smem((const void*)k.bulk, sb))
      return false;
  }
  if (k.cl) {  // two-CTA bulk: rank 1 must own phi_P and c (var >= 3); the cluster must be schedulable
    const size_t sb = k.bulk_smem(b->nF);
    if (b->V < 3 || sb > kMaxSmem || !raise_smem((const void*)k.bulk, sb)) return false;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = k.cl;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(k.cl * b->Nz * (b->Ny / k.wy), 1);
    cfg.blockDim = dim3(k.threads);
    cfg.dynamicSmemBytes = sb;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int ncl = 0;
    if (cudaOccupancyMaxActiveClusters(&ncl, (const void*)k.bulk, &cfg) != cudaSuccess || ncl < 1) {
      cudaGetLastError();
      return false;
    }
  }
  for (KernelFn f : {k.bulk, k.xj, k.imp, k.exp}) {
    if ((k.cl || k.tma) && f == k.bulk) continue;
    if (!raise_smem((const void*)f, sm)) return false;
  }
  return true;
}

// the xj pass works on one field: a variant whose bulk pass does not fit can serve it
static bool xj_ok(pf_batch* b, const XKernels& k) {
  if (b->Ny % k.wy != 0) return false;
  const size_t sm = x_smem(b->Nx, 1, k.wy);
  return sm + x_static_smem(b->Nx) <= kMaxSmem && raise_smem((const void*)k.xj, sm);
}

static void describe_variants(pf_batch* b) {
  char buf[256];
  snprintf(buf, sizeof buf, "x:wy=%d,threads=%d%s%s yz:cluster=%d,threads=%d%s%s xj:wy=%d,threads=%d%s", b->xk.wy,
           b->xk.threads, b->xk.cl ? ",cluster=2" : (b->xk.tma ? ",tma" : ""), b->xk.tag, b->yk.cluster,
           b->yk.threads, b->yk.inpl ? ",in-place" : "", b->yk.pref ? ",L2-prefetch" : "", b->xjk.wy,
           b->xjk.threads, b->xjk.tag);
  b->variant = buf;
}

static void apply_xj(pf_batch* b, const XKernels& k) {
  b->xjk = k;
  b->smem_xj = x_smem(b->Nx, 1, k.wy);
  describe_variants(b);
}

// Tensor maps of every run for the TMA x pass with wy rows per tile, written
// on the batch's stream (in order with the launches that read them).
static int write_tensor_maps(pf_batch* b, int wy) {
  for (int r = 0; r < b->nruns; ++r) {
    CUtensorMap m;
    const int rc = encode_sm_map(b->hrp[r].Sm, b->Ny, b->Nz, b->Kx, b->nF, wy, &m);
    if (rc) return rc;
    b->tmaps[r] = m;
  }
  for (int r = 0; r < b->nruns; ++r)
    PF_CUDA(cudaMemcpyAsync(const_cast<void*>(b->hrp[r].tmap_sm), &b->tmaps[r], sizeof(CUtensorMap),
                            cudaMemcpyHostToDevice, b->stream));
  return PF_OK;
}

static void apply_variants(pf_batch* b, const XKernels& xk, const YZKernels& yk) {
  b->xk = xk;
  b->yk = yk;
  b->smem_x = x_smem(b->Nx, b->nF, xk.wy);
  b->smem_bulk = (xk.cl || xk.tma) ? xk.bulk_smem(b->nF) : b->smem_x;
  if (xk.tma) {
    write_tensor_maps(b, xk.wy);  // encodable: checked by x_ok
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, (const void*)xk.bulk, xk.threads, b->smem_bulk) !=
            cudaSuccess || occ < 1) {
      cudaGetLastError();
      occ = 1;
    }
    b->tma_occ = std::min(occ, xk.tma);
  }
  b->tab.sh.nblk_x = b->Nz * (b->Ny / xk.wy);
  b->tab.sh.nblk_yz = yk.cluster * b->nF * b->Kx;
  // L2 prefetch distance of the yz variants that prefetch: the CTAs resident at once
  b->tab.sh.pref_yz = yk.pref ? yz_clusters(b, yk) * yk.cluster : 0;
  apply_xj(b, xk);
}

static int env_int(const char* name, int dflt) {
  const char* v = getenv(name);
  return v ? atoi(v) : dflt;
}

static int tune_batch(pf_batch* b) {
  XKernels xv[kMaxVariants];
  YZKernels yv[kMaxVariants];
  const int nx = get_x_variants(b->Nx, xv), ny = get_yz_variants(b->Ny, b->Nz, yv);
  std::vector<int> xs, ys;
  for (int i = 0; i < nx; ++i)
    if (x_ok(b, xv[i])) xs.push_back(i);
  for (int i = 0; i < ny; ++i)
    if (yz_ok(b, yv[i])) ys.push_back(i);
  if (xs.empty()) return fail(PF_EINVAL, "no x-pass variant fits Nx=%d, Ny=%d, var=%d", b->Nx, b->Ny, b->V);
  if (ys.empty()) return fail(PF_ECUDA, "no yz-pass variant can be scheduled for (%d, %d)", b->Ny, b->Nz);
  char key[128];
  int dev = 0;
  cudaGetDevice(&dev);
  snprintf(key, sizeof key, "%d/%d/%d/%d/%d/%d", b->Nx, b->Ny, b->Nz, b->V, b->mob, dev);
  int bx = xs[0], by = ys[0], bj = -1;
  const int fx = env_int("PFGPU_X_VARIANT", -1), fy = env_int("PFGPU_YZ_VARIANT", -1);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      bx = std::get<0>(it->second);
      by = std::get<1>(it->second);
      bj = std::get<2>(it->second);
    } else if (env_int("PFGPU_AUTOTUNE", 1) != 0 && (xs.size() > 1 || ys.size() > 1)) {
      // synthetic non-zero state so that the bulk terms take their usual branches
      const size_t nfin = (size_t)b->nF * b->Nx * b->Ny * b->Nz;
      fill_kernel<<<(unsigned)((nfin + 255) / 256), 256, 0, b->stream>>>(b->fin, nfin, 0.3f, 0.7f);
      apply_variants(b, xv[xs[0]], yv[ys[0]]);
      const dim3 g1(b->Nz * (b->Ny / b->xk.wy), 1);
      b->xk.imp<<<g1, b->xk.threads, b->smem_x, b->stream>>>(b->drp, b->tab.sh);
      cudaEvent_t e0, e1;
      cudaEventCreate(&e0);
      cudaEventCreate(&e1);
      // Whole steps are timed (kernel order and L2 contents as in the run),
      // in interleaved rounds, keeping the best time per variant: first the
      // x variants with the default yz variant, then the yz variants.
      const int ROUNDS = 3, REPS = 3;
      // warm-up steps first, so that the first variants are not timed on a GPU
      // still raising its clocks
      for (int i = 0; i < 8; ++i)
        if (enqueue_step(b, b->stream)) cudaGetLastError();
      cudaStreamSynchronize(b->stream);
      auto time_steps = [&](float& out) {
        if (enqueue_step(b, b->stream)) { cudaGetLastError(); return; }
        cudaEventRecord(e0, b->stream);
        for (int r = 0; r < REPS; ++r) enqueue_step(b, b->stream);
        cudaEventRecord(e1, b->stream);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (cudaGetLastError() == cudaSuccess) out = std::min(out, ms);
      };
      std::vector<float> tx(nx, 1e30f), ty(ny, 1e30f);
      for (int round = 0; round < ROUNDS; ++round)
        for (int i : xs) {
          apply_variants(b, xv[i], yv[by]);
          time_steps(tx[i]);
        }
      for (int i : xs)
        if (tx[i] < tx[bx]) bx = i;
      for (int round = 0; round < ROUNDS; ++round)
        for (int i : ys) {
          apply_variants(b, xv[bx], yv[i]);
          time_steps(ty[i]);
        }
      for (int i : ys)
        if (ty[i] < ty[by]) by = i;
      if (env_int("PFGPU_AUTOTUNE_REPORT", 0)) {  // every variant's best time per step, on stderr
        for (int i : xs)
          fprintf(stderr, "pfgpu autotune %s x %d wy=%d threads=%d%s%s: %.4f ms/step%s\n", key, i, xv[i].wy,
                  xv[i].threads, xv[i].cl ? ",cluster=2" : (xv[i].tma ? ",tma" : ""), xv[i].tag, tx[i] / REPS,
                  i == bx ? " (chosen)" : "");
        for (int i : ys)
          fprintf(stderr, "pfgpu autotune %s yz %d cluster=%d threads=%d%s%s: %.4f ms/step%s\n", key, i,
                  yv[i].cluster, yv[i].threads, yv[i].inpl ? ",in-place" : "", yv[i].pref ? ",L2-prefetch" : "",
                  ty[i] / REPS, i == by ? " (chosen)" : "");
      }
      // the xj pass (variable mobility) alone, over every variant that fits one field
      apply_variants(b, xv[bx], yv[by]);
      bj = bx;
      if (b->mob != MOB_CONST) {
        std::vector<float> tj(nx, 1e30f);
        const int R = b->nruns;
        for (int round = 0; round < ROUNDS; ++round)
          for (int i = 0; i < nx; ++i) {
            if (!xj_ok(b, xv[i])) continue;
            apply_xj(b, xv[i]);
            const dim3 gj(b->Nz * (b->Ny / b->xjk.wy), R);
            b->xjk.xj<<<gj, b->xjk.threads, b->smem_xj, b->stream>>>(b->drp, b->tab.sh);
            cudaEventRecord(e0, b->stream);
            for (int r = 0; r < 4 * REPS; ++r)
              b->xjk.xj<<<gj, b->xjk.threads, b->smem_xj, b->stream>>>(b->drp, b->tab.sh);
            cudaEventRecord(e1, b->stream);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (cudaGetLastError() == cudaSuccess) tj[i] = std::min(tj[i], ms);
          }
        for (int i = 0; i < nx; ++i)
          if (tj[i] < tj[bj]) bj = i;
      }
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      PF_CUDA(cudaStreamSynchronize(b->stream));
      // leave a clean state behind
      for (const RunParams& r : b->hrp) {
        const size_t fbytes = (size_t)b->nF * b->Kx * b->Ny * b->Nz * sizeof(float2);
        PF_CUDA(cudaMemsetAsync(r.Sk, 0, fbytes, b->stream));
        PF_CUDA(cudaMemsetAsync(r.Sm, 0, fbytes, b->stream));
        PF_CUDA(cudaMemsetAsync(r.D, 0, fbytes, b->stream));
        PF_CUDA(cudaMemsetAsync(r.counter, 0, 256, b->stream));  // step counter, error word
      }
      PF_CUDA(cudaStreamSynchronize(b->stream));
      g_tune_cache[key] = std::make_tuple(bx, by, bj);
    }
  }
  if (fx >= 0 && fx < nx && x_ok(b, xv[fx])) bx = fx;
  if (fy >= 0 && fy < ny && yz_ok(b, yv[fy])) by = fy;
  // PFGPU_X_VARIANT forces the xj pass too, unless PFGPU_XJ_VARIANT names its own
  const int fj = env_int("PFGPU_XJ_VARIANT", -1);
  if (bj < 0 || (fx >= 0 && fx < nx)) bj = bx;
  if (fj >= 0 && fj < nx && xj_ok(b, xv[fj])) bj = fj;
  if (!xj_ok(b, xv[bj])) bj = bx;
  apply_variants(b, xv[bx], yv[by]);
  apply_xj(b, xv[bj]);
  return PF_OK;
}

static void destroy_batch(pf_batch* b) {
  if (!b) return;
  cudaSetDevice(b->device);
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  if (b->gexec_k) cudaGraphExecDestroy(b->gexec_k);
  if (b->rec) cudaStreamDestroy(b->rec);
  if (b->ev_yz) cudaEventDestroy(b->ev_yz);
  for (cudaEvent_t ev : b->ev_rec)
    if (ev) cudaEventDestroy(ev);
  if (b->stream) cudaStreamDestroy(b->stream);
  if (b->side) cudaStreamDestroy(b->side);
  if (b->copy) cudaStreamDestroy(b->copy);
  if (b->ev_fork) cudaEventDestroy(b->ev_fork);
  if (b->ev_join) cudaEventDestroy(b->ev_join);
  if (b->ev_c) cudaEventDestroy(b->ev_c);
  cudaFree(b->drp);
  cudaFree(b->mem);
  cudaFree(b->fin);
  cudaFree(b->dstage);
  cudaFree(b->tab.base);
  delete b;
}

// Capture the one-step and the multi-step graphs on the batch's stream (again
// after pf_batch_prioritize: kernel nodes keep the priority of the stream
// they were captured on, and the graphs run with their nodes' priorities).
// The batch's graphs are replaced only when both captures succeed.
static int capture_graphs(pf_batch* b) {
  const bool branch = env_int("PFGPU_REDUCE_BRANCH", 1) != 0;
  cudaGraphExec_t ex[2] = {nullptr, nullptr};
  int rc = PF_OK;
  for (int i = 0; i < 2 && rc == PF_OK; ++i) {
    const int k = i == 0 ? 1 : kGraphSteps;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
      rc = fail(PF_ECUDA, "begin capture: %s", cudaGetErrorString(e));
      break;
    }
    rc = k == 1 ? enqueue_step(b, b->stream, branch) : enqueue_steps_overlapped(b, b->stream, k, branch);
    const cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
    if (rc == PF_OK && e2 != cudaSuccess) rc = fail(PF_ECUDA, "end capture: %s", cudaGetErrorString(e2));
    if (rc == PF_OK) {
      e = cudaGraphInstantiate(&ex[i], g, cudaGraphInstantiateFlagUseNodePriority);
      if (e != cudaSuccess) rc = fail(PF_ECUDA, "graph instantiate: %s", cudaGetErrorString(e));
    }
    if (g) cudaGraphDestroy(g);
  }
  if (rc != PF_OK) {
    for (cudaGraphExec_t x : ex)
      if (x) cudaGraphExecDestroy(x);
    cudaGetLastError();
    return rc;
  }
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  if (b->gexec_k) cudaGraphExecDestroy(b->gexec_k);
  b->gexec = ex[0];
  b->gexec_k = ex[1];
  return PF_OK;
}

static int create_batch(const pf_config* cfgs, int nruns, pf_batch** out) {
  if (!out) return fail(PF_EINVAL, "null output pointer");
  *out = nullptr;
  if (nruns < 1 || nruns > 65535) return fail(PF_EINVAL, "nruns=%d outside [1, 65535]", nruns);
  for (int i = 0; i < nruns; ++i) {
    int rc = validate(&cfgs[i]);
    if (rc) return rc;
    const pf_config& a = cfgs[0];
    const pf_config& c = cfgs[i];
    if (c.nx != a.nx || c.ny != a.ny || c.nz != a.nz || c.var != a.var || c.device != a.device)
      return fail(PF_EINVAL, "run %d: all runs of a batch need the same grid, var and device", i);
    if ((mob_mode(&c) == MOB_CONST) != (mob_mode(&a) == MOB_CONST))
      return fail(PF_EINVAL, "run %d: constant- and variable-mobility runs cannot share a batch", i);
  }
  pf_batch* b = new pf_batch();
  const pf_config& c0 = cfgs[0];
  b->nruns = nruns;
  b->device = c0.device;
  b->Nx = c0.nx; b->Ny = c0.ny; b->Nz = c0.nz; b->V = c0.var; b->nF = c0.var + 1; b->Kx = c0.nx / 2 + 1;
  b->mob = mob_mode(&c0);
  for (int i = 0; i < nruns; ++i)
    if (mob_mode(&cfgs[i]) != MOB_CONST) b->mob = mob_mode(&cfgs[i]);
  get_x_kernels(b->Nx, &b->xk);
  get_yz_kernels(b->Ny, b->Nz, &b->yk);
  auto bail = [&](int rc) { destroy_batch(b); return rc; };
  cudaError_t e = cudaSetDevice(b->device);
  if (e != cudaSuccess) return bail(fail(PF_ECUDA, "cudaSetDevice(%d): %s", b->device, cudaGetErrorString(e)));
  int rc = build_tables(b->Nx, b->Ny, b->Nz, b->tab);
  if (rc) return bail(rc);
  Shape& sh = b->tab.sh;

  // buffers
  const size_t plane = (size_t)b->Ny * b->Nz;
  const size_t fieldc = (size_t)b->Kx * plane;  // complex elements per field
  const size_t ncell = (size_t)b->Nx * b->Ny * b->Nz;
  const bool var = b->mob != MOB_CONST;
  b->ring = 1024;
  auto align = [](size_t v) { return (v + 255) & ~(size_t)255; };
  const size_t szS = align(b->nF * fieldc * sizeof(float2));
  const size_t szMob = var ? align(ncell * sizeof(float)) : 0;
  const size_t szJ = var ? align(fieldc * sizeof(float2)) : 0;  // J~ scratch
  // partial arrays sized for every variant (at least one y row per x-pass
  // block, at most 16 CTAs per yz cluster)
  const size_t szPx = align((size_t)XD_COUNT * b->Nz * b->Ny * sizeof(double));
  const size_t szPyz = align((size_t)32 * b->nF * b->Kx * sizeof(double));  // 2 parities x 2 x clusters <= 16
  const size_t szDiag = align((size_t)b->ring * DR_COUNT * sizeof(double));
  const size_t szCnt = 256;   // step counter and error word (one 64-byte line each)
  const size_t szTmap = 256;  // TMA tensor map of Sm (128 bytes, 64-byte aligned)
  const size_t per_run = 3 * szS + szMob + szJ + szPx + szPyz + szDiag + szCnt + szTmap;
  e = cudaMalloc(&b->mem, per_run * nruns);
  if (e != cudaSuccess)
    return bail(fail(PF_ENOMEM, "cudaMalloc(%zu bytes) for %d runs: %s", per_run * nruns, nruns, cudaGetErrorString(e)));
  e = cudaMemset(b->mem, 0, per_run * nruns);
  if (e != cudaSuccess) return bail(fail(PF_ECUDA, "cudaMemset: %s", cudaGetErrorString(e)));
  e = cudaMalloc(&b->fin, b->nF * ncell * sizeof(float));
  if (e != cudaSuccess) return bail(fail(PF_ENOMEM, "staging allocation: %s", cudaGetErrorString(e)));
  e = cudaMalloc(&b->dstage, b->nF * ncell * sizeof(double));
  if (e != cudaSuccess) return bail(fail(PF_ENOMEM, "staging allocation: %s", cudaGetErrorString(e)));
  b->hrp.resize(nruns);
  b->tmaps.resize(nruns);
  b->steps_done.assign(nruns, 0);
  cudaDeviceGetAttribute(&b->nsm, cudaDevAttrMultiProcessorCount, b->device);
  if (b->nsm < 1) b->nsm = 1;
  for (int i = 0; i < nruns; ++i) {
    const pf_config& c = cfgs[i];
    char* p = (char*)b->mem + per_run * i;
    RunParams& r = b->hrp[i];
    memset(&r, 0, sizeof r);
    r.Sk = (float2*)p; p += szS;
    r.Sm = (float2*)p; p += szS;
    r.D = (float2*)p; p += szS;
    r.mob = var ? (float*)p : nullptr; p += szMob;
    r.J = var ? (float2*)p : nullptr; p += szJ;
    r.part_x = (float*)p; p += szPx;
    r.part_yz = (float*)p; p += szPyz;
    r.diag = (double*)p; p += szDiag;
    r.counter = (int*)p;
    r.err = (unsigned*)(p + 128);
    p += szCnt;
    r.tmap_sm = p;
    r.fin = b->fin;
    r.L = (float)c.mob_phi;
    r.kappa_phi = (float)c.grad_coeff_phi;
    r.kappa_c = (float)c.grad_coeff_c;
    r.dt = (float)c.t_step;
    r.D_L = (float)c.D_L;
    r.D_gb = (float)c.D_gb;
    r.sigma1 = (float)c.sigma_1;
    r.sigma2 = (float)c.sigma_2;
    r.am = (float)c.am;
    r.ap = (float)c.ap;
    r.c0m = (float)c.con_0_mat;
    r.c0p = (float)c.con_0_ppt;
    r.mobility = mob_mode(&c);
    r.V = c.var;
    r.ring = b->ring;
  }
  e = cudaMalloc(&b->drp, nruns * sizeof(RunParams));
  if (e != cudaSuccess) return bail(fail(PF_ENOMEM, "run table: %s", cudaGetErrorString(e)));
  e = cudaMemcpy(b->drp, b->hrp.data(), nruns * sizeof(RunParams), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return bail(fail(PF_ECUDA, "run table copy: %s", cudaGetErrorString(e)));
  e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return bail(fail(PF_ECUDA, "stream: %s", cudaGetErrorString(e)));
  int prio_lo = 0;
  cudaDeviceGetStreamPriorityRange(&prio_lo, &b->prio_hi);
  e = cudaStreamCreateWithPriority(&b->side, cudaStreamNonBlocking, b->prio_hi);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->copy, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_c, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&b->rec, cudaStreamNonBlocking, b->prio_hi);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_yz, cudaEventDisableTiming);
  for (cudaEvent_t& ev : b->ev_rec)
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
  if (e != cudaSuccess) return bail(fail(PF_ECUDA, "stream/events: %s", cudaGetErrorString(e)));

  rc = tune_batch(b);
  if (rc) return bail(rc);

  rc = capture_graphs(b);
  if (rc) return bail(rc);
  *out = b;
  return PF_OK;
}

static int batch_set_fields(pf_batch* b, int run, const double* phi, const double* con) {
  if (!b || run < 0 || run >= b->nruns || !phi || !con) return fail(PF_EINVAL, "bad arguments to set_fields");
  PF_CUDA(cudaSetDevice(b->device));
  const size_t ncell = (size_t)b->Nx * b->Ny * b->Nz;
  double* dphi = b->dstage;
  double* dcon = b->dstage + (size_t)b->V * ncell;
  PF_CUDA(cudaMemcpyAsync(dphi, phi, (size_t)b->V * ncell * sizeof(double), cudaMemcpyHostToDevice, b->stream));
  PF_CUDA(cudaMemcpyAsync(dcon, con, ncell * sizeof(double), cudaMemcpyHostToDevice, b->stream));
  aos_to_soa_kernel<<<(unsigned)((ncell + 255) / 256), 256, 0, b->stream>>>(dphi, dcon, b->fin, b->V, ncell);
  const dim3 gx(b->Nz * (b->Ny / b->xk.wy), 1);
  b->xk.imp<<<gx, b->xk.threads, b->smem_x, b->stream>>>(b->drp + run, b->tab.sh);
  int rc = launch_yz(b, b->yk.imp, b->nF * b->Kx, b->drp + run, 1, b->stream);
  if (rc) return rc;
  PF_CUDA(cudaMemsetAsync(b->hrp[run].counter, 0, 256, b->stream));  // step counter, error word
  PF_CUDA(cudaGetLastError());
  PF_CUDA(cudaStreamSynchronize(b->stream));
  b->steps_done[run] = 0;
  return PF_OK;
}

static int batch_get_fields(pf_batch* b, int run, double* phi, double* con) {
  if (!b || run < 0 || run >= b->nruns || !phi || !con) return fail(PF_EINVAL, "bad arguments to get_fields");
  PF_CUDA(cudaSetDevice(b->device));
  const size_t ncell = (size_t)b->Nx * b->Ny * b->Nz;
  double* dphi = b->dstage;
  double* dcon = b->dstage + (size_t)b->V * ncell;
  const dim3 gx(b->Nz * (b->Ny / b->xk.wy), 1);
  b->xk.exp<<<gx, b->xk.threads, b->smem_x, b->stream>>>(b->drp + run, b->tab.sh);
  soa_to_aos_kernel<<<(unsigned)((ncell + 255) / 256), 256, 0, b->stream>>>(b->fin, dphi, dcon, b->V, ncell);
  PF_CUDA(cudaGetLastError());
  PF_CUDA(cudaMemcpyAsync(phi, dphi, (size_t)b->V * ncell * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  PF_CUDA(cudaMemcpyAsync(con, dcon, ncell * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  PF_CUDA(cudaStreamSynchronize(b->stream));
  return PF_OK;
}

// Real-space fields of run 0 of a batch in the float staging buffer fin.
static int batch_device_fields(pf_batch* b, DeviceFields* out) {
  PF_CUDA(cudaSetDevice(b->device));
  const size_t ncell = (size_t)b->Nx * b->Ny * b->Nz;
  const dim3 gx(b->Nz * (b->Ny / b->xk.wy), 1);
  b->xk.exp<<<gx, b->xk.threads, b->smem_x, b->stream>>>(b->drp, b->tab.sh);
  PF_CUDA(cudaGetLastError());
  out->phi = b->fin;
  out->con = b->fin + (size_t)b->V * ncell;
  out->is_double = 0;
  out->fstride = ncell;
  out->cstride = 1;
  out->nx = b->Nx; out->ny = b->Ny; out->nz = b->Nz; out->var = b->V; out->device = b->device;
  out->stream = b->stream;
  return PF_OK;
}

static void fill_diag(const double* d, pf_diag* o) {
  o->step = (int)d[DR_STEP];
  o->nonfinite = (int)d[DR_NONFINITE];
  o->f_int = d[DR_FINT];
  o->f_eta = d[DR_FETA];
  o->f_ch = d[DR_FCH];
  o->e_tot = d[DR_FINT] + d[DR_FCH] + d[DR_FETA];  // src/var_diff.f90:1070
  o->c_max = d[DR_CMAX];
  o->c_min = d[DR_CMIN];
  o->phi_min = d[DR_PHIMIN];
  o->phi_P_max = d[DR_PHIPMAX];
  o->mass = d[DR_MASS];
}

static int batch_step(pf_batch* b, int nsteps, pf_diag* diag) {
  if (!b || nsteps < 0) return fail(PF_EINVAL, "bad arguments to step");
  PF_CUDA(cudaSetDevice(b->device));
  int bad = 0;
  int done = 0;
  while (done < nsteps) {
    const int chunk = std::min(nsteps - done, b->ring);
    const int rl = launch_steps(b, chunk);
    if (rl) return rl;
    PF_CUDA(cudaStreamSynchronize(b->stream));
    b->hdiag.resize((size_t)b->ring * DR_COUNT);
    for (int r = 0; r < b->nruns; ++r) {
      // copy only this chunk's records (two pieces when they wrap around the ring)
      const int first = b->steps_done[r] % b->ring;
      const int n1 = std::min(chunk, b->ring - first);
      PF_CUDA(cudaMemcpy(b->hdiag.data() + (size_t)first * DR_COUNT, b->hrp[r].diag + (size_t)first * DR_COUNT,
                         (size_t)n1 * DR_COUNT * sizeof(double), cudaMemcpyDeviceToHost));
      if (chunk > n1)
        PF_CUDA(cudaMemcpy(b->hdiag.data(), b->hrp[r].diag, (size_t)(chunk - n1) * DR_COUNT * sizeof(double),
                           cudaMemcpyDeviceToHost));
      for (int s = 0; s < chunk; ++s) {
        const int step = b->steps_done[r] + s;  // 0-based
        const double* d = b->hdiag.data() + (size_t)(step % b->ring) * DR_COUNT;
        if (d[DR_NONFINITE] != 0) bad = 1;
        if (diag) fill_diag(d, &diag[(size_t)r * nsteps + done + s]);
      }
      b->steps_done[r] += chunk;
    }
    done += chunk;
  }
  if (bad) return fail(PF_ENONFINITE, "a step produced non-finite values");
  return PF_OK;
}

namespace pf {
int run_device_fields(pf_run* run, DeviceFields* out) {
  if (!run || !out) return fail(PF_EINVAL, "null argument");
  if (run->p64) return plain64_device_fields(run->p64, out);
  return batch_device_fields(run->b, out);
}
}  // namespace pf

// ---------------------------------------------------------------------------
// exported C ABI
// ---------------------------------------------------------------------------
extern "C" {

const char* pf_last_error(void) { return g_err.c_str(); }

int pf_supported_shape(int nx, int ny, int nz, int var, int precision) {
  pf_config c;
  memset(&c, 0, sizeof c);
  c.nx = nx; c.ny = ny; c.nz = nz; c.var = var; c.precision = precision; c.t_step = 0.1;
  std::string keep = g_err;
  int ok;
  if (precision == PF_FP64_PLAIN) ok = plain64_validate(&c) == PF_OK;
  else ok = validate(&c) == PF_OK;
  g_err = keep;
  return ok;
}

int pf_create(const pf_config* cfg, pf_run** out) {
  if (!cfg || !out) return fail(PF_EINVAL, "null argument");
  *out = nullptr;
  pf_run* r = new pf_run();
  r->precision = cfg->precision;
  int rc;
  if (cfg->precision == PF_FP64_PLAIN) rc = plain64_create(cfg, &r->p64);
  else if (cfg->precision == PF_FP32_FUSED || cfg->precision == 0) {
    r->precision = PF_FP32_FUSED;
    rc = create_batch(cfg, 1, &r->b);
  } else rc = fail(PF_EINVAL, "unknown precision %d", cfg->precision);
  if (rc) { delete r; return rc; }
  *out = r;
  return PF_OK;
}

int pf_set_fields(pf_run* run, const double* phi, const double* con) {
  if (!run) return fail(PF_EINVAL, "null run");
  if (run->p64) return plain64_set_fields(run->p64, phi, con);
  return batch_set_fields(run->b, 0, phi, con);
}

int pf_step(pf_run* run, int nsteps, pf_diag* diag) {
  if (!run) return fail(PF_EINVAL, "null run");
  if (run->p64) return plain64_step(run->p64, nsteps, diag);
  return batch_step(run->b, nsteps, diag);
}

int pf_get_fields(pf_run* run, double* phi, double* con) {
  if (!run) return fail(PF_EINVAL, "null run");
  if (run->p64) return plain64_get_fields(run->p64, phi, con);
  return batch_get_fields(run->b, 0, phi, con);
}

int pf_destroy(pf_run* run) {
  if (!run) return PF_OK;
  if (run->p64) plain64_destroy(run->p64);
  destroy_batch(run->b);
  delete run;
  return PF_OK;
}

int pf_batch_create(const pf_config* cfgs, int nruns, pf_batch** out) {
  if (!cfgs) return fail(PF_EINVAL, "null configs");
  for (int i = 0; i < nruns; ++i)
    if (cfgs[i].precision != PF_FP32_FUSED && cfgs[i].precision != 0)
      return fail(PF_EINVAL, "batches run on the fused FP32 path only");
  return create_batch(cfgs, nruns, out);
}
int pf_batch_set_fields(pf_batch* b, int run, const double* phi, const double* con) {
  return batch_set_fields(b, run, phi, con);
}
int pf_batch_step(pf_batch* b, int nsteps, pf_diag* diag) { return batch_step(b, nsteps, diag); }
int pf_batch_get_fields(pf_batch* b, int run, double* phi, double* con) { return batch_get_fields(b, run, phi, con); }
int pf_batch_destroy(pf_batch* b) {
  destroy_batch(b);
  return PF_OK;
}

// Internal hooks for the benchmark: enqueue steps / query the stream without
// host synchronisation.  Not part of the public header.
int pf_batch_enqueue(pf_batch* b, int nsteps) {
  if (!b) return fail(PF_EINVAL, "null batch");
  PF_CUDA(cudaSetDevice(b->device));
  const int rl = launch_steps(b, nsteps);
  if (rl) return rl;
  for (int r = 0; r < b->nruns; ++r) b->steps_done[r] += nsteps;
  return PF_OK;
}
void* pf_batch_stream(pf_batch* b) { return b ? (void*)b->stream : nullptr; }
const char* pf_batch_variant(pf_batch* b) { return b ? b->variant.c_str() : ""; }
pf_batch* pf_run_batch(pf_run* r) { return r ? r->b : nullptr; }
// Device bytes a batch of `nruns` runs of configuration `cfg` holds (the
// buffers create_batch allocates, rounded up); for admission by HBM budget.
size_t pf_batch_bytes(const pf_config* c, int nruns) {
  if (!c || nruns < 1) return 0;
  const size_t Kx = c->nx / 2 + 1, nF = c->var + 1;
  const size_t plane = (size_t)c->ny * c->nz, fieldc = Kx * plane, ncell = (size_t)c->nx * plane;
  const bool var = c->mobility == PF_MOB_C1MC || c->D_gb != 0.0;
  auto align = [](size_t v) { return (v + 255) & ~(size_t)255; };
  const size_t per_run = 3 * align(nF * fieldc * 8) + (var ? align(ncell * 4) + align(fieldc * 8) : 0) +
                         align((size_t)XD_COUNT * plane * 8) + align(32 * nF * Kx * 8) + align(1024 * DR_COUNT * 8) + 512;
  return per_run * nruns + nF * ncell * 12 + ((size_t)1 << 20);
}
// Steps run `run` has completed since its last set_fields (host count).
int pf_batch_steps_done(pf_batch* b, int run) {
  return (b && run >= 0 && run < b->nruns) ? b->steps_done[run] : -1;
}
// Records of steps first .. first+n-1 (0-based, since set_fields) of one run,
// still in the device ring (n <= the ring length).  The caller has seen those
// steps complete (an event recorded after them): the copy runs on the batch's
// copy stream, so it does not wait for steps enqueued later on the batch's
// stream, which may go on writing other slots of the ring meanwhile.
int pf_batch_records(pf_batch* b, int run, int first, int n, pf_diag* out) {
  if (!b || run < 0 || run >= b->nruns || n < 0 || n > b->ring || !out) return fail(PF_EINVAL, "bad arguments");
  PF_CUDA(cudaSetDevice(b->device));
  std::vector<double> h((size_t)n * DR_COUNT);
  const double* ring = b->hrp[run].diag;
  for (int s = 0; s < n;) {
    const int pos = (first + s) % b->ring, take = std::min(n - s, b->ring - pos);
    PF_CUDA(cudaMemcpyAsync(h.data() + (size_t)s * DR_COUNT, ring + (size_t)pos * DR_COUNT,
                            (size_t)take * DR_COUNT * sizeof(double), cudaMemcpyDeviceToHost, b->copy));
    s += take;
  }
  PF_CUDA(cudaStreamSynchronize(b->copy));
  for (int s = 0; s < n; ++s) fill_diag(h.data() + (size_t)s * DR_COUNT, &out[s]);
  return PF_OK;
}
// The k = 0 coefficient of run `run`'s concentration state (the mean of c,
// f_trans normalisation): Re and Im as doubles.  The semi-implicit update
// leaves this coefficient untouched, so the mass N^3 Re c_hat(0) is constant.
int pf_batch_c_mean(pf_batch* b, int run, double* re_im) {
  if (!b || run < 0 || run >= b->nruns || !re_im) return fail(PF_EINVAL, "bad arguments");
  PF_CUDA(cudaSetDevice(b->device));
  PF_CUDA(cudaStreamSynchronize(b->stream));
  float2 v;
  const size_t fieldc = (size_t)b->Kx * b->Ny * b->Nz;
  PF_CUDA(cudaMemcpy(&v, b->hrp[run].Sk + (size_t)b->V * fieldc, sizeof v, cudaMemcpyDeviceToHost));
  re_im[0] = v.x;
  re_im[1] = v.y;
  return PF_OK;
}
// Length of a batch's per-run record ring (steps whose records stay readable).
int pf_batch_ring(pf_batch* b) { return b ? b->ring : 0; }
// Give the batch's stream the device's highest scheduling priority (before
// any step is enqueued on it): its launches then take SMs ahead of
// lower-priority work as SMs free up.
int pf_batch_prioritize(pf_batch* b) {
  if (!b) return fail(PF_EINVAL, "null batch");
  PF_CUDA(cudaSetDevice(b->device));
  PF_CUDA(cudaStreamSynchronize(b->stream));
  cudaStream_t s = nullptr;
  PF_CUDA(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, b->prio_hi));
  cudaStream_t old = b->stream;
  b->stream = s;
  const int rc = capture_graphs(b);  // the main chain's nodes take the new stream's priority
  if (rc != PF_OK) {  // keep the batch as it was
    b->stream = old;
    cudaStreamDestroy(s);
    return rc;
  }
  cudaStreamDestroy(old);
  return PF_OK;
}
// Number of compiled x-pass and yz-pass variants of a grid (the index range
// of PFGPU_X_VARIANT / PFGPU_YZ_VARIANT).
void pf_variant_counts(int nx, int ny, int nz, int* nxv, int* nyzv) {
  XKernels xv[kMaxVariants];
  YZKernels yv[kMaxVariants];
  if (nxv) *nxv = get_x_variants(nx, xv);
  if (nyzv) *nyzv = get_yz_variants(ny, nz, yv);
}
// Launch the x pass / yz pass alone (kernel timing); returns PF_OK.
int pf_batch_enqueue_phase(pf_batch* b, int phase) {
  if (!b) return fail(PF_EINVAL, "null batch");
  const Shape sh = b->tab.sh;
  const dim3 gx(b->Nz * (b->Ny / b->xk.wy), b->nruns);
  if (phase == 0) {
    const int rc = launch_x_bulk(b, b->stream);
    if (rc) return rc;
  } else {
    int rc = launch_yz(b, b->yk.main, b->nF * b->Kx, b->drp, b->nruns, b->stream);
    if (rc) return rc;
  }
  PF_CUDA(cudaGetLastError());
  return PF_OK;
}

}  // extern "C"
