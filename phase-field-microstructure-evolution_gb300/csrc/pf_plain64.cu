// Plain FP64 GPU path and the Fortran-signature shims f_trans_, inv_trans_,
// k_space_.  Each phase of src/var_diff.f90:561-1050 is one kernel (or one
// cuFFT call) over global memory, in the reference's order, so this path does
// the reference's 7*var + 9 three-dimensional transforms per step.
#include <cuda_runtime.h>
#include <cufft.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "pf_internal.h"
#include "pf_plain64.h"

namespace pf {

static int fail64(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  set_error(buf);
  return code;
}

#define P64_CUDA(call)                                                                                   \
  do {                                                                                                   \
    cudaError_t e_ = (call);                                                                             \
    if (e_ != cudaSuccess) return fail64(PF_ECUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_),      \
                                         __FILE__, __LINE__);                                            \
  } while (0)
#define P64_FFT(call)                                                                           \
  do {                                                                                          \
    cufftResult r_ = (call);                                                                    \
    if (r_ != CUFFT_SUCCESS) return fail64(PF_ECUDA, "%s: cufft error %d", #call, (int)r_);      \
  } while (0)

static const int NB = 512;  // blocks of the grid-stride reduction kernels
static const int NT = 256;

enum P64Acc { PA_FINT = 0, PA_FETA, PA_FCH, PA_MASS, PA_CMIN, PA_CMAX, PA_PHIMIN, PA_PHIPMAX, PA_BAD, PA_COUNT };

struct Axes64 {
  const double* qx; const double* qy; const double* qz;     // q (for kf_sq, kf_4)
  const double* nx; const double* ny; const double* nz;     // Nyquist-zeroed q (kf / i)
  int Nx, Ny, Nz, Kx;
};

struct Plain64 {
  pf_config c;
  int device = 0;
  int Nx, Ny, Nz, Kx, V;
  size_t ncell, nspec;
  double* phi = nullptr;     // [V][ncell]
  double* con = nullptr;
  double* dfdphi = nullptr;  // [V][ncell]
  double* dfdc = nullptr;
  double* mob = nullptr;
  double* work = nullptr;    // 3 real work arrays
  cufftDoubleComplex* spec = nullptr;  // 5 spectra
  double* gamma = nullptr;   // [V][V]
  double* axes = nullptr;
  double* part = nullptr;    // [PA_COUNT][NB]
  double* dstage = nullptr;
  Axes64 ax;
  cufftHandle fwd = 0, inv = 0;
  cudaStream_t stream = nullptr;
  int steps = 0;
};

__device__ __forceinline__ void kidx(size_t i, const Axes64& a, int& kx, int& ky, int& kz) {
  kx = (int)(i % a.Kx);
  const size_t r = i / a.Kx;
  ky = (int)(r % a.Ny);
  kz = (int)(r / a.Ny);
}

// phase 1/3: out = in * kf_d / N^3   (kf_d = i * Nyquist-zeroed q_d)
__global__ void p64_grad_spec(const cufftDoubleComplex* __restrict__ in, cufftDoubleComplex* __restrict__ out,
                              Axes64 a, int d, double scale, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    int kx, ky, kz;
    kidx(i, a, kx, ky, kz);
    const double q = (d == 0 ? a.nx[kx] : (d == 1 ? a.ny[ky] : a.nz[kz])) * scale;
    const cufftDoubleComplex v = in[i];
    out[i] = make_cuDoubleComplex(-v.y * q, v.x * q);
  }
}

// phase 2/4: f_int += 0.5 kappa (gx^2 + gy^2 + gz^2)
__global__ void p64_fint(const double* __restrict__ g, size_t n, double coef, double* __restrict__ part) {
  double s = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    s += 0.5 * coef * (g[i] * g[i] + g[n + i] * g[n + i] + g[2 * n + i] * g[2 * n + i]);
  __shared__ double sh[NT];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = NT / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[PA_FINT * NB + blockIdx.x] += sh[0];
}

// phases 5-9 and the mobility of phase 10 (src/var_diff.f90:685-898), with the
// reference's O(var^2) loops; statistics and mass of the same fields.
__global__ void p64_bulk(const double* __restrict__ phi, const double* __restrict__ con, const double* __restrict__ gam,
                         double* __restrict__ dfdphi, double* __restrict__ dfdc, double* __restrict__ mob, int V,
                         size_t n, pf_config c, int c1mc, double* __restrict__ part) {
  double feta = 0, fch = 0, mass = 0;
  double cmin = 1.0, cmax = 0.0, pmin = 1.0, ppmax = 0.0, bad = 0;
  const int P = V - 1;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    // phase 5
    for (int iv = 0; iv < V; ++iv) {
      const double fi = phi[iv * n + i];
      feta += -0.5 * fi * fi + 0.25 * fi * fi * fi * fi;
      for (int jv = iv + 1; jv < V; ++jv) {
        const double fj = phi[jv * n + i];
        feta += gam[iv * V + jv] * fi * fi * fj * fj;
      }
    }
    // phase 6
    double num = 0, den = 0;
    for (int iv = 0; iv < V; ++iv) {
      const double f = phi[iv * n + i];
      const double f4 = f * f * f * f;
      if (iv < P) num += f4;
      den += f4;
    }
    const double cc = con[i];
    const double pm = num / den, pp = 1.0 - pm;
    fch += pm * c.am * (cc - c.con_0_mat) * (cc - c.con_0_mat) + pp * c.ap * (cc - c.con_0_ppt) * (cc - c.con_0_ppt);
    const double dc = 2.0 * pm * c.am * (cc - c.con_0_mat) + 2.0 * pp * c.ap * (cc - c.con_0_ppt);
    dfdc[i] = dc;
    // phases 7-9
    const double fmat = c.am * (cc - c.con_0_mat) * (cc - c.con_0_mat);
    const double fppt = c.ap * (cc - c.con_0_ppt) * (cc - c.con_0_ppt);
    const double fP = phi[P * n + i];
    const double t_2 = 4.0 * fP * fP * fP * (den - fP * fP * fP * fP);
    double ssq = 0;
    for (int iv = 0; iv < V; ++iv) {
      const double fi = phi[iv * n + i];
      ssq += fi * fi;
      double t2 = 0;
      for (int jv = 0; jv < V; ++jv)
        if (jv != iv) {
          const double fj = phi[jv * n + i];
          t2 += 2.0 * gam[iv * V + jv] * fi * fj * fj;
        }
      const double t1 = fi * fi * fi - fi;
      double t4;
      if (iv < P) t4 = 4.0 * fi * fi * fi * fP * fP * fP * fP * (fmat - fppt) / (den * den);
      else t4 = t_2 * (fppt - fmat) / (den * den);
      const double d = t1 + t2 + t4;
      if (!isfinite(d)) bad += 1;
      dfdphi[iv * n + i] = d;
    }
    mob[i] = c1mc ? c.D_L * (1.0 + cc * (1.0 - cc)) : c.D_L + 2.0 * (1.0 - ssq) * c.D_gb;
    // statistics of these fields (src/var_diff.f90:1082-1096)
    mass += cc;
    cmin = fmin(cmin, cc);
    cmax = fmax(cmax, cc);
    pmin = fmin(pmin, ssq);
    ppmax = fmax(ppmax, fP);
  }
  __shared__ double sh[5][NT];
  __shared__ double sm[4][NT];
  sh[0][threadIdx.x] = feta; sh[1][threadIdx.x] = fch; sh[2][threadIdx.x] = mass; sh[3][threadIdx.x] = bad;
  sm[0][threadIdx.x] = cmin; sm[1][threadIdx.x] = cmax; sm[2][threadIdx.x] = pmin; sm[3][threadIdx.x] = ppmax;
  __syncthreads();
  for (int o = NT / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      for (int q = 0; q < 4; ++q) sh[q][threadIdx.x] += sh[q][threadIdx.x + o];
      sm[0][threadIdx.x] = fmin(sm[0][threadIdx.x], sm[0][threadIdx.x + o]);
      sm[1][threadIdx.x] = fmax(sm[1][threadIdx.x], sm[1][threadIdx.x + o]);
      sm[2][threadIdx.x] = fmin(sm[2][threadIdx.x], sm[2][threadIdx.x + o]);
      sm[3][threadIdx.x] = fmax(sm[3][threadIdx.x], sm[3][threadIdx.x + o]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[PA_FETA * NB + blockIdx.x] = sh[0][0];
    part[PA_FCH * NB + blockIdx.x] = sh[1][0];
    part[PA_MASS * NB + blockIdx.x] = sh[2][0];
    part[PA_BAD * NB + blockIdx.x] = sh[3][0];
    part[PA_CMIN * NB + blockIdx.x] = sm[0][0];
    part[PA_CMAX * NB + blockIdx.x] = sm[1][0];
    part[PA_PHIMIN * NB + blockIdx.x] = sm[2][0];
    part[PA_PHIPMAX * NB + blockIdx.x] = sm[3][0];
  }
}

// phase 11: J_hat = G mu_hat - kappa_c c_hat K3   (spectra unnormalised on input)
__global__ void p64_flux(const cufftDoubleComplex* __restrict__ ch, const cufftDoubleComplex* __restrict__ mu,
                         cufftDoubleComplex* __restrict__ out, Axes64 a, double kc, double scale, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    int kx, ky, kz;
    kidx(i, a, kx, ky, kz);
    const double g = a.nx[kx] + a.ny[ky] + a.nz[kz];
    const double k3 = -(a.nx[kx] * a.qx[kx] * a.qx[kx] + a.ny[ky] * a.qy[ky] * a.qy[ky] + a.nz[kz] * a.qz[kz] * a.qz[kz]);
    // i*g*mu - kc * c * i*k3 = i (g mu - kc k3 c)
    const double re = (g * mu[i].x - kc * k3 * ch[i].x) * scale;
    const double im = (g * mu[i].y - kc * k3 * ch[i].y) * scale;
    out[i] = make_cuDoubleComplex(-im, re);
  }
}

// phase 12 (real space): J *= (mob - D_mean)
__global__ void p64_jmob(double* __restrict__ J, const double* __restrict__ mob, double dmean, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    J[i] = J[i] * (mob[i] - dmean);
}

// phase 13: c_hat = (c_hat + J'_hat dt G + D K2 dt mu_hat) / (1 + D dt kappa_c K4)
__global__ void p64_ch(cufftDoubleComplex* __restrict__ ch, const cufftDoubleComplex* __restrict__ jp,
                       const cufftDoubleComplex* __restrict__ mu, Axes64 a, double dt, double dm, double kc,
                       double scale, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    int kx, ky, kz;
    kidx(i, a, kx, ky, kz);
    const double g = a.nx[kx] + a.ny[ky] + a.nz[kz];
    const double k2 = -(a.qx[kx] * a.qx[kx] + a.qy[ky] * a.qy[ky] + a.qz[kz] * a.qz[kz]);
    const double qx2 = a.qx[kx] * a.qx[kx], qy2 = a.qy[ky] * a.qy[ky], qz2 = a.qz[kz] * a.qz[kz];
    const double k4 = qx2 * qx2 + qy2 * qy2 + qz2 * qz2;
    const double den = 1.0 + dm * dt * kc * k4;
    // J'_hat * dt * (i g)
    const double t11r = -jp[i].y * scale * dt * g, t11i = jp[i].x * scale * dt * g;
    const double t33 = dm * k2 * dt * scale;
    ch[i] = make_cuDoubleComplex((ch[i].x * scale + t11r + t33 * mu[i].x) / den,
                                 (ch[i].y * scale + t11i + t33 * mu[i].y) / den);
  }
}

// phase 14: phi_hat = (phi_hat - L dt dF_hat) / (1 - L kappa dt K2)
__global__ void p64_ac(cufftDoubleComplex* __restrict__ ph, const cufftDoubleComplex* __restrict__ df, Axes64 a,
                       double L, double dt, double kp, double scale, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    int kx, ky, kz;
    kidx(i, a, kx, ky, kz);
    const double k2 = -(a.qx[kx] * a.qx[kx] + a.qy[ky] * a.qy[ky] + a.qz[kz] * a.qz[kz]);
    const double den = 1.0 - L * kp * dt * k2;
    ph[i] = make_cuDoubleComplex((ph[i].x - L * dt * df[i].x) * scale / den, (ph[i].y - L * dt * df[i].y) * scale / den);
  }
}

__global__ void p64_finish(const double* __restrict__ part, double* __restrict__ out) {
  // one block: fixed-order sums of the block partials
  __shared__ double s[PA_COUNT];
  if (threadIdx.x < PA_COUNT) {
    const int q = threadIdx.x;
    double v = (q == PA_CMIN || q == PA_PHIMIN) ? 1.0 : ((q == PA_CMAX || q == PA_PHIPMAX) ? 0.0 : 0.0);
    for (int b = 0; b < NB; ++b) {
      const double x = part[q * NB + b];
      if (q == PA_CMIN || q == PA_PHIMIN) v = fmin(v, x);
      else if (q == PA_CMAX || q == PA_PHIPMAX) v = fmax(v, x);
      else v += x;
    }
    s[q] = v;
  }
  __syncthreads();
  if (threadIdx.x < PA_COUNT) out[threadIdx.x] = s[threadIdx.x];
}

__global__ void p64_aos_to_soa(const double* __restrict__ aos, double* __restrict__ soa, int V, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    for (int f = 0; f < V; ++f) soa[f * n + i] = aos[i * V + f];
}
__global__ void p64_soa_to_aos(const double* __restrict__ soa, double* __restrict__ aos, int V, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    for (int f = 0; f < V; ++f) aos[i * V + f] = soa[f * n + i];
}

static void host_axis(int n, int count, double* q, double* qn) {
  const double pi = std::atan(1.0) * 4.0;
  const double unit = 2.0 * pi / (double)n;
  for (int m = 0; m < count; ++m) {
    const int mp = (m <= n / 2) ? m : m - n;
    q[m] = (double)mp * unit;
    qn[m] = (2 * m == n) ? 0.0 : q[m];
  }
}

int plain64_validate(const pf_config* c) {
  if (!c) return fail64(PF_EINVAL, "null config");
  if (c->nx < 2 || c->ny < 1 || c->nz < 1 || c->nx % 2) return fail64(PF_EINVAL, "bad grid for the FP64 path");
  if ((double)c->nx * c->ny * c->nz > (double)(1u << 30)) return fail64(PF_EINVAL, "grid too large for the FP64 path");
  if (c->var < 1 || c->var > 256) return fail64(PF_EINVAL, "var=%d outside [1, 256]", c->var);
  return PF_OK;
}

void plain64_destroy(Plain64* p) {
  if (!p) return;
  cudaSetDevice(p->device);
  if (p->fwd) cufftDestroy(p->fwd);
  if (p->inv) cufftDestroy(p->inv);
  if (p->stream) cudaStreamDestroy(p->stream);
  cudaFree(p->phi); cudaFree(p->con); cudaFree(p->dfdphi); cudaFree(p->dfdc); cudaFree(p->mob);
  cudaFree(p->work); cudaFree(p->spec); cudaFree(p->gamma); cudaFree(p->axes); cudaFree(p->part);
  cudaFree(p->dstage);
  delete p;
}

int plain64_create(const pf_config* c, Plain64** out) {
  int rc = plain64_validate(c);
  if (rc) return rc;
  Plain64* p = new Plain64();
  p->c = *c;
  p->device = c->device;
  p->Nx = c->nx; p->Ny = c->ny; p->Nz = c->nz; p->Kx = c->nx / 2 + 1; p->V = c->var;
  p->ncell = (size_t)p->Nx * p->Ny * p->Nz;
  p->nspec = (size_t)p->Kx * p->Ny * p->Nz;
  auto bail = [&](int r) { plain64_destroy(p); return r; };
#define TRY(call) do { cudaError_t e_ = (call); if (e_ != cudaSuccess) \
    return bail(fail64(PF_ENOMEM, "%s: %s", #call, cudaGetErrorString(e_))); } while (0)
  TRY(cudaSetDevice(p->device));
  TRY(cudaMalloc(&p->phi, p->V * p->ncell * sizeof(double)));
  TRY(cudaMalloc(&p->con, p->ncell * sizeof(double)));
  TRY(cudaMalloc(&p->dfdphi, p->V * p->ncell * sizeof(double)));
  TRY(cudaMalloc(&p->dfdc, p->ncell * sizeof(double)));
  TRY(cudaMalloc(&p->mob, p->ncell * sizeof(double)));
  TRY(cudaMalloc(&p->work, 3 * p->ncell * sizeof(double)));
  TRY(cudaMalloc(&p->spec, 5 * p->nspec * sizeof(cufftDoubleComplex)));
  TRY(cudaMalloc(&p->gamma, (size_t)p->V * p->V * sizeof(double)));
  TRY(cudaMalloc(&p->axes, 2 * (size_t)(p->Kx + p->Ny + p->Nz) * sizeof(double)));
  TRY(cudaMalloc(&p->part, (PA_COUNT * NB + PA_COUNT) * sizeof(double)));
  TRY(cudaMalloc(&p->dstage, (p->V + 1) * p->ncell * sizeof(double)));
  TRY(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
#undef TRY
  // gamma (src/var_diff.f90:206-218)
  std::vector<double> g((size_t)p->V * p->V, 0.0);
  const int mat = p->V - 1;
  for (int j = 1; j <= p->V; ++j)
    for (int i = 1; i <= p->V; ++i) {
      double v = 0.0;
      if (i != j && i <= mat && j <= mat) v = c->sigma_1;
      if (j == p->V && i < p->V) v = c->sigma_2;
      if (i == p->V && j < p->V) v = c->sigma_2;
      g[(size_t)(i - 1) * p->V + (j - 1)] = v;
    }
  std::vector<double> ax(2 * (size_t)(p->Kx + p->Ny + p->Nz));
  double* hq = ax.data();
  double* hn = ax.data() + (p->Kx + p->Ny + p->Nz);
  host_axis(p->Nx, p->Kx, hq, hn);
  host_axis(p->Ny, p->Ny, hq + p->Kx, hn + p->Kx);
  host_axis(p->Nz, p->Nz, hq + p->Kx + p->Ny, hn + p->Kx + p->Ny);
  cudaError_t e = cudaMemcpy(p->gamma, g.data(), g.size() * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(p->axes, ax.data(), ax.size() * sizeof(double), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return bail(fail64(PF_ECUDA, "table upload: %s", cudaGetErrorString(e)));
  const double* dq = p->axes;
  const double* dn = p->axes + (p->Kx + p->Ny + p->Nz);
  p->ax.qx = dq; p->ax.qy = dq + p->Kx; p->ax.qz = dq + p->Kx + p->Ny;
  p->ax.nx = dn; p->ax.ny = dn + p->Kx; p->ax.nz = dn + p->Kx + p->Ny;
  p->ax.Nx = p->Nx; p->ax.Ny = p->Ny; p->ax.Nz = p->Nz; p->ax.Kx = p->Kx;
  if (cufftPlan3d(&p->fwd, p->Nz, p->Ny, p->Nx, CUFFT_D2Z) != CUFFT_SUCCESS ||
      cufftPlan3d(&p->inv, p->Nz, p->Ny, p->Nx, CUFFT_Z2D) != CUFFT_SUCCESS)
    return bail(fail64(PF_ECUDA, "cufftPlan3d failed"));
  cufftSetStream(p->fwd, p->stream);
  cufftSetStream(p->inv, p->stream);
  *out = p;
  return PF_OK;
}

int plain64_set_fields(Plain64* p, const double* phi, const double* con) {
  if (!p || !phi || !con) return fail64(PF_EINVAL, "bad arguments to set_fields");
  P64_CUDA(cudaSetDevice(p->device));
  P64_CUDA(cudaMemcpyAsync(p->dstage, phi, p->V * p->ncell * sizeof(double), cudaMemcpyHostToDevice, p->stream));
  p64_aos_to_soa<<<NB, NT, 0, p->stream>>>(p->dstage, p->phi, p->V, p->ncell);
  P64_CUDA(cudaMemcpyAsync(p->con, con, p->ncell * sizeof(double), cudaMemcpyHostToDevice, p->stream));
  P64_CUDA(cudaStreamSynchronize(p->stream));
  p->steps = 0;
  return PF_OK;
}

int plain64_get_fields(Plain64* p, double* phi, double* con) {
  if (!p || !phi || !con) return fail64(PF_EINVAL, "bad arguments to get_fields");
  P64_CUDA(cudaSetDevice(p->device));
  p64_soa_to_aos<<<NB, NT, 0, p->stream>>>(p->phi, p->dstage, p->V, p->ncell);
  P64_CUDA(cudaMemcpyAsync(phi, p->dstage, p->V * p->ncell * sizeof(double), cudaMemcpyDeviceToHost, p->stream));
  P64_CUDA(cudaMemcpyAsync(con, p->con, p->ncell * sizeof(double), cudaMemcpyDeviceToHost, p->stream));
  P64_CUDA(cudaStreamSynchronize(p->stream));
  return PF_OK;
}

int plain64_device_fields(Plain64* p, DeviceFields* out) {
  if (!p || !out) return fail64(PF_EINVAL, "bad arguments to device_fields");
  P64_CUDA(cudaSetDevice(p->device));
  out->phi = p->phi;
  out->con = p->con;
  out->is_double = 1;
  out->fstride = p->ncell;
  out->cstride = 1;
  out->nx = p->Nx; out->ny = p->Ny; out->nz = p->Nz; out->var = p->V; out->device = p->device;
  out->stream = p->stream;
  return PF_OK;
}

static int one_step(Plain64* p, double* acc_out) {
  const size_t n = p->ncell, ns = p->nspec;
  const double scale = 1.0 / (double)n;  // f_trans normalisation (src/f_trans.f90:12)
  cudaStream_t s = p->stream;
  cufftDoubleComplex* W0 = p->spec;
  cufftDoubleComplex* W1 = p->spec + ns;
  cufftDoubleComplex* W2 = p->spec + 2 * ns;
  cufftDoubleComplex* W3 = p->spec + 3 * ns;
  cufftDoubleComplex* W4 = p->spec + 4 * ns;
  const pf_config& c = p->c;
  P64_CUDA(cudaMemsetAsync(p->part, 0, PA_COUNT * NB * sizeof(double), s));
  // phases 1-4: gradient energy through 3 inverse transforms per field
  for (int f = 0; f <= p->V; ++f) {
    double* u = (f < p->V) ? p->phi + (size_t)f * n : p->con;
    P64_FFT(cufftExecD2Z(p->fwd, u, W0));
    for (int d = 0; d < 3; ++d) {
      p64_grad_spec<<<NB, NT, 0, s>>>(W0, W1, p->ax, d, scale, ns);
      P64_FFT(cufftExecZ2D(p->inv, W1, p->work + d * n));
    }
    p64_fint<<<NB, NT, 0, s>>>(p->work, n, f < p->V ? c.grad_coeff_phi : c.grad_coeff_c, p->part);
  }
  // phases 5-10 (bulk), statistics of the same fields
  p64_bulk<<<NB, NT, 0, s>>>(p->phi, p->con, p->gamma, p->dfdphi, p->dfdc, p->mob, p->V, n, c,
                             c.mobility == PF_MOB_C1MC, p->part);
  P64_FFT(cufftExecD2Z(p->fwd, p->con, W0));   // dft_con
  P64_FFT(cufftExecD2Z(p->fwd, p->dfdc, W1));  // dft_df_dc
  // phase 11-12: variable-mobility flux
  p64_flux<<<NB, NT, 0, s>>>(W0, W1, W2, p->ax, c.grad_coeff_c, scale, ns);
  P64_FFT(cufftExecZ2D(p->inv, W2, p->work));
  p64_jmob<<<NB, NT, 0, s>>>(p->work, p->mob, c.D_L, n);
  P64_FFT(cufftExecD2Z(p->fwd, p->work, W3));
  // phase 13
  p64_ch<<<NB, NT, 0, s>>>(W0, W3, W1, p->ax, c.t_step, c.D_L, c.grad_coeff_c, scale, ns);
  P64_FFT(cufftExecZ2D(p->inv, W0, p->con));
  // phase 14
  for (int f = 0; f < p->V; ++f) {
    P64_FFT(cufftExecD2Z(p->fwd, p->phi + (size_t)f * n, W0));
    P64_FFT(cufftExecD2Z(p->fwd, p->dfdphi + (size_t)f * n, W4));
    p64_ac<<<NB, NT, 0, s>>>(W0, W4, p->ax, c.mob_phi, c.t_step, c.grad_coeff_phi, scale, ns);
    P64_FFT(cufftExecZ2D(p->inv, W0, p->phi + (size_t)f * n));
  }
  p64_finish<<<1, 32, 0, s>>>(p->part, p->part + PA_COUNT * NB);
  P64_CUDA(cudaGetLastError());
  P64_CUDA(cudaMemcpyAsync(acc_out, p->part + PA_COUNT * NB, PA_COUNT * sizeof(double), cudaMemcpyDeviceToHost, s));
  return PF_OK;
}

int plain64_step(Plain64* p, int nsteps, pf_diag* diag) {
  if (!p || nsteps < 0) return fail64(PF_EINVAL, "bad arguments to step");
  P64_CUDA(cudaSetDevice(p->device));
  int bad = 0;
  std::vector<double> acc((size_t)std::max(nsteps, 1) * PA_COUNT);
  for (int st = 0; st < nsteps; ++st) {
    int rc = one_step(p, acc.data() + (size_t)st * PA_COUNT);
    if (rc) return rc;
  }
  P64_CUDA(cudaStreamSynchronize(p->stream));
  for (int st = 0; st < nsteps; ++st) {
    const double* a = acc.data() + (size_t)st * PA_COUNT;
    if (a[PA_BAD] != 0) bad = 1;
    if (diag) {
      pf_diag& d = diag[st];
      d.step = p->steps + st + 1;
      d.nonfinite = (int)a[PA_BAD];
      d.f_int = a[PA_FINT];
      d.f_eta = a[PA_FETA];
      d.f_ch = a[PA_FCH];
      d.e_tot = a[PA_FINT] + a[PA_FCH] + a[PA_FETA];
      d.c_max = a[PA_CMAX];
      d.c_min = a[PA_CMIN];
      d.phi_min = a[PA_PHIMIN];
      d.phi_P_max = a[PA_PHIPMAX];
      d.mass = a[PA_MASS];
    }
  }
  p->steps += nsteps;
  if (bad) return fail64(PF_ENONFINITE, "a step produced non-finite values");
  return PF_OK;
}

// ---------------------------------------------------------------------------
// Fortran shims
// ---------------------------------------------------------------------------
__global__ void p64_zyx_to_xyz(const cufftDoubleComplex* __restrict__ in, cufftDoubleComplex* __restrict__ out, int Kx,
                               int Ny, int Nz, double scale) {
  // in [z][y][kx] -> out [kx][y][z] (P3DFFT transposed order), scaled
  const size_t n = (size_t)Kx * Ny * Nz;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int kx = (int)(i % Kx);
    const size_t r = i / Kx;
    const int y = (int)(r % Ny), z = (int)(r / Ny);
    const cufftDoubleComplex v = in[i];
    out[((size_t)kx * Ny + y) * Nz + z] = make_cuDoubleComplex(v.x * scale, v.y * scale);
  }
}
__global__ void p64_xyz_to_zyx(const cufftDoubleComplex* __restrict__ in, cufftDoubleComplex* __restrict__ out, int Kx,
                               int Ny, int Nz) {
  const size_t n = (size_t)Kx * Ny * Nz;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int kx = (int)(i % Kx);
    const size_t r = i / Kx;
    const int y = (int)(r % Ny), z = (int)(r / Ny);
    out[i] = in[((size_t)kx * Ny + y) * Nz + z];
  }
}

struct ShimCtx {
  std::mutex mu;
  int device = 0;
  struct Plans {
    cufftHandle f = 0, i = 0;
    double* real = nullptr;
    cufftDoubleComplex* a = nullptr;
    cufftDoubleComplex* b = nullptr;
  };
  std::map<std::tuple<int, int, int>, Plans> plans;
};
static ShimCtx& shim() {
  static ShimCtx* s = new ShimCtx();
  return *s;
}

static int shim_plans(int Nx, int Ny, int Nz, ShimCtx::Plans** out) {
  ShimCtx& S = shim();
  auto key = std::make_tuple(Nx, Ny, Nz);
  auto it = S.plans.find(key);
  if (it != S.plans.end()) { *out = &it->second; return PF_OK; }
  ShimCtx::Plans pl;
  const size_t n = (size_t)Nx * Ny * Nz, ns = (size_t)(Nx / 2 + 1) * Ny * Nz;
  P64_CUDA(cudaMalloc(&pl.real, n * sizeof(double)));
  P64_CUDA(cudaMalloc(&pl.a, ns * sizeof(cufftDoubleComplex)));
  P64_CUDA(cudaMalloc(&pl.b, ns * sizeof(cufftDoubleComplex)));
  P64_FFT(cufftPlan3d(&pl.f, Nz, Ny, Nx, CUFFT_D2Z));
  P64_FFT(cufftPlan3d(&pl.i, Nz, Ny, Nx, CUFFT_Z2D));
  S.plans[key] = pl;
  *out = &S.plans[key];
  return PF_OK;
}

static bool single_rank(const int* ist, const int* fst) {
  return ist[0] == 1 && ist[1] == 1 && ist[2] == 1 && fst[0] == 1 && fst[1] == 1 && fst[2] == 1;
}

static void shim_report(int rc, const char* who) {
  if (rc) fprintf(stderr, "%s: %s\n", who, pf_last_error());
}

}  // namespace pf

using namespace pf;

extern "C" {

int pf_shim_device(int device) {
  ShimCtx& S = shim();
  std::lock_guard<std::mutex> lk(S.mu);
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n)
    return fail64(PF_EINVAL, "no CUDA device %d", device);
  S.device = device;
  return PF_OK;
}

static int f_trans_impl(const double* in, double* out, int Nx, int Ny, int Nz, const int* ist, const int* ien,
                        const int* fst, const int* fen) {
  if (!single_rank(ist, fst) || ien[0] != Nx || ien[1] != Ny || ien[2] != Nz || fen[0] != Nz || fen[1] != Ny ||
      fen[2] != Nx / 2 + 1)
    return fail64(PF_EINVAL, "f_trans_: only the single-rank layout ist=fst=1, ien=(Nx,Ny,Nz), fen=(Nz,Ny,Nx/2+1)");
  ShimCtx& S = shim();
  std::lock_guard<std::mutex> lk(S.mu);
  P64_CUDA(cudaSetDevice(S.device));
  ShimCtx::Plans* pl;
  int rc = shim_plans(Nx, Ny, Nz, &pl);
  if (rc) return rc;
  const size_t n = (size_t)Nx * Ny * Nz, ns = (size_t)(Nx / 2 + 1) * Ny * Nz;
  P64_CUDA(cudaMemcpy(pl->real, in, n * sizeof(double), cudaMemcpyHostToDevice));
  P64_FFT(cufftExecD2Z(pl->f, pl->real, pl->a));
  p64_zyx_to_xyz<<<NB, NT>>>(pl->a, pl->b, Nx / 2 + 1, Ny, Nz, 1.0 / (double)n);
  P64_CUDA(cudaGetLastError());
  P64_CUDA(cudaMemcpy(out, pl->b, ns * sizeof(cufftDoubleComplex), cudaMemcpyDeviceToHost));
  return PF_OK;
}

void f_trans_(const double* in, double* out, const int* Nx, const int* Ny, const int* Nz, const int* ist,
              const int* ien, const int* fst, const int* fen) {
  shim_report(f_trans_impl(in, out, *Nx, *Ny, *Nz, ist, ien, fst, fen), "f_trans_");
}

static int inv_trans_impl(const double* in, double* out, const int* ist, const int* ien, const int* fst,
                          const int* fen) {
  const int Nx = ien[0] - ist[0] + 1, Ny = ien[1] - ist[1] + 1, Nz = ien[2] - ist[2] + 1;
  if (!single_rank(ist, fst) || fen[0] != Nz || fen[1] != Ny || fen[2] != Nx / 2 + 1)
    return fail64(PF_EINVAL, "inv_trans_: only the single-rank layout is supported");
  ShimCtx& S = shim();
  std::lock_guard<std::mutex> lk(S.mu);
  P64_CUDA(cudaSetDevice(S.device));
  ShimCtx::Plans* pl;
  int rc = shim_plans(Nx, Ny, Nz, &pl);
  if (rc) return rc;
  const size_t n = (size_t)Nx * Ny * Nz, ns = (size_t)(Nx / 2 + 1) * Ny * Nz;
  P64_CUDA(cudaMemcpy(pl->b, in, ns * sizeof(cufftDoubleComplex), cudaMemcpyHostToDevice));
  p64_xyz_to_zyx<<<NB, NT>>>(pl->b, pl->a, Nx / 2 + 1, Ny, Nz);
  P64_CUDA(cudaGetLastError());
  P64_FFT(cufftExecZ2D(pl->i, pl->a, pl->real));
  P64_CUDA(cudaMemcpy(out, pl->real, n * sizeof(double), cudaMemcpyDeviceToHost));
  return PF_OK;
}

void inv_trans_(const double* in, double* out, const int* ist, const int* ien, const int* fst, const int* fen) {
  shim_report(inv_trans_impl(in, out, ist, ien, fst, fen), "inv_trans_");
}

// src/k_space.f90:13-59 on the caller's (possibly partial) spectral pencil:
// kf(3, fst(1):fen(1), fst(2):fen(2), fst(3):fen(3)) complex, dim 1 = z, dim 3 = kx.
void k_space_(const int* Nx, const int* Ny, const int* Nz, const int* fst, const int* fen, double* kf, double* kf_sq,
              double* kf_4) {
  const double pi = std::atan(1.0) * 4.0;
  const double u1 = 2.0 * pi / (double)*Nx, u2 = 2.0 * pi / (double)*Ny, u3 = 2.0 * pi / (double)*Nz;
  const int n1 = fen[0] - fst[0] + 1, n2 = fen[1] - fst[1] + 1;
  for (int i = fst[2]; i <= fen[2]; ++i) {
    const int ii = i - 1;
    const double l1 = (ii <= *Nx / 2 ? ii : ii - *Nx) * u1;
    for (int j = fst[1]; j <= fen[1]; ++j) {
      const int jj = j - 1;
      const double l2 = (jj <= *Ny / 2 ? jj : jj - *Ny) * u2;
      for (int k = fst[0]; k <= fen[0]; ++k) {
        const int kk = k - 1;
        const double l3 = (kk <= *Nz / 2 ? kk : kk - *Nz) * u3;
        const size_t cell = ((size_t)(i - fst[2]) * n2 + (j - fst[1])) * n1 + (k - fst[0]);
        double* a = kf + cell * 6;
        double* b = kf_sq + cell * 6;
        double* c = kf_4 + cell * 6;
        const double l[3] = {l1, l2, l3};
        const bool nyq[3] = {2 * ii == *Nx, 2 * jj == *Ny, 2 * kk == *Nz};
        for (int d = 0; d < 3; ++d) {
          a[2 * d] = 0.0;
          a[2 * d + 1] = nyq[d] ? 0.0 : l[d];
          b[2 * d] = -l[d] * l[d];
          b[2 * d + 1] = 0.0;
          c[2 * d] = l[d] * l[d] * l[d] * l[d];
          c[2 * d + 1] = 0.0;
        }
      }
    }
  }
}

}  // extern "C"
