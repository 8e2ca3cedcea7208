// Host-side helpers of the drop-in driver that need no GPU.
//
// pf_ran2 restates the saved-state generator ran_2 of src/ran_2.f90:1-40
// (L'Ecuyer combined generator with a 32-entry Bays-Durham shuffle).  The
// saved Fortran variables (iv, iy, idum2) live in a caller-owned state so that
// several runs can draw independent streams.
#include <cstring>

#include "../../include/pfgpu.h"

namespace {
const int IM1 = 2147483563, IM2 = 2147483399, IMM1 = IM1 - 1;
const int IA1 = 40014, IA2 = 40692, IQ1 = 53668, IQ2 = 52774, IR1 = 12211, IR2 = 3791;
const int NTAB = 32, NDIV = 1 + IMM1 / NTAB;
// am = 1./im1 is evaluated in REAL*4 (src/ran_2.f90:5): both the conversion of
// im1 and the quotient round to single precision before widening.
const double AM = (double)(1.0f / (float)IM1);
const double EPS = 1.2e-7;
const double RNMX = 1.0 - EPS;
}  // namespace

extern "C" {

void pf_ran2_init(pf_ran2_state* st) {
  memset(st, 0, sizeof *st);
  st->idum2 = 123456789;  // data idum2 /123456789/, iv /ntab*0/, iy /0/
}

double pf_ran2(pf_ran2_state* st, int* idum_p) {
  int idum = *idum_p;
  int k, j;
  if (idum <= 0) {
    idum = (-idum > 1) ? -idum : 1;
    st->idum2 = idum;
    for (j = NTAB + 8; j >= 1; --j) {
      k = idum / IQ1;
      idum = IA1 * (idum - k * IQ1) - k * IR1;
      if (idum < 0) idum += IM1;
      if (j <= NTAB) st->iv[j - 1] = idum;
    }
    st->iy = st->iv[0];
  }
  k = idum / IQ1;
  idum = IA1 * (idum - k * IQ1) - k * IR1;
  if (idum < 0) idum += IM1;
  k = st->idum2 / IQ2;
  st->idum2 = IA2 * (st->idum2 - k * IQ2) - k * IR2;
  if (st->idum2 < 0) st->idum2 += IM2;
  j = 1 + st->iy / NDIV;
  st->iy = st->iv[j - 1] - st->idum2;
  st->iv[j - 1] = idum;
  if (st->iy < 1) st->iy += IMM1;
  *idum_p = idum;
  const double v = AM * (double)st->iy;
  return v < RNMX ? v : RNMX;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Seeded initial conditions.  Fields are written in the Fortran order of the
// C ABI: phi(var, x, y, z) (var fastest) and con(x, y, z).
// ---------------------------------------------------------------------------
#include <algorithm>
#include <cmath>
#include <thread>
#include <vector>

namespace {

struct Stream {
  pf_ran2_state st;
  int idum;
  explicit Stream(int seed) {
    pf_ran2_init(&st);
    idum = -(seed + 1);  // seed 0 == the reference default iseed = -1
  }
  double next() { return pf_ran2(&st, &idum); }
};

bool bad_cfg(const pf_config* c) { return !c || c->nx < 1 || c->ny < 1 || c->nz < 1 || c->var < 1; }

// noise draws: z, y, x (x fastest); per cell var phi values, then c
void add_noise(const pf_config* c, Stream& rs, double amp_phi, double c0, double amp_c, double* phi, double* con) {
  const int V = c->var;
  const size_t ncell = (size_t)c->nx * c->ny * c->nz;
  for (size_t i = 0; i < ncell; ++i) {
    for (int f = 0; f < V; ++f) phi[i * V + f] += amp_phi * (2.0 * rs.next() - 1.0);
    con[i] = c0 + amp_c * (2.0 * rs.next() - 1.0);
  }
}

}  // namespace

extern "C" {

int pf_ic_noise(const pf_config* c, int seed, double amp_phi, double c0, double amp_c, double* phi, double* con) {
  if (bad_cfg(c) || !phi || !con) return PF_EINVAL;
  const size_t ncell = (size_t)c->nx * c->ny * c->nz;
  std::fill(phi, phi + ncell * c->var, 0.0);
  Stream rs(seed);
  add_noise(c, rs, amp_phi, c0, amp_c, phi, con);
  return PF_OK;
}

int pf_ic_voronoi(const pf_config* c, int seed, int n_grains, double amp_phi, double c0, double amp_c, double* phi,
                  double* con) {
  if (bad_cfg(c) || !phi || !con || n_grains < 1) return PF_EINVAL;
  const int Nx = c->nx, Ny = c->ny, Nz = c->nz, V = c->var;
  Stream rs(seed);
  std::vector<double> sx(n_grains), sy(n_grains), sz(n_grains);
  for (int s = 0; s < n_grains; ++s) {
    sx[s] = Nx * rs.next();
    sy[s] = Ny * rs.next();
    sz[s] = Nz * rs.next();
  }
  const size_t ncell = (size_t)Nx * Ny * Nz;
  std::fill(phi, phi + ncell * V, 0.0);
  auto mi = [](double d, int n) {
    d = std::fabs(d);
    return std::min(d, n - d);
  };
  // nearest seed (periodic minimum image, ties to the lower index); z-slabs in parallel
  auto work = [&](int z0, int z1) {
    for (int z = z0; z < z1; ++z)
      for (int y = 0; y < Ny; ++y)
        for (int x = 0; x < Nx; ++x) {
          double best = INFINITY;
          int lab = 0;
          for (int s = 0; s < n_grains; ++s) {
            const double dz = mi(z - sz[s], Nz), dy = mi(y - sy[s], Ny), dx = mi(x - sx[s], Nx);
            const double d2 = dz * dz + dy * dy + dx * dx;
            if (d2 < best) {
              best = d2;
              lab = s;
            }
          }
          const size_t i = ((size_t)z * Ny + y) * Nx + x;
          phi[i * V + (lab % V)] = 1.0;
        }
  };
  const int nth = std::max(1, std::min((int)std::thread::hardware_concurrency(), Nz));
  std::vector<std::thread> th;
  for (int t = 0; t < nth; ++t) th.emplace_back(work, (int)((long)Nz * t / nth), (int)((long)Nz * (t + 1) / nth));
  for (auto& t : th) t.join();
  add_noise(c, rs, amp_phi, c0, amp_c, phi, con);
  return PF_OK;
}

}  // extern "C"
