// Host-side files and starts of the drop-in driver (no GPU needed):
//  * input.txt reader with Fortran list-directed semantics
//    (src/var_diff.f90:104-121, format written by tests/run_phase_sim.py:112-128);
//  * data_save.NNNN / data_rerun.NNNN as Fortran unformatted sequential
//    records (src/var_diff.f90:451-461, :1134-1140), gfortran record markers;
//  * the reference's 'circle', 'plane' and 'polycryst' starts
//    (src/var_diff.f90:229-449) and the precipitate insertion at ppt_int
//    (:479-554), all on one rank (ist = 1, ien = N).
#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "../../include/pfgpu.h"

namespace {

thread_local std::string g_io_err;

int io_fail(int code, const std::string& m) {
  g_io_err = m;
  return code;
}

// ---------------------------------------------------------------------------
// Fortran list-directed input
// ---------------------------------------------------------------------------
struct ListReader {
  std::vector<std::string> lines;
  size_t line = 0;

  // Tokens of one READ statement that wants `n` items: values are separated
  // by blanks or commas, r*c repeats c, quoted strings are one value, a '/'
  // ends the statement (the remaining items keep their values), and the
  // statement continues on following lines until it has n values.  Returns
  // the values read (possibly fewer than n).
  std::vector<std::string> read(int n) {
    std::vector<std::string> out;
    bool stop = false;
    while (!stop && (int)out.size() < n && line < lines.size()) {
      const std::string& s = lines[line++];
      size_t i = 0;
      while (i < s.size() && (int)out.size() < n) {
        while (i < s.size() && (isspace((unsigned char)s[i]) || s[i] == ',')) ++i;
        if (i >= s.size()) break;
        if (s[i] == '/') {
          stop = true;
          break;
        }
        std::string tok;
        if (s[i] == '\'' || s[i] == '"') {
          const char q = s[i++];
          while (i < s.size()) {
            if (s[i] == q) {
              if (i + 1 < s.size() && s[i + 1] == q) {
                tok += q;
                i += 2;
                continue;
              }
              ++i;
              break;
            }
            tok += s[i++];
          }
        } else {
          while (i < s.size() && !isspace((unsigned char)s[i]) && s[i] != ',' && s[i] != '/') tok += s[i++];
        }
        const size_t star = tok.find('*');
        if (star != std::string::npos && star > 0 && isdigit((unsigned char)tok[0])) {
          const int r = atoi(tok.substr(0, star).c_str());
          const std::string v = tok.substr(star + 1);
          for (int k = 0; k < r && (int)out.size() < n; ++k) out.push_back(v);
        } else {
          out.push_back(tok);
        }
      }
    }
    return out;
  }
};

double fnum(const std::string& t) {
  std::string s = t;
  for (char& c : s)
    if (c == 'd' || c == 'D') c = 'e';
  return strtod(s.c_str(), nullptr);
}

int inum(const std::string& t) { return (int)strtol(t.c_str(), nullptr, 10); }

// ---------------------------------------------------------------------------
// Fortran unformatted sequential records (gfortran layout): each record is
// framed by 4-byte lengths; records above 2^31-9 bytes are split into
// sub-records whose leading marker is negative when another sub-record
// follows and whose trailing marker is negative when one precedes.
// ---------------------------------------------------------------------------
const int64_t kMaxSub = 2147483639LL;

bool write_record(FILE* f, const std::vector<std::pair<const void*, size_t>>& parts) {
  size_t total = 0;
  for (auto& p : parts) total += p.second;
  size_t done = 0, pi = 0, po = 0;
  bool first = true;
  do {
    const size_t len = std::min<size_t>(total - done, (size_t)kMaxSub);
    const bool more = done + len < total;
    const int32_t head = more ? -(int32_t)len : (int32_t)len;
    const int32_t tail = first ? (int32_t)len : -(int32_t)len;
    if (fwrite(&head, 4, 1, f) != 1) return false;
    size_t left = len;
    while (left > 0) {
      const size_t take = std::min(left, parts[pi].second - po);
      if (fwrite((const char*)parts[pi].first + po, 1, take, f) != take) return false;
      po += take;
      left -= take;
      if (po == parts[pi].second) {
        ++pi;
        po = 0;
      }
    }
    if (fwrite(&tail, 4, 1, f) != 1) return false;
    done += len;
    first = false;
  } while (done < total);
  return true;
}

// Read one record into `parts` (exact sizes required).
bool read_record(FILE* f, const std::vector<std::pair<void*, size_t>>& parts) {
  size_t want = 0;
  for (auto& p : parts) want += p.second;
  size_t got = 0, pi = 0, po = 0;
  for (;;) {
    int32_t head, tail;
    if (fread(&head, 4, 1, f) != 1) return false;
    const size_t len = (size_t)(head < 0 ? -(int64_t)head : head);
    size_t left = len;
    if (got + len > want) return false;
    while (left > 0) {
      const size_t take = std::min(left, parts[pi].second - po);
      if (fread((char*)parts[pi].first + po, 1, take, f) != take) return false;
      po += take;
      left -= take;
      if (po == parts[pi].second) {
        ++pi;
        po = 0;
      }
    }
    if (fread(&tail, 4, 1, f) != 1) return false;
    got += len;
    if (head >= 0) break;
  }
  return got == want;
}

size_t cell(const pf_config* c, int i, int j, int k) {  // 1-based Fortran indices
  return ((size_t)(k - 1) * c->ny + (j - 1)) * c->nx + (i - 1);
}

// (i/r)^2 + (j/r)^2 + (k/r)^2 <= 1 with float(i)/float(r) in REAL*4 (:303-306)
bool in_ellipsoid(int i, int j, int k, int rx, int ry, int rz) {
  const float a = (float)i / (float)rx, b = (float)j / (float)ry, c = (float)k / (float)rz;
  const double s = (double)(a * a) + (double)(b * b) + (double)(c * c);
  return s <= 1.0;
}

// The cells (i, j, k) with (i-ix)^2 + (j-jy)^2 + (k-kz)^2 <= rad, no periodic
// wrap, that the reference's precipitate placement finds by scanning the
// whole grid (src/var_diff.f90:424-447, :517-548).  Only the bounding box of
// that ball, clipped to the grid, can hold one, so both scans visit that box:
// the same cells in the same order, O(R^3) per attempt instead of O(N^3).
struct Ball {
  int ix, jy, kz, rad, i0, i1, j0, j1, k0, k1;
  Ball(const pf_config* c, int x, int y, int z, int r2) : ix(x), jy(y), kz(z), rad(r2) {
    int R = 0;  // largest offset with R^2 <= rad
    while ((R + 1) * (R + 1) <= rad) ++R;
    i0 = std::max(1, ix - R); i1 = std::min(c->nx, ix + R);
    j0 = std::max(1, jy - R); j1 = std::min(c->ny, jy + R);
    k0 = std::max(1, kz - R); k1 = std::min(c->nz, kz + R);
  }
  bool inside(int i, int j, int k) const {
    return (i - ix) * (i - ix) + (j - jy) * (j - jy) + (k - kz) * (k - kz) <= rad;
  }
  // does any cell of the ball already have phi_V > 0?
  bool hits(const pf_config* c, const double* phi) const {
    const int V = c->var;
    for (int k = k0; k <= k1; ++k)
      for (int j = j0; j <= j1; ++j)
        for (int i = i0; i <= i1; ++i)
          if (inside(i, j, k) && phi[cell(c, i, j, k) * V + (V - 1)] > 0.0) return true;
    return false;
  }
  template <class F>
  void each(F f) const {
    for (int k = k0; k <= k1; ++k)
      for (int j = j0; j <= j1; ++j)
        for (int i = i0; i <= i1; ++i)
          if (inside(i, j, k)) f(i, j, k);
  }
};

}  // namespace

extern "C" {

const char* pf_io_last_error(void) { return g_io_err.c_str(); }

int pf_read_input(const char* path, int nprocs, pf_input* in) {
  if (!path || !in) return io_fail(PF_EINVAL, "null argument");
  std::ifstream fh(path);
  if (!fh) return io_fail(PF_EIO, std::string("cannot open ") + path);
  ListReader r;
  for (std::string l; std::getline(fh, l);) r.lines.push_back(l);
  memset(in, 0, sizeof *in);
  in->seed = 0;
  in->mobility = PF_MOB_REFERENCE;
  in->precision = 0;  // 0: the caller chooses (fused FP32 where the grid is supported)
  in->amp_phi = 0.01;
  in->amp_c = 0.01;
  in->c0 = 0.5;
  in->n_grains = 8;
  snprintf(in->microstructure, sizeof in->microstructure, "mc_ivar_fin");
  in->check_fp64 = 0;
  std::vector<std::string> v;
  auto take_i = [&](int idx, int* dst, int bit) {
    if ((int)v.size() > idx) { *dst = inum(v[idx]); in->set_mask |= (1ull << bit); }
  };
  auto take_d = [&](int idx, double* dst, int bit) {
    if ((int)v.size() > idx) { *dst = fnum(v[idx]); in->set_mask |= (1ull << bit); }
  };
  v = r.read(2);  // nrun, ppt_int
  take_i(0, &in->nrun, 0); take_i(1, &in->ppt_int, 1);
  v = r.read(5);  // ppt_rad(3), N_step, ifreq
  take_i(0, &in->ppt_rad[0], 2); take_i(1, &in->ppt_rad[1], 2); take_i(2, &in->ppt_rad[2], 2);
  take_i(3, &in->N_step, 3); take_i(4, &in->ifreq, 4);
  v = r.read(4);  // i_ppt, j_ppt, k_ppt, iseed
  take_i(0, &in->i_ppt, 5); take_i(1, &in->j_ppt, 5); take_i(2, &in->k_ppt, 5); take_i(3, &in->iseed, 6);
  v = r.read(4);  // grn_rad, num_ppt, c_mat, c_ppt
  take_i(0, &in->grn_rad, 7); take_i(1, &in->num_ppt, 8); take_d(2, &in->c_mat, 9); take_d(3, &in->c_ppt, 10);
  v = r.read(8);  // Nx, Ny, Nz, var, dx, dy, dz, t_step
  take_i(0, &in->Nx, 11); take_i(1, &in->Ny, 11); take_i(2, &in->Nz, 11); take_i(3, &in->var, 12);
  take_d(4, &in->dx, 13); take_d(5, &in->dy, 13); take_d(6, &in->dz, 13); take_d(7, &in->t_step, 14);
  v = r.read(6);  // grad_coeff_phi, grad_coeff_c, D_S, D_L, D_gb, mob_phi
  take_d(0, &in->grad_coeff_phi, 15); take_d(1, &in->grad_coeff_c, 16); take_d(2, &in->D_S, 17);
  take_d(3, &in->D_L, 18); take_d(4, &in->D_gb, 19); take_d(5, &in->mob_phi, 20);
  v = r.read(2);  // sigma_1, sigma_2
  take_d(0, &in->sigma_1, 21); take_d(1, &in->sigma_2, 21);
  v = r.read(5);  // am, ap, con_0_mat, con_0_ppt, gb_force
  take_d(0, &in->am, 22); take_d(1, &in->ap, 22); take_d(2, &in->con_0_mat, 23); take_d(3, &in->con_0_ppt, 23);
  take_d(4, &in->gb_force, 24);
  v = r.read(1);  // ndim
  take_i(0, &in->ndim, 25);
  if (in->ndim == 1) {
    in->dims[0] = 1;
    in->dims[1] = nprocs;
  } else if (in->ndim == 2) {
    v = r.read(2);
    take_i(0, &in->dims[0], 26); take_i(1, &in->dims[1], 26);
  }
  v = r.read(1);  // start
  if (!v.empty()) {
    snprintf(in->start, sizeof in->start, "%s", v[0].c_str());
    in->set_mask |= (1ull << 27);
  }
  // optional trailing key=value lines (ignored by the reference): seed,
  // n_grains, amp_phi, amp_c, c0, mobility (reference|c1mc), precision (32|64)
  for (; r.line < r.lines.size(); ++r.line) {
    std::istringstream ss(r.lines[r.line]);
    std::string tok;
    while (ss >> tok) {
      const size_t eq = tok.find('=');
      if (eq == std::string::npos) continue;
      const std::string k = tok.substr(0, eq), val = tok.substr(eq + 1);
      if (k == "seed") in->seed = inum(val);
      else if (k == "n_grains") in->n_grains = inum(val);
      else if (k == "amp_phi") in->amp_phi = fnum(val);
      else if (k == "amp_c") in->amp_c = fnum(val);
      else if (k == "c0") in->c0 = fnum(val);
      else if (k == "mobility") in->mobility = (val == "c1mc") ? PF_MOB_C1MC : PF_MOB_REFERENCE;
      else if (k == "precision") in->precision = inum(val);
      else if (k == "microstructure") snprintf(in->microstructure, sizeof in->microstructure, "%s", val.c_str());
      else if (k == "check_fp64") in->check_fp64 = inum(val);
    }
  }
  if (!(in->set_mask & (1ull << 11)) || in->Nx < 1 || in->Ny < 1 || in->Nz < 1 || in->var < 1)
    return io_fail(PF_EINVAL, std::string(path) + ": grid or var missing");
  return PF_OK;
}

void pf_input_to_config(const pf_input* in, pf_config* c) {
  memset(c, 0, sizeof *c);
  c->nx = in->Nx; c->ny = in->Ny; c->nz = in->Nz; c->var = in->var;
  c->t_step = in->t_step; c->grad_coeff_phi = in->grad_coeff_phi; c->grad_coeff_c = in->grad_coeff_c;
  c->D_S = in->D_S; c->D_L = in->D_L; c->D_gb = in->D_gb; c->mob_phi = in->mob_phi;
  c->sigma_1 = in->sigma_1; c->sigma_2 = in->sigma_2;
  c->am = in->am; c->ap = in->ap; c->con_0_mat = in->con_0_mat; c->con_0_ppt = in->con_0_ppt;
  c->mobility = in->mobility;
  c->precision = in->precision ? in->precision : PF_FP32_FUSED;
}

int pf_write_data_save(const char* path, const pf_config* c, const double* phi, const double* con) {
  if (!path || !c || !phi || !con) return io_fail(PF_EINVAL, "null argument");
  FILE* f = fopen(path, "wb");
  if (!f) return io_fail(PF_EIO, std::string("cannot create ") + path + ": " + strerror(errno));
  const int32_t b[6] = {1, 1, 1, c->nx, c->ny, c->nz};  // ist(3), ien(3) of the single rank
  const size_t n = (size_t)c->nx * c->ny * c->nz;
  const bool ok = write_record(f, {{b, sizeof b}}) &&
                  write_record(f, {{phi, n * c->var * sizeof(double)}, {con, n * sizeof(double)}});
  const bool closed = fclose(f) == 0;
  return (ok && closed) ? PF_OK : io_fail(PF_EIO, std::string("write failed: ") + path);
}

int pf_read_data_save(const char* path, const pf_config* c, double* phi, double* con) {
  if (!path || !c || !phi || !con) return io_fail(PF_EINVAL, "null argument");
  FILE* f = fopen(path, "rb");
  if (!f) return io_fail(PF_EIO, std::string("cannot open ") + path);
  int32_t b[6];
  const size_t n = (size_t)c->nx * c->ny * c->nz;
  bool ok = read_record(f, {{b, sizeof b}});
  ok = ok && b[0] == 1 && b[1] == 1 && b[2] == 1 && b[3] == c->nx && b[4] == c->ny && b[5] == c->nz;
  ok = ok && read_record(f, {{phi, n * c->var * sizeof(double)}, {con, n * sizeof(double)}});
  fclose(f);
  return ok ? PF_OK : io_fail(PF_EIO, std::string("not a single-rank data_save record of this grid: ") + path);
}

// 'circle' start (src/var_diff.f90:373-449): returns the updated idum.
int pf_ic_circle(const pf_config* c, int grn_rad, const int* ppt_rad, int num_ppt, int* idum, double c_mat,
                 double con_0_ppt, pf_ran2_state* st, double* phi, double* con) {
  if (!c || !ppt_rad || !idum || !st || !phi || !con || c->var < 3)
    return io_fail(PF_EINVAL, "circle start needs var >= 3");
  const int V = c->var, Nx = c->nx, Ny = c->ny, Nz = c->nz;
  const size_t n = (size_t)Nx * Ny * Nz;
  for (size_t i = 0; i < n * V; ++i) phi[i] = 0.0;
  for (size_t i = 0; i < n; ++i) {
    phi[i * V + 0] = 1.0;
    con[i] = c_mat;
  }
  for (int k = -grn_rad; k <= grn_rad; ++k)
    for (int j = -grn_rad; j <= grn_rad; ++j)
      for (int i = -grn_rad; i <= grn_rad; ++i) {
        if (!in_ellipsoid(i, j, k, grn_rad, grn_rad, grn_rad)) continue;
        const int ii = i + Nx / 2, jj = j + Ny / 2, kk = k + Nz / 2;
        if (ii < 1 || ii > Nx || jj < 1 || jj > Ny || kk < 1 || kk > Nz) continue;
        double* p = phi + cell(c, ii, jj, kk) * V;
        p[1] = 1.0; p[0] = 0.0; p[2] = 0.0;
      }
  const int rad = ppt_rad[0] * ppt_rad[0] + ppt_rad[1] * ppt_rad[1] + ppt_rad[2] * ppt_rad[2];
  int nppt = 1;
  long guard = 0;
  while (nppt <= num_ppt) {
    if (++guard > 100000000L) return io_fail(PF_EINVAL, "circle start: no free place for a precipitate");
    const int ix = (int)(pf_ran2(st, idum) * Nx + 1.0);
    const int jy = (int)(pf_ran2(st, idum) * Ny + 1.0);
    const int kz = (int)(pf_ran2(st, idum) * Nz + 1.0);
    const Ball ball(c, ix, jy, kz, rad);
    if (ball.hits(c, phi)) continue;
    ball.each([&](int i, int j, int k) {
      double* p = phi + cell(c, i, j, k) * V;
      p[2] = 1.0; p[1] = 0.0; p[0] = 0.0;
      con[cell(c, i, j, k)] = con_0_ppt;
    });
    ++nppt;
  }
  return PF_OK;
}

// 'plane' start (src/var_diff.f90:252-371)
int pf_ic_plane(const pf_config* c, const int* ppt_rad, int i_ppt, int j_ppt, int k_ppt, double c_mat, double* phi,
                double* con) {
  if (!c || !ppt_rad || !phi || !con || c->var < 3) return io_fail(PF_EINVAL, "plane start needs var >= 3");
  const int V = c->var, Nx = c->nx, Ny = c->ny, Nz = c->nz;
  const size_t n = (size_t)Nx * Ny * Nz;
  for (size_t i = 0; i < n * V; ++i) phi[i] = 0.0;
  for (size_t i = 0; i < n; ++i) con[i] = c_mat;
  const int j1 = Ny - j_ppt + 1;
  for (int kk = 1; kk <= Nz; ++kk)
    for (int jj = 1; jj <= Ny; ++jj)
      for (int ii = 1; ii <= Nx; ++ii) {
        double* p = phi + cell(c, ii, jj, kk) * V;
        p[1] = 1.0;
        if (jj < j1 || jj >= j_ppt) {
          for (int f = 0; f < V; ++f) p[f] = 0.0;
          p[0] = 1.0;
        }
      }
  for (int jc : {j_ppt, Ny - j_ppt + 1})
    for (int k = -ppt_rad[2]; k <= ppt_rad[2]; ++k)
      for (int j = -ppt_rad[1]; j <= ppt_rad[1]; ++j)
        for (int i = -ppt_rad[0]; i <= ppt_rad[0]; ++i) {
          if (!in_ellipsoid(i, j, k, ppt_rad[0], ppt_rad[1], ppt_rad[2])) continue;
          const int ii = i + i_ppt, jj = j + jc, kk = k + k_ppt;
          if (ii < 1 || ii > Nx || jj < 1 || jj > Ny || kk < 1 || kk > Nz) continue;
          double* p = phi + cell(c, ii, jj, kk) * V;
          p[2] = 1.0; p[0] = 0.0; p[1] = 0.0;
        }
  return PF_OK;
}

// 'polycryst' start (src/var_diff.f90:232-250): Nx*Ny*Nz lines "ii jj kk ivar"
int pf_ic_polycryst(const pf_config* c, const char* path, double c_mat, double* phi, double* con) {
  if (!c || !path || !phi || !con) return io_fail(PF_EINVAL, "null argument");
  FILE* f = fopen(path, "r");
  if (!f) return io_fail(PF_EIO, std::string("cannot open microstructure file ") + path);
  const int V = c->var;
  const size_t n = (size_t)c->nx * c->ny * c->nz;
  for (size_t i = 0; i < n * V; ++i) phi[i] = 0.0;
  for (size_t i = 0; i < n; ++i) con[i] = c_mat;
  for (size_t q = 0; q < n; ++q) {
    int ii, jj, kk, iv;
    if (fscanf(f, "%d %d %d %d", &ii, &jj, &kk, &iv) != 4) {
      fclose(f);
      return io_fail(PF_EIO, std::string(path) + ": short microstructure file");
    }
    if (ii >= 1 && ii <= c->nx && jj >= 1 && jj <= c->ny && kk >= 1 && kk <= c->nz && iv >= 1 && iv <= V)
      phi[cell(c, ii, jj, kk) * V + (iv - 1)] = 1.0;
  }
  fclose(f);
  return PF_OK;
}

// Precipitate insertion at step == ppt_int (src/var_diff.f90:479-554).
int pf_insert_precipitates(const pf_config* c, const int* ppt_rad, int num_ppt, int* idum, pf_ran2_state* st,
                           double* phi) {
  if (!c || !ppt_rad || !idum || !st || !phi) return io_fail(PF_EINVAL, "null argument");
  const int V = c->var, Nx = c->nx, Ny = c->ny, Nz = c->nz, mat = V - 1;
  const int rad = ppt_rad[0] * ppt_rad[0] + ppt_rad[1] * ppt_rad[1] + ppt_rad[2] * ppt_rad[2];
  int nppt = 1;
  long guard = 0;
  while (nppt <= num_ppt) {
    if (++guard > 100000000L) return io_fail(PF_EINVAL, "precipitate insertion: no admissible place");
    const int ix = (int)(pf_ran2(st, idum) * Nx + 1.0);
    const int jy = (int)(pf_ran2(st, idum) * Ny + 1.0);
    const int kz = (int)(pf_ran2(st, idum) * Nz + 1.0);
    double s = 0.0;
    if (ix >= 1 && ix <= Nx && jy >= 1 && jy <= Ny && kz >= 1 && kz <= Nz)
      for (int f = 0; f < mat; ++f) {
        const double fi = phi[cell(c, ix, jy, kz) * V + f];
        s += fi * fi;
      }
    if (s > 0.8) continue;  // inside a grain: try again
    const Ball ball(c, ix, jy, kz, rad);
    if (ball.hits(c, phi)) continue;
    ball.each([&](int i, int j, int k) {
      double* p = phi + cell(c, i, j, k) * V;
      p[V - 1] = 1.0;
      for (int f = 0; f < mat; ++f) p[f] = 0.0;
    });
    ++nppt;
  }
  return PF_OK;
}

// Fortran Ew.d edit descriptor (0.ddddE+ee), as used by summary.dat's (i6, 8e15.7)
void pf_format_e(double x, int w, int d, char* out) {
  char body[64];
  if (!std::isfinite(x)) {
    snprintf(body, sizeof body, "%s", std::isnan(x) ? "NaN" : (x > 0 ? "Infinity" : "-Infinity"));
  } else if (x == 0.0) {
    snprintf(body, sizeof body, "%s0.%0*dE+00", std::signbit(x) ? "-" : "", d, 0);
  } else {
    // d significant digits, correctly rounded by printf: d.ddd e+XX -> 0.dddd E+(XX+1)
    char sci[64];
    snprintf(sci, sizeof sci, "%.*e", d - 1, std::fabs(x));
    std::string digits;
    const char* p = sci;
    for (; *p && *p != 'e'; ++p)
      if (isdigit((unsigned char)*p)) digits += *p;
    const int e = atoi(p + 1) + 1;
    char exp[8];
    if (std::abs(e) < 100) snprintf(exp, sizeof exp, "E%c%02d", e < 0 ? '-' : '+', std::abs(e));
    else snprintf(exp, sizeof exp, "%c%03d", e < 0 ? '-' : '+', std::abs(e));
    snprintf(body, sizeof body, "%s0.%s%s", x < 0 ? "-" : "", digits.c_str(), exp);
  }
  const int len = (int)strlen(body);
  if (len > w) {
    for (int i = 0; i < w; ++i) out[i] = '*';
    out[w] = 0;
  } else {
    snprintf(out, w + 1, "%*s", w, body);
  }
}

void pf_format_summary(int step, const pf_diag* d, char* out) {
  const double v[8] = {d->f_int, d->f_ch, d->f_eta, d->e_tot, d->c_max, d->c_min, d->phi_min, d->phi_P_max};
  int n = snprintf(out, 16, "%6d", step);
  if (n > 6) {  // i6 overflow prints asterisks
    memset(out, '*', 6);
    n = 6;
  }
  for (int i = 0; i < 8; ++i) {
    pf_format_e(v[i], 15, 7, out + n);
    n += 15;
  }
  out[n] = 0;
}

void pf_format_list_int(int v, char* out) { snprintf(out, 32, " %11d", v); }

// gfortran list-directed REAL*8: G25.17E3 with one separator blank; F form
// (right-justified in 20, then 5 blanks) for 0.1 <= |x| < 1e17 and zero,
// else 1PE25.17E3.
void pf_format_list_real(double v, char* out) {
  if (!std::isfinite(v)) {
    snprintf(out, 32, " %25s", std::isnan(v) ? "NaN" : (v > 0 ? "Infinity" : "-Infinity"));
    return;
  }
  char sci[40];
  snprintf(sci, sizeof sci, "%.16e", v);
  const char* ep = strchr(sci, 'e');
  const int e10 = v == 0.0 ? 0 : atoi(ep + 1);
  char body[48];
  if (e10 >= -1 && e10 <= 16) {
    char f[40];
    if (e10 == 16) snprintf(f, sizeof f, "%.0f.", v);  // Fortran keeps the decimal point
    else snprintf(f, sizeof f, "%.*f", 16 - e10, v);
    snprintf(body, sizeof body, "%20s     ", f);
  } else {
    std::string m(sci, ep - sci);
    snprintf(body, sizeof body, "%25s", (m + "E" + (e10 < 0 ? "-" : "+") + [&] {
                                          char b[8];
                                          snprintf(b, sizeof b, "%03d", std::abs(e10));
                                          return std::string(b);
                                        }()).c_str());
  }
  snprintf(out, 32, " %s", body);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// ASCII VTK files of paraview.f90:277-296
// ---------------------------------------------------------------------------
namespace {

template <typename T, size_t W, typename F>
int write_vtk(const char* path, int nx, int ny, int nz, const T* v, F fmt) {
  if (!path || !v || nx < 1 || ny < 1 || nz < 1) return io_fail(PF_EINVAL, "null argument to the VTK writer");
  const size_t n = (size_t)nx * ny * nz;
  FILE* f = fopen(path, "w");
  if (!f) return io_fail(PF_EIO, std::string("cannot create ") + path);
  fprintf(f, "# vtk DataFile Version 3.0\nSample Data\nASCII\nDATASET STRUCTURED_POINTS\n");
  fprintf(f, "DIMENSIONS  %6d%6d%6d\nASPECT_RATIO 1.0 1.0 1.0\nORIGIN 0.0 0.0 0.0\n", nx, ny, nz);
  fprintf(f, "POINT_DATA  %12lld\nSCALARS Field double 1\nLOOKUP_TABLE default\n", (long long)n);
  // every item has a fixed width W: format blocks of values on all cores
  const size_t block = (size_t)1 << 18;
  const int nth = std::max(1, (int)std::thread::hardware_concurrency());
  std::vector<char> buf(std::min(n, block * nth) * W + 1);
  bool ok = true;
  for (size_t base = 0; base < n && ok; base += block * nth) {
    const size_t cnt = std::min(n - base, block * nth);
    std::vector<std::thread> th;
    for (int t = 0; t < nth; ++t) {
      const size_t a = (size_t)t * block, b = std::min(cnt, a + block);
      if (a >= b) break;
      th.emplace_back([&, a, b] {
        char item[40];
        for (size_t i = a; i < b; ++i) {
          fmt(v[base + i], item);
          memcpy(&buf[i * W], item, W);
        }
      });
    }
    for (auto& t : th) t.join();
    ok = fwrite(buf.data(), 1, cnt * W, f) == cnt * W;
  }
  ok = ok && fputc('\n', f) != EOF;
  ok = (fclose(f) == 0) && ok;
  return ok ? PF_OK : io_fail(PF_EIO, std::string("write failed: ") + path);
}

}  // namespace

extern "C" {

int pf_write_vtk_real(const char* path, int nx, int ny, int nz, const double* v) {
  return write_vtk<double, 26>(path, nx, ny, nz, v, [](double x, char* out) { pf_format_list_real(x, out); });
}

int pf_write_vtk_int(const char* path, int nx, int ny, int nz, const int* v) {
  return write_vtk<int, 12>(path, nx, ny, nz, v, [](int x, char* out) { pf_format_list_int(x, out); });
}

}  // extern "C"
