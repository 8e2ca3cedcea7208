// One var_diff.x case on the host: its input record, its output and restart
// files and its host copy of the fields.  Shared by pf_var_diff (one case,
// one pf_run) and pf_sweep (many cases, batched pf_batch runs), so that both
// write the same files (src/var_diff.f90:82-95, :205-225, :1054-1153).
#pragma once

#include <sys/stat.h>
#include <sys/types.h>

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "pfgpu.h"

namespace pfcase {

// A failed case: `code` is the process exit status the drivers report
// (2: set-up or I/O error, 3: a step produced non-finite values).
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline bool mkdir_p(const std::string& dir) {
  std::string cur;
  for (size_t i = 0; i <= dir.size(); ++i) {
    if (i == dir.size() || dir[i] == '/') {
      if (!cur.empty() && cur != "." && cur != "/") {
        if (mkdir(cur.c_str(), 0755) != 0 && errno != EEXIST) return false;
      }
    }
    if (i < dir.size()) cur += dir[i];
  }
  return true;
}

inline std::string list_int(int v) {
  char b[32];
  pf_format_list_int(v, b);
  return b;
}

inline std::string list_real(double v) {
  char b[32];
  pf_format_list_real(v, b);
  return b;
}

inline std::string f8_6(double v) {  // Fortran F8.6
  char b[32];
  snprintf(b, sizeof b, "%8.6f", v);
  if (strlen(b) > 8 || !std::isfinite(v)) return "********";
  return b;
}

inline void check(int rc, const char* what) {
  if (rc == PF_OK) return;
  throw Error(2, std::string(what) + ": " + pf_last_error() + pf_io_last_error());
}

// min over cells of sum_i phi_i^2 and max of phi_var, with the reference's
// start values 1 and 0 (src/var_diff.f90:1076-1102)
inline void phi_stats(const pf_config& c, const std::vector<double>& phi, double* phi_min, double* phi_p_max) {
  const size_t n = (size_t)c.nx * c.ny * c.nz;
  double mn = 1.0, mx = 0.0;
  for (size_t i = 0; i < n; ++i) {
    double s = 0.0;
    for (int f = 0; f < c.var; ++f) s += phi[i * c.var + f] * phi[i * c.var + f];
    mn = std::min(mn, s);
    mx = std::max(mx, phi[i * c.var + c.var - 1]);
  }
  *phi_min = mn;
  *phi_p_max = mx;
}

struct Case {
  pf_input in{};
  pf_config cfg{};
  std::string prefix;   // output prefix, concatenated as given
  std::string base;     // directory that relative restart/microstructure paths start from ("" = cwd)
  FILE* log = stdout;   // where the reference's stdout lines go
  FILE *f93 = nullptr, *f95 = nullptr, *f97 = nullptr, *f98 = nullptr;
  std::vector<double> phi, con;
  pf_ran2_state rs{};
  int idum = 0;
  double run_time = 0.0;
  double ins_phi_min = NAN, ins_phi_p = NAN;  // statistics before the last insertion

  Case() = default;
  Case(const Case&) = delete;
  Case& operator=(const Case&) = delete;
  ~Case() { close(); }

  // Read the input file and settle the precision: the fused FP32 path where
  // the grid is supported, else the FP64 cuFFT path (precision=0), or the
  // one the input names.
  void load(const std::string& input_path, const std::string& out_prefix, const std::string& base_dir) {
    prefix = out_prefix;
    base = base_dir;
    if (pf_read_input(input_path.c_str(), 1, &in) != PF_OK) throw Error(2, pf_io_last_error());
    pf_input_to_config(&in, &cfg);
    if (in.precision == 0)
      cfg.precision = pf_supported_shape(in.Nx, in.Ny, in.Nz, in.var, PF_FP32_FUSED) ? PF_FP32_FUSED : PF_FP64_PLAIN;
    if (!pf_supported_shape(in.Nx, in.Ny, in.Nz, in.var, cfg.precision))
      throw Error(2, "grid " + std::to_string(in.Nx) + "x" + std::to_string(in.Ny) + "x" + std::to_string(in.Nz) +
                         " var=" + std::to_string(in.var) + " is not supported by precision " +
                         std::to_string(cfg.precision));
    if (in.ifreq < 1) throw Error(2, "ifreq must be >= 1");
  }

  // check_fp64=N: the start stepped N times on the fused and the FP64 GPU
  // paths, the run's error reported on the log (fused-path runs only)
  void report_fp64_check() {
    if (in.check_fp64 <= 0 || cfg.precision != PF_FP32_FUSED) return;
    pf_error_report rep;
    if (pf_check_fp64(&cfg, phi.data(), con.data(), in.check_fp64, &rep) != PF_OK)
      throw Error(2, std::string("pf_check_fp64: ") + pf_last_error());
    fprintf(log, " fp64 check: %d steps, phi max-abs rel %.3e l2 rel %.3e, c max-abs rel %.3e l2 rel %.3e\n",
            rep.steps, rep.phi_max_abs_rel, rep.phi_l2_rel, rep.c_max_abs_rel, rep.c_l2_rel);
    fflush(log);
  }

  std::string path_of(const char* p) const {
    if (base.empty() || p[0] == '/') return p;
    return base + "/" + p;
  }

  FILE* open_out(const std::string& path) {
    FILE* f = fopen(path.c_str(), "w");
    if (!f) throw Error(2, "cannot create " + path);
    return f;
  }

  // output files with their headers (src/var_diff.f90:82-95) and gamma (:205-225)
  void open_outputs() {
    f93 = open_out(prefix + "time_step.dat");
    fprintf(f93, "# step number, iteration duration, %s run time elapsed\n", std::string(29, ' ').c_str());
    f95 = open_out(prefix + "timing_data.dat");
    std::string h = "# step number";
    for (int i = 1; i <= 7; ++i) h += ", loop " + std::to_string(i) + " avg";
    h += "," + std::string(40, ' ');
    for (int i = 8; i <= 14; ++i) h += (i == 8 ? "loop " : ", loop ") + std::to_string(i) + " avg";
    h += "," + std::string(40, ' ') + "loop duration, run time elapsed";
    fprintf(f95, "%s\n", h.c_str());
    f97 = open_out(prefix + "gamma_matrix.dat");
    f98 = open_out(prefix + "summary.dat");
    fprintf(f98,
            "# step number, f_int_tot, f_ch_tot, %s f_eta_tot, e_tot, c_max_glob, c_min_glob, phi_min_glob, "
            "phi_3_max\n",
            std::string(7, ' ').c_str());
    const int V = in.var, P = V - 1;
    for (int i = 1; i <= V; ++i) {
      std::string l = list_int(i);
      for (int j = 1; j <= V; ++j) {
        double g = 0.0;
        if (i != j && i <= P && j <= P) g = in.sigma_1;
        if ((j == V && i < V) || (i == V && j < V)) g = in.sigma_2;
        l += list_real(g);
      }
      fprintf(f97, "%s\n", l.c_str());
    }
    fflush(f97);
  }

  // starting fields (src/var_diff.f90:196-461)
  void make_start() {
    const size_t ncell = (size_t)in.Nx * in.Ny * in.Nz;
    phi.assign(ncell * in.var, 0.0);
    con.assign(ncell, in.c_mat);
    pf_ran2_init(&rs);
    idum = in.iseed;  // iseed - myid with one rank
    const std::string start = in.start;
    if (in.nrun == 1) {
      int rc = PF_OK;
      if (start == "polycryst")
        rc = pf_ic_polycryst(&cfg, path_of(in.microstructure).c_str(), in.c_mat, phi.data(), con.data());
      else if (start == "plane")
        rc = pf_ic_plane(&cfg, in.ppt_rad, in.i_ppt, in.j_ppt, in.k_ppt, in.c_mat, phi.data(), con.data());
      else if (start == "circle")
        rc = pf_ic_circle(&cfg, in.grn_rad, in.ppt_rad, in.num_ppt, &idum, in.c_mat, in.con_0_ppt, &rs, phi.data(),
                          con.data());
      else if (start == "noise")
        rc = pf_ic_noise(&cfg, in.seed, in.amp_phi, in.c0, in.amp_c, phi.data(), con.data());
      else if (start == "voronoi")
        rc = pf_ic_voronoi(&cfg, in.seed, in.n_grains, in.amp_phi, in.c0, in.amp_c, phi.data(), con.data());
      else
        fprintf(log, " start '%s' sets no order parameter (phi = 0, con = c_mat)\n", start.c_str());
      if (rc != PF_OK) throw Error(2, std::string("start '") + start + "': " + pf_io_last_error() + pf_last_error());
    } else if (pf_read_data_save(path_of("data_rerun.0001").c_str(), &cfg, phi.data(), con.data()) != PF_OK) {
      throw Error(2, pf_io_last_error());
    }
    fprintf(log, " precipitates assigned\n");
    fflush(log);
  }

  // Last step of the chunk that starts at `step`: chunks end before the
  // insertion step and at every output step.
  int chunk_end(int step) const {
    int last = std::min(in.N_step, ((step + in.ifreq - 1) / in.ifreq) * in.ifreq);
    if (in.ppt_int > step) last = std::min(last, in.ppt_int - 1);
    return last;
  }

  // Precipitate insertion at step == ppt_int (src/var_diff.f90:479-554) into
  // the host fields (phi must be current).
  void insert() {
    phi_stats(cfg, phi, &ins_phi_min, &ins_phi_p);
    if (pf_insert_precipitates(&cfg, in.ppt_rad, in.num_ppt, &idum, &rs, phi.data()) != PF_OK)
      throw Error(2, pf_io_last_error());
    fprintf(log, " nppt= %d\n", in.num_ppt + 1);
    fflush(log);
  }

  // Records of steps step0 .. step0+n-1, each taking dt seconds.  The
  // statistics of the insertion step describe the fields before the
  // insertion, as the reference reduces them at the end of the previous step.
  void write_records(int step0, pf_diag* d, int n, double dt) {
    if (step0 == in.ppt_int && step0 > 1 && n > 0) {
      d[0].phi_min = ins_phi_min;
      d[0].phi_P_max = ins_phi_p;
    }
    for (int s = 0; s < n; ++s) {
      const int st = step0 + s;
      run_time += dt;
      fprintf(f93, "%s%s%s\n", list_int(st).c_str(), list_real(dt).c_str(), list_real(run_time).c_str());
      if (st % 2 == 0) {
        char line[160];
        pf_format_summary(st, &d[s], line);
        fprintf(f98, "%s\n", line);
      }
      char head[16];
      snprintf(head, sizeof head, "%8d", st);
      std::string l = head;
      for (int k = 0; k < 14; ++k) l += " " + f8_6(k == 13 ? dt : 0.0);
      l += " " + f8_6(dt) + " " + f8_6(run_time);
      fprintf(f95, "%s\n", l.c_str());
    }
    fflush(f93);
    fflush(f95);
    fflush(f98);
  }

  // step_NNNNNNN/data_extract_mult.in and data_save.0001 (src/var_diff.f90:1120-1142)
  void write_step_dir(int step) {
    char dn[32];
    snprintf(dn, sizeof dn, "step_%07d", step);
    const std::string dir = prefix + dn;
    if (!mkdir_p(dir)) throw Error(2, "cannot create " + dir);
    FILE* f9 = open_out(dir + "/data_extract_mult.in");
    fprintf(f9, "%s%s%s%s%s\n", list_int(in.Nx).c_str(), list_int(in.Ny).c_str(), list_int(in.Nz).c_str(),
            list_int(1).c_str(), list_int(in.var).c_str());
    // one rank wrote one data_save file: nprocs = 1, dims = (1, 1)
    fprintf(f9, "%s%s\n", list_int(1).c_str(), list_int(1).c_str());
    fclose(f9);
    if (pf_write_data_save((dir + "/data_save.0001").c_str(), &cfg, phi.data(), con.data()) != PF_OK)
      throw Error(2, pf_io_last_error());
  }

  void close() {
    for (FILE** f : {&f93, &f95, &f97, &f98})
      if (*f) {
        fclose(*f);
        *f = nullptr;
      }
    if (log && log != stdout && log != stderr) {
      fclose(log);
      log = stdout;
    }
  }
};

}  // namespace pfcase
