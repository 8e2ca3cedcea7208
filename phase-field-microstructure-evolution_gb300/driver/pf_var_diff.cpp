// pf_var_diff: the var_diff.x program (src/var_diff.f90) on one GPU.
//
//   pf_var_diff <input file> [output prefix]
//
// Same command line, input file and output files as the reference:
//   <prefix>time_step.dat     step, step duration, run time (list-directed, :1056)
//   <prefix>timing_data.dat   (I8, 16(A, F8.6)) per step (:1150-1153)
//   <prefix>gamma_matrix.dat  i, gamma(i, 1:var) (:219-224)
//   <prefix>summary.dat       (i6, 8e15.7) on even steps (:1058-1074)
//   <prefix>step_NNNNNNN/data_extract_mult.in, data_save.0001 every ifreq steps (:1120-1142)
// The prefix is concatenated as given (the reference does the same), so a
// directory prefix needs its trailing '/'.  nrun != 1 restarts from
// data_rerun.0001 in the working directory (:451-461).
//
// Differences, all visible on stdout: one rank (dims is read and ignored);
// the time step runs in the library (pf_step); timing_data.dat carries the
// step duration in the loop-duration column and zeros in the fourteen
// per-loop columns (the fused step has no separate loops); a step with
// non-finite values stops the run with exit status 3 after writing its
// records; 'polycryst' reads the `microstructure=` file (default mc_ivar_fin
// in the working directory) instead of the reference's fixed path; 'noise'
// and 'voronoi' are extra starts driven by the key=value lines.
#include <sys/stat.h>
#include <sys/types.h>

#include <algorithm>
#include <cerrno>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "pfgpu.h"

namespace {

void die(int code, const std::string& msg) {
  fprintf(stderr, "pf_var_diff: %s\n", msg.c_str());
  exit(code);
}

FILE* open_out(const std::string& path) {
  FILE* f = fopen(path.c_str(), "w");
  if (!f) die(2, "cannot create " + path);
  return f;
}

bool mkdir_p(const std::string& dir) {
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

std::string list_int(int v) {
  char b[32];
  pf_format_list_int(v, b);
  return b;
}

std::string list_real(double v) {
  char b[32];
  pf_format_list_real(v, b);
  return b;
}

std::string f8_6(double v) {  // Fortran F8.6
  char b[32];
  snprintf(b, sizeof b, "%8.6f", v);
  if (strlen(b) > 8 || !std::isfinite(v)) return "********";
  return b;
}

void check(int rc, const char* what) {
  if (rc == PF_OK) return;
  die(2, std::string(what) + ": " + pf_last_error() + pf_io_last_error());
}

// min over cells of sum_i phi_i^2 and max of phi_var, with the reference's
// start values 1 and 0 (src/var_diff.f90:1076-1102)
void phi_stats(const pf_config& c, const std::vector<double>& phi, double* phi_min, double* phi_p_max) {
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

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) {
    fprintf(stderr, "usage: pf_var_diff <input file> [output prefix]\n");
    return 1;
  }
  const std::string prefix = argc > 2 ? argv[2] : "";
  pf_input in;
  if (pf_read_input(argv[1], 1, &in) != PF_OK) die(2, pf_io_last_error());
  pf_config cfg;
  pf_input_to_config(&in, &cfg);
  if (in.precision == 0) {
    cfg.precision = pf_supported_shape(in.Nx, in.Ny, in.Nz, in.var, PF_FP32_FUSED) ? PF_FP32_FUSED : PF_FP64_PLAIN;
  }
  if (!pf_supported_shape(in.Nx, in.Ny, in.Nz, in.var, cfg.precision))
    die(2, "grid " + std::to_string(in.Nx) + "x" + std::to_string(in.Ny) + "x" + std::to_string(in.Nz) +
               " var=" + std::to_string(in.var) + " is not supported by precision " + std::to_string(cfg.precision));
  if (in.ifreq < 1) die(2, "ifreq must be >= 1");
  printf(" pf_var_diff: %d x %d x %d, var = %d, %d steps, %s path, %s mobility\n", in.Nx, in.Ny, in.Nz, in.var,
         in.N_step, cfg.precision == PF_FP64_PLAIN ? "FP64 cuFFT" : "fused FP32",
         cfg.mobility == PF_MOB_C1MC ? "c(1-c)" : "reference");
  fflush(stdout);

  // output files and their headers (src/var_diff.f90:82-95)
  FILE* f93 = open_out(prefix + "time_step.dat");
  fprintf(f93, "# step number, iteration duration, %s run time elapsed\n", std::string(29, ' ').c_str());
  FILE* f95 = open_out(prefix + "timing_data.dat");
  {
    std::string h = "# step number";
    for (int i = 1; i <= 7; ++i) h += ", loop " + std::to_string(i) + " avg";
    h += "," + std::string(40, ' ');
    for (int i = 8; i <= 14; ++i) h += (i == 8 ? "loop " : ", loop ") + std::to_string(i) + " avg";
    h += "," + std::string(40, ' ') + "loop duration, run time elapsed";
    fprintf(f95, "%s\n", h.c_str());
  }
  FILE* f97 = open_out(prefix + "gamma_matrix.dat");
  FILE* f98 = open_out(prefix + "summary.dat");
  fprintf(f98, "# step number, f_int_tot, f_ch_tot, %s f_eta_tot, e_tot, c_max_glob, c_min_glob, phi_min_glob, phi_3_max\n",
          std::string(7, ' ').c_str());

  // gamma (src/var_diff.f90:205-218)
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

  // starting fields
  const size_t ncell = (size_t)in.Nx * in.Ny * in.Nz;
  std::vector<double> phi(ncell * V, 0.0), con(ncell, in.c_mat);
  pf_ran2_state rs;
  pf_ran2_init(&rs);
  int idum = in.iseed;  // iseed - myid with one rank
  const std::string start = in.start;
  if (in.nrun == 1) {
    int rc = PF_OK;
    if (start == "polycryst") rc = pf_ic_polycryst(&cfg, in.microstructure, in.c_mat, phi.data(), con.data());
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
      printf(" start '%s' sets no order parameter (phi = 0, con = c_mat)\n", start.c_str());
    if (rc != PF_OK) die(2, std::string("start '") + start + "': " + pf_io_last_error() + pf_last_error());
  } else {
    if (pf_read_data_save("data_rerun.0001", &cfg, phi.data(), con.data()) != PF_OK) die(2, pf_io_last_error());
  }
  printf(" precipitates assigned\n");
  fflush(stdout);

  pf_run* run = nullptr;
  check(pf_create(&cfg, &run), "pf_create");
  check(pf_set_fields(run, phi.data(), con.data()), "pf_set_fields");

  // time loop (src/var_diff.f90:473-1158), advanced in chunks that end at
  // the insertion step and at every output step
  std::vector<pf_diag> diag;
  double run_time = 0.0;
  int status = 0;
  for (int step = 1; step <= in.N_step && status == 0;) {
    double ins_phi_min = NAN, ins_phi_p = NAN;
    if (step == in.ppt_int) {
      check(pf_get_fields(run, phi.data(), con.data()), "pf_get_fields");
      phi_stats(cfg, phi, &ins_phi_min, &ins_phi_p);
      const int rc = pf_insert_precipitates(&cfg, in.ppt_rad, in.num_ppt, &idum, &rs, phi.data());
      if (rc != PF_OK) die(2, pf_io_last_error());
      printf(" nppt= %d\n", in.num_ppt + 1);
      check(pf_set_fields(run, phi.data(), con.data()), "pf_set_fields");
    }
    int last = std::min(in.N_step, ((step + in.ifreq - 1) / in.ifreq) * in.ifreq);
    if (in.ppt_int > step) last = std::min(last, in.ppt_int - 1);
    const int n = last - step + 1;
    diag.resize(n);
    const auto t0 = std::chrono::steady_clock::now();
    const int rc = pf_step(run, n, diag.data());
    const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() / n;
    if (rc == PF_ENONFINITE) status = 3;
    else check(rc, "pf_step");
    // the statistics of the insertion step describe the fields before the
    // insertion, as the reference reduces them at the end of the previous step
    if (step == in.ppt_int && step > 1) {
      diag[0].phi_min = ins_phi_min;
      diag[0].phi_P_max = ins_phi_p;
    }
    for (int s = 0; s < n; ++s) {
      const int st = step + s;
      run_time += dt;
      fprintf(f93, "%s%s%s\n", list_int(st).c_str(), list_real(dt).c_str(), list_real(run_time).c_str());
      if (st % 2 == 0) {
        char line[160];
        pf_format_summary(st, &diag[s], line);
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
    if (last % in.ifreq == 0) {
      check(pf_get_fields(run, phi.data(), con.data()), "pf_get_fields");
      char dn[32];
      snprintf(dn, sizeof dn, "step_%07d", last);
      const std::string dir = prefix + dn;
      if (!mkdir_p(dir)) die(2, "cannot create " + dir);
      FILE* f9 = open_out(dir + "/data_extract_mult.in");
      fprintf(f9, "%s%s%s%s%s\n", list_int(in.Nx).c_str(), list_int(in.Ny).c_str(), list_int(in.Nz).c_str(),
              list_int(1).c_str(), list_int(in.var).c_str());
      // one rank wrote one data_save file: nprocs = 1, dims = (1, 1)
      fprintf(f9, "%s%s\n", list_int(1).c_str(), list_int(1).c_str());
      fclose(f9);
      if (pf_write_data_save((dir + "/data_save.0001").c_str(), &cfg, phi.data(), con.data()) != PF_OK)
        die(2, pf_io_last_error());
    }
    step = last + 1;
  }
  pf_destroy(run);
  fclose(f93);
  fclose(f95);
  fclose(f97);
  fclose(f98);
  if (status == 3) fprintf(stderr, "pf_var_diff: a step produced non-finite values; run stopped\n");
  return status;
}
