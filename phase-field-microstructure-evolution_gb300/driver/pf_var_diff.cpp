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
// and 'voronoi' are extra starts driven by the key=value lines; check_fp64=N
// prints the run's error against the FP64 GPU path after N steps of its start.
#include <chrono>
#include <cstdio>
#include <string>
#include <vector>

#include "pf_case.h"

int main(int argc, char** argv) {
  if (argc < 2) {
    fprintf(stderr, "usage: pf_var_diff <input file> [output prefix]\n");
    return 1;
  }
  pfcase::Case c;
  pf_run* run = nullptr;
  int status = 0;
  try {
    c.load(argv[1], argc > 2 ? argv[2] : "", "");
    printf(" pf_var_diff: %d x %d x %d, var = %d, %d steps, %s path, %s mobility\n", c.in.Nx, c.in.Ny, c.in.Nz,
           c.in.var, c.in.N_step, c.cfg.precision == PF_FP64_PLAIN ? "FP64 cuFFT" : "fused FP32",
           c.cfg.mobility == PF_MOB_C1MC ? "c(1-c)" : "reference");
    fflush(stdout);
    c.open_outputs();
    c.make_start();
    c.report_fp64_check();
    pfcase::check(pf_create(&c.cfg, &run), "pf_create");
    pfcase::check(pf_set_fields(run, c.phi.data(), c.con.data()), "pf_set_fields");
    // time loop (src/var_diff.f90:473-1158), advanced in chunks that end at
    // the insertion step and at every output step
    std::vector<pf_diag> diag;
    for (int step = 1; step <= c.in.N_step && status == 0;) {
      if (step == c.in.ppt_int) {
        pfcase::check(pf_get_fields(run, c.phi.data(), c.con.data()), "pf_get_fields");
        c.insert();
        pfcase::check(pf_set_fields(run, c.phi.data(), c.con.data()), "pf_set_fields");
      }
      const int last = c.chunk_end(step);
      const int n = last - step + 1;
      diag.resize(n);
      const auto t0 = std::chrono::steady_clock::now();
      const int rc = pf_step(run, n, diag.data());
      const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() / n;
      if (rc == PF_ENONFINITE) status = 3;
      else pfcase::check(rc, "pf_step");
      c.write_records(step, diag.data(), n, dt);
      if (last % c.in.ifreq == 0) {
        pfcase::check(pf_get_fields(run, c.phi.data(), c.con.data()), "pf_get_fields");
        c.write_step_dir(last);
      }
      step = last + 1;
    }
  } catch (const pfcase::Error& e) {
    fprintf(stderr, "pf_var_diff: %s\n", e.what());
    status = e.code;
  }
  if (run) pf_destroy(run);
  c.close();
  if (status == 3) fprintf(stderr, "pf_var_diff: a step produced non-finite values; run stopped\n");
  return status;
}
