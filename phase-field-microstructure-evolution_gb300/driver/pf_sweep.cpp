// pf_sweep: many var_diff.x cases in one process on one GPU, for parameter
// sweeps such as tests/run_phase_sim.py and tests/scaling_tests.py submit
// (one SLURM job per case there, run_phase_sim.py:130-172).
//
//   pf_sweep [--max-batch N] [--devices N|all] <case dir> [<case dir> ...]
//
// Every case directory holds an input.txt (the file run_phase_sim.py:112-128
// writes) and receives what `var_diff.x <dir>/input.txt <dir>/` writes:
// time_step.dat, timing_data.dat, gamma_matrix.dat, summary.dat and the
// step_NNNNNNN/ directories, with the program's stdout lines in <dir>/mrun.out
// (the file the reference's job script redirects them to).  Relative paths in
// a case (data_rerun.0001, microstructure=) start from its directory.
//
// Cases of the same grid, number of order parameters and mobility class run
// as one pf_batch (one set of launches per step, up to --max-batch runs; each
// run gives the same numbers as alone).  The batch is stepped in chunks that
// end at every member's insertion and output steps; a member whose N_step is
// reached stops writing records while the others go on.  time_step.dat of a
// batched case holds the batch's step time.  Cases on the FP64 path (a grid
// the fused kernels do not cover, or precision=64) run one at a time.
//
// --devices spreads the work units (batches and single cases) over N GPUs
// (all: every visible one) with pf_place_units -- largest unit first onto the
// device with the least work -- and runs each device's units in a thread of
// its own.  Cases never exchange data, so there is no collective.
//
// Exit status: 0 if every case finished, 2 if a case failed to start or to
// write, 3 if a case produced non-finite values (its records up to that step
// are written; the other cases are unaffected).
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "pf_case.h"

namespace {

using pfcase::Case;
using pfcase::check;

struct Member {
  std::unique_ptr<Case> c;
  std::string dir;
  int status = 0;  // 0 running or done, 2 / 3 failed
  bool active(int step) const { return status == 0 && step <= c->in.N_step; }
};

void fail_member(Member& m, int code, const std::string& msg) {
  m.status = code;
  fprintf(stderr, "pf_sweep: %s: %s\n", m.dir.c_str(), msg.c_str());
  if (m.c->log) {
    fprintf(m.c->log, " error: %s\n", msg.c_str());
    fflush(m.c->log);
  }
}

// one case on its own pf_run (the FP64 path)
void run_single(Member& m) {
  Case& c = *m.c;
  pf_run* run = nullptr;
  try {
    check(pf_create(&c.cfg, &run), "pf_create");
    check(pf_set_fields(run, c.phi.data(), c.con.data()), "pf_set_fields");
    std::vector<pf_diag> diag;
    for (int step = 1; step <= c.in.N_step && m.status == 0;) {
      if (step == c.in.ppt_int) {
        check(pf_get_fields(run, c.phi.data(), c.con.data()), "pf_get_fields");
        c.insert();
        check(pf_set_fields(run, c.phi.data(), c.con.data()), "pf_set_fields");
      }
      const int last = c.chunk_end(step), n = last - step + 1;
      diag.resize(n);
      const auto t0 = std::chrono::steady_clock::now();
      const int rc = pf_step(run, n, diag.data());
      const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() / n;
      if (rc != PF_ENONFINITE) check(rc, "pf_step");
      c.write_records(step, diag.data(), n, dt);
      if (rc == PF_ENONFINITE) fail_member(m, 3, "a step produced non-finite values; case stopped");
      if (last % c.in.ifreq == 0) {
        check(pf_get_fields(run, c.phi.data(), c.con.data()), "pf_get_fields");
        c.write_step_dir(last);
      }
      step = last + 1;
    }
  } catch (const pfcase::Error& e) {
    fail_member(m, e.code, e.what());
  }
  if (run) pf_destroy(run);
}

// cases of one shape and mobility class stepped together
void run_batch(std::vector<Member*>& ms) {
  const int R = (int)ms.size();
  std::vector<pf_config> cfgs;
  for (Member* m : ms) cfgs.push_back(m->c->cfg);
  pf_batch* b = nullptr;
  if (pf_batch_create(cfgs.data(), R, &b) != PF_OK) {
    const std::string msg = std::string("pf_batch_create: ") + pf_last_error();
    for (Member* m : ms) fail_member(*m, 2, msg);
    return;
  }
  int nmax = 0;
  for (int r = 0; r < R; ++r) {
    Case& c = *ms[r]->c;
    if (pf_batch_set_fields(b, r, c.phi.data(), c.con.data()) != PF_OK)
      fail_member(*ms[r], 2, std::string("pf_batch_set_fields: ") + pf_last_error());
    nmax = std::max(nmax, c.in.N_step);
  }
  std::vector<pf_diag> diag;
  for (int step = 1; step <= nmax;) {
    int last = nmax;
    bool any = false;
    for (int r = 0; r < R; ++r) {
      Member& m = *ms[r];
      if (!m.active(step)) continue;
      any = true;
      last = std::min(last, m.c->chunk_end(step));
      if (step == m.c->in.ppt_int) {
        try {
          Case& c = *m.c;
          check(pf_batch_get_fields(b, r, c.phi.data(), c.con.data()), "pf_batch_get_fields");
          c.insert();
          check(pf_batch_set_fields(b, r, c.phi.data(), c.con.data()), "pf_batch_set_fields");
        } catch (const pfcase::Error& e) {
          fail_member(m, e.code, e.what());
        }
      }
    }
    if (!any) break;
    const int n = last - step + 1;
    diag.resize((size_t)R * n);
    const auto t0 = std::chrono::steady_clock::now();
    const int rc = pf_batch_step(b, n, diag.data());
    const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() / n;
    if (rc != PF_OK && rc != PF_ENONFINITE) {
      const std::string msg = std::string("pf_batch_step: ") + pf_last_error();
      for (Member* m : ms)
        if (m->status == 0) fail_member(*m, 2, msg);
      break;
    }
    for (int r = 0; r < R; ++r) {
      Member& m = *ms[r];
      if (!m.active(step)) continue;
      Case& c = *m.c;
      try {
        const int upto = std::min(last, c.in.N_step);
        pf_diag* d = diag.data() + (size_t)r * n;
        int bad = -1;
        for (int s = 0; s < upto - step + 1; ++s)
          if (d[s].nonfinite) {
            bad = s;
            break;
          }
        c.write_records(step, d, bad < 0 ? upto - step + 1 : bad + 1, dt);
        if (bad >= 0) {
          fail_member(m, 3, "a step produced non-finite values; case stopped");
          continue;
        }
        if (upto == last && last % c.in.ifreq == 0) {
          check(pf_batch_get_fields(b, r, c.phi.data(), c.con.data()), "pf_batch_get_fields");
          c.write_step_dir(last);
        }
      } catch (const pfcase::Error& e) {
        fail_member(m, e.code, e.what());
      }
    }
    step = last + 1;
  }
  pf_batch_destroy(b);
}

}  // namespace

// a batch of same-class cases, or one FP64-path case
struct Unit {
  std::vector<Member*> ms;
  bool single = false;
  double work = 0;
};

int main(int argc, char** argv) {
  int max_batch = 64, ndev = 1;
  std::vector<std::string> dirs;
  for (int i = 1; i < argc; ++i) {
    if (!strcmp(argv[i], "--max-batch") && i + 1 < argc) {
      max_batch = std::max(1, atoi(argv[++i]));
    } else if (!strcmp(argv[i], "--devices") && i + 1 < argc) {
      ++i;
      if (!strcmp(argv[i], "all")) {
        ndev = std::max(1, pf_device_count());
      } else {
        ndev = std::max(1, atoi(argv[i]));
      }
    } else {
      dirs.push_back(argv[i]);
    }
  }
  if (dirs.empty()) {
    fprintf(stderr, "usage: pf_sweep [--max-batch N] [--devices N|all] <case dir> [<case dir> ...]\n");
    return 1;
  }
  std::vector<Member> ms(dirs.size());
  // (grid, var, variable mobility) -> batched members; FP64 members run alone
  std::map<std::tuple<int, int, int, int, int>, std::vector<Member*>> groups;
  std::vector<Member*> singles;
  for (size_t i = 0; i < dirs.size(); ++i) {
    Member& m = ms[i];
    m.dir = dirs[i];
    while (m.dir.size() > 1 && m.dir.back() == '/') m.dir.pop_back();
    m.c.reset(new Case());
    Case& c = *m.c;
    try {
      c.log = fopen((m.dir + "/mrun.out").c_str(), "w");
      if (!c.log) {
        c.log = stdout;
        throw pfcase::Error(2, "cannot create " + m.dir + "/mrun.out");
      }
      c.load(m.dir + "/input.txt", m.dir + "/", m.dir);
      fprintf(c.log, " pf_sweep case: %d x %d x %d, var = %d, %d steps, %s path\n", c.in.Nx, c.in.Ny, c.in.Nz,
              c.in.var, c.in.N_step, c.cfg.precision == PF_FP64_PLAIN ? "FP64 cuFFT" : "fused FP32");
      c.open_outputs();
      c.make_start();
      c.report_fp64_check();
    } catch (const pfcase::Error& e) {
      fail_member(m, e.code, e.what());
      continue;
    }
    if (c.cfg.precision == PF_FP64_PLAIN) {
      singles.push_back(&m);
    } else {
      const int varmob = c.cfg.mobility == PF_MOB_C1MC || c.cfg.D_gb != 0.0;
      groups[std::make_tuple(c.in.Nx, c.in.Ny, c.in.Nz, c.in.var, varmob)].push_back(&m);
    }
  }
  std::vector<Unit> units;
  size_t nbatches = 0;
  for (auto& kv : groups) {
    std::vector<Member*>& g = kv.second;
    for (size_t a = 0; a < g.size(); a += max_batch) {
      Unit u;
      u.ms.assign(g.begin() + a, g.begin() + std::min(g.size(), a + (size_t)max_batch));
      units.push_back(u);
      ++nbatches;
    }
  }
  for (Member* m : singles) {
    Unit u;
    u.ms.push_back(m);
    u.single = true;
    units.push_back(u);
  }
  // a batch steps as long as its longest member
  std::vector<double> work(units.size());
  for (size_t u = 0; u < units.size(); ++u) {
    int nmax = 0;
    for (Member* m : units[u].ms) nmax = std::max(nmax, m->c->in.N_step);
    for (Member* m : units[u].ms) units[u].work += pf_run_work(&m->c->cfg, nmax);
    work[u] = units[u].work;
  }
  std::vector<int> dev(units.size(), 0);
  pf_place_units(work.data(), (int)units.size(), ndev, dev.data(), nullptr);
  auto run_device = [&](int d) {
    for (size_t u = 0; u < units.size(); ++u) {
      if (dev[u] != d) continue;
      for (Member* m : units[u].ms) m->c->cfg.device = d;
      if (units[u].single) run_single(*units[u].ms[0]);
      else run_batch(units[u].ms);
    }
  };
  if (ndev == 1) {
    run_device(0);
  } else {
    std::vector<std::thread> th;
    for (int d = 0; d < ndev; ++d) th.emplace_back(run_device, d);
    for (auto& t : th) t.join();
  }
  int status = 0, ok = 0;
  for (Member& m : ms) {
    m.c->close();
    if (m.status == 0) ++ok;
    status = std::max(status, m.status);
  }
  printf(" pf_sweep: %d of %zu cases finished (%zu batches, %zu FP64 cases, %d device%s)\n", ok, ms.size(), nbatches,
         singles.size(), ndev, ndev == 1 ? "" : "s");
  return status;
}
