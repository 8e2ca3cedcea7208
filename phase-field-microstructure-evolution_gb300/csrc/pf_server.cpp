// Serving loop: continuous batching of independent runs on one GPU.
//
// The reference runs a parameter study as one SLURM job per run
// (tests/run_phase_sim.py:130-172, tests/scaling_tests.py); here requests are
// submitted to one process and share the GPU:
//   * a request (configuration, starting fields, number of steps) is queued
//     with a copy of its fields;
//   * a worker thread admits queued requests whenever the resident runs leave
//     room in the HBM budget and in the slot count: waiting requests of the
//     same grid, var and mobility class are admitted together as one pf_batch
//     (one set of launches per step for all of them);
//   * every resident batch has its own stream and captured step graph; the
//     worker keeps up to two chunks of steps queued on each batch and tops
//     them up as they complete, so the device has work while the worker
//     admits new requests; batches that fill the GPU by themselves take turns
//     (oldest admitted first), smaller batches overlap with them on
//     high-priority streams;
//   * a run leaves as soon as its own step count is reached (its fields and
//     last record are copied out; a batch is freed when all its runs left).
// Each run computes exactly what it computes alone: the same kernels, per-run
// reductions in a fixed order, no state shared between runs.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "../../include/pfgpu.h"

extern "C" {
// internal hooks of pf_api.cu (not in the public header)
int pf_batch_enqueue(pf_batch* b, int nsteps);
void* pf_batch_stream(pf_batch* b);
size_t pf_batch_bytes(const pf_config* c, int nruns);
int pf_batch_steps_done(pf_batch* b, int run);
int pf_batch_records(pf_batch* b, int run, int first, int n, pf_diag* out);
int pf_batch_ring(pf_batch* b);
int pf_batch_prioritize(pf_batch* b);
}

namespace {

using Clock = std::chrono::steady_clock;

thread_local std::string g_srv_err;

int srv_fail(int code, const std::string& m) {
  g_srv_err = m;
  return code;
}

struct Request {
  long long id = 0;
  pf_config cfg{};
  int nsteps = 0;
  std::vector<double> phi, con;  // inputs, then results
  pf_diag last{};
  int state = PF_REQ_QUEUED;
  int error = PF_OK;
  std::string message;
  Clock::time_point t_submit, t_start, t_done;
};

struct Chunk {
  cudaEvent_t ev = nullptr;  // recorded after the chunk's last step
  int first = 0, n = 0;      // steps first .. first+n-1 (0-based)
};

constexpr int kInFlight = 2;  // chunks queued per batch, so the GPU has work while the worker is busy
constexpr int kRing = 1024;   // per-run record ring of a batch (pf_batch_ring)
// Longest chunk: the records of all chunks in flight must fit the ring at
// once, since the newest chunk writes its slots while the oldest one's are
// copied out.
constexpr int kMaxChunk = kRing / kInFlight;
// A batch whose step touches at least this many cell-fields (runs x cells x
// (var + 1)) keeps the whole GPU busy by itself: such batches do not gain
// from running side by side, they only evict each other's data from L2 and
// fragment the SMs, so they take turns (oldest admitted first), while the
// smaller batches run beside them on high-priority streams.
constexpr double kHeavyCellFields = 16777216.0;

struct Active {
  pf_batch* b = nullptr;
  bool heavy = false;      // fills the GPU on its own (run one at a time, oldest first)
  long long seq = 0;       // admission order
  std::vector<std::shared_ptr<Request>> runs;
  std::vector<bool> left;  // run finished and copied out
  size_t bytes = 0;
  int enq = 0;             // steps enqueued so far (all runs of a batch step together)
  std::deque<Chunk> flight;
  std::vector<cudaEvent_t> spare;  // events not in use
};

}  // namespace

struct pf_server {
  pf_server_config cfg{};
  size_t budget = 0, used = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<std::shared_ptr<Request>> queue;
  std::map<long long, std::shared_ptr<Request>> all;
  long long next_id = 1;
  bool stop = false;
  std::thread worker;
  std::vector<Active> active;
  int resident = 0;
  long long next_seq = 0;
};

namespace {

std::tuple<int, int, int, int, int> klass(const pf_config& c) {
  const int varmob = c.mobility == PF_MOB_C1MC || c.D_gb != 0.0;
  return std::make_tuple(c.nx, c.ny, c.nz, c.var, varmob);
}

void finish(pf_server* s, Request& r, int state, int err, const std::string& msg) {
  std::lock_guard<std::mutex> lk(s->mu);
  r.state = state;
  r.error = err;
  r.message = msg;
  r.t_done = Clock::now();
  s->cv_done.notify_all();
}

// admit waiting requests (called by the worker without the lock held)
void admit(pf_server* s) {
  for (;;) {
    std::vector<std::shared_ptr<Request>> group;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      if (s->queue.empty()) return;
      const int slots = s->cfg.max_active - s->resident;
      if (slots <= 0) return;
      const auto key = klass(s->queue.front()->cfg);
      for (auto it = s->queue.begin(); it != s->queue.end() && (int)group.size() < slots;) {
        if (klass((*it)->cfg) == key) {
          group.push_back(*it);
          it = s->queue.erase(it);
        } else {
          ++it;
        }
      }
      // keep within the budget: shrink the group, or wait for memory
      while (!group.empty() && s->used + pf_batch_bytes(&group[0]->cfg, (int)group.size()) > s->budget) {
        s->queue.push_front(group.back());
        group.pop_back();
      }
      // restore FIFO order of what was put back
      std::stable_sort(s->queue.begin(), s->queue.end(),
                       [](const std::shared_ptr<Request>& a, const std::shared_ptr<Request>& b) { return a->id < b->id; });
      if (group.empty()) {
        if (s->resident == 0) {  // nothing will free memory: the request can never run
          auto r = s->queue.front();
          s->queue.pop_front();
          r->state = PF_REQ_FAILED;
          r->error = PF_ENOMEM;
          r->message = "request needs more device memory than the server's budget";
          r->t_done = Clock::now();
          s->cv_done.notify_all();
          continue;
        }
        return;
      }
    }
    std::vector<pf_config> cfgs;
    for (auto& r : group) cfgs.push_back(r->cfg);
    Active a;
    int rc = pf_batch_create(cfgs.data(), (int)cfgs.size(), &a.b);
    std::string msg;
    if (rc == PF_OK && pf_batch_ring(a.b) < kRing) {
      rc = PF_EINVAL;
      msg = "record ring shorter than the server's chunks need";
    }
    for (size_t i = 0; rc == PF_OK && i < group.size(); ++i)
      rc = pf_batch_set_fields(a.b, (int)i, group[i]->phi.data(), group[i]->con.data());
    for (int k = 0; rc == PF_OK && k < kInFlight; ++k) {
      cudaEvent_t ev = nullptr;
      if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) rc = PF_ECUDA;
      else a.spare.push_back(ev);
    }
    if (rc != PF_OK) {
      if (msg.empty()) msg = pf_last_error();
      if (a.b) pf_batch_destroy(a.b);
      for (cudaEvent_t ev : a.spare) cudaEventDestroy(ev);
      for (auto& r : group) finish(s, *r, PF_REQ_FAILED, rc, msg);
      continue;
    }
    a.runs = group;
    a.left.assign(group.size(), false);
    a.bytes = pf_batch_bytes(&cfgs[0], (int)cfgs.size());
    a.heavy = (double)cfgs.size() * cfgs[0].nx * cfgs[0].ny * cfgs[0].nz * (cfgs[0].var + 1) >= kHeavyCellFields;
    a.seq = s->next_seq++;
    if (!a.heavy) pf_batch_prioritize(a.b);  // best effort: default priority if it fails
    {
      std::lock_guard<std::mutex> lk(s->mu);
      const auto now = Clock::now();
      for (auto& r : group) {
        r->state = PF_REQ_RUNNING;
        r->t_start = now;
      }
      s->used += a.bytes;
      s->resident += (int)group.size();
    }
    s->active.push_back(std::move(a));
  }
}

// The oldest chunk of `a` has completed: take its records and copy out the
// runs that reached their step count (no later chunk is in flight for them:
// chunks never run past a member's end).
void leave(pf_server* s, Active& a, size_t i, int state, int err, const std::string& msg) {
  a.left[i] = true;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->resident -= 1;
  }
  finish(s, *a.runs[i], state, err, msg);
}

void harvest(pf_server* s, Active& a, const Chunk& c) {
  for (size_t i = 0; i < a.runs.size(); ++i) {
    if (a.left[i]) continue;
    Request& r = *a.runs[i];
    std::vector<pf_diag> rec(c.n);
    int rc = pf_batch_records(a.b, (int)i, c.first, c.n, rec.data());
    int bad = 0;
    for (const pf_diag& d : rec) bad |= d.nonfinite;
    if (rc == PF_OK && !rec.empty()) r.last = rec.back();
    if (rc == PF_OK && !bad && c.first + c.n < r.nsteps) continue;  // still running
    if (rc == PF_OK && !bad && !a.flight.empty()) continue;          // cannot happen: chunks stop at ends
    if (rc == PF_OK && !bad) rc = pf_batch_get_fields(a.b, (int)i, r.phi.data(), r.con.data());
    if (rc != PF_OK) leave(s, a, i, PF_REQ_FAILED, rc, pf_last_error());
    else if (bad) leave(s, a, i, PF_REQ_FAILED, PF_ENONFINITE, "a step produced non-finite values");
    else leave(s, a, i, PF_REQ_DONE, PF_OK, "");
  }
}

// steps the next chunk of `a` may take: up to the nearest member's end
int next_chunk(const pf_server* s, const Active& a) {
  int n = s->cfg.chunk_steps;
  bool any = false;
  for (size_t i = 0; i < a.runs.size(); ++i)
    if (!a.left[i]) {
      any = true;
      n = std::min(n, a.runs[i]->nsteps - a.enq);
    }
  return any ? n : 0;
}

void fail_rest(pf_server* s, Active& a, int err, const std::string& msg) {
  for (size_t i = 0; i < a.runs.size(); ++i)
    if (!a.left[i]) leave(s, a, i, PF_REQ_FAILED, err, msg);
}

void worker_loop(pf_server* s) {
  cudaSetDevice(s->cfg.device);
  for (;;) {
    {
      std::unique_lock<std::mutex> lk(s->mu);
      if (s->stop && s->active.empty()) break;
      if (s->active.empty() && s->queue.empty()) {
        s->cv_work.wait(lk, [&] { return s->stop || !s->queue.empty(); });
        if (s->stop && s->active.empty()) break;
      }
    }
    bool progressed = false;
    long long oldest_heavy = -1;  // the heavy batch whose turn it is
    for (const Active& a : s->active)
      if (a.heavy && !std::all_of(a.left.begin(), a.left.end(), [](bool v) { return v; }) &&
          (oldest_heavy < 0 || a.seq < oldest_heavy))
        oldest_heavy = a.seq;
    for (Active& a : s->active) {
      // completed chunks, oldest first
      while (!a.flight.empty() && cudaEventQuery(a.flight.front().ev) != cudaErrorNotReady) {
        const Chunk c = a.flight.front();
        a.flight.pop_front();
        a.spare.push_back(c.ev);
        harvest(s, a, c);
        progressed = true;
      }
      if (s->stop) {  // shutting down: no new work; what is in flight drains
        if (a.flight.empty()) fail_rest(s, a, PF_EINVAL, "server destroyed before the run finished");
        continue;
      }
      while ((int)a.flight.size() < kInFlight && (!a.heavy || a.seq == oldest_heavy)) {
        const int n = next_chunk(s, a);
        if (n <= 0) break;
        Chunk c;
        c.ev = a.spare.back();
        c.first = a.enq;
        c.n = n;
        int rc = pf_batch_enqueue(a.b, n);
        if (rc == PF_OK && cudaEventRecord(c.ev, (cudaStream_t)pf_batch_stream(a.b)) != cudaSuccess) rc = PF_ECUDA;
        if (rc != PF_OK) {
          fail_rest(s, a, rc, pf_last_error());
          break;
        }
        a.spare.pop_back();
        a.enq += n;
        a.flight.push_back(c);
        progressed = true;
      }
    }
    if (!s->stop) admit(s);
    // free batches whose runs all left
    for (size_t k = 0; k < s->active.size();) {
      Active& a = s->active[k];
      if (a.flight.empty() && std::all_of(a.left.begin(), a.left.end(), [](bool v) { return v; })) {
        pf_batch_destroy(a.b);
        for (cudaEvent_t ev : a.spare) cudaEventDestroy(ev);
        {
          std::lock_guard<std::mutex> lk(s->mu);
          s->used -= a.bytes;
        }
        s->active.erase(s->active.begin() + k);
        progressed = true;
      } else {
        ++k;
      }
    }
    if (!progressed) std::this_thread::sleep_for(std::chrono::microseconds(100));
  }
}

}  // namespace

extern "C" {

const char* pf_server_last_error(void) { return g_srv_err.c_str(); }

int pf_server_create(const pf_server_config* cfg, pf_server** out) {
  if (!out) return srv_fail(PF_EINVAL, "null output pointer");
  *out = nullptr;
  pf_server* s = new pf_server();
  if (cfg) s->cfg = *cfg;
  if (s->cfg.max_active <= 0) s->cfg.max_active = 64;
  if (s->cfg.chunk_steps <= 0) s->cfg.chunk_steps = 128;
  s->cfg.chunk_steps = std::min(s->cfg.chunk_steps, kMaxChunk);
  cudaError_t e = cudaSetDevice(s->cfg.device);
  size_t free_b = 0, total_b = 0;
  if (e == cudaSuccess) e = cudaMemGetInfo(&free_b, &total_b);
  if (e != cudaSuccess) {
    delete s;
    return srv_fail(PF_ECUDA, std::string("pf_server_create: ") + cudaGetErrorString(e));
  }
  s->budget = s->cfg.hbm_budget_bytes > 0 ? (size_t)s->cfg.hbm_budget_bytes : (size_t)(0.8 * (double)free_b);
  s->worker = std::thread(worker_loop, s);
  *out = s;
  return PF_OK;
}

int pf_server_submit(pf_server* s, const pf_config* cfg, const double* phi_aos, const double* con, int nsteps,
                     long long* id) {
  if (!s || !cfg || !phi_aos || !con || !id || nsteps < 1) return srv_fail(PF_EINVAL, "bad arguments to submit");
  if (cfg->precision != 0 && cfg->precision != PF_FP32_FUSED)
    return srv_fail(PF_EINVAL, "the server runs the fused FP32 path");
  if (!pf_supported_shape(cfg->nx, cfg->ny, cfg->nz, cfg->var, PF_FP32_FUSED))
    return srv_fail(PF_EINVAL, "grid or var not supported by the fused path");
  auto r = std::make_shared<Request>();
  r->cfg = *cfg;
  r->cfg.device = s->cfg.device;
  r->cfg.precision = PF_FP32_FUSED;
  r->nsteps = nsteps;
  const size_t n = (size_t)cfg->nx * cfg->ny * cfg->nz;
  r->phi.assign(phi_aos, phi_aos + n * cfg->var);
  r->con.assign(con, con + n);
  r->t_submit = Clock::now();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return srv_fail(PF_EINVAL, "server is shutting down");
    r->id = s->next_id++;
    s->queue.push_back(r);
    s->all[r->id] = r;
  }
  s->cv_work.notify_one();
  *id = r->id;
  return PF_OK;
}

int pf_server_poll(pf_server* s, long long id, int* state) {
  if (!s || !state) return srv_fail(PF_EINVAL, "bad arguments to poll");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end()) return srv_fail(PF_EINVAL, "unknown request id");
  *state = it->second->state;
  return PF_OK;
}

int pf_server_wait(pf_server* s, long long id, double timeout_s, double* phi_aos, double* con, pf_diag* last,
                   pf_request_times* times) {
  if (!s) return srv_fail(PF_EINVAL, "null server");
  std::shared_ptr<Request> r;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return srv_fail(PF_EINVAL, "unknown request id");
    r = it->second;
    auto done = [&] { return r->state == PF_REQ_DONE || r->state == PF_REQ_FAILED; };
    if (timeout_s < 0) s->cv_done.wait(lk, done);
    else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), done))
      return srv_fail(PF_EBUSY, "request not finished within the timeout");
    s->all.erase(id);
  }
  if (times) {
    const auto start = r->t_start.time_since_epoch().count() ? r->t_start : r->t_done;  // never started: 0 run time
    times->queued_s = std::chrono::duration<double>(start - r->t_submit).count();
    times->run_s = std::chrono::duration<double>(r->t_done - start).count();
    times->total_s = std::chrono::duration<double>(r->t_done - r->t_submit).count();
  }
  if (r->state == PF_REQ_FAILED) return srv_fail(r->error, r->message);
  if (phi_aos) std::copy(r->phi.begin(), r->phi.end(), phi_aos);
  if (con) std::copy(r->con.begin(), r->con.end(), con);
  if (last) *last = r->last;
  return PF_OK;
}

int pf_server_destroy(pf_server* s) {
  if (!s) return PF_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    for (auto& r : s->queue) {
      r->state = PF_REQ_FAILED;
      r->error = PF_EINVAL;
      r->message = "server destroyed before the run started";
      r->t_done = Clock::now();
    }
    s->queue.clear();
    s->cv_done.notify_all();
  }
  s->cv_work.notify_all();
  if (s->worker.joinable()) s->worker.join();
  delete s;
  return PF_OK;
}

}  // extern "C"
