// Independent runs spread over the node's GPUs: the host-side dispatcher that
// stands in for the reference's job-level fan-out (one SLURM job per run,
// tests/scaling_tests.py:88-124, tests/run_phase_sim.py:130-172).  Runs never
// communicate, so there is no collective: every device has its own pf_server
// (continuous batching on that GPU), and the dispatcher only decides where
// each run goes.
//
//   * pf_place_units: offline placement of known work units (the batches and
//     single cases of a sweep) -- largest unit first onto the device with the
//     least work so far (LPT scheduling);
//   * pf_pick_device: online placement -- the device with the least
//     outstanding work;
//   * pf_pool_*: one server per device, requests placed with pf_pick_device
//     on the work the device's unfinished requests still represent.
// The two placement functions need no GPU, so their logic is tested on the
// CPU with any device count.
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/pfgpu.h"

namespace {

thread_local std::string g_pool_err;

int pool_fail(int code, const std::string& m) {
  g_pool_err = m;
  return code;
}

struct Pending {
  long long sid;  // the device server's request id
  double work;    // cell-steps x P of the request
};

}  // namespace

struct pf_pool {
  std::vector<int> devices;
  std::vector<pf_server*> servers;
  std::mutex mu;
  std::vector<std::vector<Pending>> pending;      // per device: submitted, not yet finished
  std::map<long long, std::pair<int, long long>> ids;  // pool id -> (device index, server id)
  long long next = 1;
};

extern "C" {

const char* pf_pool_last_error(void) { return g_pool_err.c_str(); }

int pf_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

double pf_run_work(const pf_config* c, int nsteps) {
  if (!c || nsteps < 0) return 0.0;
  return (double)c->nx * c->ny * c->nz * c->var * nsteps;
}

int pf_pick_device(const double* outstanding, int ndev) {
  if (!outstanding || ndev < 1) return -1;
  int best = 0;
  for (int d = 1; d < ndev; ++d)
    if (outstanding[d] < outstanding[best]) best = d;
  return best;
}

int pf_place_units(const double* work, int nunits, int ndev, int* device_of_unit, double* load) {
  if (!work || !device_of_unit || nunits < 0 || ndev < 1) return PF_EINVAL;
  std::vector<int> order(nunits);
  std::iota(order.begin(), order.end(), 0);
  // largest first; equal work keeps the given order (stable)
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return work[a] > work[b]; });
  std::vector<double> l(ndev, 0.0);
  for (int u : order) {
    const int d = pf_pick_device(l.data(), ndev);
    device_of_unit[u] = d;
    l[d] += work[u];
  }
  if (load) std::copy(l.begin(), l.end(), load);
  return PF_OK;
}

int pf_pool_create(const pf_pool_config* cfg, pf_pool** out) {
  if (!out) return pool_fail(PF_EINVAL, "null output pointer");
  *out = nullptr;
  pf_pool_config c{};
  if (cfg) c = *cfg;
  std::vector<int> devs;
  if (c.devices && c.ndevices > 0) {
    devs.assign(c.devices, c.devices + c.ndevices);
  } else {
    int n = c.ndevices;
    if (n <= 0) {
      const cudaError_t e = cudaGetDeviceCount(&n);
      if (e != cudaSuccess || n < 1) return pool_fail(PF_ECUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
    }
    for (int d = 0; d < n; ++d) devs.push_back(d);
  }
  pf_pool* p = new pf_pool();
  p->devices = devs;
  for (int d : devs) {
    pf_server_config sc = c.server;
    sc.device = d;
    pf_server* s = nullptr;
    const int rc = pf_server_create(&sc, &s);
    if (rc != PF_OK) {
      const std::string msg = std::string("device ") + std::to_string(d) + ": " + pf_server_last_error();
      for (pf_server* t : p->servers) pf_server_destroy(t);
      delete p;
      return pool_fail(rc, msg);
    }
    p->servers.push_back(s);
  }
  p->pending.resize(devs.size());
  *out = p;
  return PF_OK;
}

int pf_pool_devices(pf_pool* p) { return p ? (int)p->devices.size() : 0; }

int pf_pool_submit(pf_pool* p, const pf_config* cfg, const double* phi_aos, const double* con, int nsteps,
                   long long* id, int* device) {
  if (!p || !cfg || !id) return pool_fail(PF_EINVAL, "bad arguments to pf_pool_submit");
  std::lock_guard<std::mutex> lk(p->mu);
  const int nd = (int)p->devices.size();
  std::vector<double> outstanding(nd, 0.0);
  for (int d = 0; d < nd; ++d) {
    auto& v = p->pending[d];
    v.erase(std::remove_if(v.begin(), v.end(),
                           [&](const Pending& q) {
                             int st = PF_REQ_DONE;
                             return pf_server_poll(p->servers[d], q.sid, &st) != PF_OK || st == PF_REQ_DONE ||
                                    st == PF_REQ_FAILED;
                           }),
            v.end());
    for (const Pending& q : v) outstanding[d] += q.work;
  }
  const int d = pf_pick_device(outstanding.data(), nd);
  long long sid = 0;
  const int rc = pf_server_submit(p->servers[d], cfg, phi_aos, con, nsteps, &sid);
  if (rc != PF_OK) return pool_fail(rc, pf_server_last_error());
  p->pending[d].push_back(Pending{sid, pf_run_work(cfg, nsteps)});
  *id = p->next++;
  p->ids[*id] = std::make_pair(d, sid);
  if (device) *device = p->devices[d];
  return PF_OK;
}

int pf_pool_wait(pf_pool* p, long long id, double timeout_s, double* phi_aos, double* con, pf_diag* last,
                 pf_request_times* times) {
  if (!p) return pool_fail(PF_EINVAL, "null pool");
  std::pair<int, long long> where;
  {
    std::lock_guard<std::mutex> lk(p->mu);
    auto it = p->ids.find(id);
    if (it == p->ids.end()) return pool_fail(PF_EINVAL, "unknown request id");
    where = it->second;
  }
  const int rc = pf_server_wait(p->servers[where.first], where.second, timeout_s, phi_aos, con, last, times);
  if (rc == PF_EBUSY) return pool_fail(rc, pf_server_last_error());
  {
    std::lock_guard<std::mutex> lk(p->mu);
    p->ids.erase(id);
    auto& v = p->pending[where.first];
    v.erase(std::remove_if(v.begin(), v.end(), [&](const Pending& q) { return q.sid == where.second; }), v.end());
  }
  return rc == PF_OK ? PF_OK : pool_fail(rc, pf_server_last_error());
}

int pf_pool_destroy(pf_pool* p) {
  if (!p) return PF_OK;
  for (pf_server* s : p->servers) pf_server_destroy(s);
  delete p;
  return PF_OK;
}

}  // extern "C"
