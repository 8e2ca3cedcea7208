#!/usr/bin/env python3
"""Throughput of the fused FP32 phase-field step on one GB300 (or N replicas).

Workload: the polycrystal run -- 128^3 periodic grid, 16 order parameters plus
the concentration, 64 Voronoi grains from seed 1 with U(-0.01, 0.01) noise on
every order parameter, c = 0.5 + U(-0.02, 0.02), concentration-dependent
mobility M(c) = M0 (1 + c (1 - c)), a = b = 1, g = 1.5, kappa = 1, L = M0 = 1,
dt = 0.1 (2000 steps for the full run).  One "step" is one semi-implicit time
step of that run; the metric is cell-steps/s x P = Nx Ny Nz * P * steps / s.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--workload large times the 256^3 grid with 32 order parameters instead (256
grains from seed 2, c = 0.4 + U(-0.02, 0.02), kappa = 2, constant mobility,
dt = 0.1; 5000 steps for the full run), with the same line; --var overrides
the number of order parameters of either grid (small profiling cases).

Under torchrun (N > 1) every rank steps its own independent replica (seed
1 + rank) on its own GPU; there is no data-path collective ("replicas only").
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path
from types import SimpleNamespace

ROOT = Path(__file__).resolve().parent
WORKLOAD = dict(Nx=128, Ny=128, Nz=128, var=16, t_step=0.1, grad_coeff_phi=1.0, grad_coeff_c=1.0, D_S=1.0, D_L=1.0,
                D_gb=0.0, mob_phi=1.0, sigma_1=1.5, sigma_2=1.5, am=0.0, ap=0.0, con_0_mat=0.0, con_0_ppt=1.0,
                mobility="c1mc")
IC = dict(seed=1, n_grains=64, amp_phi=0.01, c0=0.5, amp_c=0.02)
WORKLOAD_NAME = "polycrystal 128^3, P=16, M(c)=M0(1+c(1-c)), 64 Voronoi grains seed 1, dt=0.1"
TRAFFIC_SUFFIX = ""  # key suffix of the ncu traffic figures for a non-headline workload
_HEADLINE = (dict(WORKLOAD), dict(IC), WORKLOAD_NAME)
METRIC = "cell-steps/s x P"
FALLBACK_HBM_GBS = 6800.0


def params(**over):
    d = dict(WORKLOAD)
    d.update(over)
    return SimpleNamespace(**d)


def select_workload(name: str, var: int | None = None) -> None:
    """Point WORKLOAD / IC / WORKLOAD_NAME at the polycrystal headline grid
    or the large grid, optionally with another number of order parameters."""
    global WORKLOAD, IC, WORKLOAD_NAME, TRAFFIC_SUFFIX
    WORKLOAD, IC, WORKLOAD_NAME, TRAFFIC_SUFFIX = dict(_HEADLINE[0]), dict(_HEADLINE[1]), _HEADLINE[2], ""
    if name == "large":
        WORKLOAD = dict(WORKLOAD, Nx=256, Ny=256, Nz=256, var=32, grad_coeff_phi=2.0, grad_coeff_c=2.0,
                        mobility="reference", D_gb=0.0)
        IC = dict(seed=2, n_grains=256, amp_phi=0.01, c0=0.4, amp_c=0.02)
        WORKLOAD_NAME = "polycrystal 256^3, P=32, constant mobility, 256 Voronoi grains seed 2, c0=0.4, kappa=2, dt=0.1"
    if var is not None and var != WORKLOAD["var"]:
        WORKLOAD = dict(WORKLOAD, var=var)
        WORKLOAD_NAME = f"{WORKLOAD_NAME} [P={var} by --var]"
    if name != "polycrystal" or var is not None:
        TRAFFIC_SUFFIX = f"@{WORKLOAD['Nx']}^3xP{WORKLOAD['var']}"


# ---------------------------------------------------------------------------
# helpers
# ---------------------------------------------------------------------------
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x: float, dist=None, device: str = "cpu") -> float:
    """The largest value of x over the ranks of the process group (x itself
    without one): whole-job times are the slowest rank's."""
    if dist is None:
        return float(x)
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(cells: int, P: int, steps: int, ranks: int, seconds: float) -> float:
    """Whole-job cell-steps/s x P: every rank steps its own replica of
    `cells` cells and P order parameters `steps` times in `seconds`."""
    return cells * P * steps * ranks / seconds


def replica_seed(rank: int) -> int:
    """Voronoi seed of rank's replica (independent runs, no collective)."""
    return IC["seed"] + rank


class Clocks:
    """nvidia-smi sampler running during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None
        self.skip = 0

    def start(self):
        """Start sampling and wait for the first samples, so that nvidia-smi's
        own start-up does not overlap the timed region."""
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
            return
        t0 = time.time()
        while time.time() - t0 < 20.0:
            with open(self.path) as fh:
                if len(fh.readlines()) >= 3:
                    break
            time.sleep(0.05)
        with open(self.path) as fh:
            self.skip = len(fh.readlines())

    def mark(self):
        """Count only the samples taken from now on."""
        if self.proc is not None:
            with open(self.path) as fh:
                self.skip = len(fh.readlines())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path).readlines()[self.skip:]:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_hbm():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic(kernel_key: str):
    """Per-launch DRAM bytes of a kernel from the committed ncu summary."""
    f = ROOT / "profiles" / "ncu_traffic.txt"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        parts = line.split()
        if len(parts) >= 2 and parts[0] == kernel_key:
            try:
                return int(parts[1])
            except ValueError:
                return None
    return None


def cpu_port_throughput(p, max_seconds: float, max_steps: int, warmup: int = 1, warmup_seconds: float = 60.0):
    """FP64 CPU restatement (the oracle, faithful 7P+9 transforms) on all
    host cores, after `warmup` untimed steps (at least one, at most
    `warmup_seconds` of them): returns (value, cores, sample description,
    steps, seconds, warm-up steps done)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import numpy as np  # noqa: F401
    import pf_ref  # the checker, used here only as the timed CPU baseline

    cores = os.cpu_count() or 1
    op = pf_ref.Params(p.Nx, p.Ny, p.Nz, p.var, t_step=p.t_step, grad_coeff_phi=p.grad_coeff_phi,
                       grad_coeff_c=p.grad_coeff_c, D_S=p.D_S, D_L=p.D_L, D_gb=p.D_gb, mob_phi=p.mob_phi,
                       sigma_1=p.sigma_1, sigma_2=p.sigma_2, am=p.am, ap=p.ap, con_0_mat=p.con_0_mat,
                       con_0_ppt=p.con_0_ppt, mobility=p.mobility)
    phi, con = pf_ref.ic_voronoi(op, IC["seed"], IC["n_grains"], IC["amp_phi"], IC["c0"], IC["amp_c"])
    o = pf_ref.Oracle(op, phi, con, faithful=True, workers=cores)
    tw, nw = time.perf_counter(), 0
    while nw < max(1, warmup):  # warm-up (plans, page faults)
        o.step()
        nw += 1
        if time.perf_counter() - tw > warmup_seconds:
            break
    t0 = time.perf_counter()
    n = 0
    while n < max_steps:
        o.step()
        n += 1
        if time.perf_counter() - t0 > max_seconds:
            break
    dt = time.perf_counter() - t0
    cells = p.Nx * p.Ny * p.Nz
    value = cells * p.var * n / dt
    sample = (f"{n} step(s) of the {p.Nx}^3 x {p.var} workload after {nw} warm-up step(s), FP64, "
              f"scipy.fft with {cores} workers, {7 * p.var + 9} 3-D transforms per step")
    return value, cores, sample, n, dt, nw

ERROR_STEPS = 100  # the stated parity horizon: 1e-5 relative at 100 steps


def fp64_error(run, r64, phi_aos, con):
    """Max-abs and L2 error (relative to the FP64 field's max-abs / L2 norm)
    of phi and c after ERROR_STEPS steps of `run` (fused FP32 path) against
    `r64` (plain FP64 GPU path, pinned to the FP64 CPU oracle at 1e-10 by the
    tests), both from the start (phi_aos, con)."""
    import numpy as np

    out = []
    for r in (run, r64):
        r.set_fields_aos(phi_aos, con)
        r.step(ERROR_STEPS, raise_nonfinite=False)
        a, c = np.empty_like(phi_aos), np.empty_like(con)
        r.get_fields_aos(a, c)
        out.append((a, c))
    (ga, gc), (ha, hc) = out

    def rel(x, y):
        return float(np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-300))

    def l2(x, y):
        return float(np.linalg.norm((x - y).ravel()) / max(np.linalg.norm(y.ravel()), 1e-300))

    e = {"phi_max_abs_rel": rel(ga, ha), "phi_l2_rel": l2(ga, ha), "c_max_abs_rel": rel(gc, hc),
         "c_l2_rel": l2(gc, hc)}
    e.update({"vs": "plain FP64 GPU path (PF_FP64_PLAIN) from the same start", "steps": ERROR_STEPS,
              "tolerance": 1e-5, "within_tolerance": max(e.values()) <= 1e-5})
    return e


# ---------------------------------------------------------------------------
# reference arm: the CPU implementation of the path on the host cores
# ---------------------------------------------------------------------------
def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    p = params()
    budget = 150.0
    value, cores, sample, n, dt, nw = cpu_port_throughput(p, budget, max(1, args.steps), warmup=args.warmup)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "cell-steps/s x P", "n_gpus": ws,
        "steps": n, "warmup": nw, "ms_per_step": 1000.0 * dt / n, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Voronoi polycrystal, ran_2 stream)",
        "config": {"workload": WORKLOAD_NAME, "grid": [p.Nx, p.Ny, p.Nz], "P": p.var,
                   "sample": f"bounded to ~{budget:.0f} s of timed CPU time after at most 60 s of warm-up"},
        "cpu_baseline": {"value": value, "unit": "cell-steps/s x P", "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "cell-steps/s x P", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": ("the reference's Fortran/MPI/P3DFFT build is not available on this host (no Fortran compiler, "
                 "MPI, FFTW or P3DFFT); its FP64 algorithm is timed through the CPU restatement"),
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def run_ours(args):
    import torch

    ws, rank, local = dist_env()
    dist = None
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    sys.path.insert(0, str(ROOT))
    import __graft_entry__ as ge

    pkg = ge.load_package()
    lib = pkg.load_library()
    p = params()
    cells = p.Nx * p.Ny * p.Nz
    nF = p.var + 1
    Kx = p.Nx // 2 + 1
    var_mob = p.mobility == "c1mc" or p.D_gb != 0.0

    phi_aos, con = pkg.ic_voronoi_aos(p, replica_seed(rank), IC["n_grains"], IC["amp_phi"], IC["c0"], IC["amp_c"],
                                      pinned=True)
    run = pkg.Run(p, device=local)
    run.set_fields_aos(phi_aos, con)
    b = run.batch_handle()
    ext = torch.cuda.ExternalStream(lib.pf_batch_stream(b), device=local)

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    clocks = Clocks(local)
    clocks.start()
    # warm-up
    lib.pf_batch_enqueue(b, args.warmup)
    torch.cuda.synchronize()

    # timed region: K steps on the library's stream, bracketed by a barrier and
    # a device synchronisation on both sides; repeated until at least 1 s has
    # passed (so the clock sampler sees the timed work), the median repeat
    # reported
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    clocks.mark()
    rep_ms = []
    t_rep = time.perf_counter()
    rc = 0
    while True:
        barrier()
        ev0.record(ext)
        rc = lib.pf_batch_enqueue(b, args.steps)
        ev1.record(ext)
        ev1.synchronize()
        barrier()
        if rc != 0:
            break
        rep_ms.append(ev0.elapsed_time(ev1))
        if time.perf_counter() - t_rep >= args.min_timed_s and len(rep_ms) >= 3:
            break
    clk = clocks.stop()
    if rc != 0:
        raise RuntimeError(lib.pf_last_error().decode())
    ms = statistics.median(rep_ms)
    # confirm the run stayed finite (one more step, untimed, with its record)
    d = run.step(1)[0]
    if d["nonfinite"]:
        raise RuntimeError("non-finite values in the benchmark run")
    ms = max_over_ranks(ms, dist, f"cuda:{local}")
    value = job_throughput(cells, p.var, args.steps, ws, ms / 1000.0)

    # per-kernel timing on the same stream (each kernel alone, back to back)
    plane = p.Ny * p.Nz * Kx * 8  # bytes of one field's half spectrum (complex64)
    kernels = {
        "x_pass": dict(phase=0, bytes=2 * nF * plane + (cells * 4 if var_mob else 0)),
        # reads D~ and u_hat, writes u_hat and u~ (the c plane writes J~ instead of u~ under M(c))
        "yz_pass": dict(phase=1, bytes=4 * nF * plane),
    }
    reps = max(20, min(200, args.steps // 4))
    for name, k in kernels.items():
        # NVTX range named after the kernel: an ncu capture can select these
        # whole-grid launches with --nvtx --nvtx-include "<name>/"
        torch.cuda.nvtx.range_push(name)
        lib.pf_batch_enqueue_phase(b, k["phase"])
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        for _ in range(reps):
            lib.pf_batch_enqueue_phase(b, k["phase"])
        e1.record(ext)
        e1.synchronize()
        torch.cuda.nvtx.range_pop()
        k["ms"] = e0.elapsed_time(e1) / reps
    # bytes one whole step moves in this design: x pass + yz pass over all
    # fields, and under variable mobility the xj pass (J~ in and out, mobility
    # field in) and the C2 pass (J~ and c state in, c state out)
    step_design_bytes = kernels["x_pass"]["bytes"] + kernels["yz_pass"]["bytes"]
    if var_mob:
        step_design_bytes += (2 * plane + cells * 4) + 3 * plane
    dom_name = max(kernels, key=lambda n: kernels[n]["ms"])
    dom = kernels[dom_name]
    peak, peak_kind = measured_hbm()
    achieved = dom["bytes"] / (dom["ms"] / 1000.0) / 1e9
    traffic = ncu_traffic(dom_name + TRAFFIC_SUFFIX)

    # end to end through the C ABI with host buffers: upload the start fields
    # from pinned memory, K steps with their diagnostic records returned to the
    # host, download the fields (one output interval of K steps)
    out_phi = torch.empty(phi_aos.shape, dtype=torch.float64, pin_memory=True).numpy()
    out_con = torch.empty(con.shape, dtype=torch.float64, pin_memory=True).numpy()
    run.set_fields_aos(phi_aos, con)
    run.step(2)
    barrier()
    t0 = time.perf_counter()
    run.set_fields_aos(phi_aos, con)
    recs = run.step(args.steps)
    run.get_fields_aos(out_phi, out_con)
    t1 = time.perf_counter()
    e2e_s = t1 - t0
    e2e_s = max_over_ranks(e2e_s, dist, f"cuda:{local}")
    e2e_value = job_throughput(cells, p.var, args.steps, ws, e2e_s)
    field_bytes = (phi_aos.nbytes + con.nbytes)
    diag_bytes = 80  # sizeof(pf_diag)
    assert len(recs) == args.steps

    # x pass, yz pass (order-parameter planes and c planes as two launches on
    # the graph's two branches), xj pass, yz C2 pass, and the step's record
    # kernel; with constant mobility x pass, yz pass and record
    kernels_per_step = 6 if var_mob else 3
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "cell-steps/s x P", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Voronoi polycrystal from the ran_2 stream, no dataset)",
            "timing": {"repeats": len(rep_ms), "steps_per_repeat": args.steps,
                       "ms_per_repeat_median": statistics.median(rep_ms),
                       "ms_per_repeat_min": min(rep_ms), "ms_per_repeat_max": max(rep_ms),
                       "what": "value and ms_per_step from the median repeat of K steps (CUDA events on the "
                               "library's stream); repeats continue until at least %.1f s" % args.min_timed_s},
            "config": {"workload": WORKLOAD_NAME, "grid": [p.Nx, p.Ny, p.Nz], "P": p.var, "runs_per_gpu": 1,
                       "parallelism": f"replicas x{ws}" if ws > 1 else "single run",
                       "l2": "inputs larger than L2: %.0f MB resident state + scratch per step > 129 MB L2" %
                             ((3 * nF * plane + cells * 4 + plane) / 1e6)},
            "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                         "algorithmic_bytes_per_launch": dom["bytes"], "ms_per_launch": dom["ms"],
                         "other_kernels": {n: {"ms_per_launch": k["ms"], "algorithmic_bytes": k["bytes"],
                                               "GB_s": k["bytes"] / (k["ms"] / 1000.0) / 1e9}
                                           for n, k in kernels.items()}},
            # the whole step against the reference-shaped byte count per cell-step,
            # 4 (9P + 21) with variable mobility / 4 (9P + 9) without (FP32 fields;
            # every 3-D transform one read and one write of its field)
            "step_roofline": {"bytes_per_cell_step": 4 * (9 * p.var + (21 if var_mob else 9)),
                              "achieved": 4 * (9 * p.var + (21 if var_mob else 9)) * cells /
                                          (ms / args.steps / 1000.0) / 1e9,
                              "peak": peak, "unit": "GB/s",
                              "frac": 4 * (9 * p.var + (21 if var_mob else 9)) * cells /
                                      (ms / args.steps / 1000.0) / 1e9 / peak},
            # the whole step against the bytes this design moves per cell-step:
            # x pass 2 nF plane reads/writes, yz pass 4 nF (+ the mobility field
            # and the xj / C2 passes of the c field under variable mobility)
            "step_roofline_design": {"bytes_per_step": step_design_bytes,
                                     "bytes_per_cell_step": step_design_bytes / cells,
                                     "achieved": step_design_bytes / (ms / args.steps / 1000.0) / 1e9,
                                     "peak": peak, "unit": "GB/s",
                                     "frac": step_design_bytes / (ms / args.steps / 1000.0) / 1e9 / peak},
            "clocks": clk,
            "e2e": {"value": e2e_value, "unit": "cell-steps/s x P",
                    "h2d_bytes_per_step": field_bytes / args.steps,
                    "d2h_bytes_per_step": field_bytes / args.steps + diag_bytes,
                    "what": f"pf_set_fields (pinned host) + pf_step({args.steps}) with per-step records + "
                            "pf_get_fields, host wall clock"},
            "gpu_launches": kernels_per_step * args.steps,
            "kernel_variants": lib.pf_batch_variant(b).decode(),
        }
        if ws == 1 and not args.no_fp64:
            # the plain FP64 GPU path (cuFFT, one kernel per reference phase) on
            # the same workload: its throughput, and the error of this run's
            # fields against it after ERROR_STEPS steps from the same start
            r64 = pkg.Run(p, precision=pkg.PF_FP64_PLAIN, device=local)
            r64.set_fields_aos(phi_aos, con)
            r64.step(2)
            torch.cuda.synchronize()
            n64 = 20
            t64 = time.perf_counter()
            r64.step(n64, raise_nonfinite=False)
            t64 = time.perf_counter() - t64
            v64 = cells * p.var * n64 / t64
            line["fp64_gpu_path"] = {"value": v64, "unit": METRIC, "steps": n64,
                                     "ratio": value / v64, "what": "PF_FP64_PLAIN, host wall clock per pf_step call"}
            line["error"] = fp64_error(run, r64, phi_aos, con)
            r64.close()
        if not args.no_cpu_baseline and ws == 1 and p.Nx * p.Ny * p.Nz * p.var > (128 ** 3) * 16:
            # one FP64 CPU step of a grid this size takes minutes on the host cores
            line["cpu_baseline"] = {"value": None, "skipped": "one FP64 step of this grid on the CPU restatement "
                                                              "takes about two minutes on 16 cores"}
        elif not args.no_cpu_baseline and ws == 1:
            v, cores, sample, n, dt, _ = cpu_port_throughput(p, 20.0, 50)
            line["cpu_baseline"] = {"value": v, "unit": "cell-steps/s x P", "cores": cores, "kind": "port",
                                    "sample": sample}
        print(json.dumps(line), flush=True)
    run.close()
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return 0


# ---------------------------------------------------------------------------
# other workloads (not the headline line): the batched ensemble and a served
# request stream
# ---------------------------------------------------------------------------
def _ran2_uniform(pkg, seed: int):
    """Uniform draws from the reference's ran_2 with idum = -(seed+1)."""
    r = pkg.Ran2(-(seed + 1))
    return r.next


def ensemble_requests(pkg, n_runs: int, N: int = 64, P: int = 8, seed: int = 3):
    """Config 3: per run L ~ logU(0.1, 10), kappa ~ U(0.5, 4), g ~ U(1, 2),
    c0 ~ U(0.3, 0.7), drawn in that order from ran_2 (seed 3); the start of
    run i is the config-0 noise start from seed 1000*seed + i."""
    u = _ran2_uniform(pkg, seed)
    out = []
    for i in range(n_runs):
        L = 10 ** (-1 + 2 * u())
        kap = 0.5 + 3.5 * u()
        g = 1.0 + u()
        c0 = 0.3 + 0.4 * u()
        p = params(Nx=N, Ny=N, Nz=N, var=P, t_step=0.05, mob_phi=L, grad_coeff_phi=kap, grad_coeff_c=kap,
                   sigma_1=g, sigma_2=g, mobility="reference", D_gb=0.0)
        out.append((p, 1000 * seed + i, c0))
    return out


def run_ensemble(args):
    import torch

    torch.cuda.set_device(0)
    sys.path.insert(0, str(ROOT))
    import __graft_entry__ as ge

    pkg = ge.load_package()
    lib = pkg.load_library()
    reqs = ensemble_requests(pkg, args.runs)
    b = pkg.Batch([r[0] for r in reqs])
    for i, (p, seed, c0) in enumerate(reqs):
        phi, con = pkg.ic_noise(p, seed, 0.001, c0, 0.01)
        b.set_fields(i, phi, con)
    bh = b.h
    ext = torch.cuda.ExternalStream(lib.pf_batch_stream(bh), device=0)
    lib.pf_batch_enqueue(bh, args.warmup)
    torch.cuda.synchronize()
    clocks = Clocks(0)
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    clocks.mark()
    e0.record(ext)
    lib.pf_batch_enqueue(bh, args.steps)
    e1.record(ext)
    e1.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    p = reqs[0][0]
    cells = p.Nx * p.Ny * p.Nz
    value = cells * p.var * len(reqs) * args.steps / (ms / 1000.0)
    # the same runs one at a time (a sample), for the gain of batching
    n1, k1 = min(4, len(reqs)), 100
    t = 0.0
    for p1, seed, c0 in reqs[:n1]:
        run = pkg.Run(p1)
        phi, con = pkg.ic_noise(p1, seed, 0.001, c0, 0.01)
        run.set_fields(phi, con)
        run.step(5)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        run.step(k1)
        t += time.perf_counter() - t0
        run.close()
    alone = cells * p.var * n1 * k1 / t
    nF, Kx = p.var + 1, p.Nx // 2 + 1
    design_bytes = 6 * nF * Kx * p.Ny * p.Nz * 8 * len(reqs)
    peak, peak_kind = measured_hbm()
    achieved = design_bytes / (ms / 1000.0 / args.steps) / 1e9
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (ran_2-seeded noise starts and coefficients)",
            "config": {"workload": f"ensemble: {len(reqs)} runs of {p.Nx}^3, P={p.var}, one batch (config 3)",
                       "inputs_vs_l2": "resident working set above L2"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind, "traffic": None,
                         "what": "x + yz pass design bytes of all runs per batched step"},
            "runs_one_at_a_time": {"value": alone, "unit": METRIC, "runs": n1, "steps": k1},
            "clocks": clk, "gpu_launches": 3 * args.steps, "kernel_variants": lib.pf_batch_variant(bh).decode()}
    print(json.dumps(line), flush=True)
    b.close()
    return 0


def serve_requests(pkg, n: int, rate: float, seed: int = 4):
    """Config 4: Poisson arrivals at `rate`; grid 32/64/128/256 with
    probabilities .4/.3/.2/.1, P from {4, 8, 16}, steps ~ logU(100, 5000),
    coefficients as config 3, all from ran_2 (seed 4)."""
    import math

    u = _ran2_uniform(pkg, seed)
    t, out = 0.0, []
    for i in range(n):
        t += -math.log(max(u(), 1e-12)) / rate
        x = u()
        N = 32 if x < 0.4 else 64 if x < 0.7 else 128 if x < 0.9 else 256
        P = (4, 8, 16)[min(2, int(3 * u()))]
        steps = int(round(10 ** (2 + math.log10(50.0) * u())))
        L, kap, g, c0 = 10 ** (-1 + 2 * u()), 0.5 + 3.5 * u(), 1.0 + u(), 0.3 + 0.4 * u()
        p = params(Nx=N, Ny=N, Nz=N, var=P, t_step=0.05, mob_phi=L, grad_coeff_phi=kap, grad_coeff_c=kap,
                   sigma_1=g, sigma_2=g, mobility="reference", D_gb=0.0)
        out.append((t, p, steps, 4000 * seed + i, c0))
    return out


def _pct(xs, q):
    xs = sorted(xs)
    return xs[min(len(xs) - 1, int(round(q * (len(xs) - 1))))]


def run_serve(args):
    """Config 4 at every rate of --rates: the served stream (submitted at its
    Poisson arrival times to a pf_pool -- one continuous-batching pf_server
    per visible GPU) against serial execution of the same requests.  The
    request properties come from the same ran_2 draws at every rate; only the
    arrival times scale with 1/rate.  Serial: each request's service time alone
    (pf_create / pf_set_fields / pf_step / pf_get_fields / pf_destroy, measured
    once), replayed as a FIFO single server at each rate's arrival times."""
    import torch

    torch.cuda.set_device(0)
    sys.path.insert(0, str(ROOT))
    import __graft_entry__ as ge

    pkg = ge.load_package()
    import queue
    import threading

    import numpy as np

    rates = [float(r) for r in str(args.rates).split(",")] if args.rates else [args.rate]
    base = serve_requests(pkg, args.requests, 1.0)  # arrival times at rate 1; scaled per rate below
    # starting fields in the library's phi(var,x,y,z) layout, prepared before either leg is timed
    starts = []
    for (_, p, _, seed, c0) in base:
        phi, con = pkg.ic_noise(p, seed, 0.001, c0, 0.01)
        starts.append((pkg.to_aos(phi), np.ascontiguousarray(con, dtype=np.float64)))
    # warm the autotuner cache for every class (as a long-running server would be)
    for cls in sorted({(p.Nx, p.var) for (_, p, _, _, _) in base}):
        p = next(r[1] for r in base if (r[1].Nx, r[1].var) == cls)
        w = pkg.Run(p)
        w.close()
    torch.cuda.synchronize()
    # serial service times, measured once: create, upload, steps, download, destroy
    service = []
    for (_, p, steps, _, _), (phi_a, con) in zip(base, starts):
        tb = time.perf_counter()
        run = pkg.Run(p)
        run.set_fields_aos(phi_a, con)
        run.step(steps, raise_nonfinite=False)
        run.get_fields_aos(np.empty_like(phi_a), np.empty_like(con))
        run.close()
        service.append(time.perf_counter() - tb)
    n = len(base)
    work = sum(p.Nx * p.Ny * p.Nz * p.var * steps for (_, p, steps, _, _) in base)
    per_rate, detail = [], []
    for rate in rates:
        arrivals = [ta / rate for (ta, _, _, _, _) in base]
        pool = pkg.Pool(max_active=args.max_active)
        ids: "queue.Queue" = queue.Queue()
        done = {}

        failed = []

        def waiter():  # collects results as they finish, beside the arrivals
            while True:
                i = ids.get()
                if i is None:
                    return
                try:
                    _, _, _, tm = pool.wait_aos(i)
                except Exception as exc:  # a failed request: report it after the stream
                    failed.append((i, repr(exc)))
                    continue
                done[i] = (time.perf_counter(), tm)

        th = threading.Thread(target=waiter)
        t0 = time.perf_counter()
        th.start()
        order, t_sub = [], []
        for ta, (_, p, steps, _, _), (phi_a, con) in zip(arrivals, base, starts):
            while time.perf_counter() - t0 < ta:
                time.sleep(0.0005)
            t_sub.append(time.perf_counter() - t0)
            rid = pool.submit_aos(p, phi_a, con, steps)[0]
            order.append(rid)
            ids.put(rid)
        ids.put(None)
        th.join()
        if failed:
            pool.close()
            raise RuntimeError(f"served requests failed at rate {rate}: {failed[:3]}")
        t_served = max(done[i][0] for i in order) - t0
        lat = [done[i][1]["total_s"] for i in order]
        ndev = pool.devices
        pool.close()
        clock, lat_s = 0.0, []
        for ta, dt in zip(arrivals, service):
            clock = max(clock, ta) + dt
            lat_s.append(clock - ta)
        per_rate.append({"rate_per_s": rate, "devices": ndev,
                         "served": {"runs_per_s": n / t_served, "p50_s": _pct(lat, 0.5), "p99_s": _pct(lat, 0.99),
                                    "cell_steps_per_s_x_P": work / t_served},
                         "serial": {"runs_per_s": n / clock, "p50_s": _pct(lat_s, 0.5), "p99_s": _pct(lat_s, 0.99)}})
        for k, ((_, p, steps, _, _), i) in enumerate(zip(base, order)):
            detail.append({"rate": rate, "k": k, "N": p.Nx, "P": p.var, "steps": steps, "arrival_s": arrivals[k],
                           "submitted_s": t_sub[k], "done_s": done[i][0] - t0, "service_alone_s": service[k],
                           "serial_latency_s": lat_s[k], **done[i][1]})
    if args.serve_detail:
        with open(args.serve_detail, "w") as fh:
            for row in detail:
                fh.write(json.dumps(row) + "\n")
    top = per_rate[-1]
    line = {"metric": "served runs/s", "value": top["served"]["runs_per_s"], "unit": "runs/s", "n_gpus": top["devices"],
            "steps": None, "warmup": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic request stream (ran_2 seed 4)",
            "config": {"workload": f"served stream: {n} requests per rate, Poisson rates {rates}/s, grids 32-256, "
                                   f"P 4-16, 100-5000 steps (config 4)", "max_active": args.max_active},
            "rates": per_rate,
            "serial_what": "each request alone (pf_create/pf_set_fields/pf_step/pf_get_fields/pf_destroy), "
                           "service times measured once, FIFO single server at each rate's arrival times",
            "served_what": "requests submitted through pf_pool_submit at their arrival times (fields already in the "
                           "library's layout), results collected by a second thread as they finish; runs/s over "
                           "the time from the first arrival to the last result"}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-fp64", action="store_true",
                    help="skip the FP64 GPU path comparison (its throughput and the error against it)")
    ap.add_argument("--min-timed-s", type=float, default=1.0,
                    help="repeat the K timed steps until this many seconds have passed (median repeat reported)")
    ap.add_argument("--workload", choices=["polycrystal", "large", "ensemble", "serve"], default="polycrystal",
                    help="polycrystal (the headline line, 128^3 x 16), large (256^3 x 32), ensemble (config 3) "
                         "or serve (config 4)")
    ap.add_argument("--var", type=int, default=None,
                    help="polycrystal / large: another number of order parameters (small profiling cases)")
    ap.add_argument("--runs", type=int, default=256, help="ensemble: runs in the batch")
    ap.add_argument("--requests", type=int, default=24, help="serve: requests in the stream")
    ap.add_argument("--rate", type=float, default=8.0, help="serve: Poisson arrival rate (requests/s)")
    ap.add_argument("--rates", type=str, default=None,
                    help="serve: comma-separated arrival rates to sweep (requests/s), e.g. 2,4,8,16")
    ap.add_argument("--max-active", type=int, default=16, help="serve: resident runs at most")
    ap.add_argument("--serve-detail", type=str, default=None,
                    help="serve: write one JSON row per request and rate (arrival, submit, finish, times) to this file")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.workload in ("polycrystal", "large"):
        select_workload(args.workload, args.var)
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "ensemble":
        return run_ensemble(args)
    if args.workload == "serve":
        return run_serve(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
