"""The multi-replica path of bench.py on CPU: two gloo ranks agree on the
slowest rank's time, count every rank's work, seed distinct replicas, and only
rank 0 runs the reference arm."""
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local_ms = [12.5, 30.0][rank]
    ms = bench.max_over_ranks(local_ms, dist, "cpu")
    value = bench.job_throughput(128 ** 3, 16, 100, world, ms / 1000.0)
    out.put((rank, ms, value, bench.replica_seed(rank)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import socket

    with socket.socket() as sck:
        sck.bind(("127.0.0.1", 0))
        port = sck.getsockname()[1]
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    assert [r[1] for r in res] == [30.0, 30.0]                  # both ranks report the slowest time
    assert res[0][2] == res[1][2] == 128 ** 3 * 16 * 100 * 2 / 0.030  # whole-job work over that time
    assert res[0][3] != res[1][3]                                # independent replicas


def test_reference_arm_runs_on_rank_0_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], capture_output=True, text=True, timeout=120, env=env)
    assert r.returncode == 0 and r.stdout.strip() == ""


def test_large_workload_selection():
    """--workload large is the 256^3 x 32 polycrystal (256 grains, seed 2,
    c0 = 0.4, kappa = 2, constant mobility); --var changes only P and keys the
    ncu traffic figure by grid and P.  Run in a child process: the selection
    sets module globals."""
    code = ("import sys; sys.path.insert(0, %r); import bench\n"
            "bench.select_workload('large'); p = bench.params()\n"
            "assert (p.Nx, p.Ny, p.Nz, p.var, p.mobility, p.D_gb) == (256, 256, 256, 32, 'reference', 0.0)\n"
            "assert (p.grad_coeff_phi, p.grad_coeff_c, p.t_step) == (2.0, 2.0, 0.1)\n"
            "assert bench.IC == dict(seed=2, n_grains=256, amp_phi=0.01, c0=0.4, amp_c=0.02)\n"
            "assert bench.TRAFFIC_SUFFIX == '@256^3xP32' and bench.replica_seed(1) == 3\n"
            "bench.select_workload('polycrystal', 4)\n"
            "assert bench.params().Nx == 128 and bench.params().var == 4 and bench.TRAFFIC_SUFFIX == '@128^3xP4'\n"
            "bench.select_workload('large', 4)\n"
            "assert bench.params().Nx == 256 and bench.params().var == 4 and bench.TRAFFIC_SUFFIX == '@256^3xP4'\n"
            ) % str(ROOT)
    subprocess.run([sys.executable, "-c", code], check=True, timeout=120)
    code = ("import sys; sys.path.insert(0, %r); import bench\n"
            "bench.select_workload('polycrystal'); p = bench.params()\n"
            "assert (p.Nx, p.var, p.mobility) == (128, 16, 'c1mc') and bench.TRAFFIC_SUFFIX == ''\n") % str(ROOT)
    subprocess.run([sys.executable, "-c", code], check=True, timeout=120)
