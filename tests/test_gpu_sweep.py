"""pf_sweep (many var_diff.x cases in one process) against pf_var_diff run
case by case: summary.dat and every data_save file are identical, with
batched cases of different lengths, output periods and insertion steps, two
batch groups and one case on the FP64 path."""
import os
import subprocess

import numpy as np
import pytest

from test_io import canonical_input

pytestmark = pytest.mark.gpu


def _polycryst_file(oracle, path, var, seed):
    p = oracle.Params(Nx=32, Ny=32, Nz=32, var=var)
    rng = np.random.default_rng(seed)
    lab = (oracle.voronoi_labels(p, rng.random((6, 3)) * 32.0) % (var - 1)) + 1
    lab[:8] = rng.integers(1, var, (8, 32, 32))
    with open(path, "w") as f:
        for k in range(1, 33):
            for j in range(1, 33):
                for i in range(1, 33):
                    f.write(f"{i} {j} {k} {lab[k - 1, j - 1, i - 1]}\n")


def _cases(oracle, root):
    specs = {
        "a": dict(N_step=10, ifreq=5, ppt_int=0),
        "b": dict(N_step=6, ifreq=3, ppt_int=0, t_step=0.001, sigma_1=2.0),
        "c": dict(N_step=8, ifreq=4, ppt_int=0, start="voronoi", extra="seed=4 n_grains=5 amp_phi=0.1 c0=0.4\n"),
        "d": dict(var=4, t_step=0.005, start="polycryst", N_step=10, ifreq=5, ppt_int=5, num_ppt=3,
                  extra="microstructure=grains.txt\n"),
        "e": dict(Nx=24, Ny=24, Nz=24, N_step=4, ifreq=2, ppt_int=0, grn_rad=6, num_ppt=2),
    }
    dirs = {}
    for name, kw in specs.items():
        for side in ("sweep", "single"):
            d = root / side / f"run_{name}"
            d.mkdir(parents=True)
            canonical_input(d / "input.txt", **kw)
            if name == "d":
                _polycryst_file(oracle, d / "grains.txt", 4, 11)
            dirs.setdefault(name, {})[side] = d
    return dirs


@pytest.mark.parametrize("devices", [None, "all"])
def test_sweep_equals_single_runs(pkg, oracle, tmp_path, devices):
    """devices "all": the work units placed over every visible GPU."""
    env = dict(os.environ, PFGPU_AUTOTUNE="0")  # the same kernel variants in both processes
    dirs = _cases(oracle, tmp_path)
    extra = ["--devices", devices] if devices else []
    r = subprocess.run([str(pkg.sweep_path()), "--max-batch", "2"] + extra + [str(v["sweep"]) for v in dirs.values()],
                       capture_output=True, text=True, timeout=900, env=env)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "5 of 5 cases finished" in r.stdout and "1 FP64 cases" in r.stdout
    for name, v in dirs.items():
        s = v["single"]
        rr = subprocess.run([str(pkg.driver_path()), str(s / "input.txt"), str(s) + "/"], cwd=s, capture_output=True,
                            text=True, timeout=900, env=env)
        assert rr.returncode == 0, rr.stderr
        assert (v["sweep"] / "summary.dat").read_text() == (s / "summary.dat").read_text(), name
        assert (v["sweep"] / "gamma_matrix.dat").read_text() == (s / "gamma_matrix.dat").read_text(), name
        steps = sorted(p.name for p in s.glob("step_*"))
        assert steps and steps == sorted(p.name for p in v["sweep"].glob("step_*")), name
        for st in steps:
            a = (v["sweep"] / st / "data_save.0001").read_bytes()
            b = (s / st / "data_save.0001").read_bytes()
            assert a == b, (name, st)
        ts = [l for l in (v["sweep"] / "time_step.dat").read_text().split("\n")[1:] if l.strip()]
        n_step = {"a": 10, "b": 6, "c": 8, "d": 10, "e": 4}[name]
        assert len(ts) == n_step and int(ts[-1].split()[0]) == n_step
    assert "nppt=" in (dirs["d"]["sweep"] / "mrun.out").read_text()
