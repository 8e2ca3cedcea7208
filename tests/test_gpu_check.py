"""pf_check_fp64: a run's error against the plain FP64 GPU path, the per-run
report of max-abs and L2 error in the order parameters and c.  The device-side
comparison must equal the same comparison done on the host from the two
paths' downloaded fields, and the drop-in driver prints it for check_fp64=N."""
import subprocess

import numpy as np
import pytest

from test_gpu_parity import _l2, _rel, _run_lib
from test_io import canonical_input

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape", [(32, 32, 32, 4), (64, 32, 64, 3)])
def test_check_fp64_equals_host_comparison(pkg, oracle, shape):
    nx, ny, nz, var = shape
    p = oracle.Params(nx, ny, nz, var, t_step=0.05, mobility="c1mc")
    phi, con = pkg.ic_voronoi(p, 4, 6, 0.01, 0.5, 0.02)
    rep = pkg.check_fp64(p, phi, con, 30)
    gp, gc, _ = _run_lib(pkg, p, phi, con, 30)
    hp, hc, _ = _run_lib(pkg, p, phi, con, 30, precision=64)
    want = dict(phi_max_abs_rel=_rel(gp, hp), phi_l2_rel=_l2(gp, hp), c_max_abs_rel=_rel(gc, hc), c_l2_rel=_l2(gc, hc))
    assert rep["steps"] == 30
    for k, v in want.items():
        assert abs(rep[k] - v) <= 1e-9 * v + 1e-15, (k, rep[k], v)
        assert rep[k] < 1e-5, (k, rep[k])


def test_driver_prints_the_fp64_check(pkg, tmp_path):
    inp = canonical_input(tmp_path / "input.txt", N_step=4, ifreq=4, ppt_int=0, extra="check_fp64=20\n")
    r = subprocess.run([str(pkg.driver_path()), str(inp), str(tmp_path) + "/"], cwd=tmp_path, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    line = next(l for l in r.stdout.splitlines() if "fp64 check" in l)
    vals = [float(t) for t in line.replace(",", " ").split() if t[0].isdigit() and "e" in t]
    assert "20 steps" in line and len(vals) == 4 and max(vals) < 1e-5, line
