"""Every compiled kernel variant (x pass: rows and threads per CTA; yz pass:
one CTA per plane or clusters) gives the oracle's fields and diagnostics,
whichever one the autotuner would pick.  Each variant is forced through
PFGPU_X_VARIANT / PFGPU_YZ_VARIANT for one run."""
import os

import numpy as np
import pytest

from test_gpu_parity import TOL32, _check_diag, _check_fields

pytestmark = pytest.mark.gpu

# (80^3, 102^3 and 160^3 are the reference's weak-scaling grids,
# inputs/config.yaml:71-106)
SHAPES = [(32, 32, 32, 5), (64, 64, 64, 4), (96, 96, 96, 3), (128, 128, 128, 3), (64, 32, 64, 3), (80, 80, 80, 4),
          (102, 102, 102, 3), (160, 160, 160, 3)]


def _run(pkg, p, phi, con, steps, env):
    old = {k: os.environ.get(k) for k in env}
    os.environ.update(env)
    try:
        run = pkg.Run(p)
        run.set_fields(phi, con)
        d = run.step(steps)
        gp, gc = run.get_fields()
        var = pkg.load_library().pf_batch_variant(run.batch_handle()).decode()
        run.close()
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    return gp, gc, d, var


@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "x".join(map(str, s)))
def test_every_variant_matches_oracle(pkg, oracle, shape):
    nx, ny, nz, var = shape
    p = oracle.Params(nx, ny, nz, var, t_step=0.01, mobility="c1mc", am=0.5, ap=2.0, con_0_mat=0.3, con_0_ppt=0.7)
    phi, con = oracle.ic_voronoi(p, 5, 6, 0.02, 0.45, 0.02)
    steps = 3
    op, oc, od = oracle.run(p, phi, con, steps, faithful=False, workers=8)
    nxv, nyzv = pkg.variant_counts(nx, ny, nz)
    assert nxv >= 1 and nyzv >= 1
    seen = set()
    for i in range(nxv):
        gp, gc, gd, name = _run(pkg, p, phi, con, steps, {"PFGPU_X_VARIANT": str(i), "PFGPU_YZ_VARIANT": "0"})
        _check_fields(gp, gc, op, oc, TOL32)
        _check_diag(gd, od, TOL32, oracle.stats(phi, con))
        seen.add(name)
    for j in range(nyzv):
        gp, gc, gd, name = _run(pkg, p, phi, con, steps, {"PFGPU_X_VARIANT": "0", "PFGPU_YZ_VARIANT": str(j)})
        _check_fields(gp, gc, op, oc, TOL32)
        _check_diag(gd, od, TOL32, oracle.stats(phi, con))
        seen.add(name)
    assert len(seen) >= nxv  # every x variant ran (a yz variant that cannot be scheduled falls back)


@pytest.mark.parametrize("n,var", [(256, 16), (200, 8)])
def test_every_variant_large(pkg, oracle, n, var):
    """256^3 and 200^3 (the largest of the reference's weak-scaling grids):
    each variant against the FP64 GPU path (the oracle would take minutes per
    step at this size), with enough fields that every x variant's per-warp
    reductions are exercised."""
    p = oracle.Params(n, n, n, var, t_step=0.02, am=0.5, ap=2.0, con_0_mat=0.3, con_0_ppt=0.7)
    phi, con = pkg.ic_voronoi(p, 2, 24, 0.01, 0.4, 0.02)
    steps = 2
    run = pkg.Run(p, precision=pkg.PF_FP64_PLAIN)
    run.set_fields(phi, con)
    hd = run.step(steps)
    hp, hc = run.get_fields()
    run.close()
    nxv, nyzv = pkg.variant_counts(n, n, n)
    envs = [{"PFGPU_X_VARIANT": str(i), "PFGPU_YZ_VARIANT": "0"} for i in range(nxv)]
    envs += [{"PFGPU_X_VARIANT": "0", "PFGPU_YZ_VARIANT": str(j)} for j in range(1, nyzv)]
    for env in envs:
        gp, gc, gd, name = _run(pkg, p, phi, con, steps, env)
        _check_fields(gp, gc, hp, hc, TOL32)
        for a, b in zip(gd, hd):
            for k in ("f_int", "f_eta", "f_ch", "c_min", "c_max", "phi_min", "phi_P_max"):
                assert abs(a[k] - b[k]) <= TOL32 * max(1.0, abs(b[k])), (name, a["step"], k, a[k], b[k])
            assert a["nonfinite"] == 0, name


def test_runs_of_one_grid_with_different_var_coexist(pkg, oracle):
    """Kernels are shared by every run of a grid: creating a run with fewer
    fields must not shrink the shared-memory limit a live run with more fields
    needs."""
    pa = oracle.Params(64, 64, 64, 12, t_step=0.05)
    pb = oracle.Params(64, 64, 64, 3, t_step=0.05)
    fa = oracle.ic_noise(pa, 1, 0.001, 0.5, 0.01)
    fb = oracle.ic_noise(pb, 2, 0.001, 0.5, 0.01)
    ra = pkg.Run(pa)
    ra.set_fields(*fa)
    rb = pkg.Run(pb)
    rb.set_fields(*fb)
    ra.step(3)
    rb.step(3)
    gp, gc = ra.get_fields()
    ra.close()
    rb.close()
    op, oc, _ = oracle.run(pa, fa[0], fa[1], 3, faithful=False, workers=8)
    _check_fields(gp, gc, op, oc, TOL32)
