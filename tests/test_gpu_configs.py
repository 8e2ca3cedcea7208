"""Parity at the configurations the benchmark runs (bench.py builds the same
workloads, so these tests use its own definitions):

* polycrystal 128^3, P = 16, M(c), 64 Voronoi grains from seed 1, dt = 0.1
  (the headline line): 100 steps against the plain FP64 GPU path, and 5 steps
  against the FP64 CPU oracle directly;
* the large grid 256^3, P = 32, 256 grains from seed 2, c0 = 0.4, kappa = 2:
  10 steps against the FP64 GPU path (the oracle takes minutes per step here);
* the batched ensemble (16 runs of 64^3, P = 8, per-run L, kappa, g, c0 drawn
  from ran_2 seed 3): batched equals alone bit for bit, and every run matches
  the oracle;
* the mass of c over 1000 steps: the k = 0 coefficient of c never changes,
  and the compensated sum of the cell values stays at N^3 Re c_hat(0) to the
  FP32 rounding of those values.

Tolerance: max-abs and L2 error of every field relative to the reference's
max-abs / L2 norm <= 1e-5 (FP32 path); diagnostics <= 1e-5 relative.  The
plain FP64 GPU path is itself held to the oracle at 1e-10
(test_gpu_parity.py::test_fp64_plain_vs_oracle).
"""
import numpy as np
import pytest

import bench
from test_gpu_parity import TOL32, _check_diag, _check_fields, _l2, _rel, _run_lib

pytestmark = pytest.mark.gpu

# The mass is the compensated FP64 sum of the FP32 cell values the x pass
# sees; those values carry the rounding of the inverse transforms, which for a
# field close to a constant leans the same way in most cells (up to half an
# FP32 ulp of c each: 3e-8 relative at c = 0.4).  Measured on the GB300:
# 3e-8 to 7e-8 against the FP64 path and against N^3 Re c_hat(0).
MASS_TOL = 2e-7


def _workload(name):
    bench.select_workload(name)
    try:
        return bench.params(), dict(bench.IC)
    finally:
        bench.select_workload("polycrystal")


def _start(pkg, p, ic, seed=None):
    return pkg.ic_voronoi(p, ic["seed"] if seed is None else seed, ic["n_grains"], ic["amp_phi"], ic["c0"],
                          ic["amp_c"])


def _check_records(gd, hd, tol):
    for a, b in zip(gd, hd):
        assert a["step"] == b["step"] and a["nonfinite"] == 0
        for k in ("f_int", "f_eta", "f_ch", "c_min", "c_max", "phi_min", "phi_P_max"):
            assert abs(a[k] - b[k]) <= tol * max(1.0, abs(b[k])), (a["step"], k, a[k], b[k])
        assert abs(a["mass"] - b["mass"]) <= MASS_TOL * abs(b["mass"]), (a["step"], a["mass"], b["mass"])


def test_polycrystal_128_P16_vs_fp64_path_100_steps(pkg):
    p, ic = _workload("polycrystal")
    assert (p.Nx, p.var, p.mobility, p.t_step) == (128, 16, "c1mc", 0.1)
    phi, con = _start(pkg, p, ic)
    gp, gc, gd = _run_lib(pkg, p, phi, con, 100)
    hp, hc, hd = _run_lib(pkg, p, phi, con, 100, precision=64)
    errs = dict(phi_max=_rel(gp, hp), phi_l2=_l2(gp, hp), c_max=_rel(gc, hc), c_l2=_l2(gc, hc))
    print("polycrystal 128^3 x 16, 100 steps vs FP64 path:", {k: f"{v:.2e}" for k, v in errs.items()})
    _check_fields(gp, gc, hp, hc, TOL32)
    _check_records(gd, hd, TOL32)


def test_polycrystal_128_P16_vs_oracle_5_steps(pkg, oracle):
    p, ic = _workload("polycrystal")
    phi, con = _start(pkg, p, ic)
    op_ = oracle.Params(**bench.WORKLOAD)
    gp, gc, gd = _run_lib(pkg, p, phi, con, 5)
    o_phi, o_con, od = oracle.run(op_, phi, con, 5, faithful=False, workers=16)
    _check_fields(gp, gc, o_phi, o_con, TOL32)
    _check_diag(gd, od, TOL32, oracle.stats(phi, con))


def test_large_256_P32_vs_fp64_path_10_steps(pkg):
    p, ic = _workload("large")
    assert (p.Nx, p.var, p.grad_coeff_phi, ic["n_grains"], ic["c0"]) == (256, 32, 2.0, 256, 0.4)
    phi, con = _start(pkg, p, ic)
    gp, gc, gd = _run_lib(pkg, p, phi, con, 10)
    hp, hc, hd = _run_lib(pkg, p, phi, con, 10, precision=64)
    _check_fields(gp, gc, hp, hc, TOL32)
    _check_records(gd, hd, TOL32)


def test_ensemble_batch_equals_alone_and_oracle(pkg, oracle):
    reqs = bench.ensemble_requests(pkg, 16)
    starts = [pkg.ic_noise(p, seed, 0.001, c0, 0.01) for p, seed, c0 in reqs]
    b = pkg.Batch([r[0] for r in reqs])
    try:
        for i, (phi, con) in enumerate(starts):
            b.set_fields(i, phi, con)
        steps = 5
        bd = b.step(steps)
        fields = [b.get_fields(i) for i in range(len(reqs))]
    finally:
        b.close()
    for i, (p, _, _) in enumerate(reqs):
        gp, gc = fields[i]
        sp, sc, sd = _run_lib(pkg, p, starts[i][0], starts[i][1], steps)
        assert np.array_equal(gp, sp) and np.array_equal(gc, sc), f"run {i}: batched differs from alone"
        assert [d["f_int"] for d in bd[i]] == [d["f_int"] for d in sd]
        assert [d["mass"] for d in bd[i]] == [d["mass"] for d in sd]
        op_ = oracle.Params(**{k: getattr(p, k) for k in vars(oracle.Params(1, 1, 1, 1))})
        o_phi, o_con, od = oracle.run(op_, starts[i][0], starts[i][1], steps, faithful=False, workers=8)
        _check_fields(gp, gc, o_phi, o_con, TOL32)
        _check_diag(bd[i], od, TOL32, oracle.stats(*starts[i]))


@pytest.mark.parametrize("workload", ["noise64", "polycrystal"])
def test_mass_is_the_k0_coefficient_over_1000_steps(pkg, oracle, workload):
    """The update never touches the k = 0 coefficient of c, so the mass
    N^3 Re c_hat(0) is constant bit for bit; the recorded mass (a compensated
    FP64 sum of the FP32 cell values the x pass sees) follows it up to the
    FP32 rounding of the inverse transforms, and its first value is the exact
    sum of the FP32 cell values."""
    if workload == "noise64":
        p = oracle.Params(64, 64, 64, 4, t_step=0.05)
        phi, con = oracle.ic_noise(p, 0, 0.001, 0.5, 0.01)
    else:
        p, ic = _workload("polycrystal")
        phi, con = _start(pkg, p, ic)
    n3 = p.Nx * p.Ny * p.Nz
    run = pkg.Run(p)
    try:
        run.set_fields(phi, con)
        k0 = run.c_mean()
        gd = run.step(1000)
        k1 = run.c_mean()
    finally:
        run.close()
    assert k0 == k1, (k0, k1)
    ref = n3 * k0.real
    dev = max(abs(d["mass"] - ref) for d in gd) / abs(ref)
    drift = max(abs(d["mass"] - gd[0]["mass"]) for d in gd) / abs(ref)
    exact = float(np.sum(con.astype(np.float32).astype(np.float64), dtype=np.float64))
    print(f"{workload}: |mass - N^3 Re c_hat(0)| <= {dev:.2e}, drift {drift:.2e}, "
          f"start vs sum of the FP32 start values {abs(gd[0]['mass'] - exact) / abs(exact):.2e}")
    assert dev < MASS_TOL and drift < MASS_TOL
    # the x pass sees c after one FP32 round trip through the transforms
    assert abs(gd[0]["mass"] - exact) <= 2e-8 * abs(exact)
