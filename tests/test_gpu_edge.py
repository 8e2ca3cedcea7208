"""Edge cases of the fused step on the GPU: one and two order parameters,
dt = 0, non-finite input, cells whose order parameters are tiny (the
rescaled h = N4/S4 branch) or all zero (0/0 in the reference), and the largest
number of order parameters a grid allows, against the oracle or the FP64 GPU
path."""
import numpy as np
import pytest

from test_gpu_parity import TOL32, _check_diag, _check_fields, _rel, _run_lib

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("var,mob", [(1, "reference"), (2, "c1mc"), (1, "c1mc")])
def test_few_order_parameters(pkg, oracle, var, mob):
    # the explicit variable-mobility term bounds dt (larger dt grows without bound in FP64 too)
    p = oracle.Params(32, 32, 32, var, t_step=0.002 if mob == "reference" else 0.01, am=0.5, ap=2.0,
                      con_0_mat=0.3, con_0_ppt=0.7, mobility=mob, D_gb=0.5 if mob == "reference" else 0.0)
    rng = np.random.default_rng(var)
    phi = 0.5 + 0.3 * (rng.random((var,) + p.shape) - 0.5)
    con = 0.5 + 0.02 * (rng.random(p.shape) - 0.5)
    gp, gc, gd = _run_lib(pkg, p, phi, con, 20)
    op, oc, od = oracle.run(p, phi, con, 20, faithful=False, workers=8)
    _check_fields(gp, gc, op, oc, TOL32)
    _check_diag(gd, od, TOL32, oracle.stats(phi, con))


def test_zero_time_step_keeps_the_fields(pkg, oracle):
    p = oracle.Params(64, 64, 64, 4, t_step=0.0, mobility="c1mc", am=0.5, ap=2.0, con_0_mat=0.3, con_0_ppt=0.7)
    phi, con = oracle.ic_voronoi(p, 3, 7, 0.02, 0.5, 0.02)
    gp, gc, _ = _run_lib(pkg, p, phi, con, 3)
    assert _rel(gp, phi) < 1e-6 and _rel(gc, con) < 1e-6


def test_non_finite_input_is_reported_and_the_run_recovers(pkg, oracle):
    p = oracle.Params(32, 32, 32, 3, t_step=0.01)
    phi, con = oracle.ic_noise(p, 4, 0.01, 0.5, 0.01)
    bad = phi.copy()
    bad[1, 5, 6, 7] = np.nan
    run = pkg.Run(p)
    try:
        run.set_fields(bad, con)
        with pytest.raises(pkg.PFError) as e:
            run.step(2)
        assert e.value.code == pkg.PF_ENONFINITE
        recs = run.step(1, raise_nonfinite=False)
        assert recs[0]["nonfinite"] != 0
        run.set_fields(phi, con)  # a fresh start on the same run
        d = run.step(5)
        assert all(r["nonfinite"] == 0 for r in d)
        gp, gc = run.get_fields()
    finally:
        run.close()
    op, oc, _ = oracle.run(p, phi, con, 5, faithful=False)
    _check_fields(gp, gc, op, oc, TOL32)


def test_tiny_order_parameters_take_the_rescaled_branch(pkg, oracle):
    """|phi| ~ 1e-9 makes S4 = sum phi^4 ~ 1e-36, below FP32's normal range;
    the kernel rescales by 1/max|phi| and must still match the FP64 oracle."""
    p = oracle.Params(32, 32, 32, 3, t_step=1e-16, am=0.5, ap=2.0, con_0_mat=0.3, con_0_ppt=0.7)
    rng = np.random.default_rng(11)
    phi = 1e-9 * (0.5 + rng.random((3,) + p.shape))
    con = 0.5 + 0.02 * (rng.random(p.shape) - 0.5)
    gp, gc, gd = _run_lib(pkg, p, phi, con, 1)
    op, oc, od = oracle.run(p, phi, con, 1, faithful=False)
    assert np.all(np.isfinite(op))  # the oracle's FP64 does not need the rescaling
    _check_fields(gp, gc, op, oc, 1e-4)
    assert abs(gd[0]["f_ch"] - od[0].f_ch) <= 1e-5 * abs(od[0].f_ch)


def test_all_zero_order_parameters(pkg, oracle):
    """Where every phi_i is 0, the reference's h = N4/S4 is 0/0 (NaN, and so
    is the oracle's); the library takes h = 0 and term4 = 0 there, so f_ch is
    the sum of ap (c - c0p)^2 and the step stays finite.  A documented
    deviation from the reference."""
    p = oracle.Params(16, 16, 16, 3, t_step=0.01, am=0.5, ap=2.0, con_0_mat=0.3, con_0_ppt=0.7)
    phi = np.zeros((3,) + p.shape)
    rng = np.random.default_rng(2)
    con = 0.5 + 0.02 * (rng.random(p.shape) - 0.5)
    gp, gc, gd = _run_lib(pkg, p, phi, con, 1)
    assert np.all(np.isfinite(gp)) and np.all(np.isfinite(gc)) and gd[0]["nonfinite"] == 0
    want = float(np.sum(p.ap * (con - p.con_0_ppt) ** 2))
    assert abs(gd[0]["f_ch"] - want) <= 1e-5 * want
    _, oc, od = oracle.run(p, phi, con, 1, faithful=False)
    assert np.isnan(od[0].f_ch)


def test_largest_var_for_the_grid(pkg, oracle):
    """150 order parameters on 32^3 (the x pass holds 151 field rows of 8 y
    rows in shared memory): fused path against the FP64 path."""
    p = oracle.Params(32, 32, 32, 150, t_step=0.01, am=0.5, ap=2.0, con_0_mat=0.3, con_0_ppt=0.7, mobility="c1mc")
    assert pkg.load_library().pf_supported_shape(32, 32, 32, 150, 32) == 1
    phi, con = oracle.ic_voronoi(p, 5, 200, 0.02, 0.5, 0.02)
    gp, gc, gd = _run_lib(pkg, p, phi, con, 3)
    hp, hc, hd = _run_lib(pkg, p, phi, con, 3, precision=64)
    _check_fields(gp, gc, hp, hc, TOL32)
    for a, b in zip(gd, hd):
        for k in ("f_int", "f_eta", "f_ch"):
            assert abs(a[k] - b[k]) <= TOL32 * max(1.0, abs(b[k])), (k, a[k], b[k])
