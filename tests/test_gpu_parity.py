"""Parity of the CUDA library against the FP64 CPU oracle (runs on the GPU).

Tolerances
----------
* fused FP32 path: max-abs and L2 error of every field, relative to the
  oracle's max-abs / L2 norm, <= 1e-5 after 100 steps (the stated target);
  shorter runs use the same bound;
* plain FP64 path: <= 1e-10 relative;
* diagnostics (f_int, f_eta, f_ch): <= 1e-5 relative (FP32), 1e-9 (FP64).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL32 = 1e-5
TOL64 = 1e-10


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def _check_fields(gp, gc, op, oc, tol):
    assert _rel(gp, op) < tol, f"phi max rel err {_rel(gp, op):.3e}"
    assert _l2(gp, op) < tol, f"phi l2 rel err {_l2(gp, op):.3e}"
    assert _rel(gc, oc) < tol, f"con max rel err {_rel(gc, oc):.3e}"
    assert _l2(gc, oc) < tol, f"con l2 rel err {_l2(gc, oc):.3e}"


def _check_diag(gd, od, tol, initial_stats):
    """gd: library records (fields at the start of each step); od: oracle
    Diag (energies at the start, statistics at the end of each step)."""
    for t in range(len(gd)):
        for k in ("f_int", "f_eta", "f_ch"):
            ref = getattr(od[t], k)
            scale = max(abs(ref), 1e-30)
            if ref == 0.0:
                assert abs(gd[t][k]) < 1e-12, (t, k, gd[t][k])
            else:
                assert abs(gd[t][k] - ref) / scale < tol, (t, k, gd[t][k], ref)
        prev = initial_stats if t == 0 else dict(c_min=od[t - 1].c_min, c_max=od[t - 1].c_max,
                                                   phi_min=od[t - 1].phi_min, phi_P_max=od[t - 1].phi_P_max)
        for k in ("c_min", "c_max", "phi_P_max"):
            assert abs(gd[t][k] - prev[k]) <= tol * max(1.0, abs(prev[k])), (t, k, gd[t][k], prev[k])
        assert abs(gd[t]["phi_min"] - prev["phi_min"]) <= tol * max(1e-3, abs(prev["phi_min"])) + 1e-7, t


def _run_lib(pkg, p, phi, con, steps, precision=32):
    run = pkg.Run(p, precision=precision)
    run.set_fields(phi, con)
    d = run.step(steps)
    gp, gc = run.get_fields()
    run.close()
    return gp, gc, d


# Parameter sets are kept inside the stable range of the explicit chemical and
# variable-mobility terms (larger dt blows up in FP64 too); noise starts are
# used only with am = ap = 0, where term4 is identically zero.
CASES = {
    # name: (params kwargs, ic, steps)
    "c0_noise_32": (dict(Nx=32, Ny=32, Nz=32, var=4, t_step=0.05), ("noise", 0, 0.001, 0.5, 0.01), 100),
    "chem_refvar_32": (dict(Nx=32, Ny=32, Nz=32, var=3, t_step=0.002, D_gb=1.0, am=0.5, ap=2.0, con_0_mat=0.3,
                            con_0_ppt=0.7, sigma_1=6.0, sigma_2=3.0), ("voronoi", 3, 5, 0.05, 0.5, 0.02), 50),
    "c1mc_32": (dict(Nx=32, Ny=32, Nz=32, var=4, t_step=0.1, mobility="c1mc"), ("voronoi", 1, 6, 0.01, 0.5, 0.02),
                50),
    "noncubic_64x32x64": (dict(Nx=64, Ny=32, Nz=64, var=2, t_step=0.005, am=0.5, ap=2.0, con_0_mat=0.3,
                               con_0_ppt=0.7), ("voronoi", 5, 4, 0.05, 0.5, 0.01), 30),
    "noncubic_16x32x16": (dict(Nx=16, Ny=32, Nz=16, var=3, t_step=0.005, D_gb=0.5), ("noise", 6, 0.05, 0.5, 0.01),
                          30),
    "cube16": (dict(Nx=16, Ny=16, Nz=16, var=5, t_step=0.05, mobility="c1mc"), ("voronoi", 7, 4, 0.01, 0.4, 0.02),
               40),
}


def _make(oracle, kw, ic):
    p = oracle.Params(**kw)
    if ic[0] == "noise":
        phi, con = oracle.ic_noise(p, ic[1], ic[2], ic[3], ic[4])
    else:
        phi, con = oracle.ic_voronoi(p, ic[1], ic[2], ic[3], ic[4], ic[5])
    return p, phi, con


@pytest.mark.parametrize("name", list(CASES))
def test_fp32_fused_vs_oracle(pkg, oracle, name):
    kw, ic, steps = CASES[name]
    p, phi, con = _make(oracle, kw, ic)
    gp, gc, gd = _run_lib(pkg, p, phi, con, steps)
    op, oc, od = oracle.run(p, phi, con, steps, faithful=False, workers=4)
    _check_fields(gp, gc, op, oc, TOL32)
    _check_diag(gd, od, TOL32, oracle.stats(phi, con))


def test_fp32_config0_64cube_100_steps(pkg, oracle):
    """The 64^3, var=4 noise case (seed 0, dt 0.05) at the 100-step parity horizon."""
    p = oracle.Params(64, 64, 64, 4, t_step=0.05)
    phi, con = oracle.ic_noise(p, 0, 0.001, 0.5, 0.01)
    gp, gc, gd = _run_lib(pkg, p, phi, con, 100)
    op, oc, od = oracle.run(p, phi, con, 100, faithful=False, workers=8)
    _check_fields(gp, gc, op, oc, TOL32)
    _check_diag(gd, od, TOL32, oracle.stats(phi, con))
    # mass: sum of c at the start of every step is conserved to FP32 round-off
    m0 = gd[0]["mass"]
    assert max(abs(d["mass"] - m0) for d in gd) / abs(m0) < 1e-6


def test_fp32_128cube_cluster(pkg, oracle):
    p = oracle.Params(128, 128, 128, 2, t_step=0.02, mobility="c1mc", am=0.5, ap=2.0, con_0_mat=0.3, con_0_ppt=0.7)
    phi, con = oracle.ic_voronoi(p, 1, 8, 0.01, 0.5, 0.02)
    gp, gc, gd = _run_lib(pkg, p, phi, con, 6)
    op, oc, od = oracle.run(p, phi, con, 6, faithful=False, workers=8)
    _check_fields(gp, gc, op, oc, TOL32)
    _check_diag(gd, od, TOL32, oracle.stats(phi, con))


def test_fp32_256cube_cluster(pkg, oracle):
    p = oracle.Params(256, 256, 256, 2, t_step=0.02, am=0.5, ap=2.0, con_0_mat=0.3, con_0_ppt=0.7)
    phi, con = oracle.ic_voronoi(p, 2, 6, 0.01, 0.4, 0.02)
    gp, gc, gd = _run_lib(pkg, p, phi, con, 2)
    op, oc, od = oracle.run(p, phi, con, 2, faithful=False, workers=8)
    _check_fields(gp, gc, op, oc, TOL32)


def test_fp32_96cube_reference_grid(pkg, oracle):
    """The reference's own grid (96^3, inputs/config.yaml) with variable mobility."""
    p = oracle.Params(96, 96, 96, 8, t_step=0.005, D_gb=0.5, am=0.5, ap=2.0, con_0_mat=0.3, con_0_ppt=0.7)
    phi, con = oracle.ic_voronoi(p, 8, 12, 0.02, 0.4, 0.02)
    gp, gc, gd = _run_lib(pkg, p, phi, con, 20)
    op, oc, od = oracle.run(p, phi, con, 20, faithful=False, workers=8)
    _check_fields(gp, gc, op, oc, TOL32)
    _check_diag(gd, od, TOL32, oracle.stats(phi, con))


def test_fp32_many_order_parameters(pkg, oracle):
    """var = 55 (the reference's baseline configuration) on a 32^3 grid."""
    p = oracle.Params(32, 32, 32, 55, t_step=0.005, D_gb=1.0, am=0.5, ap=5.0, con_0_mat=0.1, con_0_ppt=1.0)
    phi, con = oracle.ic_voronoi(p, 9, 40, 0.02, 0.5, 0.02)
    gp, gc, gd = _run_lib(pkg, p, phi, con, 10)
    op, oc, od = oracle.run(p, phi, con, 10, faithful=False, workers=8)
    _check_fields(gp, gc, op, oc, TOL32)
    _check_diag(gd, od, TOL32, oracle.stats(phi, con))


def test_fp32_vs_fp64_reference_baseline_config(pkg, oracle):
    """inputs/config.yaml's baseline (96^3, var = 55, am 0.5, ap 5, c0 0.1/1,
    D_gb 1, dt 1e-4) on both GPU paths: the fused FP32 path against the FP64
    cuFFT path over 20 steps."""
    p = oracle.Params(96, 96, 96, 55, t_step=1e-4, D_gb=1.0, am=0.5, ap=5.0, con_0_mat=0.1, con_0_ppt=1.0)
    phi, con = oracle.ic_voronoi(p, 11, 64, 0.02, 0.5, 0.02)
    gp, gc, gd = _run_lib(pkg, p, phi, con, 20)
    hp, hc, hd = _run_lib(pkg, p, phi, con, 20, precision=64)
    _check_fields(gp, gc, hp, hc, TOL32)
    for a, b in zip(gd, hd):
        for k in ("f_int", "f_eta", "f_ch", "c_min", "c_max", "phi_min", "phi_P_max"):
            assert abs(a[k] - b[k]) <= TOL32 * max(1.0, abs(b[k])), (a["step"], k, a[k], b[k])


@pytest.mark.parametrize("mob", ["reference", "c1mc"])
def test_fp64_plain_vs_oracle(pkg, oracle, mob):
    p = oracle.Params(16, 16, 16, 3, t_step=0.01, D_gb=1.0, am=0.5, ap=2.0, con_0_mat=0.3, con_0_ppt=0.7,
                      sigma_1=6.0, sigma_2=3.0, mobility=mob)
    phi, con = oracle.ic_voronoi(p, 3, 5, 0.05, 0.5, 0.02)
    gp, gc, gd = _run_lib(pkg, p, phi, con, 10, precision=64)
    op, oc, od = oracle.run(p, phi, con, 10, faithful=True)
    _check_fields(gp, gc, op, oc, TOL64)
    _check_diag(gd, od, 1e-9, oracle.stats(phi, con))


def test_batch_equals_single(pkg, oracle):
    """Runs stepped together give the same numbers as each run alone."""
    ps, ics = [], []
    for i, (L, kap, g, c0) in enumerate([(0.3, 0.8, 1.2, 0.35), (2.0, 2.5, 1.8, 0.6), (7.0, 1.0, 1.5, 0.5)]):
        p = oracle.Params(32, 32, 32, 3, t_step=0.05, mob_phi=L, grad_coeff_phi=kap, grad_coeff_c=kap,
                          sigma_1=g, sigma_2=g)
        ps.append(p)
        ics.append(oracle.ic_noise(p, 10 + i, 0.001, c0, 0.01))
    b = pkg.Batch(ps)
    for i, (phi, con) in enumerate(ics):
        b.set_fields(i, phi, con)
    bd = b.step(20)
    for i, p in enumerate(ps):
        gp, gc = b.get_fields(i)
        sp, sc, sd = _run_lib(pkg, p, ics[i][0], ics[i][1], 20)
        assert np.array_equal(gp, sp) and np.array_equal(gc, sc), f"run {i} differs alone vs batched"
        assert [d["f_eta"] for d in bd[i]] == [d["f_eta"] for d in sd]
        op, oc, od = oracle.run(p, ics[i][0], ics[i][1], 20, faithful=False)
        _check_fields(gp, gc, op, oc, TOL32)
    b.close()


def test_set_get_roundtrip(pkg, oracle):
    p = oracle.Params(64, 64, 64, 3)
    phi, con = oracle.ic_voronoi(p, 4, 7, 0.01, 0.5, 0.02)
    run = pkg.Run(p)
    run.set_fields(phi, con)
    gp, gc = run.get_fields()
    run.close()
    assert _rel(gp, phi) < 1e-6 and _rel(gc, con) < 1e-6


def test_fortran_shims(lib, oracle):
    import ctypes as C

    Nx, Ny, Nz = 32, 16, 8
    rng = np.random.default_rng(0)
    u = rng.standard_normal((Nz, Ny, Nx))
    ist = (C.c_int * 3)(1, 1, 1)
    ien = (C.c_int * 3)(Nx, Ny, Nz)
    fst = (C.c_int * 3)(1, 1, 1)
    fen = (C.c_int * 3)(Nz, Ny, Nx // 2 + 1)
    out = np.zeros((Nx // 2 + 1, Ny, Nz, 2))
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    ci = lambda v: C.byref(C.c_int(v))
    lib.f_trans_(dp(u), dp(out), ci(Nx), ci(Ny), ci(Nz), ist, ien, fst, fen)
    ref = np.fft.rfftn(u, axes=(0, 1, 2)) / (Nx * Ny * Nz)  # [z][y][kx]
    got = (out[..., 0] + 1j * out[..., 1]).transpose(2, 1, 0)
    assert np.max(np.abs(got - ref)) < 1e-14
    back = np.zeros((Nz, Ny, Nx))
    lib.inv_trans_(dp(out), dp(back), ist, ien, fst, fen)
    assert np.max(np.abs(back - u)) < 1e-12


@pytest.mark.parametrize("name", ["noise_const_16", "voronoi_refvar_16", "voronoi_c1mc_16"])
def test_fp32_fused_vs_golden_fixture(pkg, name):
    """The CUDA path against the committed oracle fixtures (starts regenerated
    by the library's own seeded generators)."""
    import json
    from pathlib import Path
    from types import SimpleNamespace

    ref = np.load(Path(__file__).resolve().parent / "golden" / f"{name}.npz")
    meta = json.loads(str(ref["meta"]))
    case = meta["case"]
    base = dict(t_step=0.05, grad_coeff_phi=1.0, grad_coeff_c=1.0, D_S=1.0, D_L=1.0, D_gb=0.0, mob_phi=1.0,
                sigma_1=1.5, sigma_2=1.5, am=0.0, ap=0.0, con_0_mat=0.0, con_0_ppt=1.0, mobility="reference")
    base.update(case["params"])
    p = SimpleNamespace(**base)
    ic = case["ic"]
    phi, con = (pkg.ic_noise(p, *ic[1:]) if ic[0] == "noise" else pkg.ic_voronoi(p, *ic[1:]))
    gp, gc, gd = _run_lib(pkg, p, phi, con, case["steps"])
    _check_fields(gp, gc, ref["phi"], ref["con"], TOL32)
    keys = meta["diag_keys"]
    for t in range(case["steps"]):
        for k in ("f_int", "f_eta", "f_ch"):
            r = ref["diag"][t][keys.index(k)]
            if r != 0:
                assert abs(gd[t][k] - r) / abs(r) < TOL32, (t, k)
