"""Pins of the CPU oracle (no GPU).

The reference ships no tests, fixtures or golden vectors for this path, and
its Fortran (P3DFFT/FFTW/MPI) cannot be built here, so the oracle is pinned by
known answers of the discretised equations, by invariants, by the committed
regression fixtures in tests/golden/ and by a second, independent restatement
of ran_2 (the library's C code).
"""
import math

import numpy as np
import pytest


def test_ran2_am_constant(oracle):
    # am = 1./im1 in REAL*4: 2^-31 (1 + 2^-23)
    assert oracle.Ran2.AM == 2.0 ** -31 * (1 + 2.0 ** -23)
    assert abs(oracle.Ran2.AM - 4.6566134e-10) < 1e-16


def test_ran2_python_vs_c(oracle, pkg):
    for idum0 in (-1, -2, -12345, 0, 7):
        a = oracle.Ran2()
        b = pkg.Ran2(idum0)
        ia = idum0
        for _ in range(2000):
            va, ia = a(ia)
            vb = b.next()
            assert va == vb
        assert ia == b.idum.value


def test_ran2_range_and_seed_mapping(oracle):
    s0 = oracle.Ran2Stream(0).take(1000)
    s1 = oracle.Ran2Stream(1).take(1000)
    ref = oracle.Ran2Stream(idum=-1).take(1000)
    assert np.array_equal(s0, ref)  # seed 0 == reference default iseed = -1
    assert not np.array_equal(s0, s1)
    assert s0.min() > 0 and s0.max() < 1


def test_k_space_tables(oracle):
    q, qn = oracle.axis_wavenumbers(8)
    pi = math.atan(1.0) * 4
    assert np.allclose(q, [0, 1, 2, 3, 4, -3, -2, -1] * (np.ones(8) * 2 * pi / 8))
    assert qn[4] == 0 and q[4] != 0  # kf zeroed at Nyquist, kf_sq is not
    G, K2, K3, K4 = oracle.k_space(8, 6, 4)
    assert G.shape == (4, 6, 5)
    assert np.all(G.real == 0) and np.all(K3.real == 0)
    # K4 = sum q^4 (not |q|^4)
    qx, _ = oracle.axis_wavenumbers(8, half=True)
    qy, _ = oracle.axis_wavenumbers(6)
    qz, _ = oracle.axis_wavenumbers(4)
    assert np.isclose(K4[1, 2, 3], qx[3] ** 4 + qy[2] ** 4 + qz[1] ** 4)
    assert np.isclose(K2[1, 2, 3], -(qx[3] ** 2 + qy[2] ** 2 + qz[1] ** 2))


def test_fft_normalisation(oracle):
    p = oracle.Params(8, 6, 4, 1)
    o = oracle.Oracle(p, np.zeros((1, 4, 6, 8)), np.zeros((4, 6, 8)))
    u = np.random.default_rng(1).standard_normal((4, 6, 8))
    uh = o.F(u)
    assert np.isclose(uh[0, 0, 0], u.mean())  # f_trans divides by Nx*Ny*Nz
    assert np.allclose(o.Finv(uh), u)  # inv_trans is un-normalised


def _mode(shape, kx=1, ky=2, kz=1):
    Nz, Ny, Nx = shape
    z, y, x = np.meshgrid(np.arange(Nz), np.arange(Ny), np.arange(Nx), indexing="ij")
    return np.cos(2 * np.pi * (kx * x / Nx + ky * y / Ny + kz * z / Nz))


def test_known_answer_ch_mode_decay(oracle):
    """am = ap = 0, constant mobility: each Fourier mode of c is divided by
    1 + D dt kappa_c K4 per step (src/var_diff.f90:976-983), exactly."""
    p = oracle.Params(16, 8, 8, 1, t_step=0.3, grad_coeff_c=1.7, D_L=0.9)
    shape = p.shape
    eps = 0.01
    con = 0.5 + eps * _mode(shape, 2, 1, 3)
    phi = np.full((1,) + shape, 0.3)
    o = oracle.Oracle(p, phi, con)
    q = lambda m, n: 2 * np.pi * ((m if m <= n // 2 else m - n)) / n
    K4 = q(2, 16) ** 4 + q(1, 8) ** 4 + q(3, 8) ** 4
    fac = 1.0 / (1 + p.D_L * p.t_step * p.grad_coeff_c * K4)
    for n in range(1, 6):
        o.step()
        assert np.allclose(o.con - 0.5, eps * fac ** n * _mode(shape, 2, 1, 3), atol=1e-14)


def test_known_answer_ac_mode_growth(oracle):
    """One order parameter, am = ap = 0: for |phi| << 1 the Allen-Cahn update
    multiplies a Fourier mode by (1 + L dt) / (1 + L kappa dt |q|^2)
    (src/var_diff.f90:1015-1024); the cubic term adds O(eps^2) relative."""
    p = oracle.Params(8, 16, 8, 1, t_step=0.05, mob_phi=1.3, grad_coeff_phi=0.7)
    eps = 1e-6
    phi = eps * _mode(p.shape, 1, 3, 2)[None]
    o = oracle.Oracle(p, phi, np.full(p.shape, 0.5))
    q = lambda m, n: 2 * np.pi * ((m if m <= n // 2 else m - n)) / n
    qq = q(1, 8) ** 2 + q(3, 16) ** 2 + q(2, 8) ** 2
    fac = (1 + p.mob_phi * p.t_step) / (1 + p.mob_phi * p.grad_coeff_phi * p.t_step * qq)
    for n in range(1, 6):
        o.step()
        assert np.allclose(o.phi[0], eps * fac ** n * _mode(p.shape, 1, 3, 2), rtol=0, atol=1e-9 * eps)


def test_mass_conservation(oracle):
    p = oracle.Params(16, 16, 16, 3, t_step=0.01, D_gb=1.0, am=0.5, ap=2.0, con_0_mat=0.3, con_0_ppt=0.7)
    phi, con = oracle.ic_voronoi(p, 3, 5, 0.05, 0.5, 0.02)
    m0 = con.sum()
    _, c, d = oracle.run(p, phi, con, 10)
    assert abs(c.sum() - m0) / m0 < 1e-12
    assert abs(d[-1].mass - m0) / m0 < 1e-12


@pytest.mark.parametrize("mob,dgb", [("reference", 0.0), ("reference", 1.0), ("c1mc", 0.0)])
def test_faithful_equals_fast(oracle, mob, dgb):
    p = oracle.Params(16, 8, 16, 3, t_step=0.01, D_gb=dgb, am=0.5, ap=2.0, con_0_mat=0.3, con_0_ppt=0.7,
                      mobility=mob)
    phi, con = oracle.ic_voronoi(p, 9, 4, 0.05, 0.5, 0.02)
    a = oracle.run(p, phi, con, 5, faithful=True)
    b = oracle.run(p, phi, con, 5, faithful=False)
    assert np.allclose(a[0], b[0], rtol=0, atol=1e-12)
    assert np.allclose(a[1], b[1], rtol=0, atol=1e-12)
    for x, y in zip(a[2], b[2]):
        assert math.isclose(x.f_int, y.f_int, rel_tol=1e-11)


def test_stats_clamps(oracle):
    # reference start values 1.0 / 0.0 act as clamps (src/var_diff.f90:1076-1080)
    phi = np.full((2, 2, 2, 2), -0.5)
    con = np.full((2, 2, 2), 3.0)
    s = oracle.stats(phi, con)
    assert s["phi_P_max"] == 0.0 and s["c_min"] == 1.0 and s["c_max"] == 3.0 and s["phi_min"] == 0.5


def test_fortran_layout_roundtrip(oracle):
    phi = np.random.default_rng(2).standard_normal((3, 4, 5, 6))
    buf = oracle.to_fortran_aos(phi)
    # phi(var, x, y, z): element (ivar=1, x=2, y=3, z=1) sits at ivar + var*(x + Nx*(y + Ny*z))
    assert buf[1 + 3 * (2 + 6 * (3 + 5 * 1))] == phi[1, 1, 3, 2]
    assert np.array_equal(oracle.from_fortran_aos(buf, 3, 6, 5, 4), phi)


def test_gamma_matrix(oracle):
    g = oracle.gamma_matrix(4, 6.0, 3.0)
    assert np.array_equal(np.diag(g), np.zeros(4))
    assert g[0, 1] == 6.0 and g[0, 3] == 3.0 and g[3, 2] == 3.0 and np.array_equal(g, g.T)


def test_circle_ic_shape(oracle):
    p = oracle.Params(24, 24, 24, 3)
    phi, con, idum = oracle.ic_circle(p, grn_rad=6, ppt_rad=(2, 2, 2), num_ppt=3, iseed=-1, c_mat=0.3,
                                      con_0_ppt=0.7)
    assert np.all(np.isin(phi, (0.0, 1.0)))
    assert np.all(phi.sum(axis=0) == 1.0)
    assert phi[1, 12, 12, 12] in (0.0, 1.0)
    assert (phi[2] == 1).sum() > 0 and np.all(con[phi[2] == 1] == 0.7)


@pytest.mark.parametrize("name", ["noise_const_16", "voronoi_refvar_16", "voronoi_c1mc_16"])
def test_oracle_regression_fixtures(oracle, name):
    import importlib.util
    from pathlib import Path

    here = Path(__file__).resolve().parent / "golden"
    spec = importlib.util.spec_from_file_location("make_golden", here / "make_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    ref = np.load(here / f"{name}.npz")
    ph, c, diag = mg.compute(mg.CASES[name])
    assert np.allclose(ph, ref["phi"], rtol=0, atol=1e-12)
    assert np.allclose(c, ref["con"], rtol=0, atol=1e-12)
    assert np.allclose(diag, ref["diag"], rtol=1e-10, atol=1e-14)
