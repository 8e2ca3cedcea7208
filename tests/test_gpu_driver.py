"""pf_var_diff (the var_diff.x drop-in) end to end on the GPU, against the
oracle driven through the same protocol: the 'circle' and 'polycryst'
starts, precipitates inserted at step ppt_int, summary.dat records on even
steps (statistics lagged by one step), data_save files every ifreq steps, and
a restart from data_rerun.0001.

Precipitates are inserted into a polycrystal without precipitates, as the
reference's runs do: once phi_var has gone through a transform it is no
longer exactly zero anywhere, and the insertion's test "phi_var > 0 in the
sphere" then rejects every position."""
import shutil
import subprocess

import numpy as np
import pytest

from test_io import HEADER_SUMMARY, HEADER_TIME_STEP, canonical_input

pytestmark = pytest.mark.gpu

TOL = 2e-5  # FP32 fields against the FP64 oracle over 10 steps


def _params(oracle, **kw):
    q = dict(Nx=32, Ny=32, Nz=32, var=3, t_step=0.002, D_L=1.0, D_gb=0.5, sigma_1=1.5, sigma_2=1.5, am=0.5,
             ap=2.0, con_0_mat=0.3, con_0_ppt=0.7)
    q.update(kw)
    return oracle.Params(**q)


def _circle(oracle, p, num_ppt, grn_rad):
    gen = oracle.Ran2()
    phi, con, idum = oracle.ic_circle(p, grn_rad, (2, 2, 2), num_ppt, -1, 0.3, 0.7, gen=gen)
    return phi, con, idum, gen


def _oracle_protocol(oracle, p, start, n_step, ppt_int=0, ppt_rad=(2, 2, 2), num_ppt=0):
    phi, con, idum, gen = start
    orc = oracle.Oracle(p, phi, con, faithful=False)
    rows, fields = {}, {}
    prev = None
    for step in range(1, n_step + 1):
        if step == ppt_int:
            idum = oracle.insert_precipitates(p, orc.phi, ppt_rad, num_ppt, idum, gen)
        d = orc.step()
        if step % 2 == 0:
            rows[step] = [d.f_int, d.f_ch, d.f_eta, d.f_int + d.f_ch + d.f_eta,
                          prev.c_max, prev.c_min, prev.phi_min, prev.phi_P_max]
        prev = d
        fields[step] = (orc.phi.copy(), orc.con.copy())
    return rows, fields


def _summary(path):
    rows = {}
    for line in path.read_text().split("\n")[1:]:
        if line.strip():
            v = line.split()
            rows[int(v[0])] = [float(x) for x in v[1:]]
    return rows


def _check_rows(got, want, p):
    """Columns f_int, f_ch, f_eta, e_tot, c_max, c_min, phi_min, phi_P_max.
    f_ch (and e_tot) also get an absolute floor: the FP32 h = N4 * (1/S4) is
    within 2 ulp of 1 where phi_var = 0, so each cell adds up to
    2 eps32 ap (c - c0p)^2 <= 2 eps32 (am + ap) even where the oracle's term is 0."""
    floor = p.Nx * p.Ny * p.Nz * 2 * 1.2e-7 * (p.am + p.ap)
    assert sorted(got) == sorted(want)
    for s in want:
        for col, (g, w) in enumerate(zip(got[s], want[s])):
            tol = TOL * max(1.0, abs(w)) + 5e-7 * abs(w) + (floor if col in (1, 3) else 0.0)
            assert abs(g - w) <= tol, (s, col, got[s], want[s])


def _run(exe, inp, cwd, prefix):
    r = subprocess.run([exe, str(inp), prefix], cwd=cwd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r


def test_driver_circle_run_matches_oracle(pkg, oracle, tmp_path):
    exe = str(pkg.driver_path())
    inp = canonical_input(tmp_path / "input.txt", N_step=10, ifreq=5, ppt_int=0, num_ppt=3)
    out = tmp_path / "out"
    out.mkdir()
    r = _run(exe, inp, tmp_path, str(out) + "/")
    assert "fused FP32" in r.stdout
    p = _params(oracle)
    want_rows, want_fields = _oracle_protocol(oracle, p, _circle(oracle, p, 3, 8), 10)
    assert (out / "summary.dat").read_text().split("\n")[0] == HEADER_SUMMARY
    _check_rows(_summary(out / "summary.dat"), want_rows, p)
    ts = (out / "time_step.dat").read_text().split("\n")
    assert ts[0] == HEADER_TIME_STEP and len([x for x in ts[1:] if x.strip()]) == 10
    # run_phase_sim.py's reader: csv with ' ' and skipinitialspace, row[2] = run time
    last = [x for x in ts[1:] if x.strip()][-1].split()
    assert int(last[0]) == 10 and float(last[2]) > 0
    for step in (5, 10):
        d = out / f"step_{step:07d}"
        assert (d / "data_extract_mult.in").read_text().split() == ["32", "32", "32", "1", "3", "1", "1"]
        phi, con = pkg.read_data_save(d / "data_save.0001", p)
        wphi, wcon = want_fields[step]
        assert np.max(np.abs(phi - wphi)) < TOL and np.max(np.abs(con - wcon)) < TOL


def test_driver_polycryst_with_insertion(pkg, oracle, tmp_path):
    """'polycryst' start (grains of three variants, a slab of single-cell
    grains) and four precipitates inserted at step 5."""
    exe = str(pkg.driver_path())
    p = _params(oracle, var=4, t_step=0.005)
    rng = np.random.default_rng(11)
    lab = (oracle.voronoi_labels(p, rng.random((6, 3)) * 32.0) % 3) + 1
    lab[:8] = rng.integers(1, 4, (8, 32, 32))
    with open(tmp_path / "grains.txt", "w") as f:
        for k in range(1, 33):
            for j in range(1, 33):
                for i in range(1, 33):
                    f.write(f"{i} {j} {k} {lab[k - 1, j - 1, i - 1]}\n")
    inp = canonical_input(tmp_path / "input.txt", var=4, t_step=0.005, start="polycryst", N_step=10, ifreq=10,
                          ppt_int=5, num_ppt=4, extra="microstructure=grains.txt\n")
    _run(exe, inp, tmp_path, "")
    phi0 = np.zeros((4,) + p.shape)
    for v in range(3):
        phi0[v][lab == v + 1] = 1.0
    start = (phi0, np.full(p.shape, 0.3), -1, oracle.Ran2())
    want_rows, want = _oracle_protocol(oracle, p, start, 10, ppt_int=5, num_ppt=4)
    _check_rows(_summary(tmp_path / "summary.dat"), want_rows, p)
    phi, con = pkg.read_data_save(tmp_path / "step_0000010" / "data_save.0001", p)
    assert np.max(np.abs(phi - want[10][0])) < TOL and np.max(np.abs(con - want[10][1])) < TOL
    assert np.count_nonzero(phi[3] > 0.5) > 100


def test_driver_restart_from_data_rerun(pkg, oracle, tmp_path):
    """nrun = 2 reads data_rerun.0001 from the working directory and steps on."""
    exe = str(pkg.driver_path())
    first = tmp_path / "a"
    first.mkdir()
    inp = canonical_input(first / "input.txt", N_step=4, ifreq=4, ppt_int=0)
    r = subprocess.run([exe, str(inp), str(first) + "/"], cwd=first, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    second = tmp_path / "b"
    second.mkdir()
    shutil.copy(first / "step_0000004" / "data_save.0001", second / "data_rerun.0001")
    inp2 = canonical_input(second / "input.txt", N_step=4, ifreq=4, ppt_int=0)
    txt = inp2.read_text().replace("1 0       / nrun", "2 0       / nrun")
    inp2.write_text(txt)
    r = subprocess.run([exe, str(inp2), str(second) + "/"], cwd=second, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    p = _params(oracle)
    _, want = _oracle_protocol(oracle, p, _circle(oracle, p, 3, 8), 8)
    phi, con = pkg.read_data_save(second / "step_0000004" / "data_save.0001", p)
    assert np.max(np.abs(phi - want[8][0])) < TOL and np.max(np.abs(con - want[8][1])) < TOL


def test_driver_fp64_path_for_other_grids(pkg, oracle, tmp_path):
    """A grid the fused kernels do not cover (24^3) runs on the FP64 cuFFT path."""
    exe = str(pkg.driver_path())
    inp = canonical_input(tmp_path / "input.txt", Nx=24, Ny=24, Nz=24, N_step=4, ifreq=4, ppt_int=0, grn_rad=6,
                          num_ppt=2)
    r = subprocess.run([exe, str(inp), str(tmp_path) + "/"], cwd=tmp_path, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    assert "FP64 cuFFT" in r.stdout
    p = _params(oracle, Nx=24, Ny=24, Nz=24)
    want_rows, want = _oracle_protocol(oracle, p, _circle(oracle, p, 2, 6), 4)
    phi, con = pkg.read_data_save(tmp_path / "step_0000004" / "data_save.0001", p)
    assert np.max(np.abs(phi - want[4][0])) < 1e-9 and np.max(np.abs(con - want[4][1])) < 1e-9
    got = _summary(tmp_path / "summary.dat")
    for s in want_rows:
        for g, w in zip(got[s], want_rows[s]):
            assert abs(g - w) <= 5e-7 * abs(w) + 1e-12


def test_driver_weak_scaling_grid_80_baseline(pkg, oracle, tmp_path):
    """One of the reference's weak-scaling grids (80^3, inputs/config.yaml:76-79)
    with its baseline coefficients (var 55, dt 1e-4, am 0.5, ap 5, c0 0.1 / 1,
    d_gb 1) runs on the fused FP32 path and matches the oracle."""
    exe = str(pkg.driver_path())
    kw = dict(Nx=80, Ny=80, Nz=80, var=55, t_step=1e-4, am=0.5, ap=5.0, con_0_mat=0.1, con_0_ppt=1.0)
    inp = canonical_input(tmp_path / "input.txt", N_step=4, ifreq=4, ppt_int=0, grn_rad=10, num_ppt=6,
                          c_mat=0.5, c_ppt=0.5, d_gb=1.0, ijk_ppt=(40, 40, 40), **kw)
    r = _run(exe, inp, tmp_path, str(tmp_path) + "/")
    assert "fused FP32" in r.stdout, r.stdout
    p = _params(oracle, D_gb=1.0, **kw)
    gen = oracle.Ran2()
    phi, con, idum = oracle.ic_circle(p, 10, (2, 2, 2), 6, -1, 0.5, 1.0, gen=gen)
    want_rows, want = _oracle_protocol(oracle, p, (phi, con, idum, gen), 4)
    _check_rows(_summary(tmp_path / "summary.dat"), want_rows, p)
    gphi, gcon = pkg.read_data_save(tmp_path / "step_0000004" / "data_save.0001", p)
    assert np.max(np.abs(gphi - want[4][0])) < TOL and np.max(np.abs(gcon - want[4][1])) < TOL
