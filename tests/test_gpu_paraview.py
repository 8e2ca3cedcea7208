"""GPU voxel analysis of paraview.x against the oracle (bit for bit), in situ
on resident runs, and the pf_paraview tool end to end on pf_var_diff output
(VTK files byte for byte, the stdout lines run_phase_sim.py parses)."""
import struct
import subprocess

import numpy as np
import pytest

from test_io import canonical_input

pytestmark = pytest.mark.gpu

ARRAYS = ("phi_sq", "var_num", "phi_3", "grad_phi_3", "boundary")


@pytest.fixture(scope="module")
def pv():
    import pf_paraview

    return pf_paraview


def _random_fields(oracle, p, seed):
    rng = np.random.default_rng(seed)
    phi = rng.random((p.var,) + p.shape) ** 3      # many values near 0, some above 0.8
    con = rng.random(p.shape)
    return phi, con


@pytest.mark.parametrize("shape,var,thr", [((32, 32, 32), 4, 0.2), ((16, 32, 64), 3, 0.5), ((3, 5, 7), 6, 0.1)])
def test_analyze_fields_bit_exact(pkg, oracle, pv, shape, var, thr):
    nz, ny, nx = shape
    p = oracle.Params(Nx=nx, Ny=ny, Nz=nz, var=var)
    phi, con = _random_fields(oracle, p, seed=var)
    got = pkg.analyze_fields(p, phi, con, thr)
    want = pv.analyze(phi, con, thr)
    for k in ARRAYS:
        assert np.array_equal(got[k], want[k]), k
    for k in ("precipitate_voxels", "boundary_voxels", "precipitate_fraction"):
        assert got[k] == want[k], k
    assert want["boundary_voxels"] > 0 and want["precipitate_voxels"] > 0


def test_analyze_rejects_var_below_3(pkg, oracle):
    p = oracle.Params(Nx=4, Ny=4, Nz=4, var=2)
    with pytest.raises(pkg.PFError):
        pkg.analyze_fields(p, np.zeros((2, 4, 4, 4)), np.zeros((4, 4, 4)), 0.2)


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_analyze_run_in_situ(pkg, oracle, pv, precision):
    """Counts and arrays of a resident run equal those of its downloaded fields."""
    p = oracle.Params(Nx=32, Ny=32, Nz=32, var=4, t_step=0.01, mobility="c1mc", am=0.5, ap=2.0, con_0_mat=0.3,
                      con_0_ppt=0.7)
    phi0, con0 = oracle.ic_voronoi(p, 3, 10, 0.05, 0.4, 0.02)
    prec = pkg.PF_FP32_FUSED if precision == "fp32" else pkg.PF_FP64_PLAIN
    run = pkg.Run(p, precision=prec)
    try:
        run.set_fields(phi0, con0)
        run.step(5)
        got = pkg.analyze_run(run, 0.2, want=ARRAYS + ("con",))
        counts = pkg.analyze_run(run, 0.2)
        phi, con = run.get_fields()
        run.step(1)  # the run steps on after an analysis
    finally:
        run.close()
    want = pv.analyze(phi, con, 0.2)
    for k in ARRAYS:
        assert np.array_equal(got[k], want[k]), k
    assert np.array_equal(got["con"], con)
    for k in ("precipitate_voxels", "boundary_voxels"):
        assert got[k] == want[k] == counts[k]
    assert want["boundary_voxels"] > 0


def _read(path):
    return path.read_text()


def test_paraview_tool_on_driver_output(pkg, oracle, pv, tmp_path):
    exe = str(pkg.driver_path())
    inp = canonical_input(tmp_path / "input.txt", N_step=6, ifreq=3, ppt_int=0, start="voronoi",
                          extra="seed=1 n_grains=6 amp_phi=0.3 c0=0.4 amp_c=0.02\n")
    run_dir = tmp_path / "run"
    run_dir.mkdir()
    r = subprocess.run([exe, str(inp), str(run_dir) + "/"], cwd=tmp_path, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    vis = tmp_path / "vis"
    vis.mkdir()
    r = subprocess.run([str(pkg.paraview_path()), str(run_dir), str(vis), "0.2"], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip("\n").split("\n")
    assert lines[0] == pv.HEADER and len(lines) == 3
    p = oracle.Params(Nx=32, Ny=32, Nz=32, var=3)
    for line, step in zip(lines[1:], ("0000003", "0000006")):
        phi, con = pkg.read_data_save(run_dir / f"step_{step}" / "data_save.0001", p)
        want = pv.analyze(phi, con, 0.2)
        assert line == pv.stdout_line(step, want)
        # run_phase_sim.py:225 takes the fourth column of the last line
        assert float(line.split()[3]) == float("%.2f" % want["precipitate_fraction"])
        for name in pv.VTK_NAMES:
            text = _read(vis / f"{name}_{step}.vtk")
            assert text == pv.vtk_text(32, 32, 32, want[name], integer=(name == "var_num")), name
    assert want["boundary_voxels"] > 0 and want["precipitate_voxels"] > 0


def test_paraview_tool_reads_several_ranks(pkg, oracle, pv, tmp_path):
    """A step directory written by 2 x 2 ranks (y and z split, each file with
    its own ist/ien record) gives the same result as one file."""
    p = oracle.Params(Nx=8, Ny=8, Nz=6, var=3)
    phi, con = _random_fields(oracle, p, seed=21)
    d = tmp_path / "run" / "step_0000100"
    d.mkdir(parents=True)
    (d / "data_extract_mult.in").write_text(" 8 8 6 4 3\n 2 2\n")
    fn = 0
    for (z0, z1) in ((1, 3), (4, 6)):
        for (y0, y1) in ((1, 5), (6, 8)):
            fn += 1
            sub_phi = phi[:, z0 - 1:z1, y0 - 1:y1, :]
            sub_con = con[z0 - 1:z1, y0 - 1:y1, :]
            payload = np.concatenate([oracle.to_fortran_aos(sub_phi), sub_con.reshape(-1)]).astype("<f8").tobytes()
            rec1 = struct.pack("<6i", 1, y0, z0, 8, y1, z1)
            data = (struct.pack("<i", 24) + rec1 + struct.pack("<i", 24) + struct.pack("<i", len(payload)) + payload
                    + struct.pack("<i", len(payload)))
            (d / f"data_save.{fn:04d}").write_bytes(data)
    vis = tmp_path / "vis"
    vis.mkdir()
    r = subprocess.run([str(pkg.paraview_path()), str(tmp_path / "run"), str(vis), "0.3"], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    want = pv.analyze(phi, con, 0.3)
    assert r.stdout.strip("\n").split("\n")[1] == pv.stdout_line("0000100", want)
    assert _read(vis / "boundary_0000100.vtk") == pv.vtk_text(8, 8, 6, want["boundary"])
    assert _read(vis / "con_0000100.vtk") == pv.vtk_text(8, 8, 6, con)
