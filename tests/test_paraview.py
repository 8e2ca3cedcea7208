"""The post-processor paraview.x: its oracle against hand-computed answers, the
VTK writer against the oracle's text (byte for byte), and the pf_paraview
tool's directory handling.  No GPU (the analysis kernels are in
test_gpu_paraview.py)."""
import subprocess
import sys

import numpy as np
import pytest


@pytest.fixture(scope="module")
def pv():
    import pf_paraview

    return pf_paraview


def test_oracle_known_answers(pv):
    # 1 x 1 x 4 voxels, var = 3, threshold 0.2
    phi = np.zeros((3, 1, 1, 4))
    phi[:, 0, 0, 0] = [1.0, 0.0, 0.0]      # grain 1: var_num 1, not boundary
    phi[:, 0, 0, 1] = [0.5, 0.5, 0.0]      # boundary of 1 and 2
    phi[:, 0, 0, 2] = [0.3, 0.1, 0.9]      # boundary with precipitate (phi_3 = 0.9 > 0.8)
    phi[:, 0, 0, 3] = [0.85, 0.9, 0.25]    # three above 0.2: boundary + precipitate; last > 0.8 is 2
    con = np.array([[[0.1, 0.2, 0.3, 0.4]]])
    r = pv.analyze(phi, con, 0.2)
    assert r["var_num"].reshape(-1).tolist() == [1, 0, 3, 2]
    assert r["boundary"].reshape(-1).tolist() == [0.0, 1.0, 1.0, 1.0]
    assert (r["boundary_voxels"], r["precipitate_voxels"]) == (3, 2)
    assert r["precipitate_fraction"] == 2 / 3
    assert np.allclose(r["phi_sq"].reshape(-1), [1.0, 0.5, 0.91, 0.85 ** 2 + 0.81 + 0.0625])
    assert np.all(r["grad_phi_3"] == 0.0)  # no interior cell on a 1 x 1 x 4 grid
    assert pv.stdout_line("0000010", r) == "0000010       2       3  0.67"


def test_oracle_gradient_interior_only(pv):
    z, y, x = np.meshgrid(np.arange(5.0), np.arange(4.0), np.arange(6.0), indexing="ij")
    f = 2.0 * x + 3.0 * y - z
    g = pv.grad_mag(f)
    want = np.sqrt(4.0 + 9.0 + 1.0)
    assert np.all(g[1:-1, 1:-1, 1:-1] == want)
    g[1:-1, 1:-1, 1:-1] = 0.0
    assert np.all(g == 0.0)


def test_vtk_writer_matches_oracle(pkg, pv, tmp_path):
    rng = np.random.default_rng(5)
    v = rng.standard_normal((3, 4, 5)) * 10.0 ** rng.integers(-20, 20, (3, 4, 5))
    v.reshape(-1)[:6] = [0.0, 1.0, 0.5, 1.5e-3, 123456.0, 9.999999999999999e16]
    path = tmp_path / "phi_sq_0000010.vtk"
    pkg.write_vtk(path, v)
    assert path.read_text() == pv.vtk_text(5, 4, 3, v)
    iv = rng.integers(0, 17, (3, 4, 5)).astype(np.int32)
    pkg.write_vtk(tmp_path / "var_num.vtk", iv)
    assert (tmp_path / "var_num.vtk").read_text() == pv.vtk_text(5, 4, 3, iv, integer=True)
    lines = path.read_text().split("\n")
    assert lines[4] == "DIMENSIONS       5     4     3" and lines[7] == "POINT_DATA            60"
    assert len(lines[10]) == 60 * 26


def test_vtk_writer_large_parallel(pkg, pv, tmp_path):
    """More values than one formatting block per thread."""
    v = np.linspace(-1.0, 1.0, 64 * 64 * 80).reshape(80, 64, 64)
    pkg.write_vtk(tmp_path / "big.vtk", v)
    body = (tmp_path / "big.vtk").read_text().split("\n")[10]
    assert len(body) == v.size * 26
    idx = [0, 1, 262143, 262144, 262145, v.size - 1]
    for i in idx:
        assert body[i * 26:(i + 1) * 26] == pv.list_real(float(v.reshape(-1)[i]))


def test_paraview_tool_directory_handling(pkg, oracle, pv, tmp_path):
    """The header line, the step order and var_dist come before any GPU work;
    without a GPU the tool then stops with status 2."""
    exe = str(pkg.paraview_path())
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "usage" in r.stderr
    p = oracle.Params(Nx=4, Ny=4, Nz=4, var=3)
    src = tmp_path / "run"
    for s in ("0000020", "0000010"):
        d = src / f"step_{s}"
        d.mkdir(parents=True)
        (d / "data_extract_mult.in").write_text("           4           4           4           1           3\n"
                                                "           1           1\n")
        phi = np.zeros((3,) + p.shape)
        phi[0] = 1.0
        pkg.write_data_save(d / "data_save.0001", p, phi, np.full(p.shape, 0.3))
    out = tmp_path / "vis"
    out.mkdir()
    r = subprocess.run([exe, str(src), str(out), "0.2"], capture_output=True, text=True, timeout=300)
    lines = r.stdout.split("\n")
    assert lines[0] == pv.HEADER
    assert (src / "step_0000010" / "var_dist").exists()
    if r.returncode == 0:
        assert lines[1:3] == ["0000010       0       0  0.00", "0000020       0       0  0.00"]
    else:
        assert r.returncode == 2 and "analysis" in r.stderr
