"""CPU oracle of the post-processor ``paraview.x`` (``src/paraview.f90``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/`` as the checker of the GPU
analysis kernel and of the ``pf_paraview`` tool; the product never imports it.

Restates, for one step directory written by one rank:

* ``src/paraview.f90:189-244``  per-voxel classification: phi_sq = sum phi_i^2
  (i = 1..var in order), var_num = the LAST variant with phi > 0.8 (0 if
  none; ``phi_max`` stays 0.8), phi_3 = phi(3, ...) whatever var is (:206),
  boundary = 1 where more than one variant exceeds the threshold, and the
  counts of boundary voxels and of boundary voxels with phi_var > threshold;
* ``src/paraview.f90:380-429``  |grad phi_3| by central differences on the
  interior cells only (the boundary layer of the reference's array is never
  written; 0 here);
* ``src/paraview.f90:263-300``  the six ASCII VTK files (fixed header, the
  values as ONE gfortran list-directed record);
* ``src/paraview.f90:109-110,311-318``  the stdout lines.

Parity of the text is pinned to gfortran's documented list-directed layout
(INTEGER*4: a blank and I11; REAL*8: a blank and G25.17E3 with 1P for the E
form); no gfortran is available to run the reference itself.
"""
from __future__ import annotations

import numpy as np

HEADER = "# step, precipitate_voxels," + " " * 22 + "boundary_voxels, precipitate_fraction"
VTK_NAMES = ("phi_sq", "con", "var_num", "phi_3", "grad_phi_3", "boundary")


def classify(phi: np.ndarray, con: np.ndarray, threshold: float):
    """phi[var, z, y, x], con[z, y, x] -> dict of the per-voxel arrays and counts."""
    var = phi.shape[0]
    phi_sq = np.zeros(phi.shape[1:])
    var_num = np.zeros(phi.shape[1:], dtype=np.int32)
    above = np.zeros(phi.shape[1:], dtype=np.int32)
    for ii in range(var):
        f = phi[ii]
        phi_sq = phi_sq + f * f
        var_num[f > 0.8] = ii + 1
        above += (f > threshold)
    boundary = (above > 1)
    prec = int(np.count_nonzero(boundary & (phi[var - 1] > threshold)))
    nb = int(np.count_nonzero(boundary))
    return dict(phi_sq=phi_sq, con=np.array(con, dtype=np.float64), var_num=var_num,
                phi_3=np.array(phi[2], dtype=np.float64), boundary=boundary.astype(np.float64),
                precipitate_voxels=prec, boundary_voxels=nb,
                precipitate_fraction=(prec / nb) if nb > 0 else 0.0)


def grad_mag(f: np.ndarray) -> np.ndarray:
    """|grad f| with (f(i+1) - f(i-1)) / 2 on 2..N-1 of every axis; 0 elsewhere."""
    g = np.zeros_like(f, dtype=np.float64)
    if min(f.shape) < 3:
        return g
    c = (slice(1, -1),) * 3
    gx = (f[1:-1, 1:-1, 2:] - f[1:-1, 1:-1, :-2]) / 2.0
    gy = (f[1:-1, 2:, 1:-1] - f[1:-1, :-2, 1:-1]) / 2.0
    gz = (f[2:, 1:-1, 1:-1] - f[:-2, 1:-1, 1:-1]) / 2.0
    g[c] = np.sqrt(gx * gx + gy * gy + gz * gz)
    return g


def analyze(phi: np.ndarray, con: np.ndarray, threshold: float):
    out = classify(phi, con, threshold)
    out["grad_phi_3"] = grad_mag(out["phi_3"])
    return out


def list_real(v: float) -> str:
    """One gfortran list-directed REAL*8 item (a blank, then G25.17E3)."""
    if v == 0.0:
        return " " + "%20s     " % (("-" if np.signbit(v) else "") + "0.0000000000000000")
    m, e = ("%.16e" % v).split("e")
    e = int(e)
    if -1 <= e <= 16:
        body = ("%.0f." % v) if e == 16 else ("%.*f" % (16 - e, v))
        return " " + "%20s     " % body
    return " " + "%25s" % (m + "E" + ("-" if e < 0 else "+") + "%03d" % abs(e))


def list_int(v: int) -> str:
    return " %11d" % v


def vtk_text(nx: int, ny: int, nz: int, values: np.ndarray, integer: bool = False) -> str:
    head = ["# vtk DataFile Version 3.0", "Sample Data", "ASCII", "DATASET STRUCTURED_POINTS",
            "DIMENSIONS  %6d%6d%6d" % (nx, ny, nz), "ASPECT_RATIO 1.0 1.0 1.0", "ORIGIN 0.0 0.0 0.0",
            "POINT_DATA  %12d" % (nx * ny * nz), "SCALARS Field double 1", "LOOKUP_TABLE default"]
    flat = np.asarray(values).reshape(-1)
    fmt = list_int if integer else list_real
    body = "".join(fmt(int(v)) if integer else fmt(float(v)) for v in flat)
    return "\n".join(head) + "\n" + body + "\n"


def stdout_line(step_string: str, res) -> str:
    """'(A, 2(I8), F6.2)' of paraview.f90:318."""
    return "%s%8d%8d%6.2f" % (step_string.strip(), res["precipitate_voxels"], res["boundary_voxels"],
                               res["precipitate_fraction"])
