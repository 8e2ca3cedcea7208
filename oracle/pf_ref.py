"""CPU oracle for the semi-implicit Fourier-spectral phase-field step.

TEST INFRASTRUCTURE ONLY.  This module is the checker: it is imported by
``tests/``, by ``__graft_entry__.smoke()`` and by the CPU-baseline leg of
``bench.py``.  The product path (the CUDA library behind ``include/pfgpu.h``)
never imports, links or calls it.

What it is
----------
A loop-for-loop FP64 NumPy/SciPy restatement of the time step of the
reference program ``var_diff.x``:

* ``src/var_diff.f90:474-1118``  one time step (14 timed phases) and the
  diagnostics/statistics that follow it;
* ``src/k_space.f90:13-59``      wavenumber tables;
* ``src/f_trans.f90:11-12``      forward R2C FFT normalised by 1/(Nx*Ny*Nz);
* ``src/inv_trans.f90:10``       un-normalised inverse C2R FFT;
* ``src/ran_2.f90:1-40``         L'Ecuyer combined generator with shuffle;
* ``src/var_diff.f90:196-449``   gamma matrix and the 'circle'/'plane'
  initial conditions.

The reference's FFTs come from P3DFFT 2.7.9 on top of FFTW 3.3.10
(``src/Makefile:8-9``); neither is vendored, and the Fortran cannot be built
where this oracle runs (no Fortran compiler, MPI, FFTW or P3DFFT).  SciPy's
pocketfft computes the same mathematical transform (DFT with e^{-i k x} in the
forward direction), so this restatement follows the published algorithm, not
the reference binary.  The reference ships no golden vectors or tests for this
path, so **parity is unpinned**: the oracle is instead pinned by known-answer
tests (single Fourier-mode decay rates, FFT round trips, mass conservation,
the published first outputs of the ran_2 generator recomputed by a separate C
restatement) in ``tests/test_oracle.py``.

Array layout used here: ``phi[ivar, z, y, x]`` (C order, x fastest) and
``con[z, y, x]``.  The Fortran arrays are ``phi(var, x, y, z)`` (var fastest);
``to_fortran_aos``/``from_fortran_aos`` convert.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Optional

import numpy as np

try:  # scipy.fft honours float32 and can use several threads
    import scipy.fft as _fft

    def _rfftn(a, workers):
        return _fft.rfftn(a, axes=(-3, -2, -1), norm="forward", workers=workers)

    def _irfftn(a, shape, workers):
        return _fft.irfftn(a, s=shape, axes=(-3, -2, -1), norm="forward", workers=workers)
except ImportError:  # pragma: no cover - numpy fallback for the checker only
    def _rfftn(a, workers):
        return np.fft.rfftn(a, axes=(-3, -2, -1), norm="forward")

    def _irfftn(a, shape, workers):
        return np.fft.irfftn(a, s=shape, axes=(-3, -2, -1), norm="forward")


# ---------------------------------------------------------------------------
# Parameters (the records of input.txt that the step uses)
# ---------------------------------------------------------------------------
@dataclasses.dataclass
class Params:
    """Coefficients of one run, named as in ``src/var_diff.f90:104-121``.

    ``mobility`` selects the concentration mobility:
      * ``"reference"``: mob = D_L + 2(1 - sum_i phi_i^2) D_gb
        (``src/var_diff.f90:893-898``; D_bulk(var) = D_L, ``:188-194``);
      * ``"c1mc"``: mob = D_L * (1 + c(1 - c)), the concentration-dependent
        form M(c) = M0 (1 + c (1 - c)) with M0 = D_L.
    In both cases the implicit mean mobility is D_mean = D_L (``:916``).
    """
    Nx: int
    Ny: int
    Nz: int
    var: int
    t_step: float = 0.05
    grad_coeff_phi: float = 1.0
    grad_coeff_c: float = 1.0
    D_S: float = 1.0
    D_L: float = 1.0
    D_gb: float = 0.0
    mob_phi: float = 1.0
    sigma_1: float = 1.5
    sigma_2: float = 1.5
    am: float = 0.0
    ap: float = 0.0
    con_0_mat: float = 0.0
    con_0_ppt: float = 1.0
    mobility: str = "reference"

    @property
    def shape(self):
        return (self.Nz, self.Ny, self.Nx)


def gamma_matrix(var: int, sigma_1: float, sigma_2: float) -> np.ndarray:
    """gamma(i,j) of ``src/var_diff.f90:206-218`` (0-based here)."""
    g = np.zeros((var, var))
    mat = var - 1
    for j in range(var):
        for i in range(var):
            if i != j and i < mat and j < mat:
                g[i, j] = sigma_1
            if j == var - 1 and i < var - 1:
                g[i, j] = sigma_2
            if i == var - 1 and j < var - 1:
                g[i, j] = sigma_2
    return g


# ---------------------------------------------------------------------------
# Wavenumbers: src/k_space.f90:13-59
# ---------------------------------------------------------------------------
def axis_wavenumbers(n: int, half: bool = False):
    """Per-axis q (for kf_sq/kf_4) and Nyquist-zeroed q (for kf).

    ``src/k_space.f90``: m' = m if m <= n/2 else m - n, lamda = m' * (2*pi/n)
    (``unit1 = unit/float(Nx)`` is formed first, then multiplied by float(m')),
    kf = i*lamda except kf = 0 where 2m = n (``:51-53``); kf_sq = lamda^2,
    kf_4 = lamda^4 are NOT zeroed at Nyquist (``:54-59``).
    ``half`` selects the R2C-halved axis (m = 0..n/2).
    """
    pi = math.atan(1.0) * 4.0
    unit = 2.0 * pi / float(n)
    m = np.arange(n // 2 + 1 if half else n)
    mp = np.where(m <= n // 2, m, m - n).astype(np.float64)
    q = mp * unit
    qz = np.where(2 * m == n, 0.0, q)
    return q, qz


def k_space(Nx: int, Ny: int, Nz: int):
    """Return (G, K2, K3, K4) on the (Nz, Ny, Nx//2+1) half spectrum.

    G  = sum_d kf_d            (pure imaginary, Nyquist-zeroed)   var_diff.f90:932
    K2 = sum_d kf_sq_d = -sum q_d^2                              var_diff.f90:933
    K3 = sum_d kf_d*kf_sq_d = -i sum_d qz_d q_d^2                var_diff.f90:934-935
    K4 = sum_d kf_4_d = sum_d q_d^4 (not |q|^4)                  var_diff.f90:980
    """
    qx, qzx = axis_wavenumbers(Nx, half=True)
    qy, qzy = axis_wavenumbers(Ny)
    qz, qzz = axis_wavenumbers(Nz)
    X = (slice(None), None, None)
    qx3, qy3, qz3 = qx[None, None, :], qy[None, :, None], qz[:, None, None]
    zx3, zy3, zz3 = qzx[None, None, :], qzy[None, :, None], qzz[:, None, None]
    G = 1j * (zx3 + zy3 + zz3)
    K2 = -(qx3 * qx3 + qy3 * qy3 + qz3 * qz3)
    K3 = -1j * (zx3 * qx3 * qx3 + zy3 * qy3 * qy3 + zz3 * qz3 * qz3)
    K4 = qx3 ** 4 + qy3 ** 4 + qz3 ** 4
    del X
    return G, K2, K3, K4


# ---------------------------------------------------------------------------
# ran_2: src/ran_2.f90:1-40
# ---------------------------------------------------------------------------
class Ran2:
    """Restatement of the saved-state function ``ran_2(idum)``.

    ``am = 1./im1`` is evaluated in REAL*4 (``src/ran_2.f90:5``): the integer
    2147483563 rounds to the float 2147483520 and the quotient rounds to
    2^-31 (1 + 2^-23) = 4.6566134e-10, which is then widened.
    """
    IM1, IM2 = 2147483563, 2147483399
    IA1, IA2 = 40014, 40692
    IQ1, IQ2 = 53668, 52774
    IR1, IR2 = 12211, 3791
    NTAB = 32
    IMM1 = IM1 - 1
    NDIV = 1 + IMM1 // NTAB
    AM = float(np.float32(1.0) / np.float32(IM1))
    EPS = 1.2e-7
    RNMX = 1.0 - EPS

    def __init__(self):
        self.idum2 = 123456789
        self.iv = [0] * self.NTAB
        self.iy = 0

    def __call__(self, idum: int):
        """Return (value, new_idum) exactly like ``ran_2(idum)``."""
        if idum <= 0:
            idum = max(-idum, 1)
            self.idum2 = idum
            for j in range(self.NTAB + 8, 0, -1):
                k = idum // self.IQ1
                idum = self.IA1 * (idum - k * self.IQ1) - k * self.IR1
                if idum < 0:
                    idum += self.IM1
                if j <= self.NTAB:
                    self.iv[j - 1] = idum
            self.iy = self.iv[0]
        k = idum // self.IQ1
        idum = self.IA1 * (idum - k * self.IQ1) - k * self.IR1
        if idum < 0:
            idum += self.IM1
        k = self.idum2 // self.IQ2
        self.idum2 = self.IA2 * (self.idum2 - k * self.IQ2) - k * self.IR2
        if self.idum2 < 0:
            self.idum2 += self.IM2
        j = 1 + self.iy // self.NDIV
        self.iy = self.iv[j - 1] - self.idum2
        self.iv[j - 1] = idum
        if self.iy < 1:
            self.iy += self.IMM1
        return min(self.AM * self.iy, self.RNMX), idum


class Ran2Stream:
    """Convenience wrapper: a generator seeded like the drop-in's ``seed`` key.

    ``idum = -(seed + 1)`` so that seed 0 reproduces the reference default
    ``iseed = -1`` (``tests/run_phase_sim.py:118``) and seeds 0/1 do not
    collide through ``max(-idum, 1)`` (``src/ran_2.f90:14-15``).
    """

    def __init__(self, seed: int = 0, idum: Optional[int] = None):
        self.gen = Ran2()
        self.idum = -(seed + 1) if idum is None else idum

    def next(self) -> float:
        v, self.idum = self.gen(self.idum)
        return v

    def take(self, n: int) -> np.ndarray:
        out = np.empty(n)
        for i in range(n):
            out[i] = self.next()
        return out


# ---------------------------------------------------------------------------
# Initial conditions
# ---------------------------------------------------------------------------
def ic_noise(p: Params, seed: int, amp_phi: float, c0: float, amp_c: float):
    """Uniform-noise start: draw order z, y, x (x fastest), per cell var phi
    values then c; U(-a, a) = a (2 r - 1).  phi_i ~ U(-amp_phi, amp_phi),
    c = c0 + U(-amp_c, amp_c)."""
    rs = Ran2Stream(seed)
    n = p.Nx * p.Ny * p.Nz * (p.var + 1)
    r = rs.take(n).reshape(p.Nz, p.Ny, p.Nx, p.var + 1)
    phi = np.ascontiguousarray(np.moveaxis(amp_phi * (2.0 * r[..., :p.var] - 1.0), -1, 0))
    con = c0 + amp_c * (2.0 * r[..., p.var] - 1.0)
    return phi, np.ascontiguousarray(con)


def voronoi_labels(p: Params, seeds: np.ndarray) -> np.ndarray:
    """Grain index (0-based) of every cell: nearest seed by periodic
    minimum-image distance, cells at integer coordinates, ties to the lower
    seed index."""
    nseed = seeds.shape[0]
    z = np.arange(p.Nz, dtype=np.float64)
    y = np.arange(p.Ny, dtype=np.float64)
    x = np.arange(p.Nx, dtype=np.float64)
    best = np.full(p.shape, np.inf)
    lab = np.zeros(p.shape, dtype=np.int64)

    def mi(d, n):
        d = np.abs(d)
        return np.minimum(d, n - d)

    for s in range(nseed):
        sx, sy, sz = seeds[s]
        dz = mi(z - sz, p.Nz)[:, None, None]
        dy = mi(y - sy, p.Ny)[None, :, None]
        dx = mi(x - sx, p.Nx)[None, None, :]
        d2 = dz * dz + dy * dy + dx * dx
        upd = d2 < best
        best = np.where(upd, d2, best)
        lab = np.where(upd, s, lab)
    return lab


def ic_voronoi(p: Params, seed: int, n_grains: int, amp_phi: float, c0: float, amp_c: float):
    """Voronoi polycrystal start: n_grains seed points (x, y, z) = (Nx r, Ny r,
    Nz r) drawn first; grain s (1-based) gets variant ((s-1) mod var)+1 set to
    1; then the noise of ``ic_noise`` is added with the same stream."""
    rs = Ran2Stream(seed)
    seeds = np.empty((n_grains, 3))
    for s in range(n_grains):
        seeds[s, 0] = p.Nx * rs.next()
        seeds[s, 1] = p.Ny * rs.next()
        seeds[s, 2] = p.Nz * rs.next()
    lab = voronoi_labels(p, seeds)
    phi = np.zeros((p.var,) + p.shape)
    variant = lab % p.var
    for i in range(p.var):
        phi[i][variant == i] = 1.0
    n = p.Nx * p.Ny * p.Nz * (p.var + 1)
    r = rs.take(n).reshape(p.Nz, p.Ny, p.Nx, p.var + 1)
    phi += np.moveaxis(amp_phi * (2.0 * r[..., :p.var] - 1.0), -1, 0)
    con = c0 + amp_c * (2.0 * r[..., p.var] - 1.0)
    return np.ascontiguousarray(phi), np.ascontiguousarray(con)


def _f32(x):
    return float(np.float32(x))


def _ellipsoid_offsets(rx: int, ry: int, rz: int):
    """Offsets (i, j, k) with (i/rx)^2+(j/ry)^2+(k/rz)^2 <= 1, evaluated in
    REAL*4 like ``float(i)/float(ppt_rad(1))`` (``src/var_diff.f90:303-306``)."""
    out = []
    for k in range(-rz, rz + 1):
        for j in range(-ry, ry + 1):
            for i in range(-rx, rx + 1):
                t1 = np.float32(np.float32(i) / np.float32(rx)) ** 2
                t2 = np.float32(np.float32(j) / np.float32(ry)) ** 2
                t3 = np.float32(np.float32(k) / np.float32(rz)) ** 2
                # term_1..3 are REAL*8 variables: the squares are taken in REAL*4
                # and widened, the sum is REAL*8.
                s = float(t1) + float(t2) + float(t3)
                if s <= 1.0:
                    out.append((i, j, k))
    return out


def ic_circle(p: Params, grn_rad: int, ppt_rad, num_ppt: int, iseed: int,
              c_mat: float, con_0_ppt: float, gen: Optional["Ran2"] = None):
    """'circle' start, ``src/var_diff.f90:373-449`` (one rank: ist=1, ien=N).

    phi_1 = 1 everywhere, a spherical grain of variant 2 at the centre, then
    num_ppt precipitates (variant 3, c = con_0_ppt) placed at ran_2 positions
    that are rejected while any cell of the sphere already has phi_var > 0.
    ``gen`` carries ran_2's saved state on to a later precipitate insertion.
    Returns (phi, con, idum_after)."""
    var = p.var
    phi = np.zeros((var,) + p.shape)
    con = np.full(p.shape, float(c_mat))
    phi[0] = 1.0
    for (i, j, k) in _ellipsoid_offsets(grn_rad, grn_rad, grn_rad):
        ii, jj, kk = i + p.Nx // 2, j + p.Ny // 2, k + p.Nz // 2
        if 1 <= ii <= p.Nx and 1 <= jj <= p.Ny and 1 <= kk <= p.Nz:
            phi[1, kk - 1, jj - 1, ii - 1] = 1.0
            phi[0, kk - 1, jj - 1, ii - 1] = 0.0
            phi[2, kk - 1, jj - 1, ii - 1] = 0.0
    gen = Ran2() if gen is None else gen
    idum = iseed
    rad_ppt = ppt_rad[0] ** 2 + ppt_rad[1] ** 2 + ppt_rad[2] ** 2
    zz, yy, xx = np.meshgrid(np.arange(1, p.Nz + 1), np.arange(1, p.Ny + 1),
                             np.arange(1, p.Nx + 1), indexing="ij")
    nppt = 1
    while nppt <= num_ppt:
        r, idum = gen(idum)
        ix = int(r * p.Nx + 1.0)
        r, idum = gen(idum)
        jy = int(r * p.Ny + 1.0)
        r, idum = gen(idum)
        kz = int(r * p.Nz + 1.0)
        rad = (xx - ix) ** 2 + (yy - jy) ** 2 + (zz - kz) ** 2
        inside = rad <= rad_ppt
        if np.any(inside & (phi[var - 1] > 0.0)):
            continue
        phi[2][inside] = 1.0
        phi[1][inside] = 0.0
        phi[0][inside] = 0.0
        con[inside] = con_0_ppt
        nppt += 1
    return phi, con, idum


def ic_plane(p: Params, ppt_rad, i_ppt: int, j_ppt: int, k_ppt: int, c_mat: float):
    """'plane' start, ``src/var_diff.f90:252-371`` (one rank)."""
    var = p.var
    phi = np.zeros((var,) + p.shape)
    con = np.full(p.shape, float(c_mat))
    phi[1] = 1.0
    j1 = p.Ny - j_ppt + 1
    jj = np.arange(1, p.Ny + 1)
    low = jj < j1
    phi[:, :, low, :] = 0.0
    phi[0, :, low, :] = 1.0
    high = jj >= j_ppt
    phi[:, :, high, :] = 0.0
    phi[0, :, high, :] = 1.0
    offs = _ellipsoid_offsets(*ppt_rad)
    for jc in (j_ppt, p.Ny - j_ppt + 1):
        for (i, j, k) in offs:
            ii, jj_, kk = i + i_ppt, j + jc, k + k_ppt
            if 1 <= ii <= p.Nx and 1 <= jj_ <= p.Ny and 1 <= kk <= p.Nz:
                phi[2, kk - 1, jj_ - 1, ii - 1] = 1.0
                phi[0, kk - 1, jj_ - 1, ii - 1] = 0.0
                phi[1, kk - 1, jj_ - 1, ii - 1] = 0.0
    return phi, con


def insert_precipitates(p: Params, phi: np.ndarray, ppt_rad, num_ppt: int, idum: int, gen: "Ran2",
                        max_attempts: int = 10 ** 8):
    """Precipitates added at step ``ppt_int``, ``src/var_diff.f90:479-554``
    (one rank).  A ran_2 position is rejected while the matrix variants there
    have sum phi_i^2 > 0.8 (inside a grain) or any cell of the sphere already
    has phi_var > 0; an accepted sphere gets phi_var = 1 and the matrix
    variants 0 (con is left as it is).  Modifies phi in place; returns
    idum_after.  The reference loops until it succeeds; here more than
    ``max_attempts`` draws raise RuntimeError (the library gives up after
    1e8 with PF_EINVAL)."""
    var = p.var
    rad_ppt = ppt_rad[0] ** 2 + ppt_rad[1] ** 2 + ppt_rad[2] ** 2
    zz, yy, xx = np.meshgrid(np.arange(1, p.Nz + 1), np.arange(1, p.Ny + 1),
                             np.arange(1, p.Nx + 1), indexing="ij")
    nppt = 1
    attempts = 0
    while nppt <= num_ppt:
        attempts += 1
        if attempts > max_attempts:
            raise RuntimeError("precipitate insertion: no admissible place")
        r, idum = gen(idum)
        ix = int(r * p.Nx + 1.0)
        r, idum = gen(idum)
        jy = int(r * p.Ny + 1.0)
        r, idum = gen(idum)
        kz = int(r * p.Nz + 1.0)
        s = 0.0
        if 1 <= ix <= p.Nx and 1 <= jy <= p.Ny and 1 <= kz <= p.Nz:
            for f in range(var - 1):
                s += float(phi[f, kz - 1, jy - 1, ix - 1]) ** 2
        if s > 0.8:
            continue
        rad = (xx - ix) ** 2 + (yy - jy) ** 2 + (zz - kz) ** 2
        inside = rad <= rad_ppt
        if np.any(inside & (phi[var - 1] > 0.0)):
            continue
        phi[var - 1][inside] = 1.0
        for f in range(var - 1):
            phi[f][inside] = 0.0
        nppt += 1
    return idum


# ---------------------------------------------------------------------------
# One time step: src/var_diff.f90:556-1050 and the statistics at :1076-1118
# ---------------------------------------------------------------------------
def bulk_energies(p: Params, phi: np.ndarray, con: np.ndarray, gamma=None, dtype=np.float64):
    """Phases 5-6 of one step from the fields at its start:
    f_eta (``src/var_diff.f90:685-719``), h = phi_mat = N4/S4, f_ch and df_dc
    (``:723-757``).  Returns (f_eta, f_ch, phi_mat, S4, df_dc); an all-zero
    cell gives phi_mat = 0/0 = NaN, as in the reference."""
    var = p.var
    P = var - 1
    g = gamma_matrix(var, p.sigma_1, p.sigma_2) if gamma is None else gamma
    f_eta_c = np.zeros(p.shape, dtype=dtype)
    for i in range(var):
        fi2 = phi[i] * phi[i]
        f_eta_c += -0.5 * fi2 + 0.25 * fi2 * fi2
        for j in range(i + 1, var):
            f_eta_c += g[i, j] * fi2 * (phi[j] * phi[j])
    f_eta = float(np.sum(f_eta_c))
    num = np.zeros(p.shape, dtype=dtype)
    den = np.zeros(p.shape, dtype=dtype)
    for i in range(var):
        f4 = phi[i] ** 4
        if i < P:
            num += f4
        den += f4
    with np.errstate(invalid="ignore", divide="ignore"):
        phi_mat = num / den
    phi_ppt = 1.0 - phi_mat
    dcm = con - p.con_0_mat
    dcp = con - p.con_0_ppt
    f_ch = float(np.sum(phi_mat * p.am * dcm ** 2 + phi_ppt * p.ap * dcp ** 2))
    df_dc = 2.0 * phi_mat * p.am * dcm + 2.0 * phi_ppt * p.ap * dcp
    return f_eta, f_ch, phi_mat, den, df_dc


@dataclasses.dataclass
class Diag:
    """Per-step diagnostics.  f_int, f_eta, f_ch use the fields at the START
    of the step; c_min, c_max, phi_min (min over cells of sum_i phi_i^2) and
    phi_P_max (max of the last order parameter) use the fields at the END of
    the step (``src/var_diff.f90:1076-1102``, with the reference's initial
    values 1.0, 0.0, 1.0, 0.0)."""
    f_int: float
    f_eta: float
    f_ch: float
    c_min: float
    c_max: float
    phi_min: float
    phi_P_max: float
    mass: float


class Oracle:
    """Stateful FP64 restatement of ``var_diff.x``'s loop body.

    ``faithful=True`` performs exactly the 7P+9 transforms of the reference
    (gradients by three inverse FFTs per field, the variable-mobility chain
    even when it multiplies by zero).  ``faithful=False`` computes f_int by
    Parseval and skips the correction chain when D_gb = 0 under the reference
    mobility; both give the same numbers to round-off (tested).
    """

    def __init__(self, p: Params, phi: np.ndarray, con: np.ndarray,
                 faithful: bool = True, workers: int = 1, dtype=np.float64):
        self.p = p
        self.dtype = np.dtype(dtype)
        self.phi = np.array(phi, dtype=self.dtype, copy=True)
        self.con = np.array(con, dtype=self.dtype, copy=True)
        self.faithful = faithful
        self.workers = workers
        self.gamma = gamma_matrix(p.var, p.sigma_1, p.sigma_2)
        G, K2, K3, K4 = k_space(p.Nx, p.Ny, p.Nz)
        cdt = np.complex64 if self.dtype == np.float32 else np.complex128
        self.G, self.K3 = G.astype(cdt), K3.astype(cdt)
        self.K2, self.K4 = K2.astype(self.dtype), K4.astype(self.dtype)
        qx, zx = axis_wavenumbers(p.Nx, half=True)
        qy, zy = axis_wavenumbers(p.Ny)
        qz, zz = axis_wavenumbers(p.Nz)
        self._kf = (zx[None, None, :], zy[None, :, None], zz[:, None, None])
        self.step_no = 0

    # f_trans / inv_trans
    def F(self, a):
        return _rfftn(a, self.workers)

    def Finv(self, a):
        return _irfftn(a, self.p.shape, self.workers)

    def _f_int(self):
        p = self.p
        kfx, kfy, kfz = self._kf
        f_int = 0.0
        if self.faithful:
            # phases 1-4, src/var_diff.f90:561-678
            for i in range(p.var):
                ph = self.F(self.phi[i])
                gx = self.Finv(ph * (1j * kfx))
                gy = self.Finv(ph * (1j * kfy))
                gz = self.Finv(ph * (1j * kfz))
                f_int += float(np.sum(0.5 * p.grad_coeff_phi * (gx * gx + gy * gy + gz * gz)))
            ch = self.F(self.con)
            gx = self.Finv(ch * (1j * kfx))
            gy = self.Finv(ch * (1j * kfy))
            gz = self.Finv(ch * (1j * kfz))
            f_int += float(np.sum(0.5 * p.grad_coeff_c * (gx * gx + gy * gy + gz * gz)))
            return f_int
        # Parseval: sum_x |g|^2 = N^3 sum_k |g_hat|^2 over the full spectrum
        n3 = float(p.Nx * p.Ny * p.Nz)
        k2z = kfx * kfx + kfy * kfy + kfz * kfz
        w = np.full(p.Nx // 2 + 1, 2.0)
        w[0] = 1.0
        if p.Nx % 2 == 0:
            w[-1] = 1.0
        w = w[None, None, :]
        for i in range(p.var):
            ph = self.F(self.phi[i])
            f_int += 0.5 * p.grad_coeff_phi * n3 * float(np.sum(w * k2z * (ph.real ** 2 + ph.imag ** 2)))
        ch = self.F(self.con)
        f_int += 0.5 * p.grad_coeff_c * n3 * float(np.sum(w * k2z * (ch.real ** 2 + ch.imag ** 2)))
        return f_int

    def step(self) -> Diag:
        p = self.p
        phi, con = self.phi, self.con
        var = p.var
        P = var - 1  # index of the precipitate order parameter
        g = self.gamma

        f_int = self._f_int()

        f_eta, f_ch, phi_mat, den, df_dc = bulk_energies(p, phi, con, g, self.dtype)
        dcm = con - p.con_0_mat
        dcp = con - p.con_0_ppt

        # phase 7: term1, term2 (src/var_diff.f90:767-803)
        df_dphi = np.empty_like(phi)
        for i in range(var):
            fi = phi[i]
            t2 = np.zeros(p.shape, dtype=self.dtype)
            for j in range(var):
                if j != i:
                    t2 += 2.0 * g[i, j] * fi * phi[j] ** 2
            df_dphi[i] = (fi ** 3 - fi) + t2
        # phase 8: term4 (src/var_diff.f90:810-844); phase 9 sums the terms
        fch_mat = p.am * dcm ** 2
        fch_ppt = p.ap * dcp ** 2
        fP = phi[P]
        term_2 = 4.0 * fP ** 3 * (den - fP ** 4)
        with np.errstate(invalid="ignore", divide="ignore"):
            den2 = den ** 2
            for i in range(var):
                if i < P:
                    term_1 = 4.0 * phi[i] ** 3 * fP ** 4
                    df_dphi[i] += term_1 * (fch_mat - fch_ppt) / den2
                else:
                    df_dphi[i] += term_2 * (fch_ppt - fch_mat) / den2

        # phase 10: FFT(c), FFT(df_dc), mobility (src/var_diff.f90:868-916)
        c_hat = self.F(con)
        mu_hat = self.F(df_dc)
        D_mean = p.D_L
        if p.mobility == "reference":
            phi_sum = np.zeros(p.shape, dtype=self.dtype)
            for i in range(var):
                phi_sum += phi[i] * phi[i]
            mob = p.D_L + 2.0 * (1.0 - phi_sum) * p.D_gb
            skip_chain = (not self.faithful) and p.D_gb == 0.0
        elif p.mobility == "c1mc":
            mob = p.D_L * (1.0 + con * (1.0 - con))
            skip_chain = False
        else:
            raise ValueError(p.mobility)

        dt = p.t_step
        if skip_chain:
            corr = 0.0
        else:
            # phase 11: J_hat = G mu_hat - kappa_c c_hat K3 ; J = F^-1 (:923-945)
            J = self.Finv(self.G * mu_hat - p.grad_coeff_c * c_hat * self.K3)
            # phase 12: J *= (mob - D_mean) ; F (:947-965)
            Jp = self.F(J * (mob - D_mean))
            corr = Jp * dt * self.G
        # phase 13: CH update (:969-995)
        den_c = 1.0 + D_mean * dt * p.grad_coeff_c * self.K4
        c_hat = (c_hat + corr + D_mean * self.K2 * dt * mu_hat) / den_c
        self.con = self.Finv(c_hat)

        # phase 14: AC update per field (:999-1050)
        den_a = 1.0 - p.mob_phi * p.grad_coeff_phi * dt * self.K2
        new_phi = np.empty_like(phi)
        for i in range(var):
            ph = self.F(phi[i])
            dh = self.F(df_dphi[i])
            new_phi[i] = self.Finv((ph - p.mob_phi * dt * dh) / den_a)
        self.phi = new_phi
        self.step_no += 1
        return Diag(f_int=f_int, f_eta=f_eta, f_ch=f_ch, mass=float(np.sum(self.con, dtype=np.float64)),
                    **stats(self.phi, self.con))


def stats(phi: np.ndarray, con: np.ndarray) -> dict:
    """End-of-step statistics, ``src/var_diff.f90:1076-1102``: note the
    starting values (phi_min 1.0, phi_3 0.0, c_max 0.0, c_min 1.0) act as
    clamps."""
    sq = np.sum(phi.astype(np.float64) ** 2, axis=0)
    return dict(
        c_min=min(1.0, float(np.min(con))),
        c_max=max(0.0, float(np.max(con))),
        phi_min=min(1.0, float(np.min(sq))),
        phi_P_max=max(0.0, float(np.max(phi[-1]))),
    )


def run(p: Params, phi, con, steps: int, faithful: bool = True, workers: int = 1, dtype=np.float64):
    """Run ``steps`` steps; return (phi, con, [Diag per step])."""
    o = Oracle(p, phi, con, faithful=faithful, workers=workers, dtype=dtype)
    diags = [o.step() for _ in range(steps)]
    return o.phi, o.con, diags


# ---------------------------------------------------------------------------
# Layout helpers for the Fortran phi(var, x, y, z) order
# ---------------------------------------------------------------------------
def to_fortran_aos(phi: np.ndarray) -> np.ndarray:
    """phi[ivar, z, y, x] -> flat buffer in Fortran phi(var, x, y, z) order."""
    return np.ascontiguousarray(np.moveaxis(phi, 0, -1)).reshape(-1)


def from_fortran_aos(buf: np.ndarray, var: int, Nx: int, Ny: int, Nz: int) -> np.ndarray:
    return np.ascontiguousarray(np.moveaxis(np.asarray(buf).reshape(Nz, Ny, Nx, var), -1, 0))
