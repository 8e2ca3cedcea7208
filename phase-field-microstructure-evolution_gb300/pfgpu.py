"""ctypes binding of libpfgpu.so (include/pfgpu.h).

Field arrays on the Python side use the layout ``phi[ivar, z, y, x]`` and
``con[z, y, x]`` (C order, x fastest); they are converted to the Fortran
``phi(var, x, y, z)`` order of the C ABI on the way in and out.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path
from typing import List, Optional, Sequence

import numpy as np

from . import build as _build

PF_OK, PF_EINVAL, PF_ECUDA, PF_ENOMEM, PF_ENONFINITE, PF_EIO, PF_EBUSY = 0, -1, -2, -3, -4, -5, -6
PF_REQ_QUEUED, PF_REQ_RUNNING, PF_REQ_DONE, PF_REQ_FAILED = 0, 1, 2, 3
PF_MOB_REFERENCE, PF_MOB_C1MC = 0, 1
PF_FP32_FUSED, PF_FP64_PLAIN = 32, 64

EXPORTED = (
    "pf_create", "pf_supported_shape", "pf_set_fields", "pf_step", "pf_get_fields", "pf_destroy",
    "pf_last_error", "pf_batch_create", "pf_batch_set_fields", "pf_batch_step", "pf_batch_get_fields",
    "pf_batch_destroy", "f_trans_", "inv_trans_", "k_space_", "pf_shim_device", "pf_ran2_init", "pf_ran2",
    "pf_ic_noise", "pf_ic_voronoi", "pf_diag_fields_noalloc", "pf_io_last_error", "pf_read_input",
    "pf_input_to_config", "pf_write_data_save", "pf_read_data_save", "pf_ic_circle", "pf_ic_plane",
    "pf_ic_polycryst", "pf_insert_precipitates", "pf_format_e", "pf_format_summary", "pf_format_list_int",
    "pf_format_list_real", "pf_analyze_fields", "pf_analyze_run", "pf_write_vtk_real", "pf_write_vtk_int",
    "pf_server_create", "pf_server_submit", "pf_server_poll", "pf_server_wait", "pf_server_destroy",
    "pf_server_last_error", "pf_check_fp64", "pf_device_count", "pf_run_work", "pf_pick_device", "pf_place_units", "pf_pool_create", "pf_pool_devices",
    "pf_pool_submit", "pf_pool_wait", "pf_pool_destroy", "pf_pool_last_error",
)


class PFError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"pfgpu error {code}: {msg}")
        self.code = code


class Config(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("var", C.c_int),
        ("t_step", C.c_double), ("grad_coeff_phi", C.c_double), ("grad_coeff_c", C.c_double),
        ("D_S", C.c_double), ("D_L", C.c_double), ("D_gb", C.c_double), ("mob_phi", C.c_double),
        ("sigma_1", C.c_double), ("sigma_2", C.c_double),
        ("am", C.c_double), ("ap", C.c_double), ("con_0_mat", C.c_double), ("con_0_ppt", C.c_double),
        ("mobility", C.c_int), ("precision", C.c_int), ("device", C.c_int), ("reserved", C.c_int * 5),
    ]


class Diag(C.Structure):
    _fields_ = [
        ("step", C.c_int), ("nonfinite", C.c_int),
        ("f_int", C.c_double), ("f_eta", C.c_double), ("f_ch", C.c_double), ("e_tot", C.c_double),
        ("c_max", C.c_double), ("c_min", C.c_double), ("phi_min", C.c_double), ("phi_P_max", C.c_double),
        ("mass", C.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Ran2State(C.Structure):
    _fields_ = [("idum2", C.c_int), ("iy", C.c_int), ("iv", C.c_int * 32), ("initialised", C.c_int),
                ("pad", C.c_int * 5)]


class Input(C.Structure):
    """pf_input: the values of input.txt plus the key=value extensions."""
    _fields_ = [
        ("nrun", C.c_int), ("ppt_int", C.c_int), ("ppt_rad", C.c_int * 3), ("N_step", C.c_int),
        ("ifreq", C.c_int), ("i_ppt", C.c_int), ("j_ppt", C.c_int), ("k_ppt", C.c_int), ("iseed", C.c_int),
        ("grn_rad", C.c_int), ("num_ppt", C.c_int), ("c_mat", C.c_double), ("c_ppt", C.c_double),
        ("Nx", C.c_int), ("Ny", C.c_int), ("Nz", C.c_int), ("var", C.c_int),
        ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double), ("t_step", C.c_double),
        ("grad_coeff_phi", C.c_double), ("grad_coeff_c", C.c_double), ("D_S", C.c_double),
        ("D_L", C.c_double), ("D_gb", C.c_double), ("mob_phi", C.c_double),
        ("sigma_1", C.c_double), ("sigma_2", C.c_double),
        ("am", C.c_double), ("ap", C.c_double), ("con_0_mat", C.c_double), ("con_0_ppt", C.c_double),
        ("gb_force", C.c_double), ("ndim", C.c_int), ("dims", C.c_int * 2), ("start", C.c_char * 16),
        ("set_mask", C.c_ulonglong),
        ("seed", C.c_int), ("n_grains", C.c_int), ("mobility_code", C.c_int), ("precision", C.c_int),
        ("amp_phi", C.c_double), ("amp_c", C.c_double), ("c0", C.c_double), ("microstructure", C.c_char * 256),
        ("check_fp64", C.c_int),
    ]

    @property
    def mobility(self):
        return "c1mc" if self.mobility_code == PF_MOB_C1MC else "reference"


class ErrorReport(C.Structure):
    _fields_ = [("steps", C.c_int), ("pad", C.c_int), ("phi_max_abs_rel", C.c_double), ("phi_l2_rel", C.c_double),
                ("c_max_abs_rel", C.c_double), ("c_l2_rel", C.c_double)]


class ServerConfig(C.Structure):
    _fields_ = [("device", C.c_int), ("max_active", C.c_int), ("hbm_budget_bytes", C.c_double),
                ("chunk_steps", C.c_int), ("reserved", C.c_int * 5)]


class PoolConfig(C.Structure):
    _fields_ = [("ndevices", C.c_int), ("devices", C.POINTER(C.c_int)), ("server", ServerConfig)]


class RequestTimes(C.Structure):
    _fields_ = [("queued_s", C.c_double), ("run_s", C.c_double), ("total_s", C.c_double)]


class VoxelCounts(C.Structure):
    _fields_ = [("precipitate_voxels", C.c_longlong), ("boundary_voxels", C.c_longlong),
                ("precipitate_fraction", C.c_double)]


class AnalysisOut(C.Structure):
    _fields_ = [("phi_sq", C.POINTER(C.c_double)), ("var_num", C.POINTER(C.c_int)),
                ("phi_3", C.POINTER(C.c_double)), ("grad_phi_3", C.POINTER(C.c_double)),
                ("boundary", C.POINTER(C.c_double)), ("con", C.POINTER(C.c_double))]


_LIB = None


def library_path() -> Path:
    return _build.LIB


def load_library(build_if_missing: bool = True) -> C.CDLL:
    """Load (building first if needed) the in-tree libpfgpu.so."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if not path.exists():
        if not build_if_missing:
            raise FileNotFoundError(f"{path} is missing: run build() first")
        _build.build()
    lib = C.CDLL(str(path))
    P = C.POINTER
    dp = P(C.c_double)
    ip = P(C.c_int)
    sig = {
        "pf_create": (C.c_int, [P(Config), P(C.c_void_p)]),
        "pf_supported_shape": (C.c_int, [C.c_int] * 5),
        "pf_set_fields": (C.c_int, [C.c_void_p, dp, dp]),
        "pf_step": (C.c_int, [C.c_void_p, C.c_int, P(Diag)]),
        "pf_get_fields": (C.c_int, [C.c_void_p, dp, dp]),
        "pf_destroy": (C.c_int, [C.c_void_p]),
        "pf_last_error": (C.c_char_p, []),
        "pf_batch_create": (C.c_int, [P(Config), C.c_int, P(C.c_void_p)]),
        "pf_batch_set_fields": (C.c_int, [C.c_void_p, C.c_int, dp, dp]),
        "pf_batch_step": (C.c_int, [C.c_void_p, C.c_int, P(Diag)]),
        "pf_batch_get_fields": (C.c_int, [C.c_void_p, C.c_int, dp, dp]),
        "pf_batch_destroy": (C.c_int, [C.c_void_p]),
        "pf_batch_enqueue": (C.c_int, [C.c_void_p, C.c_int]),
        "pf_batch_enqueue_phase": (C.c_int, [C.c_void_p, C.c_int]),
        "pf_batch_stream": (C.c_void_p, [C.c_void_p]),
        "pf_batch_variant": (C.c_char_p, [C.c_void_p]),
        "pf_run_batch": (C.c_void_p, [C.c_void_p]),
        "pf_batch_c_mean": (C.c_int, [C.c_void_p, C.c_int, dp]),
        "pf_batch_ring": (C.c_int, [C.c_void_p]),
        "pf_variant_counts": (None, [C.c_int, C.c_int, C.c_int, ip, ip]),
        "f_trans_": (None, [dp, dp, ip, ip, ip, ip, ip, ip, ip]),
        "inv_trans_": (None, [dp, dp, ip, ip, ip, ip]),
        "k_space_": (None, [ip, ip, ip, ip, ip, dp, dp, dp]),
        "pf_shim_device": (C.c_int, [C.c_int]),
        "pf_ran2_init": (None, [P(Ran2State)]),
        "pf_ran2": (C.c_double, [P(Ran2State), ip]),
        "pf_ic_noise": (C.c_int, [P(Config), C.c_int, C.c_double, C.c_double, C.c_double, dp, dp]),
        "pf_ic_voronoi": (C.c_int, [P(Config), C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, dp, dp]),
        "pf_diag_fields_noalloc": (C.c_int, [P(Config), C.c_void_p, P(Diag), C.c_void_p]),
        "pf_io_last_error": (C.c_char_p, []),
        "pf_read_input": (C.c_int, [C.c_char_p, C.c_int, P(Input)]),
        "pf_input_to_config": (None, [P(Input), P(Config)]),
        "pf_write_data_save": (C.c_int, [C.c_char_p, P(Config), dp, dp]),
        "pf_read_data_save": (C.c_int, [C.c_char_p, P(Config), dp, dp]),
        "pf_ic_circle": (C.c_int, [P(Config), C.c_int, ip, C.c_int, ip, C.c_double, C.c_double, P(Ran2State),
                                   dp, dp]),
        "pf_ic_plane": (C.c_int, [P(Config), ip, C.c_int, C.c_int, C.c_int, C.c_double, dp, dp]),
        "pf_ic_polycryst": (C.c_int, [P(Config), C.c_char_p, C.c_double, dp, dp]),
        "pf_insert_precipitates": (C.c_int, [P(Config), ip, C.c_int, ip, P(Ran2State), dp]),
        "pf_format_e": (None, [C.c_double, C.c_int, C.c_int, C.c_char_p]),
        "pf_format_summary": (None, [C.c_int, P(Diag), C.c_char_p]),
        "pf_format_list_int": (None, [C.c_int, C.c_char_p]),
        "pf_format_list_real": (None, [C.c_double, C.c_char_p]),
        "pf_analyze_fields": (C.c_int, [P(Config), dp, dp, C.c_double, P(AnalysisOut), P(VoxelCounts)]),
        "pf_analyze_run": (C.c_int, [C.c_void_p, C.c_double, P(AnalysisOut), P(VoxelCounts)]),
        "pf_write_vtk_real": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_int, dp]),
        "pf_write_vtk_int": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_int, P(C.c_int)]),
        "pf_server_create": (C.c_int, [P(ServerConfig), P(C.c_void_p)]),
        "pf_server_submit": (C.c_int, [C.c_void_p, P(Config), dp, dp, C.c_int, P(C.c_longlong)]),
        "pf_server_poll": (C.c_int, [C.c_void_p, C.c_longlong, ip]),
        "pf_server_wait": (C.c_int, [C.c_void_p, C.c_longlong, C.c_double, dp, dp, P(Diag), P(RequestTimes)]),
        "pf_server_destroy": (C.c_int, [C.c_void_p]),
        "pf_server_last_error": (C.c_char_p, []),
        "pf_device_count": (C.c_int, []),
        "pf_check_fp64": (C.c_int, [P(Config), dp, dp, C.c_int, P(ErrorReport)]),
        "pf_run_work": (C.c_double, [P(Config), C.c_int]),
        "pf_pick_device": (C.c_int, [dp, C.c_int]),
        "pf_place_units": (C.c_int, [dp, C.c_int, C.c_int, ip, dp]),
        "pf_pool_create": (C.c_int, [P(PoolConfig), P(C.c_void_p)]),
        "pf_pool_devices": (C.c_int, [C.c_void_p]),
        "pf_pool_submit": (C.c_int, [C.c_void_p, P(Config), dp, dp, C.c_int, P(C.c_longlong), ip]),
        "pf_pool_wait": (C.c_int, [C.c_void_p, C.c_longlong, C.c_double, dp, dp, P(Diag), P(RequestTimes)]),
        "pf_pool_destroy": (C.c_int, [C.c_void_p]),
        "pf_pool_last_error": (C.c_char_p, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def _check(rc: int):
    if rc != PF_OK:
        msg = load_library().pf_last_error().decode()
        raise PFError(rc, msg)


def make_config(p, precision: int = PF_FP32_FUSED, device: int = 0) -> Config:
    """Config from any object with the input.txt attribute names (e.g. the
    oracle's Params or the input-file reader's record)."""
    c = Config()
    c.nx, c.ny, c.nz, c.var = p.Nx, p.Ny, p.Nz, p.var
    for k in ("t_step", "grad_coeff_phi", "grad_coeff_c", "D_S", "D_L", "D_gb", "mob_phi",
              "sigma_1", "sigma_2", "am", "ap", "con_0_mat", "con_0_ppt"):
        setattr(c, k, float(getattr(p, k)))
    mob = getattr(p, "mobility", "reference")
    c.mobility = PF_MOB_C1MC if mob in ("c1mc", PF_MOB_C1MC) else PF_MOB_REFERENCE
    c.precision = precision
    c.device = device
    return c


def to_aos(phi: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(np.moveaxis(np.asarray(phi, dtype=np.float64), 0, -1))


def from_aos(buf: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(np.moveaxis(buf, -1, 0))


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Run:
    """One run behind pf_create/pf_set_fields/pf_step/pf_get_fields."""

    def __init__(self, params, precision: int = PF_FP32_FUSED, device: int = 0):
        self.lib = load_library()
        self.p = params
        self.cfg = make_config(params, precision, device)
        h = C.c_void_p()
        _check(self.lib.pf_create(C.byref(self.cfg), C.byref(h)))
        self.h = h

    def set_fields(self, phi: np.ndarray, con: np.ndarray):
        a = to_aos(phi)
        c = np.ascontiguousarray(con, dtype=np.float64)
        _check(self.lib.pf_set_fields(self.h, _dp(a), _dp(c)))

    def set_fields_aos(self, phi_aos: np.ndarray, con: np.ndarray):
        """Upload buffers already in the Fortran phi(var,x,y,z) layout."""
        _check(self.lib.pf_set_fields(self.h, _dp(phi_aos), _dp(con)))

    def get_fields_aos(self, phi_aos: np.ndarray, con: np.ndarray):
        _check(self.lib.pf_get_fields(self.h, _dp(phi_aos), _dp(con)))

    def step(self, n: int, raise_nonfinite: bool = True) -> List[dict]:
        d = (Diag * max(n, 1))()
        rc = self.lib.pf_step(self.h, n, d)
        if rc != PF_ENONFINITE or raise_nonfinite:
            _check(rc)
        return [d[i].as_dict() for i in range(n)]

    def get_fields(self):
        p = self.p
        a = np.empty((p.Nz, p.Ny, p.Nx, p.var))
        c = np.empty((p.Nz, p.Ny, p.Nx))
        _check(self.lib.pf_get_fields(self.h, _dp(a), _dp(c)))
        return from_aos(a), c

    def batch_handle(self):
        return self.lib.pf_run_batch(self.h)

    def c_mean(self) -> complex:
        """The k = 0 coefficient of the resident concentration state (fused
        path): the mean of c, so N^3 times its real part is the mass."""
        v = (C.c_double * 2)()
        _check(self.lib.pf_batch_c_mean(self.batch_handle(), 0, v))
        return complex(v[0], v[1])

    def close(self):
        if getattr(self, "h", None):
            self.lib.pf_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Same-shape runs stepped by one set of launches (pf_batch_*)."""

    def __init__(self, params_list: Sequence, device: int = 0):
        self.lib = load_library()
        self.ps = list(params_list)
        arr = (Config * len(self.ps))(*[make_config(p, PF_FP32_FUSED, device) for p in self.ps])
        self._cfgs = arr
        h = C.c_void_p()
        _check(self.lib.pf_batch_create(arr, len(self.ps), C.byref(h)))
        self.h = h

    def set_fields(self, run: int, phi, con):
        a = to_aos(phi)
        c = np.ascontiguousarray(con, dtype=np.float64)
        _check(self.lib.pf_batch_set_fields(self.h, run, _dp(a), _dp(c)))

    def step(self, n: int) -> List[List[dict]]:
        R = len(self.ps)
        d = (Diag * max(R * n, 1))()
        _check(self.lib.pf_batch_step(self.h, n, d))
        return [[d[r * n + i].as_dict() for i in range(n)] for r in range(R)]

    def get_fields(self, run: int):
        p = self.ps[run]
        a = np.empty((p.Nz, p.Ny, p.Nx, p.var))
        c = np.empty((p.Nz, p.Ny, p.Nx))
        _check(self.lib.pf_batch_get_fields(self.h, run, _dp(a), _dp(c)))
        return from_aos(a), c

    def close(self):
        if getattr(self, "h", None):
            self.lib.pf_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def check_fp64(p, phi: np.ndarray, con: np.ndarray, nsteps: int, device: int = 0) -> dict:
    """The run's error against the FP64 GPU path after nsteps steps of the
    start (phi[ivar,z,y,x], con[z,y,x]): max-abs and L2 differences relative to
    the FP64 fields' max-abs and L2 norms (pf_check_fp64)."""
    lib = load_library()
    cfg = make_config(p, PF_FP32_FUSED, device)
    a = to_aos(phi)
    c = np.ascontiguousarray(con, dtype=np.float64)
    rep = ErrorReport()
    _check(lib.pf_check_fp64(C.byref(cfg), _dp(a), _dp(c), int(nsteps), C.byref(rep)))
    return {k: getattr(rep, k) for k, _ in rep._fields_ if k != "pad"}


def _ic_buffers(p, pinned: bool):
    shape_phi = (p.Nz, p.Ny, p.Nx, p.var)
    shape_c = (p.Nz, p.Ny, p.Nx)
    if pinned:
        import torch

        a = torch.empty(shape_phi, dtype=torch.float64, pin_memory=True).numpy()
        c = torch.empty(shape_c, dtype=torch.float64, pin_memory=True).numpy()
        return a, c
    return np.empty(shape_phi), np.empty(shape_c)


def ic_noise_aos(p, seed: int, amp_phi: float, c0: float, amp_c: float, pinned: bool = False):
    """Noise start in the Fortran layout of the C ABI: (phi(var,x,y,z), con)."""
    lib = load_library()
    a, c = _ic_buffers(p, pinned)
    cfg = make_config(p)
    _check(lib.pf_ic_noise(C.byref(cfg), seed, amp_phi, c0, amp_c, _dp(a), _dp(c)))
    return a, c


def ic_voronoi_aos(p, seed: int, n_grains: int, amp_phi: float, c0: float, amp_c: float, pinned: bool = False):
    lib = load_library()
    a, c = _ic_buffers(p, pinned)
    cfg = make_config(p)
    _check(lib.pf_ic_voronoi(C.byref(cfg), seed, n_grains, amp_phi, c0, amp_c, _dp(a), _dp(c)))
    return a, c


def ic_noise(p, seed, amp_phi, c0, amp_c):
    a, c = ic_noise_aos(p, seed, amp_phi, c0, amp_c)
    return from_aos(a), c


def ic_voronoi(p, seed, n_grains, amp_phi, c0, amp_c):
    a, c = ic_voronoi_aos(p, seed, n_grains, amp_phi, c0, amp_c)
    return from_aos(a), c


class Ran2:
    """The library's C restatement of ran_2 (for cross-checks and host ICs)."""

    def __init__(self, idum: int):
        self.lib = load_library()
        self.st = Ran2State()
        self.lib.pf_ran2_init(C.byref(self.st))
        self.idum = C.c_int(idum)

    def next(self) -> float:
        return self.lib.pf_ran2(C.byref(self.st), C.byref(self.idum))


# ---------------------------------------------------------------------------
# input.txt, restart files, the reference's starts and output formats
# ---------------------------------------------------------------------------
def _check_io(rc: int):
    if rc != PF_OK:
        raise PFError(rc, load_library().pf_io_last_error().decode())


def driver_path() -> Path:
    """The pf_var_diff executable (built next to the library)."""
    return _build.EXE


def read_input(path, nprocs: int = 1) -> Input:
    """input.txt with Fortran list-directed rules (pf_read_input)."""
    lib = load_library()
    rec = Input()
    _check_io(lib.pf_read_input(str(path).encode(), nprocs, C.byref(rec)))
    return rec


def input_to_config(rec: Input) -> Config:
    c = Config()
    load_library().pf_input_to_config(C.byref(rec), C.byref(c))
    return c


def write_data_save(path, p, phi: np.ndarray, con: np.ndarray):
    """data_save file of phi[ivar,z,y,x], con[z,y,x] (REAL*8, Fortran unformatted)."""
    lib = load_library()
    cfg = make_config(p)
    a = to_aos(phi)
    c = np.ascontiguousarray(con, dtype=np.float64)
    _check_io(lib.pf_write_data_save(str(path).encode(), C.byref(cfg), _dp(a), _dp(c)))


def read_data_save(path, p):
    lib = load_library()
    cfg = make_config(p)
    a = np.empty((p.Nz, p.Ny, p.Nx, p.var))
    c = np.empty((p.Nz, p.Ny, p.Nx))
    _check_io(lib.pf_read_data_save(str(path).encode(), C.byref(cfg), _dp(a), _dp(c)))
    return from_aos(a), c


def _ints(v):
    return (C.c_int * len(v))(*[int(x) for x in v])


def ic_circle(p, grn_rad: int, ppt_rad, num_ppt: int, iseed: int, c_mat: float, con_0_ppt: float,
              rng: Optional["Ran2"] = None):
    """'circle' start; returns (phi, con, rng) with rng advanced (its idum too)."""
    lib = load_library()
    rng = rng or Ran2(iseed)
    cfg = make_config(p)
    a, c = _ic_buffers(p, False)
    _check_io(lib.pf_ic_circle(C.byref(cfg), grn_rad, _ints(ppt_rad), num_ppt, C.byref(rng.idum), c_mat,
                               con_0_ppt, C.byref(rng.st), _dp(a), _dp(c)))
    return from_aos(a), c, rng


def ic_plane(p, ppt_rad, i_ppt: int, j_ppt: int, k_ppt: int, c_mat: float):
    lib = load_library()
    cfg = make_config(p)
    a, c = _ic_buffers(p, False)
    _check_io(lib.pf_ic_plane(C.byref(cfg), _ints(ppt_rad), i_ppt, j_ppt, k_ppt, c_mat, _dp(a), _dp(c)))
    return from_aos(a), c


def ic_polycryst(p, path, c_mat: float):
    lib = load_library()
    cfg = make_config(p)
    a, c = _ic_buffers(p, False)
    _check_io(lib.pf_ic_polycryst(C.byref(cfg), str(path).encode(), c_mat, _dp(a), _dp(c)))
    return from_aos(a), c


def insert_precipitates(p, phi: np.ndarray, ppt_rad, num_ppt: int, rng: "Ran2") -> np.ndarray:
    """Precipitate insertion of step ppt_int; returns the new phi (rng advanced)."""
    lib = load_library()
    cfg = make_config(p)
    a = to_aos(phi)
    _check_io(lib.pf_insert_precipitates(C.byref(cfg), _ints(ppt_rad), num_ppt, C.byref(rng.idum),
                                         C.byref(rng.st), _dp(a)))
    return from_aos(a)


def format_e(x: float, w: int, d: int) -> str:
    buf = C.create_string_buffer(w + 8)
    load_library().pf_format_e(x, w, d, buf)
    return buf.value.decode()


def format_summary(step: int, diag: Diag) -> str:
    buf = C.create_string_buffer(256)
    load_library().pf_format_summary(step, C.byref(diag), buf)
    return buf.value.decode()


def format_list_int(v: int) -> str:
    buf = C.create_string_buffer(64)
    load_library().pf_format_list_int(v, buf)
    return buf.value.decode()


def format_list_real(v: float) -> str:
    buf = C.create_string_buffer(64)
    load_library().pf_format_list_real(v, buf)
    return buf.value.decode()


# ---------------------------------------------------------------------------
# voxel analysis of paraview.x and its VTK files
# ---------------------------------------------------------------------------
ANALYSIS_FIELDS = ("phi_sq", "var_num", "phi_3", "grad_phi_3", "boundary", "con")


def _analysis_out(shape, want):
    arrays, out = {}, AnalysisOut()
    for k in ANALYSIS_FIELDS:
        if k in want:
            a = np.empty(shape, dtype=np.int32 if k == "var_num" else np.float64)
            arrays[k] = a
            setattr(out, k, a.ctypes.data_as(C.POINTER(C.c_int if k == "var_num" else C.c_double)))
    return arrays, out


def _counts(c: VoxelCounts) -> dict:
    return dict(precipitate_voxels=c.precipitate_voxels, boundary_voxels=c.boundary_voxels,
                precipitate_fraction=c.precipitate_fraction)


def analyze_fields(p, phi: np.ndarray, con: np.ndarray, threshold: float, device: int = 0,
                   want=ANALYSIS_FIELDS[:5]) -> dict:
    """GPU voxel analysis of phi[ivar,z,y,x], con[z,y,x]; arrays are [z,y,x]."""
    lib = load_library()
    cfg = make_config(p, device=device)
    a = to_aos(phi)
    c = np.ascontiguousarray(con, dtype=np.float64)
    arrays, out = _analysis_out((p.Nz, p.Ny, p.Nx), [k for k in want if k != "con"])
    cnt = VoxelCounts()
    _check(lib.pf_analyze_fields(C.byref(cfg), _dp(a), _dp(c), threshold, C.byref(out), C.byref(cnt)))
    arrays.update(_counts(cnt))
    return arrays


def analyze_run(run: "Run", threshold: float, want=()) -> dict:
    """In-situ analysis of a run's resident fields (counts, plus the arrays in want)."""
    lib = load_library()
    p = run.p
    arrays, out = _analysis_out((p.Nz, p.Ny, p.Nx), want)
    cnt = VoxelCounts()
    _check(lib.pf_analyze_run(run.h, threshold, C.byref(out) if want else None, C.byref(cnt)))
    arrays.update(_counts(cnt))
    return arrays


def write_vtk(path, values: np.ndarray):
    """ASCII VTK file of values[z, y, x] (float64 or int32) in paraview.x's layout."""
    lib = load_library()
    nz, ny, nx = values.shape
    if values.dtype.kind in "iu":
        v = np.ascontiguousarray(values, dtype=np.int32)
        rc = lib.pf_write_vtk_int(str(path).encode(), nx, ny, nz, v.ctypes.data_as(C.POINTER(C.c_int)))
    else:
        v = np.ascontiguousarray(values, dtype=np.float64)
        rc = lib.pf_write_vtk_real(str(path).encode(), nx, ny, nz, _dp(v))
    _check_io(rc)


def paraview_path() -> Path:
    """The pf_paraview executable (built next to the library)."""
    return _build.PARAVIEW_EXE


def sweep_path() -> Path:
    """The pf_sweep executable (built next to the library)."""
    return _build.SWEEP_EXE


def sweep(case_dirs, max_batch: int = 64, timeout: Optional[float] = None):
    """Run var_diff.x cases (directories holding an input.txt) through
    pf_sweep; returns the CompletedProcess (exit status 0 when every case
    finished, 2 or 3 when one failed; see pf_sweep.cpp)."""
    import subprocess

    cmd = [str(sweep_path()), "--max-batch", str(max_batch)] + [str(d) for d in case_dirs]
    return subprocess.run(cmd, capture_output=True, text=True, timeout=timeout)


def variant_counts(nx: int, ny: int, nz: int):
    """(x-pass, yz-pass) compiled variants of a grid: the ranges of
    PFGPU_X_VARIANT and PFGPU_YZ_VARIANT."""
    a, b = C.c_int(0), C.c_int(0)
    load_library().pf_variant_counts(nx, ny, nz, C.byref(a), C.byref(b))
    return a.value, b.value


# ---------------------------------------------------------------------------
# serving: continuous batching of independent runs
# ---------------------------------------------------------------------------
class Server:
    """pf_server: submit runs, poll or wait for them (see include/pfgpu.h)."""

    def __init__(self, device: int = 0, max_active: int = 0, hbm_budget_bytes: float = 0.0, chunk_steps: int = 0):
        self.lib = load_library()
        cfg = ServerConfig()
        cfg.device, cfg.max_active, cfg.hbm_budget_bytes, cfg.chunk_steps = device, max_active, hbm_budget_bytes, \
            chunk_steps
        h = C.c_void_p()
        rc = self.lib.pf_server_create(C.byref(cfg), C.byref(h))
        if rc != PF_OK:
            raise PFError(rc, self.lib.pf_server_last_error().decode())
        self.h = h
        self.device = device
        self._shape = {}

    def _check(self, rc):
        if rc != PF_OK:
            raise PFError(rc, self.lib.pf_server_last_error().decode())

    def submit(self, params, phi: np.ndarray, con: np.ndarray, nsteps: int) -> int:
        """Queue a run (fields phi[ivar,z,y,x], con[z,y,x]); returns its id."""
        cfg = make_config(params, PF_FP32_FUSED, self.device)
        a = to_aos(phi)
        c = np.ascontiguousarray(con, dtype=np.float64)
        rid = C.c_longlong()
        self._check(self.lib.pf_server_submit(self.h, C.byref(cfg), _dp(a), _dp(c), int(nsteps), C.byref(rid)))
        self._shape[rid.value] = (params.var, params.Nz, params.Ny, params.Nx)
        return rid.value

    def poll(self, rid: int) -> int:
        st = C.c_int()
        self._check(self.lib.pf_server_poll(self.h, rid, C.byref(st)))
        return st.value

    def wait(self, rid: int, timeout: float = -1.0):
        """(phi, con, last record dict, times dict) of a finished run."""
        var, nz, ny, nx = self._shape.pop(rid)
        a = np.empty((nz, ny, nx, var))
        c = np.empty((nz, ny, nx))
        d = Diag()
        t = RequestTimes()
        rc = self.lib.pf_server_wait(self.h, rid, timeout, _dp(a), _dp(c), C.byref(d), C.byref(t))
        if rc == PF_EBUSY:
            self._shape[rid] = (var, nz, ny, nx)
        self._check(rc)
        return from_aos(a), c, d.as_dict(), {k: getattr(t, k) for k, _ in t._fields_}

    def close(self):
        if getattr(self, "h", None):
            self.lib.pf_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# independent runs over the node's GPUs (placement only, no collective)
# ---------------------------------------------------------------------------
def place_units(work, ndev: int):
    """LPT placement of work units on ndev devices (pf_place_units): returns
    (device of each unit, work per device)."""
    lib = load_library()
    w = np.ascontiguousarray(work, dtype=np.float64)
    dev = np.empty(len(w), dtype=np.int32)
    load = np.empty(ndev, dtype=np.float64)
    _check(lib.pf_place_units(_dp(w), len(w), ndev, dev.ctypes.data_as(C.POINTER(C.c_int)), _dp(load)))
    return dev, load


def pick_device(outstanding) -> int:
    o = np.ascontiguousarray(outstanding, dtype=np.float64)
    return load_library().pf_pick_device(_dp(o), len(o))


class Pool:
    """pf_pool: one pf_server per device, each run placed on the device with
    the least outstanding work."""

    def __init__(self, ndevices: int = 0, max_active: int = 0, hbm_budget_bytes: float = 0.0, chunk_steps: int = 0):
        self.lib = load_library()
        cfg = PoolConfig()
        cfg.ndevices = ndevices
        cfg.server.max_active, cfg.server.hbm_budget_bytes, cfg.server.chunk_steps = max_active, hbm_budget_bytes, \
            chunk_steps
        h = C.c_void_p()
        rc = self.lib.pf_pool_create(C.byref(cfg), C.byref(h))
        if rc != PF_OK:
            raise PFError(rc, self.lib.pf_pool_last_error().decode())
        self.h = h
        self.devices = self.lib.pf_pool_devices(h)
        self._shape = {}

    def submit(self, params, phi: np.ndarray, con: np.ndarray, nsteps: int):
        """Queue a run; returns (id, device ordinal)."""
        return self.submit_aos(params, to_aos(phi), np.ascontiguousarray(con, dtype=np.float64), nsteps)

    def submit_aos(self, params, phi_aos: np.ndarray, con: np.ndarray, nsteps: int):
        """submit() with the order parameters already in the Fortran
        phi(var,x,y,z) layout (C-contiguous float64 [z][y][x][var]), which the
        library copies as they are."""
        assert phi_aos.dtype == np.float64 and phi_aos.flags.c_contiguous and con.flags.c_contiguous
        cfg = make_config(params, PF_FP32_FUSED, 0)
        rid, dev = C.c_longlong(), C.c_int()
        rc = self.lib.pf_pool_submit(self.h, C.byref(cfg), _dp(phi_aos), _dp(con), int(nsteps), C.byref(rid),
                                     C.byref(dev))
        if rc != PF_OK:
            raise PFError(rc, self.lib.pf_pool_last_error().decode())
        self._shape[rid.value] = (params.var, params.Nz, params.Ny, params.Nx)
        return rid.value, dev.value

    def wait(self, rid: int, timeout: float = -1.0):
        a, c, d, t = self.wait_aos(rid, timeout)
        return from_aos(a), c, d, t

    def wait_aos(self, rid: int, timeout: float = -1.0):
        """wait() returning the order parameters in the phi(var,x,y,z) layout."""
        var, nz, ny, nx = self._shape.pop(rid)
        a = np.empty((nz, ny, nx, var))
        c = np.empty((nz, ny, nx))
        d = Diag()
        t = RequestTimes()
        rc = self.lib.pf_pool_wait(self.h, rid, timeout, _dp(a), _dp(c), C.byref(d), C.byref(t))
        if rc == PF_EBUSY:
            self._shape[rid] = (var, nz, ny, nx)
        if rc != PF_OK:
            raise PFError(rc, self.lib.pf_pool_last_error().decode())
        return a, c, d.as_dict(), {k: getattr(t, k) for k, _ in t._fields_}

    def close(self):
        if getattr(self, "h", None):
            self.lib.pf_pool_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
