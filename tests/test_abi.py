"""The C-ABI library loads and exports every entry point of include/pfgpu.h
(no GPU needed; no compute calls)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def _declared():
    txt = (ROOT / "include" / "pfgpu.h").read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    names = re.findall(r"\b(?:int|void|double|const char\*)\s+\**\s*([A-Za-z_][A-Za-z0-9_]*)\s*\(", txt)
    return sorted(set(names))


def test_header_symbols_exported(lib):
    names = _declared()
    assert "pf_create" in names and "f_trans_" in names and len(names) >= 18
    for n in names:
        assert hasattr(lib, n), f"{n} declared in pfgpu.h but not exported"


def test_python_binding_covers_header(pkg):
    assert set(pkg.EXPORTED) <= set(_declared())


def test_supported_shapes(lib):
    assert lib.pf_supported_shape(128, 128, 128, 16, 32) == 1
    assert lib.pf_supported_shape(256, 256, 256, 32, 32) == 1
    assert lib.pf_supported_shape(64, 32, 64, 4, 32) == 1
    assert lib.pf_supported_shape(96, 96, 96, 55, 32) == 1  # the reference's own grid and var
    assert lib.pf_supported_shape(48, 48, 48, 4, 32) == 0  # not a fused-path size
    assert lib.pf_supported_shape(48, 48, 48, 4, 64) == 1  # the FP64 path takes any even Nx
    # the x pass's tile of every field plus its static tables within 227 KB
    assert lib.pf_supported_shape(128, 128, 128, 97, 32) == 1
    assert lib.pf_supported_shape(128, 128, 128, 98, 32) == 0  # x-pass rows no longer fit
    assert lib.pf_supported_shape(96, 96, 96, 129, 32) == 1
    assert lib.pf_supported_shape(96, 96, 96, 130, 32) == 0
    assert lib.pf_supported_shape(256, 256, 256, 195, 32) == 1  # one-row tiles of 196 fields
    assert lib.pf_supported_shape(256, 256, 256, 196, 32) == 0
    assert lib.pf_supported_shape(64, 64, 64, 256, 32) == 0  # var limit


def test_create_rejects_bad_config(pkg, oracle):
    with pytest.raises(pkg.PFError) as e:
        pkg.Run(oracle.Params(48, 48, 48, 4))
    assert e.value.code == -1 and "Nx=48" in str(e.value)


def test_k_space_shim_matches_oracle(lib, oracle):
    Nx, Ny, Nz = 8, 6, 4
    fst = (C.c_int * 3)(1, 1, 1)
    fen = (C.c_int * 3)(Nz, Ny, Nx // 2 + 1)
    n = Nz * Ny * (Nx // 2 + 1)
    kf, ksq, k4 = (np.zeros((n, 3, 2)) for _ in range(3))
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    ci = lambda v: C.byref(C.c_int(v))
    lib.k_space_(ci(Nx), ci(Ny), ci(Nz), fst, fen, dp(kf), dp(ksq), dp(k4))
    # layout kf(3, z, y, kx): index = ((kx*Ny + y)*Nz + z)
    G, K2, K3, K4 = oracle.k_space(Nx, Ny, Nz)  # [z][y][kx]
    kfc = (kf[..., 0] + 1j * kf[..., 1]).reshape(Nx // 2 + 1, Ny, Nz, 3).transpose(2, 1, 0, 3)
    assert np.allclose(kfc.sum(-1), G, atol=1e-15)
    assert np.allclose(ksq[..., 0].reshape(Nx // 2 + 1, Ny, Nz, 3).transpose(2, 1, 0, 3).sum(-1), K2)
    assert np.allclose(k4[..., 0].reshape(Nx // 2 + 1, Ny, Nz, 3).transpose(2, 1, 0, 3).sum(-1), K4)


@pytest.mark.parametrize("kind", ["noise", "voronoi"])
def test_library_ics_match_oracle(pkg, oracle, kind):
    p = oracle.Params(12, 10, 8, 3)
    if kind == "noise":
        a = pkg.ic_noise(p, 3, 0.01, 0.45, 0.02)
        b = oracle.ic_noise(p, 3, 0.01, 0.45, 0.02)
    else:
        a = pkg.ic_voronoi(p, 4, 7, 0.01, 0.5, 0.02)
        b = oracle.ic_voronoi(p, 4, 7, 0.01, 0.5, 0.02)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_create_without_gpu_fails_cleanly(pkg, oracle):
    """On a host without a usable GPU, pf_create reports a CUDA error (no
    crash, no CPU fallback)."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(pkg.PFError) as e:
        pkg.Run(oracle.Params(32, 32, 32, 4))
    assert e.value.code == -2


def test_server_create_without_gpu(pkg):
    """The serving API exists and, without a GPU, refuses to start."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(pkg.PFError) as e:
        pkg.Server()
    assert e.value.code == pkg.PF_ECUDA
