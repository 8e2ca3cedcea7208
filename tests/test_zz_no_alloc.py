"""pf_diag_fields_noalloc: diagnostics of device-resident fields without any
device allocation, for callers that must not allocate (see include/pfgpu.h).

Checked two ways: against the existing entry point (the record pf_step
returns for its first step describes the fields at the start of that step)
and against the FP64 oracle evaluated on the same FP32 fields, both within
the FP32 tolerance of the other GPU tests (1e-5 relative).  Calls follow one
another on grids of different sizes (so the shared scratch is reused with
different block counts, up to the largest grid the entry point accepts), on
the default stream and on a side stream; tiny order parameters take the
rescaled h = N4/S4 branch; non-finite values are counted cell by cell while
large finite ones are not flagged.  This file is collected last on purpose.
"""
import ctypes as C
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5
MAX_CELLS = 256 ** 3  # PF_NOALLOC_MAX_CELLS


def _bind(lib, pkg):
    fn = lib.pf_diag_fields_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.POINTER(pkg.Config), C.c_void_p, C.POINTER(pkg.Diag), C.c_void_p]
    return fn


def _close(a, b, scale=None):
    s = abs(b) if scale is None else scale
    return abs(a - b) <= TOL * max(s, 1e-30)


def _device_fields(phi, con):
    import torch

    return torch.tensor(np.concatenate([phi, con[None]]), dtype=torch.float32, device="cuda").contiguous()


def _call(pkg, lib, p, fields, stream=None):
    fn = _bind(lib, pkg)
    cfg = pkg.make_config(p)
    out = pkg.Diag()
    rc = fn(C.byref(cfg), C.c_void_p(fields.data_ptr()), C.byref(out), C.c_void_p(stream) if stream else None)
    return rc, out.as_dict()


def _oracle_record(oracle, p, phi, con):
    """The oracle's start-of-step quantities on the fields as the device holds
    them (rounded to FP32)."""
    phi32 = phi.astype(np.float32).astype(np.float64)
    con32 = con.astype(np.float32).astype(np.float64)
    f_eta, f_ch, _, _, _ = oracle.bulk_energies(p, phi32, con32)
    rec = dict(f_eta=f_eta, f_ch=f_ch, mass=math.fsum(con32.ravel()))
    rec.update(oracle.stats(phi32, con32))
    return rec


def _check_against(got, ref, what, exact_mass=False):
    """exact_mass: ref["mass"] is the exact sum of the same FP32 values, which
    the compensated sum reproduces to FP64 round-off."""
    assert math.isnan(got["f_int"]) and math.isnan(got["e_tot"])
    for k in ("f_eta", "f_ch", "mass"):
        assert _close(got[k], ref[k], max(abs(ref[k]), 1.0)), (what, k, got[k], ref[k])
    for k in ("c_min", "c_max", "phi_min", "phi_P_max"):
        assert _close(got[k], ref[k], 1.0), (what, k, got[k], ref[k])
    if exact_mass:
        assert abs(got["mass"] - ref["mass"]) <= 1e-13 * abs(ref["mass"]), (what, got["mass"], ref["mass"])


def test_noalloc_diag_matches_pf_step_and_oracle(pkg, lib, oracle):
    p = oracle.Params(64, 64, 64, 4, t_step=0.01, am=0.5, ap=2.0, con_0_mat=0.3, con_0_ppt=0.7,
                      sigma_1=1.5, sigma_2=1.2, mobility="c1mc")
    for seed in (3, 8):  # two calls in a row, different fields
        phi, con = pkg.ic_voronoi(p, seed, 7, 0.02, 0.45 + 0.01 * seed, 0.02)
        run = pkg.Run(p)
        run.set_fields(phi, con)
        ref = run.step(1)[0]
        run.close()
        fields = _device_fields(phi, con)
        import torch

        torch.cuda.synchronize()
        rc, got = _call(pkg, lib, p, fields)
        assert rc == 0, lib.pf_last_error().decode()
        assert got["nonfinite"] == 0
        _check_against(got, ref, f"pf_step seed {seed}")
        _check_against(got, _oracle_record(oracle, p, phi, con), f"oracle seed {seed}", exact_mass=True)


def test_noalloc_grid_sizes_streams_and_the_limit(pkg, lib, oracle):
    """The largest accepted grid (256^3 cells, var = 1, on a side stream),
    then a small grid right after (fewer blocks: nothing left over in the
    shared scratch may leak into it), then var = 1 on the default stream."""
    import torch

    cases = [
        (oracle.Params(256, 256, 256, 1, am=0.5, ap=2.0, con_0_mat=0.3, con_0_ppt=0.7), 11, True),
        (oracle.Params(32, 32, 32, 3, am=0.5, ap=2.0, con_0_mat=0.3, con_0_ppt=0.7), 12, False),
        (oracle.Params(48 * 2, 32, 16, 1, am=0.2, ap=1.0, con_0_mat=0.2, con_0_ppt=0.9), 13, False),
    ]
    assert cases[0][0].Nx * cases[0][0].Ny * cases[0][0].Nz == MAX_CELLS
    side = torch.cuda.Stream()
    for p, seed, on_side in cases:
        rng = np.random.default_rng(seed)
        phi = rng.uniform(-0.2, 1.1, (p.var,) + p.shape)
        con = rng.uniform(0.1, 0.9, p.shape)
        fields = _device_fields(phi, con)
        torch.cuda.synchronize()
        rc, got = _call(pkg, lib, p, fields, side.cuda_stream if on_side else None)
        assert rc == 0, lib.pf_last_error().decode()
        assert got["nonfinite"] == 0
        _check_against(got, _oracle_record(oracle, p, phi, con), (p.Nx, p.Ny, p.Nz, p.var), exact_mass=True)


def test_noalloc_tiny_order_parameters_take_the_rescaled_branch(pkg, lib, oracle):
    """|phi| ~ 1e-9: S4 = sum phi^4 ~ 1e-36 is below FP32's reach (1e-30), h
    comes from phi / max|phi|; f_ch depends on h through am != ap."""
    import torch

    p = oracle.Params(32, 32, 32, 3, am=0.5, ap=2.0, con_0_mat=0.3, con_0_ppt=0.7)
    rng = np.random.default_rng(21)
    phi = 1e-9 * rng.uniform(0.2, 1.0, (p.var,) + p.shape) * rng.choice([-1.0, 1.0], (p.var,) + p.shape)
    con = rng.uniform(0.2, 0.8, p.shape)
    ref = _oracle_record(oracle, p, phi, con)
    s4 = np.sum(phi.astype(np.float32).astype(np.float64) ** 4, axis=0)
    assert np.max(s4) < 1e-30
    fields = _device_fields(phi, con)
    torch.cuda.synchronize()
    rc, got = _call(pkg, lib, p, fields)
    assert rc == 0, lib.pf_last_error().decode()
    _check_against(got, ref, "tiny phi", exact_mass=True)


def test_noalloc_counts_non_finite_cells_value_by_value(pkg, lib, oracle):
    """NaN in one cell's phi and Inf in another cell's c are counted (two
    cells, PF_ENONFINITE); values whose fourth powers overflow FP32 but that
    are themselves finite are not."""
    import torch

    p = oracle.Params(32, 32, 32, 3, am=0.5, ap=2.0, con_0_mat=0.3, con_0_ppt=0.7)
    rng = np.random.default_rng(5)
    phi = rng.uniform(0.0, 1.0, (p.var,) + p.shape)
    con = rng.uniform(0.2, 0.8, p.shape)
    big = phi.copy()
    big[0, 1, 2, 3] = 3e37  # finite in FP32, its square is not
    big[2, 4, 5, 6] = -1e20
    rc, got = _call(pkg, lib, p, _device_fields(big, con))
    assert rc == 0 and got["nonfinite"] == 0, (rc, got["nonfinite"])
    bad_phi, bad_con = phi.copy(), con.copy()
    bad_phi[1, 7, 8, 9] = np.nan
    bad_con[10, 11, 12] = np.inf
    bad_phi[2, 10, 11, 12] = np.nan  # same cell as the Inf in c: still one cell
    torch.cuda.synchronize()
    rc, got = _call(pkg, lib, p, _device_fields(bad_phi, bad_con))
    assert rc == pkg.PF_ENONFINITE and got["nonfinite"] == 2, (rc, got["nonfinite"])
    # a clean call right after: nothing carried over
    rc, got = _call(pkg, lib, p, _device_fields(phi, con))
    assert rc == 0 and got["nonfinite"] == 0
    _check_against(got, _oracle_record(oracle, p, phi, con), "after non-finite")


def test_noalloc_rejects_grids_above_the_limit_and_captured_streams(pkg, lib, oracle):
    import torch

    dummy = torch.zeros(4, dtype=torch.float32, device="cuda")
    rc, _ = _call(pkg, lib, oracle.Params(512, 256, 256, 1), dummy)
    assert rc == pkg.PF_EINVAL and "exceed" in lib.pf_last_error().decode()
    # a stream that is being captured: rejected before any work is enqueued
    p = oracle.Params(16, 16, 16, 2)
    fields = torch.zeros((3, 16, 16, 16), dtype=torch.float32, device="cuda")
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.stream(s):
        g.capture_begin()
        try:
            rc, _ = _call(pkg, lib, p, fields, s.cuda_stream)
            fields.add_(1.0)  # keep the captured graph non-empty
        finally:
            g.capture_end()
    assert rc == pkg.PF_EINVAL and "captured" in lib.pf_last_error().decode()
    g.replay()
    torch.cuda.synchronize()
    rc, got = _call(pkg, lib, p, fields)
    assert rc == 0 and got["mass"] == 16 ** 3
