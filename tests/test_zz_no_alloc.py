"""pf_diag_fields_noalloc: diagnostics of device-resident fields without any
device allocation, for callers that must not allocate (see include/pfgpu.h).

Checked against the existing entry point: the record pf_step returns for its
first step describes the fields at the start of that step, so it must agree
with the no-allocation call on the same fields, within the FP32 tolerance of
the other GPU tests (1e-5 relative).  Two calls in a row on different fields
show that the shared scratch carries nothing from one call to the next.
This file is collected last on purpose.
"""
import ctypes as C
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _bind(lib, pkg):
    fn = lib.pf_diag_fields_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.POINTER(pkg.Config), C.c_void_p, C.POINTER(pkg.Diag), C.c_void_p]
    return fn


def _close(a, b, scale=None):
    s = abs(b) if scale is None else scale
    return abs(a - b) <= TOL * max(s, 1e-30)


def test_noalloc_diag_matches_pf_step(pkg, lib, oracle):
    import torch

    fn = _bind(lib, pkg)
    p = oracle.Params(64, 64, 64, 4, t_step=0.01, am=0.5, ap=2.0, con_0_mat=0.3, con_0_ppt=0.7,
                      sigma_1=1.5, sigma_2=1.2, mobility="c1mc")
    cfg = pkg.make_config(p)
    for seed in (3, 8):  # two calls in a row, different fields
        phi, con = pkg.ic_voronoi(p, seed, 7, 0.02, 0.45 + 0.01 * seed, 0.02)
        run = pkg.Run(p)
        run.set_fields(phi, con)
        ref = run.step(1)[0]
        run.close()
        fields = torch.tensor(np.concatenate([phi, con[None]]), dtype=torch.float32, device="cuda").contiguous()
        torch.cuda.synchronize()
        out = pkg.Diag()
        rc = fn(C.byref(cfg), C.c_void_p(fields.data_ptr()), C.byref(out), None)
        assert rc == 0, lib.pf_last_error().decode()
        got = out.as_dict()
        assert math.isnan(got["f_int"]) and math.isnan(got["e_tot"])
        for k in ("f_eta", "f_ch", "mass"):
            assert _close(got[k], ref[k]), (seed, k, got[k], ref[k])
        for k in ("c_min", "c_max", "phi_P_max"):
            assert _close(got[k], ref[k], 1.0), (seed, k, got[k], ref[k])
        assert _close(got["phi_min"], ref["phi_min"], 1.0), (seed, got["phi_min"], ref["phi_min"])
        assert got["nonfinite"] == 0


def test_noalloc_rejects_grids_above_the_limit(pkg, lib, oracle):
    import torch

    fn = _bind(lib, pkg)
    cfg = pkg.make_config(oracle.Params(512, 256, 256, 1))
    dummy = torch.zeros(4, dtype=torch.float32, device="cuda")
    rc = fn(C.byref(cfg), C.c_void_p(dummy.data_ptr()), C.byref(pkg.Diag()), None)
    assert rc == -1 and "exceed" in lib.pf_last_error().decode()
