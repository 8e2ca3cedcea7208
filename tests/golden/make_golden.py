"""Regenerate the oracle regression fixtures in this directory.

    python tests/golden/make_golden.py

Each fixture holds the parameters, the seeded start (by its generator
arguments), the fields after `steps` steps of the FP64 oracle (faithful 7P+9
transform mode) and the per-step diagnostics.  The reference ships no golden
data for this path; these pin the oracle against unintended changes.
"""
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1] / "oracle"))
import pf_ref  # noqa: E402

CASES = {
    "noise_const_16": dict(params=dict(Nx=16, Ny=16, Nz=16, var=3, t_step=0.05),
                           ic=["noise", 0, 0.001, 0.5, 0.01], steps=6),
    "voronoi_refvar_16": dict(params=dict(Nx=16, Ny=16, Nz=16, var=3, t_step=0.002, D_gb=1.0, am=0.5, ap=2.0,
                                          con_0_mat=0.3, con_0_ppt=0.7, sigma_1=6.0, sigma_2=3.0),
                              ic=["voronoi", 3, 5, 0.05, 0.5, 0.02], steps=6),
    "voronoi_c1mc_16": dict(params=dict(Nx=16, Ny=16, Nz=16, var=4, t_step=0.05, mobility="c1mc", am=0.5, ap=2.0,
                                        con_0_mat=0.3, con_0_ppt=0.7),
                            ic=["voronoi", 1, 6, 0.01, 0.5, 0.02], steps=6),
}

DIAG_KEYS = ("f_int", "f_eta", "f_ch", "c_min", "c_max", "phi_min", "phi_P_max", "mass")


def start(case):
    p = pf_ref.Params(**case["params"])
    ic = case["ic"]
    if ic[0] == "noise":
        phi, con = pf_ref.ic_noise(p, *ic[1:])
    else:
        phi, con = pf_ref.ic_voronoi(p, *ic[1:])
    return p, phi, con


def compute(case):
    p, phi, con = start(case)
    ph, c, d = pf_ref.run(p, phi, con, case["steps"], faithful=True)
    diag = np.array([[getattr(x, k) for k in DIAG_KEYS] for x in d])
    return ph, c, diag


def main():
    for name, case in CASES.items():
        ph, c, diag = compute(case)
        np.savez_compressed(HERE / f"{name}.npz", phi=ph, con=c, diag=diag,
                            meta=json.dumps(dict(case=case, diag_keys=DIAG_KEYS)))
        print(name, ph.shape)


if __name__ == "__main__":
    main()
