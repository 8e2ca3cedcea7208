"""The step graphs: pf_step runs four-step graphs, in which each step's record
runs beside the next step's x pass and the steps alternate two sets of
diagnostic partials, then single-step graphs for the remainder.  Both must
give the same fields and records bit for bit, and so must the captured step
without its second branch (PFGPU_REDUCE_BRANCH=0)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _params(oracle, mobility):
    return oracle.Params(64, 64, 64, 4, t_step=0.02, am=0.5, ap=2.0, con_0_mat=0.3, con_0_ppt=0.7,
                         sigma_1=1.5, sigma_2=1.5, mobility=mobility)


def _run(pkg, p, phi, con, chunks, env=None):
    old = {k: os.environ.get(k) for k in (env or {})}
    os.environ.update(env or {})
    try:
        run = pkg.Run(p)
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    try:
        run.set_fields(phi, con)
        recs = []
        for n in chunks:
            recs += run.step(n)
        gp, gc = run.get_fields()
    finally:
        run.close()
    return gp, gc, recs


@pytest.mark.parametrize("mobility", ["c1mc", "reference"])
def test_multi_step_graphs_equal_single_steps(pkg, oracle, mobility):
    p = _params(oracle, mobility)
    phi, con = pkg.ic_voronoi(p, 5, 9, 0.02, 0.45, 0.02)
    # 10 steps: two four-step graphs and two single steps; then one step at a time
    ap, ac, ad = _run(pkg, p, phi, con, [10])
    bp, bc, bd = _run(pkg, p, phi, con, [1] * 10)
    assert np.array_equal(ap, bp) and np.array_equal(ac, bc)
    assert len(ad) == len(bd) == 10
    for a, b in zip(ad, bd):
        assert a == b, (a, b)
    assert [d["step"] for d in ad] == list(range(1, 11))  # the records in order, one per step


def test_serial_chain_equals_branches(pkg, oracle):
    p = _params(oracle, "c1mc")
    phi, con = pkg.ic_voronoi(p, 6, 9, 0.02, 0.45, 0.02)
    ap, ac, ad = _run(pkg, p, phi, con, [9])
    bp, bc, bd = _run(pkg, p, phi, con, [9], env={"PFGPU_REDUCE_BRANCH": "0"})
    assert np.array_equal(ap, bp) and np.array_equal(ac, bc)
    for a, b in zip(ad, bd):
        assert a == b, (a, b)
