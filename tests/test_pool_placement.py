"""Placement of independent runs over a node's GPUs (no collective): the
offline LPT placement pf_sweep --devices uses and the online choice of
pf_pool, checked on the CPU with made-up device counts (no GPU needed)."""
import itertools

import numpy as np
import pytest


@pytest.mark.parametrize("ndev", [1, 2, 3, 4, 8])
def test_lpt_placement_is_complete_and_balanced(pkg, ndev):
    rng = np.random.default_rng(ndev)
    # a sweep's units: many small batches, a few large single runs
    work = np.concatenate([rng.uniform(1, 10, 40), rng.uniform(50, 200, 5)])
    dev, load = pkg.place_units(work, ndev)
    assert dev.shape == work.shape and set(dev.tolist()) <= set(range(ndev))
    for d in range(ndev):
        assert load[d] == pytest.approx(work[dev == d].sum())
    # Graham's bound for LPT: makespan <= (4/3 - 1/(3 m)) OPT, OPT >= max(mean load, largest unit)
    opt_lb = max(work.sum() / ndev, work.max())
    assert load.max() <= (4.0 / 3.0 - 1.0 / (3 * ndev)) * opt_lb + 1e-9
    if ndev <= len(work):
        assert np.all(load > 0)  # no device left idle


def test_lpt_placement_small_cases_exact(pkg):
    # equal units: round robin in the given order
    dev, load = pkg.place_units([5.0] * 6, 3)
    assert dev.tolist() == [0, 1, 2, 0, 1, 2] and load.tolist() == [10.0, 10.0, 10.0]
    # largest first onto the least loaded device
    dev, load = pkg.place_units([1.0, 7.0, 3.0, 3.0, 2.0], 2)
    assert dev.tolist() == [0, 0, 1, 1, 1] and load.tolist() == [8.0, 8.0]
    # the best of all assignments for a tiny case is reached here
    w = [4.0, 3.0, 3.0, 2.0, 2.0]
    best = min(max(sum(x for x, a in zip(w, asg) if a == d) for d in range(2))
               for asg in itertools.product(range(2), repeat=len(w)))
    assert pkg.place_units(w, 2)[1].max() <= best * 7 / 6 + 1e-12
    # more devices than units
    dev, load = pkg.place_units([2.0, 1.0], 4)
    assert dev.tolist() == [0, 1] and load.tolist() == [2.0, 1.0, 0.0, 0.0]


def test_online_pick_takes_least_outstanding_work(pkg):
    assert pkg.pick_device([3.0, 1.0, 2.0]) == 1
    assert pkg.pick_device([2.0, 2.0, 5.0]) == 0  # ties: lowest ordinal
    assert pkg.pick_device([0.0]) == 0
    # a stream of equal requests onto 4 idle devices fills them in turn
    out, seen = [0.0] * 4, []
    for _ in range(8):
        d = pkg.pick_device(out)
        seen.append(d)
        out[d] += 1.0
    assert seen == [0, 1, 2, 3, 0, 1, 2, 3]


def test_run_work_is_cell_steps_times_P(pkg, oracle):
    lib = pkg.load_library()
    import ctypes as C

    cfg = pkg.make_config(oracle.Params(64, 32, 16, 5))
    assert lib.pf_run_work(C.byref(cfg), 100) == 64 * 32 * 16 * 5 * 100
