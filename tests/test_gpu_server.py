"""pf_server (continuous batching): requests of several shapes, submitted
while others run, finish with exactly the fields and records they get when run
alone; admission respects the memory budget."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _requests(oracle):
    specs = [
        # (params kwargs, ic, steps, delay before submit [s])
        (dict(Nx=32, Ny=32, Nz=32, var=4, t_step=0.1, mobility="c1mc"), ("voronoi", 1, 6, 0.01, 0.5, 0.02), 150, 0.0),
        (dict(Nx=64, Ny=64, Nz=64, var=8, t_step=0.05), ("noise", 2, 0.001, 0.5, 0.01), 100, 0.0),
        (dict(Nx=32, Ny=32, Nz=32, var=4, t_step=0.05, mobility="c1mc", mob_phi=2.0, grad_coeff_phi=0.7),
         ("voronoi", 3, 5, 0.01, 0.45, 0.02), 60, 0.0),
        (dict(Nx=16, Ny=16, Nz=16, var=5, t_step=0.05, mobility="c1mc"), ("voronoi", 4, 4, 0.01, 0.4, 0.02), 80, 0.05),
        (dict(Nx=64, Ny=64, Nz=64, var=8, t_step=0.02, sigma_1=1.2, sigma_2=1.2), ("noise", 5, 0.001, 0.4, 0.01), 120,
         0.1),
        (dict(Nx=32, Ny=32, Nz=32, var=4, t_step=0.1, mobility="c1mc"), ("voronoi", 6, 6, 0.01, 0.5, 0.02), 40, 0.15),
    ]
    out = []
    for kw, ic, steps, delay in specs:
        p = oracle.Params(**kw)
        if ic[0] == "noise":
            phi, con = oracle.ic_noise(p, *ic[1:])
        else:
            phi, con = oracle.ic_voronoi(p, *ic[1:])
        out.append((p, phi, con, steps, delay))
    return out


def test_server_results_equal_runs_alone(pkg, oracle):
    reqs = _requests(oracle)
    srv = pkg.Server(max_active=8, chunk_steps=32)
    try:
        ids = []
        t0 = time.perf_counter()
        for p, phi, con, steps, delay in reqs:
            while time.perf_counter() - t0 < delay:
                time.sleep(0.005)
            ids.append(srv.submit(p, phi, con, steps))
        results = [srv.wait(i, timeout=600.0) for i in ids]
    finally:
        srv.close()
    for (p, phi, con, steps, _), (gp, gc, last, times) in zip(reqs, results):
        run = pkg.Run(p)
        run.set_fields(phi, con)
        d = run.step(steps)
        ap, ac = run.get_fields()
        run.close()
        assert np.array_equal(gp, ap) and np.array_equal(gc, ac), (p.Nx, p.var, steps)
        assert last["step"] == steps and last["f_eta"] == d[-1]["f_eta"] and last["mass"] == d[-1]["mass"]
        assert times["total_s"] >= times["run_s"] > 0 and times["queued_s"] >= 0


def test_server_budget_and_states(pkg, oracle):
    p = oracle.Params(Nx=64, Ny=64, Nz=64, var=8, t_step=0.05)
    phi, con = oracle.ic_noise(p, 7, 0.001, 0.5, 0.01)
    # a budget below one run: the request fails cleanly instead of waiting forever
    srv = pkg.Server(hbm_budget_bytes=1e6)
    try:
        rid = srv.submit(p, phi, con, 10)
        with pytest.raises(pkg.PFError) as e:
            srv.wait(rid, timeout=120.0)
        assert e.value.code == pkg.PF_ENOMEM
    finally:
        srv.close()
    # room for one run at a time: the second waits in the queue, both finish
    srv = pkg.Server(max_active=1, chunk_steps=16)
    try:
        a = srv.submit(p, phi, con, 200)
        b = srv.submit(p, phi, con, 20)
        assert srv.poll(b) in (pkg.PF_REQ_QUEUED, pkg.PF_REQ_RUNNING)
        ra = srv.wait(a, timeout=600.0)
        rb = srv.wait(b, timeout=600.0)
        assert rb[3]["queued_s"] >= ra[3]["run_s"] * 0.5  # b was admitted only after a left
        with pytest.raises(pkg.PFError):
            srv.poll(a)  # forgotten after wait
    finally:
        srv.close()


def test_server_long_chunks_keep_their_records(pkg, oracle):
    """chunk_steps above 512 is cut to 512, so that the records of the two
    chunks kept in flight both fit the per-run ring of 1024: the last record
    and the fields of a 1500-step run equal those of the run alone."""
    p = oracle.Params(16, 16, 16, 3, t_step=0.05)
    phi, con = oracle.ic_noise(p, 9, 0.001, 0.5, 0.01)
    srv = pkg.Server(chunk_steps=1000)
    try:
        rid = srv.submit(p, phi, con, 1500)
        gp, gc, last, _ = srv.wait(rid, timeout=600.0)
    finally:
        srv.close()
    run = pkg.Run(p)
    run.set_fields(phi, con)
    d = run.step(1500)
    ap, ac = run.get_fields()
    run.close()
    assert np.array_equal(gp, ap) and np.array_equal(gc, ac)
    assert last == d[-1], (last, d[-1])


def test_pool_over_visible_devices_equals_runs_alone(pkg, oracle):
    """pf_pool: one server per visible GPU, every request placed on the device
    with the least outstanding work; results equal the runs alone."""
    reqs = _requests(oracle)[:4]
    pool = pkg.Pool(max_active=8, chunk_steps=32)
    try:
        assert pool.devices == pkg.load_library().pf_device_count() >= 1
        subs = [pool.submit(p, phi, con, steps) for p, phi, con, steps, _ in reqs]
        assert all(0 <= d < pool.devices for _, d in subs)
        results = [pool.wait(i, timeout=600.0) for i, _ in subs]
    finally:
        pool.close()
    for (p, phi, con, steps, _), (gp, gc, last, _) in zip(reqs, results):
        run = pkg.Run(p)
        run.set_fields(phi, con)
        d = run.step(steps)
        ap, ac = run.get_fields()
        run.close()
        assert np.array_equal(gp, ap) and np.array_equal(gc, ac)
        assert last == d[-1]
