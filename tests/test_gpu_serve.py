"""Serving pool: continuous batching with HBM-footprint admission.  Each
result must be bitwise the result of the same run alone, whatever else was
resident while it ran."""
import threading
import time

import numpy as np
import pytest

from qgw_gb300 import configs as C

pytestmark = pytest.mark.gpu


def alone(capi, p, prec, q0, n):
    r = capi.Run(p, prec)
    r.set_q(q0)
    r.fix_dt(p["dt"])
    r.step(n)
    out = r.get()
    r.close()
    return out


def test_pool_results_equal_alone(qgwlib):
    # the first request is long, so the later ones arrive while it runs; the
    # last two are a periodic basin and a stochastically forced periodic
    # basin (batched apart from the closed basins)
    forced = dict(NX=32, NY=32, nl=1, Lx=1.0, f0=2.0, beta=0.0, tau0=0.0, k_f=20.0, sigma_f=3.0,
                  bc_fac=-1.0, dh=[1.0], N2=[0.0], nu=0.01, hEkb=0.0, tend=1e12, cfl=0.2, dt=2e-4)
    reqs = [(C.cfg1(64), 0, 3000), (C.cfg2(128, 5), 1, 40), (dict(C.cfg1(64), NY=32), 1, 7),
            (C.cfg2(64, 10), 0, 31), (C.basin_params(32, 2, dt=900.0), 1, 50), (C.cfg1(128), 0, 12),
            (dict(C.cfg1(64), bc_fac=-1.0), 0, 17), (forced, 0, 25)]
    pool = qgwlib.Pool(budget_bytes=0, steps_per_tick=8)
    ids = []
    for k, (p, prec, n) in enumerate(reqs):
        ids.append(pool.submit(p, C.noise_ic(p, 900 + k), prec, n))
        time.sleep(0.002)  # arrivals while the first runs
    for rid in ids:
        assert pool.poll(rid, wait_ms=60000) == 0
    st = pool.stats()
    assert st["completed"] == len(reqs) and st["max_resident"] >= 2
    for k, ((p, prec, n), rid) in enumerate(zip(reqs, ids)):
        psi, q, tm, lat = pool.fetch(rid)
        psi_a, q_a = alone(qgwlib, p, prec, C.noise_ic(p, 900 + k), n)
        assert np.array_equal(q, q_a) and np.array_equal(psi, psi_a), k
        assert tm["t"] == pytest.approx(n * p["dt"])
        assert lat[2] >= lat[1] >= 0
    pool.close()


def test_pool_admission_by_footprint(qgwlib):
    small = C.cfg1(64)
    fp = qgwlib.footprint(small, 0)
    pool = qgwlib.Pool(budget_bytes=int(fp * 1.5), steps_per_tick=4)  # one resident at a time
    ids = [pool.submit(small, C.noise_ic(small, k), 0, 10) for k in range(3)]
    big = C.cfg2(256, 10)
    too_big = pool.submit(big, C.noise_ic(big, 1), 0, 5)
    for rid in ids:
        assert pool.poll(rid, wait_ms=60000) == 0
    assert pool.poll(too_big, wait_ms=60000) == -9  # QGW_ERR_ADMISSION
    assert pool.stats()["max_resident"] == 1
    pool.close()


def test_pool_refuses_chirp_z_grids(qgwlib):
    """The pool batches runs through the ensemble kernels, which hold the
    half-length transforms only: a request on a grid that needs the chirp-z
    transform (NX = 22, half-length 11) ends with QGW_ERR_UNSUPPORTED, and
    the requests around it still complete."""
    pool = qgwlib.Pool(steps_per_tick=4)
    ok = C.cfg1(64)
    chirp = C.cfg1(22)
    a = pool.submit(ok, C.noise_ic(ok, 3), 0, 8)
    b = pool.submit(chirp, C.noise_ic(chirp, 4), 0, 8)
    c = pool.submit(ok, C.noise_ic(ok, 5), 1, 8)
    assert pool.poll(a, wait_ms=60000) == 0
    assert pool.poll(b, wait_ms=60000) == -6  # QGW_ERR_UNSUPPORTED
    assert pool.poll(c, wait_ms=60000) == 0
    pool.close()


def test_pool_concurrent_submitters(qgwlib):
    pool = qgwlib.Pool(steps_per_tick=16)
    out = {}

    def client(k):
        p = C.basin_params(64, 3, dt=1200.0)
        rid = pool.submit(p, C.noise_ic(p, 100 + k), k % 2, 20 + k)
        assert pool.poll(rid, wait_ms=60000) == 0
        out[k] = pool.fetch(rid)

    th = [threading.Thread(target=client, args=(k,)) for k in range(8)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert len(out) == 8
    pool.close()
