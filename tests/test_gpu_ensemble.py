"""Ensembles of uneven runs (one launch per step stage over all members,
CUDA-graph replay, autotuned persistent grids): every member's result must
be bitwise the result of the same run alone."""
import numpy as np
import pytest

from qgw_gb300 import configs as C

pytestmark = pytest.mark.gpu


def members():
    # the last two are not powers of two (mixed-radix transforms)
    return [C.cfg1(64), C.cfg2(128, 5), dict(C.cfg1(64), NY=32), C.cfg2(64, 10), C.basin_params(32, 2, dt=900.0),
            dict(C.cfg1(96), NY=60), C.cfg2(70, 5)]


def alone(capi, p, prec, q0, n):
    r = capi.Run(p, prec)
    r.set_q(q0)
    r.fix_dt(p["dt"])
    info = r.step(n)
    assert info.steps_taken == n
    out = r.get()
    r.close()
    return out


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("graph", [True, False])
def test_ensemble_members_equal_alone(qgwlib, prec, graph):
    ps = members()
    q0s = [C.noise_ic(p, 300 + i) for i, p in enumerate(ps)]
    ens = qgwlib.Ensemble(ps, prec)
    for i, (p, q0) in enumerate(zip(ps, q0s)):
        ens.set_q(i, q0)
        ens.fix_dt(i, p["dt"])
    caps = [12, 0, 5, 12, 9, 7, 0]  # 0: no cap (12 steps)
    infos = ens.step(12, max_steps=caps, graph=graph)
    for i, (p, q0) in enumerate(zip(ps, q0s)):
        n = caps[i] or 12
        assert infos[i].steps_taken == n
        psi, q = ens.get(i)
        psi_a, q_a = alone(qgwlib, p, prec, q0, n)
        assert np.array_equal(q, q_a), (i, np.abs(q - q_a).max())
        assert np.array_equal(psi, psi_a), (i, np.abs(psi - psi_a).max())
    ens.close()


def test_ensemble_tune_then_run(qgwlib):
    ps = members()
    ens = qgwlib.Ensemble(ps, 1)
    q0s = [C.noise_ic(p, 500 + i) for i, p in enumerate(ps)]
    for i, (p, q0) in enumerate(zip(ps, q0s)):
        ens.set_q(i, q0)
        ens.fix_dt(i, p["dt"])
    ms, grids = ens.tune(2)
    # blocks per SM of each stage's grid (0: one block per work item)
    assert all(g in (0, 1, 2, 3, 4, 5, 6, 8) for g in grids) and all(m > 0 for m in ms)
    for i, (p, q0) in enumerate(zip(ps, q0s)):  # the trials advanced the state
        ens.set_q(i, q0)
        ens.fix_dt(i, p["dt"])
    ens.step(7)
    for i, (p, q0) in enumerate(zip(ps, q0s)):
        psi, q = ens.get(i)
        psi_a, q_a = alone(qgwlib, p, 1, q0, 7)
        assert np.array_equal(q, q_a) and np.array_equal(psi, psi_a)
    ens.close()
