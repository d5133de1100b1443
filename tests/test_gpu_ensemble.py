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


# every non-default work-tile shape: 32-row RHS tiles, half-width column
# tiles, two modes per block in both row kernels
ALT_SHAPE = dict(rhs_tile_rows=32, row_group_fwd=2, row_group_inv=2)


def alt_shape(prec):
    return dict(ALT_SHAPE, col_tile=4 if prec else 2)


@pytest.mark.parametrize("prec", [0, 1])
def test_shape_leaves_results_bitwise(qgwlib, prec):
    """The work-tile shape (RHS tile height, column-tile width, modes per
    row-kernel block) changes which block computes a value, never the
    arithmetic: a run gives bitwise the same psi and q in every shape, also
    with bottom drag, topography, hyperviscosity and a doubly periodic
    basin."""
    cases = [C.cfg2(128, 5), dict(C.cfg1(96), NY=60), dict(C.cfg2(64, 10), bc_fac=-1.0),
             dict(C.cfg1(64), n_hyper=6, nu_hyper=1e8, bc_fac=0.6)]
    for p in cases:
        q0 = C.noise_ic(p, 41)
        psi_a, q_a = alone(qgwlib, p, prec, q0, 9)
        assert np.isfinite(q_a).all()
        r = qgwlib.Run(p, prec)
        r.set_shape(**alt_shape(prec))
        sh = r.get_shape()
        assert sh["rhs_tile_rows"] == 32 and sh["col_tile"] == alt_shape(prec)["col_tile"], sh
        r.set_q(q0)
        r.fix_dt(p["dt"])
        assert r.step(9).steps_taken == 9
        psi, q = r.get()
        r.close()
        assert np.array_equal(q, q_a), (p["NX"], np.abs(q - q_a).max())
        assert np.array_equal(psi, psi_a), (p["NX"], np.abs(psi - psi_a).max())


def test_shape_refuses_unknown_values(qgwlib):
    r = qgwlib.Run(C.cfg1(64), 1)
    before = r.get_shape()
    for bad in (dict(rhs_tile_rows=24), dict(col_tile=6), dict(row_group_fwd=17)):
        with pytest.raises(qgwlib.QgwError):
            r.set_shape(**bad)
        assert r.get_shape() == before
    r.close()


@pytest.mark.parametrize("prec", [0, 1])
def test_ensemble_nondefault_shape_equals_alone(qgwlib, prec):
    """An ensemble in a non-default shape against each member alone in the
    default shape: bitwise equal."""
    ps = members()
    q0s = [C.noise_ic(p, 700 + i) for i, p in enumerate(ps)]
    ens = qgwlib.Ensemble(ps, prec)
    ens.set_shape(**alt_shape(prec))
    assert ens.get_shape(0)["rhs_tile_rows"] == 32
    for i, (p, q0) in enumerate(zip(ps, q0s)):
        ens.set_q(i, q0)
        ens.fix_dt(i, p["dt"])
    ens.step(8)
    for i, (p, q0) in enumerate(zip(ps, q0s)):
        psi, q = ens.get(i)
        psi_a, q_a = alone(qgwlib, p, prec, q0, 8)
        assert np.array_equal(q, q_a), (i, np.abs(q - q_a).max())
        assert np.array_equal(psi, psi_a), (i, np.abs(psi - psi_a).max())
    ens.close()


def test_ensemble_tuner_picks_a_shape(qgwlib):
    """The tuner's shape is one of its candidates, and the tuned ensemble
    still matches each run alone bitwise."""
    ps = members()[:4]
    ens = qgwlib.Ensemble(ps, 1)
    q0s = [C.noise_ic(p, 900 + i) for i, p in enumerate(ps)]
    for i, (p, q0) in enumerate(zip(ps, q0s)):
        ens.set_q(i, q0)
        ens.fix_dt(i, p["dt"])
    ens.tune(1)
    sh = ens.get_shape(0)
    assert sh["rhs_tile_rows"] in (16, 32) and sh["col_tile"] in (4, 8), sh
    for i, (p, q0) in enumerate(zip(ps, q0s)):
        ens.set_q(i, q0)
        ens.fix_dt(i, p["dt"])
    ens.step(5)
    for i, (p, q0) in enumerate(zip(ps, q0s)):
        psi, q = ens.get(i)
        psi_a, q_a = alone(qgwlib, p, 1, q0, 5)
        assert np.array_equal(q, q_a) and np.array_equal(psi, psi_a), i
    ens.close()


def test_ensemble_of_mixed_column_widths(qgwlib):
    """A 2048^2 FP32c member takes 16-byte column tiles (its 32-byte-row
    buffers would pass the shared memory a block can have) while a small
    member defaults to 32-byte ones: the ensemble gives both the narrower
    width and each member still equals its run alone bitwise."""
    ps = [C.cfg2(2048, 2), C.cfg2(128, 5)]
    q0s = [C.noise_ic(p, 1100 + i) for i, p in enumerate(ps)]
    ens = qgwlib.Ensemble(ps, 1)
    assert [ens.get_shape(i)["col_tile"] for i in range(2)] == [4, 4]
    for i, (p, q0) in enumerate(zip(ps, q0s)):
        ens.set_q(i, q0)
        ens.fix_dt(i, p["dt"])
    ens.step(3)
    for i, (p, q0) in enumerate(zip(ps, q0s)):
        psi, q = ens.get(i)
        psi_a, q_a = alone(qgwlib, p, 1, q0, 3)
        assert np.array_equal(q, q_a) and np.array_equal(psi, psi_a), i
    ens.close()
