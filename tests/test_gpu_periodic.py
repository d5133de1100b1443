"""Doubly periodic basin (bc_fac = -1) on the GPU: the reference inverts
with FFTW's 2-D r2c / c2r (src/elliptic.h:32-47,103-118) and wraps the
ghost rings (src/domain.h:225-256).  The golden fixtures of the reference
itself are covered by test_gpu_parity.test_fp64_matches_reference_golden
(the periodic_* cases); this file adds larger sizes against the C port,
the analytic Fourier-mode inversion, the compensated path, ensembles and
the refusals.  Tolerances as in test_gpu_parity: FP64 rel-L2 <= 1e-12 after
100 steps, FP32c within 1e-5 of FP64 after 100 steps."""
import numpy as np
import pytest

from qgw_gb300 import configs as C
from test_gpu_parity import TOL32C, TOL64, gpu_run, rel

pytestmark = pytest.mark.gpu


def periodic(p, **kw):
    q = dict(p, bc_fac=-1.0)
    q.update(kw)
    return q


@pytest.mark.parametrize("case", ["cfg1_256", "cfg2_256_nl10", "topo_128"])
def test_periodic_fp64_vs_port_100_steps(qgwlib, oracle_mod, case):
    if case == "cfg1_256":
        p, dt = periodic(C.cfg1(256)), 1200.0
    elif case == "cfg2_256_nl10":
        p, dt = periodic(C.cfg2(256, 10)), 600.0
    else:
        p, dt = periodic(C.cfg1(128), h_topo=300.0, w_topo=4e5), 1200.0
    q0 = C.noise_ic(p, 3001)
    o = oracle_mod.run_port(p, q0, 100, dt_fixed=dt)
    psi, q, _ = gpu_run(qgwlib, p, q0, 100, dt)
    assert rel(q, o["q"]) <= TOL64, rel(q, o["q"])
    assert rel(psi, o["psi"]) <= TOL64, rel(psi, o["psi"])


def test_periodic_analytic_mode_inversion(qgwlib):
    """Known answer: q = sin(2 pi a X/L) cos(2 pi b Y/L) on one vertical
    mode m (X = (i-1) Delta) inverts to q / -((2 pi a/L)^2 + (2 pi b/L)^2
    + iRd2_m) exactly, including the Nyquist wavenumber along y."""
    p = periodic(C.cfg2(512, 10))
    cl, cm, ird = qgwlib.eigmode(p)
    n = 512
    L = p["Lx"]
    D = L / n
    X = (np.arange(n + 2) - 1) * D
    Y = ((np.arange(n + 2) - 1) * D)[:, None]
    for a, b, m in [(1, 0, 0), (3, 7, 4), (200, 5, 9), (17, 256, 3)]:
        shape = np.sin(2 * np.pi * a * X / L) * np.cos(2 * np.pi * b * Y / L)
        q = cm[:, m][:, None, None] * shape[None]
        r = qgwlib.Run(p)
        r.set_q(q)
        psi, _ = r.get()
        r.close()
        expect = q / -((2 * np.pi * a / L) ** 2 + (2 * np.pi * b / L) ** 2 + ird[m])
        assert rel(psi, expect) <= 1e-12, (a, b, m, rel(psi, expect))


def test_periodic_mean_is_removed(qgwlib):
    """A uniform q has no periodic inverse: the reference zeroes the (0, 0)
    coefficient of every mode, so psi = 0."""
    p = periodic(C.cfg1(64))
    q = np.full((3, 66, 66), 1e-6)
    r = qgwlib.Run(p)
    r.set_q(q)
    psi, _ = r.get()
    r.close()
    assert np.abs(psi).max() < 1e-9 * np.abs(q).max() * (p["Lx"] / 64) ** 2 * 64 ** 2


@pytest.mark.parametrize("nx", [256, 1024])
def test_periodic_fp32c_vs_fp64_100_steps(qgwlib, nx):
    p = periodic(C.cfg2(nx, 10))
    q0 = C.noise_ic(p, 35)
    psi64, q64, _ = gpu_run(qgwlib, p, q0, 100, 600.0, precision=0)
    psi32, q32, _ = gpu_run(qgwlib, p, q0, 100, 600.0, precision=1)
    assert rel(q32, q64) <= TOL32C, rel(q32, q64)
    assert rel(psi32, psi64) <= TOL32C, rel(psi32, psi64)


def test_periodic_ghosts_wrap(qgwlib):
    p = periodic(C.cfg1(64))
    r = qgwlib.Run(p)
    r.set_q(C.noise_ic(p, 4))
    r.fix_dt(1200.0)
    r.step(5)
    psi, q = r.get()
    r.close()
    for f in (psi, q):
        assert np.array_equal(f[:, 0, :], f[:, -2, :]) and np.array_equal(f[:, -1, :], f[:, 1, :])
        assert np.array_equal(f[:, :, 0], f[:, :, -2]) and np.array_equal(f[:, :, -1], f[:, :, 1])


def test_periodic_budget_matches_numpy(qgwlib):
    p = periodic(C.cfg1(128))
    r = qgwlib.Run(p)
    r.set_q(C.noise_ic(p, 9))
    r.fix_dt(1200.0)
    r.step(10)
    b = r.budget()
    psi, q = r.get()
    r.close()
    dh = np.array(p["dh"])
    w = dh / dh.sum()
    D = p["Lx"] / p["NX"]
    scale = D * D / (p["Lx"] * p["Lx"])
    P, Q = psi[:, 1:-1, 1:-1], q[:, 1:-1, 1:-1]
    u = (psi[:, 1:-1, 2:] - P) / D
    v = (psi[:, 2:, 1:-1] - P) / D
    ke = (w[:, None, None] * 0.5 * (u ** 2 + v ** 2)).sum() * scale
    assert b["ke"] == pytest.approx(ke, rel=1e-12)


def test_periodic_ensemble_alone_equals_mix(qgwlib):
    ps = [periodic(C.cfg1(64)), periodic(C.cfg2(128, 5)), periodic(C.cfg2(32, 2))]
    for prec in (0, 1):
        ens = qgwlib.Ensemble(ps, prec)
        q0s = [C.noise_ic(p, 900 + i) for i, p in enumerate(ps)]
        for i, (p, q0) in enumerate(zip(ps, q0s)):
            ens.set_q(i, q0)
            ens.fix_dt(i, p["dt"])
        ens.step(6)
        for i, (p, q0) in enumerate(zip(ps, q0s)):
            psi, q = ens.get(i)
            r = qgwlib.Run(p, prec)
            r.set_q(q0)
            r.fix_dt(p["dt"])
            r.step(6)
            psi_a, q_a = r.get()
            r.close()
            assert np.array_equal(q, q_a) and np.array_equal(psi, psi_a), (prec, i)
        ens.close()


def test_periodic_refusals(qgwlib):
    # the reference's periodic layout needs a square grid; an ensemble holds
    # one boundary kind
    with pytest.raises(qgwlib.QgwError) as e:
        qgwlib.Run(periodic(C.cfg1(64), NY=32))
    assert e.value.status == -6
    with pytest.raises(qgwlib.QgwError) as e:
        qgwlib.Ensemble([periodic(C.cfg1(64)), C.cfg1(64)], 0)
    assert e.value.status == -6
