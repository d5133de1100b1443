"""The oracle itself: pinned against scipy's DST-I, numpy's LAPACK
eigensolver, the reference's golden fixtures, and (where the reference
sources are present) the reference compiled in place."""
import numpy as np
import pytest
import scipy.fft as sf

import golden_cases as G
from qgw_gb300 import configs as C


@pytest.mark.parametrize("n", [1, 3, 7, 31, 63, 255, 1023, 100, 257])
def test_dst_matches_scipy(oracle_mod, n):
    x = np.random.default_rng(n).standard_normal((4, n))
    ref = sf.dst(x, type=1, axis=1)
    for fast in (True, False):
        y = oracle_mod.dst1(x, fast=fast)
        assert np.abs(y - ref).max() <= 1e-13 * np.abs(ref).max()


def _numpy_modes(p):
    """compute_eigmode restated with numpy.linalg.eig (LAPACK dgeev)."""
    nl = p["nl"]
    dh = np.array(p["dh"], float)
    N2 = np.array(p["N2"], float)
    f0 = p["f0"]
    dhc = 0.5 * (dh[:-1] + dh[1:])
    G_ = np.zeros((nl, nl))
    for l in range(nl):
        if l > 0:
            G_[l, l - 1] = -f0 ** 2 / N2[l - 1] / (dhc[l - 1] * dh[l])
        if l < nl - 1:
            G_[l, l + 1] = -f0 ** 2 / N2[l] / (dhc[l] * dh[l])
        G_[l, l] = -G_[l].sum()
    w, vr = np.linalg.eig(G_)
    wl, vl = np.linalg.eig(G_.T)
    o, ol = np.argsort(w.real), np.argsort(wl.real)
    w, vr, vl = w.real[o], vr.real[:, o], vl.real[:, ol]
    H = dh.sum()
    for m in range(nl):
        vr[:, m] *= np.sign(vr[0, m]) * np.sqrt(H / np.sum(dh * vr[:, m] ** 2))
        vl[:, m] /= np.dot(vr[:, m], vl[:, m])
    ird = w.copy()
    ird[0] = 0.0
    return vl.T.copy(), vr.copy(), ird


@pytest.mark.parametrize("nl", [2, 3, 5, 10, 20])
def test_eigmodes_match_lapack(oracle_mod, nl):
    p = C.basin_params(64, nl)
    port = oracle_mod.Port(p)
    cl, cm, ird = port.modes()
    ncl, ncm, nird = _numpy_modes(p)
    assert np.allclose(cl, ncl, rtol=1e-10, atol=1e-12 * np.abs(ncl).max())
    assert np.allclose(cm, ncm, rtol=1e-10, atol=1e-12 * np.abs(ncm).max())
    assert np.allclose(ird, nird, rtol=1e-10, atol=0)
    # known answers: cl2m . cm2l = I, sum_k dh_k cm2l[k,m]^2 = H, ascending
    assert np.allclose(cl @ cm, np.eye(nl), atol=1e-12)
    dh = np.array(p["dh"])
    assert np.allclose((dh[:, None] * cm ** 2).sum(0), dh.sum(), rtol=1e-12)
    assert ird[0] == 0.0 and np.all(np.diff(ird) > 0)


def test_ab3_constant_dt_coefficients():
    # doc/timestep.org:44 -- constant dt gives 23/12, -16/12, 5/12
    dt = dt0 = dt1 = 600.0
    c0 = dt * (2 * dt ** 2 + 3 * dt * (2 * dt0 + dt1) + 6 * dt0 * (dt0 + dt1)) / (6 * dt0 * (dt0 + dt1))
    c1 = dt ** 2 * (-dt / 3 - dt0 / 2 - dt1 / 2) / (dt0 * dt1)
    c2 = dt ** 2 * (dt / 3 + dt0 / 2) / (dt1 * (dt0 + dt1))
    assert np.allclose([c0 / dt, c1 / dt, c2 / dt], [23 / 12, -16 / 12, 5 / 12], rtol=1e-15)


@pytest.mark.parametrize("name", G.names())
def test_port_matches_reference_golden(oracle_mod, name):
    meta, d = G.load(name)
    p = meta["params"]
    frec = d.get("frec")
    r = oracle_mod.run_port(p, d["q0"], meta["nsteps"], dt_fixed=meta["dt_fixed"], fast_dst=False,
                            forcing_records=frec)
    # same DST algorithm as the golden run: bit-identical
    assert np.array_equal(r["q"], d["q"])
    assert np.array_equal(r["psi"], d["psi"])
    for k in ("t", "dt", "dt0", "dt1"):
        assert r["time"][k] == meta["time"][k]
    # the fast DST differs only by round-off
    r2 = oracle_mod.run_port(p, d["q0"], meta["nsteps"], dt_fixed=meta["dt_fixed"], fast_dst=True,
                             forcing_records=frec)
    assert oracle_mod.rel_l2(r2["q"], d["q"]) < 1e-13
    assert oracle_mod.rel_l2(r2["psi"], d["psi"]) < 1e-13


def test_port_matches_reference_live(oracle_mod):
    if not oracle_mod.ref_available():
        pytest.skip("reference sources not present")
    p = C.cfg2(32, 5)
    q0 = C.noise_ic(p, 11)
    r = oracle_mod.run_ref(p, q0, 20, dt_fixed=600.0)
    s = oracle_mod.run_port(p, q0, 20, dt_fixed=600.0, fast_dst=False)
    assert np.array_equal(r["q"], s["q"]) and np.array_equal(r["psi"], s["psi"])


def test_arakawa_identities(oracle_mod):
    """Sums of psi*J and q*J vanish to round-off with psi = 0 walls: the
    energy and enstrophy conservation the Arakawa scheme is built for."""
    p = C.basin_params(32, 1, tau_nm2=0.0, dt=1.0)
    p.update(beta=0.0, nu=0.0, hEkb=0.0, tau0=0.0, cfl=1e30)  # dt never CFL-limited
    q0 = C.noise_ic(p, 3, std=1.0)
    port = oracle_mod.Port(p)
    port.set_q(q0)
    port.fix_dt(1.0)
    port.invert()
    psi, q = port.get()
    port.step(1)
    _, q1 = port.get()
    # with f1 = f2 = 0 and constant dt: q1 = q + 23/12 dt * (-J)
    J = -(q1 - q)[:, 1:-1, 1:-1] / (23.0 / 12.0)
    s = np.abs(J).sum()
    assert abs((psi[:, 1:-1, 1:-1] * J).sum()) < 1e-14 * s * np.abs(psi).max()
    assert abs((q[:, 1:-1, 1:-1] * J).sum()) < 1e-14 * s * np.abs(q).max()
