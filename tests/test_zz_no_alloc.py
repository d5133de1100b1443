"""The allocation-free PV inversion (qgw_invert_pv_noalloc) against the
library's ordinary inversion path.

It serves callers that cannot allocate device memory (a host model that
owns every device buffer, or a loop that must not call cudaMalloc/cudaFree).
The test owns the device arrays (torch allocates them here, as such a
caller's memory manager would) and calls the entry point twice in a row
through the C ABI, each time comparing psi and the q ghost ring with the
existing qgw_create/qgw_set_q/qgw_get path within the FP64 tolerance of the
parity tests.  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

from qgw_gb300 import configs as C
from qgw_gb300.params import to_struct

pytestmark = pytest.mark.gpu

TOL64 = 1e-12


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def test_noalloc_inversion_matches_library_path(qgwlib):
    torch = pytest.importorskip("torch")
    lib = qgwlib.load()
    fn = lib.qgw_invert_pv_noalloc
    fn.argtypes = [ctypes.POINTER(type(to_struct({}))), ctypes.POINTER(ctypes.c_double),
                   ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    p = dict(C.cfg2(256, 6), bc_fac=0.5)
    s = to_struct(p)
    cl, cm, ird = qgwlib.eigmode(p)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    for seed in (11, 12):  # two calls in a row
        q0 = C.noise_ic(p, seed)
        run = qgwlib.Run(p)
        run.set_q(q0)
        psi_ref, q_ref = run.get()
        run.close()
        qd = torch.from_numpy(q0.copy()).to(dev)
        psid = torch.full(qd.shape, 7.0, dtype=torch.float64, device=dev)
        rc = fn(ctypes.byref(s), _dp(cl), _dp(cm), _dp(ird), ctypes.c_void_p(qd.data_ptr()),
                ctypes.c_void_p(psid.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, qgwlib.STATUS.get(rc)
        torch.cuda.synchronize(dev)
        psi = psid.cpu().numpy()
        q = qd.cpu().numpy()
        assert rel(psi, psi_ref) <= TOL64, rel(psi, psi_ref)
        assert rel(q, q_ref) <= TOL64, rel(q, q_ref)
        assert np.all(psi[:, 0, :] == 0) and np.all(psi[:, :, -1] == 0)


def _noalloc_vs_library(qgwlib, torch, p, seed):
    """One call of the entry point on the caller's device arrays, compared
    with qgw_create/qgw_set_q/qgw_get on the same q."""
    lib = qgwlib.load()
    fn = lib.qgw_invert_pv_noalloc
    fn.argtypes = [ctypes.POINTER(type(to_struct({}))), ctypes.POINTER(ctypes.c_double),
                   ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    s = to_struct(p)
    cl, cm, ird = qgwlib.eigmode(p)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    q0 = C.noise_ic(p, seed)
    run = qgwlib.Run(p)
    run.set_q(q0)
    psi_ref, q_ref = run.get()
    run.close()
    qd = torch.from_numpy(q0.copy()).to(dev)
    psid = torch.full(qd.shape, 7.0, dtype=torch.float64, device=dev)
    rc = fn(ctypes.byref(s), _dp(cl), _dp(cm), _dp(ird), ctypes.c_void_p(qd.data_ptr()),
            ctypes.c_void_p(psid.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    assert rc == 0, qgwlib.STATUS.get(rc)
    torch.cuda.synchronize(dev)
    psi, q = psid.cpu().numpy(), qd.cpu().numpy()
    assert rel(psi, psi_ref) <= TOL64, rel(psi, psi_ref)
    assert rel(q, q_ref) <= TOL64, rel(q, q_ref)


def test_noalloc_set_ups_alternate(qgwlib):
    """The scratch keeps the last call's tables; a call with other sizes or
    modes rebuilds them.  Set-ups alternate here (a non-square 6-layer grid,
    a square 3-layer one, a mixed-radix grid with half-lengths 48 = 2^4 3 and
    30 = 2 3 5, the 1024^2 single-layer grid at the size limit, then the
    first again), every call against the library path."""
    torch = pytest.importorskip("torch")
    a = dict(C.cfg2(256, 6), NY=128, bc_fac=0.5)
    b = C.cfg1(128)
    c = dict(C.cfg1(96), NY=60)
    d = dict(C.cfg2(1024, 1), n_hyper=0, nu_hyper=0.0)
    for k, p in enumerate((a, b, c, d, a, b)):
        _noalloc_vs_library(qgwlib, torch, p, 20 + k)


@pytest.mark.parametrize("case", ["oversize", "periodic", "prime_half_length", "odd"])
def test_noalloc_rejects_what_it_cannot_hold(qgwlib, case):
    """QGW_ERR_UNSUPPORTED before any device work (the array arguments are
    never touched): 10 * 1025^2 doubles exceed the scratch array; the
    periodic basin; NX = 2 * 11 and NY = 99, lengths that the run path takes
    as chirp-z transforms and the allocation-free path does not hold."""
    lib = qgwlib.load()
    p = {"oversize": C.cfg2(1024, 10), "periodic": dict(C.cfg1(64), bc_fac=-1.0),
         "prime_half_length": dict(C.cfg1(64), NX=22),
         "odd": dict(C.cfg1(64), NY=99)}[case]
    s = to_struct(p)
    cl, cm, ird = qgwlib.eigmode(p)
    fn = lib.qgw_invert_pv_noalloc
    fn.argtypes = [ctypes.c_void_p] * 7
    rc = fn(ctypes.addressof(s), cl.ctypes.data, cm.ctypes.data, ird.ctypes.data,
            ctypes.c_void_p(16), ctypes.c_void_p(16), None)
    assert rc == -6
