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


def test_noalloc_rejects_oversize(qgwlib):
    lib = qgwlib.load()
    p = C.cfg2(1024, 10)  # 10 * 1025^2 doubles exceed the scratch array
    s = to_struct(p)
    cl, cm, ird = qgwlib.eigmode(p)
    fn = lib.qgw_invert_pv_noalloc
    fn.argtypes = [ctypes.c_void_p] * 7
    rc = fn(ctypes.addressof(s), cl.ctypes.data, cm.ctypes.data, ird.ctypes.data,
            ctypes.c_void_p(16), ctypes.c_void_p(16), None)
    assert rc == -6
