"""ctypes binding of libqgw_gpu.so (include/qgw_gpu.h).

``Run`` mirrors the reference's step interface on one GPU run:

    reference (src/)                      this binding
    read_params(params, "params.in")      read_params(path) -> dict-like struct
    compute_eigmode()                     eigmode(params)
    check_timestep()                      check_timestep(params)
    invert_pv(q, psi)                     Run.invert()
    timestep(q)                           Run.step(n)
    q, psi globals                        Run.get() / Run.set_q()

The library is loaded from the package's ``lib/`` directory; there is no
fallback: a missing or unloadable library raises ``ImportError``.
"""
from __future__ import annotations

import ctypes
import os
from typing import Dict, Optional

import numpy as np

from .params import QgwBudget, QgwParams, QgwShape, QgwStepInfo, QgwTime, halo_shape, to_struct

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libqgw_gpu.so")

FP64 = 0
FP32C = 1

STATUS = {
    0: "ok", -1: "invalid parameter", -2: "params file not found", -3: "CUDA runtime error",
    -4: "out of memory", -5: "non-finite value in the state", -6: "configuration not supported",
    -7: "eigensolver failed", -8: "call out of order", -9: "request exceeds the HBM budget",
    -10: "device wait timed out", -11: "result not ready",
}

# Every entry point declared in include/qgw_gpu.h (checked by the CPU tests).
EXPORTS = [
    "qgw_params_default", "qgw_params_read", "qgw_eigmode", "qgw_check_timestep", "qgw_topo",
    "qgw_create", "qgw_destroy", "qgw_set_q", "qgw_set_q_device", "qgw_put_q", "qgw_get_time", "qgw_set_time",
    "qgw_set_forcing_seed", "qgw_set_forcing_records", "qgw_ensemble_set_forcing_records",
    "qgw_step", "qgw_step_host", "qgw_invert", "qgw_get", "qgw_budget", "qgw_footprint", "qgw_stream",
    "qgw_kernels_per_step", "qgw_profile_kernels", "qgw_probe_fp_rates", "qgw_strerror", "qgw_abi_version",
    "qgw_invert_pv_noalloc", "qgw_nc_create", "qgw_nc_write", "qgw_nc_close", "qgw_nc_read",
    "qgw_ensemble_create", "qgw_ensemble_destroy", "qgw_ensemble_size", "qgw_ensemble_member",
    "qgw_ensemble_set_q", "qgw_ensemble_set_time", "qgw_ensemble_get", "qgw_ensemble_step",
    "qgw_ensemble_tune", "qgw_ensemble_grids", "qgw_ensemble_set_shape", "qgw_ensemble_shape",
    "qgw_set_shape", "qgw_get_shape",
    "qgw_pool_create", "qgw_pool_submit", "qgw_pool_poll", "qgw_pool_fetch", "qgw_pool_stats",
    "qgw_pool_destroy",
]


class QgwError(RuntimeError):
    def __init__(self, status: int, where: str):
        super().__init__(f"{where}: {STATUS.get(status, 'unknown')} ({status})")
        self.status = status


_lib = None


def load(path: str = LIB_PATH):
    """Load the library once; raises ImportError when it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: run qgw_gb300.build.build() first")
    lib = ctypes.CDLL(path)
    P, D, I, V = ctypes.POINTER, ctypes.POINTER(ctypes.c_double), ctypes.c_int, ctypes.c_void_p
    pp = P(QgwParams)
    lib.qgw_params_default.argtypes = [pp]
    lib.qgw_params_default.restype = None
    lib.qgw_params_read.argtypes = [pp, ctypes.c_char_p]
    lib.qgw_eigmode.argtypes = [pp, D, D, D]
    lib.qgw_check_timestep.argtypes = [pp, D, D]
    lib.qgw_topo.argtypes = [pp, D]
    lib.qgw_create.argtypes = [pp, D, D, D, D, I, P(V)]
    lib.qgw_destroy.argtypes = [V]
    lib.qgw_destroy.restype = None
    lib.qgw_set_q.argtypes = [V, D]
    lib.qgw_set_q_device.argtypes = [V, V]
    lib.qgw_put_q.argtypes = [V, D]
    lib.qgw_get_time.argtypes = [V, P(QgwTime)]
    lib.qgw_set_time.argtypes = [V, P(QgwTime)]
    lib.qgw_step.argtypes = [V, I, ctypes.c_double, ctypes.c_double, P(QgwStepInfo)]
    lib.qgw_step_host.argtypes = [V, I, ctypes.c_double, ctypes.c_double, D, D, P(QgwStepInfo)]
    lib.qgw_invert.argtypes = [V]
    lib.qgw_get.argtypes = [V, D, D]
    lib.qgw_budget.argtypes = [V, P(QgwBudget)]
    lib.qgw_footprint.argtypes = [pp, I, P(ctypes.c_size_t)]
    lib.qgw_stream.argtypes = [V]
    lib.qgw_stream.restype = V
    lib.qgw_kernels_per_step.argtypes = [V]
    lib.qgw_set_forcing_records.argtypes = [V, D, I]
    lib.qgw_ensemble_set_forcing_records.argtypes = [V, I, D, I]
    lib.qgw_set_forcing_seed.argtypes = [V, ctypes.c_uint]
    lib.qgw_profile_kernels.argtypes = [V, I, P(ctypes.c_float)]
    lib.qgw_probe_fp_rates.argtypes = [D, D]
    lib.qgw_strerror.argtypes = [I]
    lib.qgw_strerror.restype = ctypes.c_char_p
    lib.qgw_abi_version.argtypes = []
    lib.qgw_ensemble_create.argtypes = [I, pp, I, P(V)]
    lib.qgw_ensemble_destroy.argtypes = [V]
    lib.qgw_ensemble_destroy.restype = None
    lib.qgw_ensemble_size.argtypes = [V]
    lib.qgw_ensemble_member.argtypes = [V, I]
    lib.qgw_ensemble_member.restype = V
    lib.qgw_ensemble_set_q.argtypes = [V, I, D]
    lib.qgw_ensemble_set_time.argtypes = [V, I, P(QgwTime)]
    lib.qgw_ensemble_get.argtypes = [V, I, D, D]
    lib.qgw_ensemble_step.argtypes = [V, I, P(I), I, P(QgwStepInfo)]
    lib.qgw_ensemble_tune.argtypes = [V, I, P(ctypes.c_float)]
    lib.qgw_ensemble_grids.argtypes = [V, P(I)]
    lib.qgw_ensemble_set_shape.argtypes = [V, P(QgwShape)]
    lib.qgw_ensemble_shape.argtypes = [V, I, P(QgwShape)]
    lib.qgw_set_shape.argtypes = [V, P(QgwShape)]
    lib.qgw_get_shape.argtypes = [V, P(QgwShape)]
    LL = ctypes.c_longlong
    lib.qgw_pool_create.argtypes = [ctypes.c_size_t, I, P(V)]
    lib.qgw_pool_submit.argtypes = [V, pp, D, I, I, P(LL)]
    lib.qgw_pool_poll.argtypes = [V, LL, I, P(I)]
    lib.qgw_pool_fetch.argtypes = [V, LL, D, D, P(QgwTime), D]
    lib.qgw_pool_stats.argtypes = [V, D]
    lib.qgw_pool_destroy.argtypes = [V]
    lib.qgw_pool_destroy.restype = None
    lib.qgw_nc_create.argtypes = [ctypes.c_char_p, I, I, I, ctypes.c_double]
    lib.qgw_nc_create.restype = V
    lib.qgw_nc_write.argtypes = [V, ctypes.c_double, D, D]
    lib.qgw_nc_close.argtypes = [V]
    lib.qgw_nc_close.restype = None
    lib.qgw_nc_read.argtypes = [ctypes.c_char_p, ctypes.c_char_p, I, D, ctypes.c_long]
    lib.qgw_nc_read.restype = ctypes.c_long
    _lib = lib
    return lib


def _check(rc: int, where: str):
    if rc != 0:
        raise QgwError(rc, where)


def _dp(a: Optional[np.ndarray]):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def read_params(path: str) -> QgwParams:
    lib = load()
    s = QgwParams()
    lib.qgw_params_default(ctypes.byref(s))
    _check(lib.qgw_params_read(ctypes.byref(s), path.encode()), "qgw_params_read")
    return s


def eigmode(params: Dict[str, object]):
    lib = load()
    s = to_struct(params)
    nl = s.nl
    a, b, c = np.empty((nl, nl)), np.empty((nl, nl)), np.empty(nl)
    _check(lib.qgw_eigmode(ctypes.byref(s), _dp(a), _dp(b), _dp(c)), "qgw_eigmode")
    return a, b, c


def check_timestep(params: Dict[str, object]):
    lib = load()
    s = to_struct(params)
    DT, dt = ctypes.c_double(), ctypes.c_double()
    _check(lib.qgw_check_timestep(ctypes.byref(s), ctypes.byref(DT), ctypes.byref(dt)), "qgw_check_timestep")
    return DT.value, dt.value


def probe_fp_rates():
    """Measured (FP64, FP32) FMA throughput of the current GPU in TFLOP/s."""
    lib = load()
    a, b = ctypes.c_double(), ctypes.c_double()
    _check(lib.qgw_probe_fp_rates(ctypes.byref(a), ctypes.byref(b)), "qgw_probe_fp_rates")
    return a.value, b.value


def footprint(params: Dict[str, object], precision: int = FP64) -> int:
    lib = load()
    s = to_struct(params)
    b = ctypes.c_size_t()
    _check(lib.qgw_footprint(ctypes.byref(s), int(precision), ctypes.byref(b)), "qgw_footprint")
    return int(b.value)


class Ensemble:
    """Independent runs of uneven sizes advanced together (one launch per
    step stage over all members, replayed as a CUDA graph)."""

    def __init__(self, params_list, precision: int = FP32C):
        self.lib = load()
        self.params = list(params_list)
        n = len(self.params)
        arr = (QgwParams * n)(*[to_struct(p) for p in self.params])
        self._arr = arr
        h = ctypes.c_void_p()
        _check(self.lib.qgw_ensemble_create(n, arr, int(precision), ctypes.byref(h)), "qgw_ensemble_create")
        self.h = h
        self.shapes = [halo_shape(p) for p in self.params]

    def __len__(self):
        return len(self.params)

    def close(self):
        if getattr(self, "h", None):
            self.lib.qgw_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_q(self, i: int, q: np.ndarray):
        q = np.ascontiguousarray(q, dtype=np.float64)
        _check(self.lib.qgw_ensemble_set_q(self.h, int(i), _dp(q)), "qgw_ensemble_set_q")

    def fix_dt(self, i: int, dt: float):
        tm = QgwTime(0.0, dt, dt, dt, dt)
        _check(self.lib.qgw_ensemble_set_time(self.h, int(i), ctypes.byref(tm)), "qgw_ensemble_set_time")

    def step(self, n: int, max_steps=None, graph: bool = True):
        m = len(self.params)
        infos = (QgwStepInfo * m)()
        ms = None if max_steps is None else (ctypes.c_int * m)(*[int(x) for x in max_steps])
        _check(self.lib.qgw_ensemble_step(self.h, int(n), ms, int(graph), infos), "qgw_ensemble_step")
        return list(infos)

    def get(self, i: int):
        psi, q = np.empty(self.shapes[i]), np.empty(self.shapes[i])
        _check(self.lib.qgw_ensemble_get(self.h, int(i), _dp(psi), _dp(q)), "qgw_ensemble_get")
        return psi, q

    def set_forcing_records(self, i: int, rec: np.ndarray):
        """The 4-D forcing's records of member i, (nrec,) + the reference layout."""
        rec = np.ascontiguousarray(rec, dtype=np.float64)
        _check(self.lib.qgw_ensemble_set_forcing_records(self.h, int(i), _dp(rec), rec.shape[0]),
               "qgw_ensemble_set_forcing_records")

    def tune(self, trial_steps: int = 3):
        """Tune the work-tile shape, then each stage's persistent grid;
        returns (step ms after each stage's grid choice, blocks per SM)."""
        ms = (ctypes.c_float * 4)()
        _check(self.lib.qgw_ensemble_tune(self.h, int(trial_steps), ms), "qgw_ensemble_tune")
        g = (ctypes.c_int * 4)()
        _check(self.lib.qgw_ensemble_grids(self.h, g), "qgw_ensemble_grids")
        return list(ms), list(g)

    def set_shape(self, **kw):
        """One work-tile shape for every member (keys of QgwShape; 0 or absent keeps a value)."""
        sh = QgwShape(**{k: int(v) for k, v in kw.items()})
        _check(self.lib.qgw_ensemble_set_shape(self.h, ctypes.byref(sh)), "qgw_ensemble_set_shape")

    def get_shape(self, i: int = 0) -> dict:
        """Member i's work-tile shape."""
        sh = QgwShape()
        _check(self.lib.qgw_ensemble_shape(self.h, int(i), ctypes.byref(sh)), "qgw_ensemble_shape")
        return sh.as_dict()


class Pool:
    """Continuous-batching serving pool (worker thread in the library)."""

    def __init__(self, budget_bytes: int = 0, steps_per_tick: int = 32):
        self.lib = load()
        h = ctypes.c_void_p()
        _check(self.lib.qgw_pool_create(int(budget_bytes), int(steps_per_tick), ctypes.byref(h)), "qgw_pool_create")
        self.h = h
        self.shapes = {}

    def submit(self, params, q0: np.ndarray, precision: int, nsteps: int) -> int:
        s = to_struct(params)
        q0 = np.ascontiguousarray(q0, dtype=np.float64)
        rid = ctypes.c_longlong()
        _check(self.lib.qgw_pool_submit(self.h, ctypes.byref(s), _dp(q0), int(precision), int(nsteps),
                                        ctypes.byref(rid)), "qgw_pool_submit")
        self.shapes[rid.value] = halo_shape(params)
        return rid.value

    def poll(self, rid: int, wait_ms: int = 0):
        """None while running, else the request's status."""
        st = ctypes.c_int()
        rc = self.lib.qgw_pool_poll(self.h, ctypes.c_longlong(rid), int(wait_ms), ctypes.byref(st))
        if rc == -11:
            return None
        _check(rc, "qgw_pool_poll")
        return st.value

    def fetch(self, rid: int):
        shape = self.shapes.pop(rid)
        psi, q = np.empty(shape), np.empty(shape)
        tm = QgwTime()
        lat = np.zeros(3)
        _check(self.lib.qgw_pool_fetch(self.h, ctypes.c_longlong(rid), _dp(psi), _dp(q), ctypes.byref(tm),
                                       _dp(lat)), "qgw_pool_fetch")
        return psi, q, {"t": tm.t, "dt": tm.dt}, lat

    def stats(self):
        s = np.zeros(6)
        _check(self.lib.qgw_pool_stats(self.h, _dp(s)), "qgw_pool_stats")
        keys = ["completed", "admitted", "ticks", "max_resident", "lgp_steps", "bytes_in_use"]
        return dict(zip(keys, s.tolist()))

    def close(self):
        if getattr(self, "h", None):
            self.lib.qgw_pool_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class NcWriter:
    """vars.nc in the reference's layout (netCDF-3, written by the library)."""

    def __init__(self, path: str, nl: int, ny_out: int, nx_out: int, Delta: float):
        self.lib = load()
        self.h = self.lib.qgw_nc_create(path.encode(), nl, ny_out, nx_out, float(Delta))
        if not self.h:
            raise QgwError(-2, "qgw_nc_create")

    def write(self, t: float, psi: np.ndarray, q: np.ndarray):
        psi = np.ascontiguousarray(psi, dtype=np.float64)
        q = np.ascontiguousarray(q, dtype=np.float64)
        _check(self.lib.qgw_nc_write(self.h, float(t), _dp(psi), _dp(q)), "qgw_nc_write")

    def close(self):
        if self.h:
            self.lib.qgw_nc_close(self.h)
            self.h = None


def nc_read(path: str, name: str, shape, rec: int = 0) -> np.ndarray:
    """Record `rec` of a netCDF-3 variable as float64 of the given shape."""
    out = np.empty(shape, dtype=np.float64)
    n = load().qgw_nc_read(path.encode(), name.encode(), int(rec), _dp(out), int(out.size))
    if n < 0:
        raise QgwError(int(n), f"qgw_nc_read({name})")
    return out


class Run:
    """One qgw run resident on the current CUDA device."""

    def __init__(self, params: Dict[str, object], precision: int = FP64,
                 topo: Optional[np.ndarray] = None, modes=None):
        self.lib = load()
        self.params = params
        self.precision = precision
        self._s = to_struct(params)
        self.shape = halo_shape(params)
        h = ctypes.c_void_p()
        cl = cm = ird = None
        if modes is not None:
            cl, cm, ird = (np.ascontiguousarray(m, dtype=np.float64) for m in modes)
        tp = None if topo is None else np.ascontiguousarray(topo, dtype=np.float64)
        _check(self.lib.qgw_create(ctypes.byref(self._s), _dp(cl), _dp(cm), _dp(ird), _dp(tp),
                                   int(precision), ctypes.byref(h)), "qgw_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.qgw_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_q(self, q: np.ndarray):
        q = np.ascontiguousarray(q, dtype=np.float64)
        if q.shape != self.shape:
            raise ValueError(f"q has shape {q.shape}, expected {self.shape}")
        _check(self.lib.qgw_set_q(self.h, _dp(q)), "qgw_set_q")

    def put_q(self, q: np.ndarray):
        """Replace q, keeping the AB3 history (per-step host driver)."""
        _check(self.lib.qgw_put_q(self.h, _dp(q)), "qgw_put_q")

    def step_host(self, n: int, q_in: Optional[np.ndarray], q_out: Optional[np.ndarray],
                  t_out: float = 0.0, tend: float = 0.0) -> "QgwStepInfo":
        """qgw_step with the caller's q in and out (timestep(q) on a host
        array); q_in / q_out in the reference layout, either may be None or
        both the same array."""
        info = QgwStepInfo()
        _check(self.lib.qgw_step_host(self.h, int(n), float(t_out), float(tend),
                                      None if q_in is None else _dp(q_in),
                                      None if q_out is None else _dp(q_out), ctypes.byref(info)),
               "qgw_step_host")
        return info

    def set_q_device(self, ptr: int):
        _check(self.lib.qgw_set_q_device(self.h, ctypes.c_void_p(ptr)), "qgw_set_q_device")

    def time(self) -> Dict[str, float]:
        t = QgwTime()
        _check(self.lib.qgw_get_time(self.h, ctypes.byref(t)), "qgw_get_time")
        return {"t": t.t, "dt": t.dt, "dt0": t.dt0, "dt1": t.dt1, "DT_max": t.DT_max}

    def set_time(self, t=0.0, dt=0.0, dt0=None, dt1=None, DT_max=None):
        tm = QgwTime(t, dt, dt if dt0 is None else dt0, dt if dt1 is None else dt1,
                     dt if DT_max is None else DT_max)
        _check(self.lib.qgw_set_time(self.h, ctypes.byref(tm)), "qgw_set_time")

    def set_forcing_records(self, rec: np.ndarray):
        """The 4-D forcing's records, (nrec,) + the reference layout."""
        rec = np.ascontiguousarray(rec, dtype=np.float64)
        _check(self.lib.qgw_set_forcing_records(self.h, _dp(rec), rec.shape[0]), "qgw_set_forcing_records")

    def set_forcing_seed(self, seed: int):
        """Restart the stochastic forcing's noise sequence as srand(seed)."""
        _check(self.lib.qgw_set_forcing_seed(self.h, int(seed)), "qgw_set_forcing_seed")

    def fix_dt(self, dt: float):
        self.set_time(0.0, dt, dt, dt, dt)

    def step(self, n: int = 1, t_out: float = 0.0, tend: float = 0.0) -> QgwStepInfo:
        info = QgwStepInfo()
        _check(self.lib.qgw_step(self.h, int(n), float(t_out), float(tend), ctypes.byref(info)), "qgw_step")
        return info

    def invert(self):
        _check(self.lib.qgw_invert(self.h), "qgw_invert")

    def get(self, psi: Optional[np.ndarray] = None, q: Optional[np.ndarray] = None, want=("psi", "q")):
        if psi is None and "psi" in want:
            psi = np.empty(self.shape)
        if q is None and "q" in want:
            q = np.empty(self.shape)
        _check(self.lib.qgw_get(self.h, _dp(psi), _dp(q)), "qgw_get")
        return psi, q

    def budget(self) -> Dict[str, float]:
        b = QgwBudget()
        _check(self.lib.qgw_budget(self.h, ctypes.byref(b)), "qgw_budget")
        return {"ke": b.ke, "energy": b.energy, "enstrophy": b.enstrophy, "wind_work": b.wind_work}

    def stream(self) -> int:
        return int(self.lib.qgw_stream(self.h) or 0)

    def set_shape(self, **kw):
        """Work-tile shape of the step kernels (keys of QgwShape; 0 or absent keeps a value)."""
        sh = QgwShape(**{k: int(v) for k, v in kw.items()})
        _check(self.lib.qgw_set_shape(self.h, ctypes.byref(sh)), "qgw_set_shape")

    def get_shape(self) -> dict:
        """The work-tile shape of the step kernels."""
        sh = QgwShape()
        _check(self.lib.qgw_get_shape(self.h, ctypes.byref(sh)), "qgw_get_shape")
        return sh.as_dict()

    def profile_kernels(self, nsteps: int):
        ms = (ctypes.c_float * 4)()
        _check(self.lib.qgw_profile_kernels(self.h, int(nsteps), ms), "qgw_profile_kernels")
        return [float(x) for x in ms]
