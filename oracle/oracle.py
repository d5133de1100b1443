"""Python access to the oracle (TEST INFRASTRUCTURE ONLY).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this module; the product library never does.

Two oracles:
  * ``Port``   -- the C restatement of the reference step (qgw_port.c),
                  loaded with ctypes from ``oracle/_build/libqgw_port.so``;
  * ``run_ref`` -- the reference's own ``src/qg.c`` compiled in place with
                  project shims (``oracle/_ref/qgw_ref``), run as a
                  subprocess.  It exists only where the reference sources
                  were available at build time.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys
import tempfile
from typing import Dict, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from qgw_gb300.params import QgwParams, QgwTime, halo_shape, to_struct, write_params  # noqa: E402

PORT_SO = os.path.join(HERE, "_build", "libqgw_port.so")
REF_BIN = os.path.join(HERE, "_ref", "qgw_ref")


def build(ref: bool = True) -> None:
    """Compile the port (always) and the in-place reference build (the
    recipe, oracle/Makefile, builds it where the reference sources exist --
    QGW_REF_SRC names their directory -- and skips it elsewhere)."""
    subprocess.check_call(["make", "-s", "-C", HERE, "port"])
    if ref:
        subprocess.check_call(["make", "-s", "-C", HERE, "ref"], stdout=subprocess.DEVNULL)


def ref_source_dir() -> str:
    """The reference source directory the recipe reads (QGW_REF_SRC, or the
    recipe's usual location)."""
    return subprocess.check_output(["make", "-s", "-C", HERE, "print-ref-src"], text=True).strip()


def ref_available() -> bool:
    return os.path.exists(REF_BIN)


_lib = None


def _port_lib():
    global _lib
    if _lib is None:
        if not os.path.exists(PORT_SO):
            build(ref=False)
        lib = ctypes.CDLL(PORT_SO)
        vp, dp, ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_int
        lib.port_create.restype = vp
        lib.port_create.argtypes = [ctypes.POINTER(QgwParams), ip]
        lib.port_destroy.argtypes = [vp]
        lib.port_sizes.argtypes = [vp, ctypes.POINTER(ip), ctypes.POINTER(ip), ctypes.POINTER(ip)]
        for fn in ("port_set_q", "port_set_topo"):
            getattr(lib, fn).argtypes = [vp, dp]
        lib.port_get.argtypes = [vp, dp, dp]
        lib.port_get_modes.argtypes = [vp, dp, dp, dp]
        lib.port_get_time.argtypes = [vp, ctypes.POINTER(QgwTime), dp]
        lib.port_set_time.argtypes = [vp, ctypes.POINTER(QgwTime), ctypes.c_double]
        lib.port_invert.argtypes = [vp]
        lib.port_timestep.argtypes = [vp]
        lib.port_run_steps.argtypes = [vp, ip, ip]
        lib.port_set_forcing_records.argtypes = [vp, dp, ip]
        lib.port_run_steps.restype = ip
        lib.port_dst1.argtypes = [ip, ip, dp, ip]
        lib.port_params_read.argtypes = [ctypes.POINTER(QgwParams), ctypes.c_char_p]
        lib.port_params_default.argtypes = [ctypes.POINTER(QgwParams)]
        _lib = lib
    return _lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def dst1(x: np.ndarray, fast: bool = True) -> np.ndarray:
    """DST-I (FFTW RODFT00) of each row of a 2-D array."""
    y = np.ascontiguousarray(x, dtype=np.float64).copy()
    _port_lib().port_dst1(y.shape[-1], y.size // y.shape[-1], _dp(y), int(fast))
    return y


class Port:
    """The C restatement of the reference step on one run."""

    def __init__(self, params: Dict[str, object], fast_dst: bool = True):
        self.lib = _port_lib()
        self.params = params
        self._s = to_struct(params)
        self.h = self.lib.port_create(ctypes.byref(self._s), int(fast_dst))
        self.shape = halo_shape(params)

    def close(self):
        if self.h:
            self.lib.port_destroy(self.h)
            self.h = None

    __del__ = close

    def set_q(self, q: np.ndarray):
        q = np.ascontiguousarray(q, dtype=np.float64)
        assert q.shape == self.shape
        self.lib.port_set_q(self.h, _dp(q))

    def set_topo(self, topo: np.ndarray):
        topo = np.ascontiguousarray(topo, dtype=np.float64)
        self.lib.port_set_topo(self.h, _dp(topo))

    def set_forcing_records(self, rec: np.ndarray):
        """The 4-D forcing's records, (nrec,) + the reference layout."""
        rec = np.ascontiguousarray(rec, dtype=np.float64)
        assert rec.shape[1:] == self.shape
        self.lib.port_set_forcing_records(self.h, _dp(rec), rec.shape[0])

    def get(self):
        psi, q = np.empty(self.shape), np.empty(self.shape)
        self.lib.port_get(self.h, _dp(psi), _dp(q))
        return psi, q

    def modes(self):
        nl = self.shape[0]
        a, b, c = np.empty((nl, nl)), np.empty((nl, nl)), np.empty(nl)
        self.lib.port_get_modes(self.h, _dp(a), _dp(b), _dp(c))
        return a, b, c

    def time(self):
        t = QgwTime()
        tout = ctypes.c_double()
        self.lib.port_get_time(self.h, ctypes.byref(t), ctypes.byref(tout))
        return {"t": t.t, "dt": t.dt, "dt0": t.dt0, "dt1": t.dt1, "DT_max": t.DT_max,
                "t_out": tout.value}

    def set_time(self, t=0.0, dt=0.0, dt0=None, dt1=None, DT_max=None, t_out=0.0):
        tm = QgwTime(t, dt, dt if dt0 is None else dt0, dt if dt1 is None else dt1,
                     dt if DT_max is None else DT_max)
        self.lib.port_set_time(self.h, ctypes.byref(tm), float(t_out))

    def fix_dt(self, dt: float):
        """The harness's fixed-step mode: dt = dt0 = dt1 = DT_max, no t_out."""
        self.set_time(0.0, dt, dt, dt, dt, 0.0)

    def invert(self):
        self.lib.port_invert(self.h)

    def step(self, n: int = 1, snap: bool = False) -> int:
        return self.lib.port_run_steps(self.h, int(n), int(snap))


def forcing_file_shape(params, nrec):
    """Shape of the q_forcing_3d records read_nc expects in input_vars.nc
    (src/netcdf_io.h:286-382): the full grid with walls, or the interior of
    a periodic basin."""
    nl, nyp2, nxp2 = halo_shape(params)
    ibc = 1 if float(params.get("bc_fac", 0.0)) == -1 else 0
    return (nrec, nl, nyp2 - 2 * ibc, nxp2 - 2 * ibc)


def forcing_records_layout(params, frec_file: np.ndarray) -> np.ndarray:
    """File records -> the reference layout read_nc fills (doubles)."""
    nl, nyp2, nxp2 = halo_shape(params)
    out = np.zeros((frec_file.shape[0], nl, nyp2, nxp2))
    if float(params.get("bc_fac", 0.0)) == -1:
        out[:, :, 1:-1, 1:-1] = frec_file
    else:
        out[:] = frec_file
    return out


def write_forcing_file(path, params, frec_file: np.ndarray):
    """input_vars.nc with q_forcing_3d(time, level, y, x), float."""
    from scipy.io import netcdf_file
    f = netcdf_file(path, "w", version=2)
    f.createDimension("time", None)
    f.createDimension("level", frec_file.shape[1])
    f.createDimension("y", frec_file.shape[2])
    f.createDimension("x", frec_file.shape[3])
    v = f.createVariable("q_forcing_3d", "f4", ("time", "level", "y", "x"))
    v[:] = frec_file.astype(np.float32)
    f.close()


def run_port(params, q0, nsteps, dt_fixed=None, topo=None, fast_dst=True, forcing_records=None):
    """Port counterpart of ``run_ref``: returns psi, q after ``nsteps``.
    ``forcing_records``: the 4-D forcing's records in the file layout."""
    p = Port(params, fast_dst)
    if forcing_records is not None:
        p.set_forcing_records(forcing_records_layout(params, forcing_records))
    if topo is not None:
        p.set_topo(topo)
    p.set_q(q0)
    p.invert()
    if dt_fixed:
        p.fix_dt(dt_fixed)
        p.step(nsteps, snap=False)
    else:
        p.step(nsteps, snap=True)
    p.invert()
    psi, q = p.get()
    tm = p.time()
    modes = p.modes()
    p.close()
    return {"psi": psi, "q": q, "time": tm, "modes": modes}


def run_ref(params, q0: Optional[np.ndarray], nsteps: int, dt_fixed: Optional[float] = None,
            mode: str = "step", topo: Optional[np.ndarray] = None, fast_dst: bool = False,
            forcing_records: Optional[np.ndarray] = None):
    """Run the reference's own step code (compiled in place) and return its
    outputs.  ``params`` may carry the extra ``dt`` key; it is written to the
    params file but the reference ignores it."""
    if not ref_available():
        raise RuntimeError("reference build oracle/_ref/qgw_ref is missing")
    shape = halo_shape(params)
    with tempfile.TemporaryDirectory() as d:
        pf = os.path.join(d, "params.in")
        write_params(pf, {k: v for k, v in params.items() if not k.startswith("_")})
        qf = "-"
        if q0 is not None:
            qf = os.path.join(d, "q0.bin")
            np.ascontiguousarray(q0, dtype=np.float64).tofile(qf)
        args = [REF_BIN, pf, qf, os.path.join(d, "out"), str(nsteps),
                repr(float(dt_fixed or 0.0)), mode]
        if topo is not None:
            tf = os.path.join(d, "topo.bin")
            np.ascontiguousarray(topo, dtype=np.float64).tofile(tf)
            args.append(tf)
        if forcing_records is not None:  # read by the reference itself (src/forcing.h:270-271)
            write_forcing_file(os.path.join(d, "input_vars.nc"), params, forcing_records)
        env = dict(os.environ)
        env["QGW_SHIM_DST"] = "fast" if fast_dst else "direct"
        subprocess.run(args, check=True, cwd=d, env=env, stdout=subprocess.DEVNULL)
        out = {
            "psi": np.fromfile(os.path.join(d, "out.psi")).reshape(shape),
            "q": np.fromfile(os.path.join(d, "out.q")).reshape(shape),
        }
        nl = shape[0]
        m = np.fromfile(os.path.join(d, "out.modes"))
        out["modes"] = (m[:nl * nl].reshape(nl, nl), m[nl * nl:2 * nl * nl].reshape(nl, nl),
                        m[2 * nl * nl:])
        if mode == "rhs":
            out["rhs"] = np.fromfile(os.path.join(d, "out.rhs")).reshape(shape)
        vals = open(os.path.join(d, "out.time")).read().split()
        out["time"] = dict(zip(["t", "dt", "dt0", "dt1", "DT_max", "t_out"], map(float, vals[:6])))
        out["time"]["steps"] = int(vals[6])
    return out


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    """||a - b||_2 / ||b||_2 (0 when both vanish)."""
    nb = float(np.linalg.norm(b))
    na = float(np.linalg.norm(a - b))
    return na / nb if nb > 0 else na
