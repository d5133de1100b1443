"""params.in model of qgw and the ctypes mirror of ``qgw_params``.

The reference reads its configuration from a ``params.in`` file of
``key = value`` / ``key = [a, b, ...]`` lines (``src/extra.h:118-153``) into
the globals registered at ``src/qg.c:113-137``.  This module holds the same
key set with the reference defaults (``src/qg.c:57-83``,
``src/forcing.h:13-14,38-39``), writes ``params.in`` text, and converts a
dict into the ``qgw_params`` C struct of ``include/qgw_gpu.h``.  Parsing a
file is done by the C library (``qgw_params_read``) so that there is a single
parser implementation on the product path.
"""
from __future__ import annotations

import ctypes
from typing import Dict, Iterable

NL_MAX = 1000  # QGW_NL_MAX in include/qgw_gpu.h

INT_KEYS = ("NX", "NY", "nl", "n_hyper")
ARRAY_KEYS = ("dh", "N2")
DOUBLE_KEYS = ("Lx", "tau0", "forc_mode", "f0", "beta", "nu", "nu_hyper", "hEkb",
               "Ld", "h_topo", "w_topo", "bc_fac", "tend", "dt_out", "dt_forc",
               "dt_forc_period", "sigma_f", "k_f", "cfl", "dt")

# reference defaults (src/qg.c:57-83, src/forcing.h:13-14,38-39); `dt` is the
# optional fixed-step key of this library (0 = adaptive, as the reference)
DEFAULTS: Dict[str, object] = {
    "NX": 0, "NY": 0, "nl": 1, "n_hyper": 0, "Lx": 0.0, "dh": [1.0], "N2": [1.0],
    "tau0": 0.0, "forc_mode": 1.0, "f0": 1e-5, "beta": 0.0, "nu": 0.0,
    "nu_hyper": 0.0, "hEkb": 0.0, "Ld": 0.0, "h_topo": 0.0, "w_topo": 1.0,
    "bc_fac": 0.0, "tend": 1.0, "dt_out": 0.1, "dt_forc": 0.0,
    "dt_forc_period": 0.0, "sigma_f": 1.0, "k_f": 0.0, "cfl": 0.2, "dt": 0.0,
}


class QgwParams(ctypes.Structure):
    """ctypes layout of ``qgw_params`` (include/qgw_gpu.h)."""

    _fields_ = ([(k, ctypes.c_int) for k in INT_KEYS]
                + [("Lx", ctypes.c_double),
                   ("dh", ctypes.c_double * NL_MAX),
                   ("N2", ctypes.c_double * NL_MAX)]
                + [(k, ctypes.c_double) for k in
                   ("tau0", "forc_mode", "f0", "beta", "nu", "nu_hyper", "hEkb", "Ld",
                    "h_topo", "w_topo", "bc_fac", "tend", "dt_out", "dt_forc",
                    "dt_forc_period", "sigma_f", "k_f", "cfl", "dt")])


class QgwTime(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in ("t", "dt", "dt0", "dt1", "DT_max")]


class QgwStepInfo(ctypes.Structure):
    _fields_ = [("time", QgwTime), ("steps_taken", ctypes.c_int),
                ("stop_reason", ctypes.c_int), ("nonfinite", ctypes.c_int)]


class QgwShape(ctypes.Structure):
    """Work-tile shape of a run's step kernels (qgw_shape)."""
    _fields_ = [(k, ctypes.c_int) for k in ("rhs_tile_rows", "col_tile", "row_group_fwd", "row_group_inv")]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


class QgwBudget(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in ("ke", "energy", "enstrophy", "wind_work")]


def full(params: Dict[str, object]) -> Dict[str, object]:
    """Defaults overlaid with ``params`` (unknown keys are kept, as the
    reference ignores them)."""
    out = dict(DEFAULTS)
    out["dh"] = list(DEFAULTS["dh"])
    out["N2"] = list(DEFAULTS["N2"])
    out.update(params)
    return out


def to_struct(params: Dict[str, object]) -> QgwParams:
    p = full(params)
    s = QgwParams()
    for k in INT_KEYS:
        setattr(s, k, int(p[k]))
    for k in DOUBLE_KEYS:
        setattr(s, k, float(p[k]))
    for k in ARRAY_KEYS:
        vals = list(p[k])
        if len(vals) > NL_MAX:
            raise ValueError(f"{k} has {len(vals)} entries, at most {NL_MAX} supported")
        arr = getattr(s, k)
        for i, v in enumerate(vals):
            arr[i] = float(v)
    return s


def _fmt(v) -> str:
    if isinstance(v, (list, tuple)):
        return "[" + ", ".join(repr(float(x)) for x in v) + "]"
    if isinstance(v, int):
        return str(v)
    return repr(float(v))


def params_text(params: Dict[str, object], keys: Iterable[str] | None = None) -> str:
    """``params.in`` text for ``params`` (only the given keys; all by default)."""
    keys = list(params.keys()) if keys is None else list(keys)
    lines = ["# qgw params.in"]
    for k in keys:
        lines.append(f"{k} = {_fmt(params[k])}")
    return "\n".join(lines) + "\n"


def write_params(path: str, params: Dict[str, object]) -> None:
    with open(path, "w") as f:
        f.write(params_text(params))


def interior_shape(params: Dict[str, object]):
    """(nl, ny, nx) interior sizes; closed basins drop one point per side
    (src/domain.h:71-74)."""
    p = full(params)
    nx, ny = int(p["NX"]), int(p["NY"])
    if float(p["bc_fac"]) >= 0:
        nx, ny = nx - 1, ny - 1
    return int(p["nl"]), ny, nx


def halo_shape(params: Dict[str, object]):
    nl, ny, nx = interior_shape(params)
    return nl, ny + 2, nx + 2
