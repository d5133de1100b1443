"""Workload definitions: the closed-basin double-gyre runs the engine is
measured on, written as reference ``params.in`` settings, and the seeded
synthetic initial conditions.

Physical settings -> reference keys:
  * wind stress 0.08 (1 - cos(2 pi y / L)) N/m^2 with rho0 = 1000 is the
    kinematic ``tau0 = 8e-5`` with ``forc_mode = 2`` (src/domain.h:33);
  * reduced gravity g'_l at interface l is ``N2_l = g'_l / dhc_l`` with
    ``dhc_l = (dh_l + dh_{l+1}) / 2`` (src/eigmode.h:19-20, :108-118);
  * linear bottom drag r is ``hEkb = 2 r dh_{nl-1} / f0`` (src/dynamics.h:68);
  * free-slip walls are ``bc_fac = 0``; ``NX = 256`` gives 255 interior
    points per side (src/domain.h:71-74), the DST length whose FFT size is a
    power of two;
  * the fixed time step uses the optional ``dt`` key (the reference has no
    such key and always adapts dt; its parser ignores unknown keys).
"""
from __future__ import annotations

import math
from typing import Dict, List

import numpy as np

from .params import halo_shape

RHO0 = 1000.0
LX = 4.0e6
F0 = 1e-4
BETA = 2e-11
DRAG = 1e-7


def layer_profile(nl: int, total: float = 4000.0, ratio: float = 1.3,
                  gp_top: float = 0.02, gp_bottom: float = 0.002):
    """Geometrically stretched thicknesses summing to ``total`` and reduced
    gravities decreasing geometrically from ``gp_top`` to ``gp_bottom``."""
    if nl == 1:
        return [total], []
    if nl == 3:  # the 3-layer basin profile
        return [500.0, 1000.0, 2500.0], [0.02, 0.01]
    dh0 = total * (ratio - 1.0) / (ratio ** nl - 1.0)
    dh = [dh0 * ratio ** k for k in range(nl)]
    if nl == 2:
        gp = [gp_top]
    else:
        gp = [gp_top * (gp_bottom / gp_top) ** (l / (nl - 2)) for l in range(nl - 1)]
    return dh, gp


def basin_params(NX: int, nl: int, *, tau_nm2: float = 0.08, dt: float = 1200.0,
                 nu: float = 0.0, n_hyper: int = 0, nu_hyper: float = 0.0,
                 tend: float = 1e12, dt_out: float = 1e12) -> Dict[str, object]:
    dh, gp = layer_profile(nl)
    dhc = [0.5 * (dh[l] + dh[l + 1]) for l in range(nl - 1)]
    N2 = [gp[l] / dhc[l] for l in range(nl - 1)] or [1.0]
    return {
        "NX": NX, "NY": NX, "nl": nl, "Lx": LX, "dh": dh, "N2": N2,
        "f0": F0, "beta": BETA, "tau0": tau_nm2 / RHO0, "forc_mode": 2.0,
        "nu": nu, "n_hyper": n_hyper, "nu_hyper": nu_hyper,
        "hEkb": 2.0 * DRAG * dh[-1] / F0, "bc_fac": 0.0,
        "tend": tend, "dt_out": dt_out, "dt": dt,
    }


def cfg1(NX: int = 256) -> Dict[str, object]:
    """3 layers, Laplacian viscosity 50 m^2/s on q, dt = 1200 s."""
    return basin_params(NX, 3, dt=1200.0, nu=50.0)


def cfg2(NX: int = 1024, nl: int = 10) -> Dict[str, object]:
    """10 stretched layers, biharmonic viscosity 1e9 m^4/s, dt = 600 s."""
    return basin_params(NX, nl, dt=600.0, nu=0.0, n_hyper=4, nu_hyper=1e9)


def noise_ic(params: Dict[str, object], seed: int, std: float = 1e-7) -> np.ndarray:
    """Seeded FP64 Gaussian q on interior points, zero ghost ring, in the
    reference layout (nl, ny+2, nx+2)."""
    nl, nyp2, nxp2 = halo_shape(params)
    rng = np.random.Generator(np.random.PCG64(seed))
    q = np.zeros((nl, nyp2, nxp2))
    q[:, 1:-1, 1:-1] = rng.normal(0.0, std, size=(nl, nyp2 - 2, nxp2 - 2))
    return q


def ensemble_members(n: int = 64, seed: int = 4000) -> List[Dict[str, object]]:
    """Uneven ensemble: grids from {128, 256, 512, 1024}^2, nl from
    {2, 3, 5, 10}, wind amplitude uniform in [0.04, 0.12] N/m^2."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for m in range(n):
        NX = int(rng.choice([128, 256, 512, 1024]))
        nl = int(rng.choice([2, 3, 5, 10]))
        tau = float(rng.uniform(0.04, 0.12))
        p = basin_params(NX, nl, tau_nm2=tau, dt=600.0, n_hyper=4, nu_hyper=1e9)
        p["_seed"] = seed + m
        out.append(p)
    return out


def lgp(params: Dict[str, object]) -> int:
    """Layer-gridpoints of one step: nl * (NX-1) * (NY-1)."""
    nl, nyp2, nxp2 = halo_shape(params)
    return nl * (nyp2 - 2) * (nxp2 - 2)


def public(params: Dict[str, object]) -> Dict[str, object]:
    """Drop private (underscore) keys before writing params.in."""
    return {k: v for k, v in params.items() if not k.startswith("_")}


__all__ = ["basin_params", "cfg1", "cfg2", "noise_ic", "ensemble_members", "lgp",
           "layer_profile", "public", "math"]
