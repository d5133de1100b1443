"""Domain diagnostics of a state in the reference layout, in numpy: the
checker of ``qgw_budget``.

Energy and enstrophy follow the reference's own diagnostic
(test/test_energy_injection.py:24-25: energy = -sum(psi q) Delta^2 / Lx^2,
enstrophy = sum(q^2) Delta^2 / Lx^2), weighted by the layer thicknesses
dh_k / H; KE uses the one-sided differences of the CFL rule
(src/timestep.h:77-78); the wind work is -dh_0/H psi_0 forcing_q, with
forcing_q the reference's surface PV forcing (src/domain.h:33) at the row's
coordinate Y_j = (j + J0) Delta (J0 = 0 closed, -1 periodic,
src/domain.h:144-148,163-168).  Every sum runs over interior points and is
scaled by Delta^2 / (Lx Ly)."""
import numpy as np


def budget_np(params, psi, q):
    """psi, q: (nl, ny+2, nx+2) with the ghost ring the reference holds after
    invert_pv (walls 0 in a closed basin, wrapped values when periodic)."""
    NX, NY = int(params["NX"]), int(params.get("NY", params["NX"]))
    Lx = float(params["Lx"])
    D = Lx / NX
    Ly = NY * D
    dh = np.asarray(params["dh"][: psi.shape[0]], dtype=np.float64)
    w = (dh / dh.sum())[:, None, None]
    P, Q = psi[:, 1:-1, 1:-1], q[:, 1:-1, 1:-1]
    u = (psi[:, 1:-1, 2:] - P) / D
    v = (psi[:, 2:, 1:-1] - P) / D
    scale = D * D / (Lx * Ly)
    ke = float((w * 0.5 * (u * u + v * v)).sum() * scale)
    energy = float(-(w * P * Q).sum() * scale)
    enstrophy = float((w * Q * Q).sum() * scale)
    periodic = float(params.get("bc_fac", 0.0)) == -1.0
    j0 = -1 if periodic else 0
    ny = P.shape[1]
    Y = (np.arange(1, ny + 1) + j0) * D
    fm = float(params.get("forc_mode", 0.0))
    fq = -float(params.get("tau0", 0.0)) / float(params["dh"][0]) * fm * np.pi / Ly * np.sin(fm * np.pi * Y / Ly)
    wind = float(-(w[0, 0, 0] * P[0] * fq[:, None]).sum() * scale)
    return {"ke": ke, "energy": energy, "enstrophy": enstrophy, "wind_work": wind}
