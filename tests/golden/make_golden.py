"""Generate the golden fixtures of tests/golden/ from the REFERENCE ITSELF.

Each case runs the reference's own src/qg.c (compiled in place with the
oracle shims, oracle/_ref/qgw_ref) from a seeded initial condition and
stores inputs and outputs as compressed npz.  One case is driven by the
parameter file the reference ships as test/params_03.in (read here from the
reference tree; the fixture stores the parsed values, not the file).

Run in the container that holds the reference sources:
    python tests/golden/make_golden.py            # every case
    python tests/golden/make_golden.py NAME ...   # only these (index merged)
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402
from qgw_gb300 import configs as C  # noqa: E402

# the reference's test/ directory beside the src/ that the oracle recipe reads
REF_TEST = os.environ.get("QGW_REF_TEST") or os.path.join(os.path.dirname(O.ref_source_dir()), "test")


def parse_params_in(path):
    """Minimal reader of a params.in for the fixture metadata (the reference
    parser itself is what the run uses)."""
    out = {}
    ints = {"NX", "NY", "nl", "n_hyper"}
    for line in open(path):
        line = line.replace(" ", "").strip()
        if "=" not in line or line.startswith("#"):
            continue
        k, v = line.split("=", 1)
        if v.startswith("["):
            out[k] = [float(x) for x in v.strip("[]").split(",")]
        else:
            try:
                out[k] = int(v) if k in ints else float(v.rstrip(";"))
            except ValueError:
                pass
    return out


def cases():
    out = []
    p = C.cfg1(64)
    out.append(("cfg1_nx64_fixed", p, 100, 1200.0, None))
    p = C.cfg2(32, 10)
    out.append(("cfg2_nx32_nl10_fixed", p, 100, 600.0, None))
    p = C.cfg1(32)
    p = {k: v for k, v in p.items() if k != "dt"}
    p.update(tend=1e9, dt_out=86400.0 * 2)
    out.append(("cfg1_nx32_adaptive", p, 40, None, None))
    p = C.cfg1(32)
    p.update(bc_fac=0.6, h_topo=150.0, w_topo=3e5)
    out.append(("noslip_topo_nx32", p, 50, 1200.0, None))
    p = C.cfg1(64)
    p["NY"] = 32
    out.append(("cfg1_nx64_ny32", p, 30, 1200.0, None))
    ref03 = os.path.join(REF_TEST, "params_03.in")
    if os.path.exists(ref03):
        p = parse_params_in(ref03)
        p["tend"] = 1e12
        out.append(("ref_params03", p, 30, None, None))
    # periodic basin (bc_fac = -1): r2c/c2r inversion, periodic ghosts
    p = C.cfg1(32)
    p.update(bc_fac=-1.0)
    out.append(("periodic_nx32", p, 50, 1200.0, None))
    p = C.cfg2(32, 10)
    p.update(bc_fac=-1.0)
    out.append(("periodic_nx32_nl10_hyper", p, 50, 600.0, None))
    p = C.cfg1(64)
    p.update(bc_fac=-1.0, h_topo=150.0, w_topo=3e5)
    out.append(("periodic_topo_nx64", p, 30, 1200.0, None))
    # stochastic ring forcing (src/forcing.h:67-201), the reference's own
    # test configurations scaled down (test/params_05.in periodic,
    # test/params_02.in closed): rand() from a fresh process
    p = stochastic_params(32, -1.0)
    out.append(("stochastic_periodic_nx32", p, 30, 5e-4, None))
    p = stochastic_params(64, 0.0)
    p.update(k_f=30.0)
    out.append(("stochastic_closed_nx64", p, 20, 5e-4, None))
    # 4-D forcing from input_vars.nc (src/forcing.h:226-288): 3 records of
    # q_forcing_3d, period 3 dt_forc, the run crossing record boundaries
    for name, bc, nx in (("forcing4d_closed_nx32", 0.0, 32), ("forcing4d_periodic_nx32", -1.0, 32)):
        p = C.cfg1(nx)
        p.update(bc_fac=bc, dt_forc=7200.0, dt_forc_period=3 * 7200.0)
        rng = np.random.Generator(np.random.PCG64(8100 + int(nx) + int(bc)))
        frec = (rng.normal(0.0, 1e-11, size=O.forcing_file_shape(p, 3))).astype(np.float32)
        out.append((name, p, 40, 1200.0, None, frec))
    # grids that are not powers of two (FFTW plans any length): DST-I of
    # 95 x 59 points (half-lengths 48 = 8*2*3, 30 = 2*3*5), hyperviscous
    # 49^2 x 10 (25 = 5*5), a periodic 48^2 basin (24 = 8*3, 48)
    p = C.cfg1(96)
    p["NY"] = 60
    out.append(("mixed_radix_nx96_ny60", p, 50, 1200.0, None))
    p = C.cfg2(50, 10)
    out.append(("mixed_radix_nx50_nl10_hyper", p, 40, 600.0, None))
    p = C.cfg1(48)
    p.update(bc_fac=-1.0)
    out.append(("periodic_nx48", p, 40, 1200.0, None))
    # many layers: 20 stretched layers with hyperviscosity (the row kernels'
    # mode and layer groups for more than 10 layers); dh and N2 to 6 digits,
    # since the reference reads params.in lines into 300 characters
    # (src/extra.h:121-122) and would cut a longer list short
    p = C.cfg2(32, 20)
    p["dh"] = [float(f"{x:.6g}") for x in p["dh"]]
    p["N2"] = [float(f"{x:.6g}") for x in p["N2"]]
    out.append(("cfg2_nx32_nl20_hyper", p, 40, 600.0, None))
    # lengths whose half-length FFT would need a radix above 7, or that are
    # odd (FFTW plans them; the GPU runs them as chirp-z transforms): 22^2
    # (half-length 11), 45 x 26 with hyperviscosity (odd; half-length 13)
    out.append(("chirp_z_nx22", C.cfg1(22), 40, 1200.0, None))
    p = C.cfg2(45, 5)
    p["NY"] = 26
    out.append(("chirp_z_nx45_ny26_hyper", p, 40, 600.0, None))
    return out


def stochastic_params(NX, bc_fac):
    return dict(NX=NX, NY=NX, nl=1, Lx=1.0, f0=2.0, beta=0.0, tau0=0.0, forc_mode=4.0, k_f=20.0,
                sigma_f=3.0, bc_fac=bc_fac, dh=[1.0], N2=[0.0], nu=0.01, hEkb=0.0, tend=1e12,
                dt_out=0.01, cfl=0.2, n_hyper=0, nu_hyper=0.0)


def main():
    O.build(ref=True)
    if not O.ref_available():
        raise SystemExit("reference build unavailable")
    only = set(sys.argv[1:])
    index_path = os.path.join(HERE, "index.json")
    index = {}
    if only and os.path.exists(index_path):
        with open(index_path) as f:
            index = json.load(f)
    for n, case in enumerate(cases()):
        name, params, nsteps, dt, topo = case[:5]
        frec = case[5] if len(case) > 5 else None
        if only and name not in only:
            continue
        seed = 7000 + n
        q0 = C.noise_ic(params, seed)
        r = O.run_ref(params, q0, nsteps, dt_fixed=dt, fast_dst=False, forcing_records=frec)
        extra = {} if frec is None else {"frec": frec}
        np.savez_compressed(os.path.join(HERE, name + ".npz"), q0=q0, psi=r["psi"], q=r["q"],
                            cl2m=r["modes"][0], cm2l=r["modes"][1], iRd2=r["modes"][2], **extra)
        index[name] = {"params": params, "nsteps": nsteps, "dt_fixed": dt, "seed": seed,
                       "time": r["time"]}
        print(name, r["time"])
    with open(index_path, "w") as f:
        json.dump(index, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
