"""Run a few time steps of one configuration, for profiler captures (the
commands of the profiles/ summaries run this file).

    python tests/profile_step.py --nx 1024 --nl 10 --precision 0 --warmup 2 --steps 3

The warm-up steps and the captured steps are separate qgw_step calls, so a
profiler can skip the warm-up launches by count: each call launches one
begin kernel, 4 kernels per step (7 with stochastic forcing), and a flush
pair (2 kernels).
"""
import argparse
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
from qgw_gb300 import build, capi, configs  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--nx", type=int, default=1024)
    ap.add_argument("--nl", type=int, default=10)
    ap.add_argument("--precision", type=int, default=0)
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--variant", default="closed", choices=("closed", "periodic", "stochastic", "forcing4d"),
                    help="closed basin; doubly periodic; periodic with stochastic ring forcing "
                         "(ring radius 40 wavenumbers); closed with 4-D forcing (4 records)")
    args = ap.parse_args()
    build.build()
    p = configs.cfg2(args.nx, args.nl)
    if args.variant in ("periodic", "stochastic"):
        p = dict(p, bc_fac=-1.0)
    if args.variant == "stochastic":
        p = dict(p, k_f=2 * np.pi * 40 / p["Lx"], sigma_f=1e-12)
    if args.variant == "forcing4d":
        p = dict(p, dt_forc=3600.0, dt_forc_period=4 * 3600.0)
    run = capi.Run(p, args.precision)
    if args.variant == "forcing4d":
        shape = (4,) + tuple(configs.noise_ic(p, 1).shape)
        run.set_forcing_records(np.random.Generator(np.random.PCG64(7)).normal(0.0, 1e-12, size=shape))
    run.set_q(configs.noise_ic(p, 2000))
    run.fix_dt(600.0)
    run.step(args.warmup)
    t0 = time.perf_counter()
    info = run.step(args.steps)
    dt = time.perf_counter() - t0
    assert info.steps_taken == args.steps
    print(f"{args.steps} steps of {args.nx}^2 x {args.nl} {args.variant} (precision {args.precision}): "
          f"{dt / args.steps * 1e3:.3f} ms/step (host timer)")
    run.close()


if __name__ == "__main__":
    main()
