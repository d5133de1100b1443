"""Run a few time steps of one configuration, for profiler captures.

    python -m qgw_gb300.profile_step --nx 1024 --nl 10 --precision 0 --warmup 2 --steps 3

The warm-up steps and the captured steps are separate qgw_step calls, so a
profiler can skip the warm-up launches by count: each call launches one
begin kernel, 4 kernels per step, and a flush pair (2 kernels).
"""
import argparse
import time

from . import build, capi, configs


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--nx", type=int, default=1024)
    ap.add_argument("--nl", type=int, default=10)
    ap.add_argument("--precision", type=int, default=0)
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--steps", type=int, default=3)
    args = ap.parse_args()
    build.build()
    p = configs.cfg2(args.nx, args.nl)
    run = capi.Run(p, args.precision)
    run.set_q(configs.noise_ic(p, 2000))
    run.fix_dt(600.0)
    run.step(args.warmup)
    t0 = time.perf_counter()
    info = run.step(args.steps)
    dt = time.perf_counter() - t0
    assert info.steps_taken == args.steps
    print(f"{args.steps} steps of {args.nx}^2 x {args.nl} (precision {args.precision}): "
          f"{dt / args.steps * 1e3:.3f} ms/step (host timer)")
    run.close()


if __name__ == "__main__":
    main()
