"""Run a few steps of one benchmark problem, for profilers (ncu) to attach to.

    python -m pluto_gb300.profile_case --problem blast --n 128 --precision mixed --steps 2

Runs ``--steps`` steps eagerly on a fresh solver (no CUDA graph, so every
kernel is a separate launch a profiler can select with -k/-s/-c).
"""
from __future__ import annotations

import argparse

from . import Solver, problems


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--problem", default="blast", choices=["blast", "turb", "ot"])
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "mixed_dw", "fp64"])
    ap.add_argument("--steps", type=int, default=2)
    args = ap.parse_args()
    if args.problem == "blast":
        spec, vc, faces = problems.blast3d(args.n)
    elif args.problem == "turb":
        spec, vc, faces = problems.turbulence3d(args.n)
    else:
        spec, vc, faces = problems.orszag_tang(args.n)
    s = Solver(spec, precision=args.precision)
    s.upload(vc, faces)
    dt = spec["first_dt"]
    for _ in range(args.steps):
        inv, _, _ = s.advance(dt)
        dt = min((1.0 / inv) * spec["cfl"], 1.1 * dt)
    print(f"ok {args.problem} n={args.n} {args.precision} steps={args.steps} next_dt={dt:.3e}")


if __name__ == "__main__":
    main()
