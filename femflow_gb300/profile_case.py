"""Small driver for profilers: the two-cube scene stepped by the resident solver.

    python -m femflow_gb300.profile_case [--n-per-cube N] [--res R] [--warmup W] [--steps K]

Runs W + K substeps with direct launches (no CUDA graph, so every kernel shows up by name),
synchronises, checks the device status word and prints one line.
"""
from __future__ import annotations

import argparse
import time

import torch

from .scenes import two_cubes
from .solver import MPMSolver


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n-per-cube", type=int, default=524_288)
    ap.add_argument("--res", type=int, default=128)
    ap.add_argument("--dt", type=float, default=5e-5)
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--dtype", choices=["f32", "f64"], default="f32")
    ap.add_argument("--variant", type=int, default=0, help="kernel variant flags (see ffmpm_params.variant)")
    ap.add_argument("--block-size", type=int, default=0)
    ap.add_argument("--sort-every", type=int, default=8, help="substeps between re-sorts")
    ap.add_argument("--deterministic", action="store_true", help="bit-reproducible P2G (re-sorts every substep)")
    args = ap.parse_args()
    s = two_cubes(args.n_per_cube)
    dtype = torch.float32 if args.dtype == "f32" else torch.float64
    solver = MPMSolver(torch.tensor(s["x"]), res=args.res, dt=args.dt, gravity=-9.8, volume=s["vol"],
                       mass=s["mass"], mu_0=s["mu"], lambda_0=s["lam"], v=torch.tensor(s["v"]), dtype=dtype,
                       variant=args.variant, block_size=args.block_size, sort_every=args.sort_every,
                       deterministic=args.deterministic)
    solver.step(args.warmup)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    solver.step(args.steps)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    solver.check()
    prof = solver.profile(args.steps)
    per = {k: round(v[0] / v[1] * 1e3, 2) for k, v in prof.items() if v[1]}
    print(f"profile_case: {s['n']} particles, res {args.res}, {args.steps} substeps in {dt * 1e3:.2f} ms "
          f"({s['n'] * args.steps / dt:.3e} particle-substeps/s), plan {solver.plan_info()}, "
          f"us per launch {per}")


if __name__ == "__main__":
    main()
