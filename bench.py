#!/usr/bin/env python
"""Throughput of the MLS-MPM substep (particle-substeps/s) on the 1,048,576-particle scene.

Workload (the 3D float32 configuration): two seeded-uniform cubes of edge 0.2 centred at
(0.35,0.5,0.5) and (0.65,0.5,0.5) with x-velocities +1 and -1 m/s, 524,288 particles each,
128^3 grid, rho=1, nu=0.3, gravity -9.8, dt=5e-5.  E is 4.5e3 (elastic CFL number 0.5): at
E=5e4 the scene is past the explicit stability limit (CFL 1.66) and diverges in the float64
reference itself, so the stable variant with the same particles, grid, dt and memory traffic is
measured.  One step = one substep over all particles.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`ours`: the resident block-sorted solver replayed from CUDA graphs (value), the
reference-facing solve_mls_mpm_3d on pinned host arrays with the copies inside the timed region
(e2e), per-kernel CUDA-event times for the roofline, a float64 GPU run for the position error,
and the float64 C port of the reference timed on one host core (cpu_baseline).
`reference`: the float64 C port of the reference's numba loops (the reference is Python-only and
numba is not installed) on all host cores, on the same scene.
With N>1 (torchrun) every rank runs an independent replica of the scene (no collective on the
data path); the step time is the maximum over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "particle-substeps/s at 1M"
UNIT = "particle-substeps/s"
N_PER_CUBE = 524_288
RES, DT, GRAVITY, E_YOUNG, NU, EDGE = 128, 5e-5, -9.8, 4.5e3, 0.3, 0.2
WORKLOAD = "two_cubes_1M_res128"
SORT_EVERY = 8  # substeps between re-sorts by block (earlier when a particle leaves its block's neighbourhood)


def scene(seed: int = 0):
    from femflow_gb300.scenes import two_cubes

    return two_cubes(N_PER_CUBE, edge=EDGE, speed=1.0, E=E_YOUNG, nu=NU, seed=seed)


def config(extra=None):
    c = {"workload": WORKLOAD, "particles": 2 * N_PER_CUBE, "grid": f"{RES}^3", "dt": DT, "E": E_YOUNG, "nu": NU,
         "rho": 1.0, "material": "fixed-corotated ('neo_hookean' of the reference)",
         "l2": "no flush: a substep streams ~0.25 GB of particle state (> 129 MB L2)"}
    c.update(extra or {})
    return c


# --------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi samples (every 100 ms) of SM clock and throttle reasons, with wall timestamps."""

    FIELDS = "index,pci.bus_id,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown," \
             "clocks_event_reasons.sw_power_cap"

    def __init__(self, bus_id: str | None):
        self.samples = []
        self.bus = (bus_id or "").lower()
        self.proc = None
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            if self.bus and self.bus[-12:] not in parts[1].lower():
                continue
            try:
                self.samples.append((time.time(), float(parts[2]), float(parts[3]), parts[5:9]))
            except ValueError:
                pass

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, t0, t1):
        win = [s for s in self.samples if t0 - 0.15 <= s[0] <= t1 + 0.15] or self.samples
        if not win:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        seen = sorted({names[i] for s in win for i, v in enumerate(s[3]) if v.lower().startswith("active")})
        return {"sm_mhz": statistics.median(s[1] for s in win), "sm_max_mhz": max(s[2] for s in win),
                "reasons": seen, "samples": len(win)}


def measured_peak_hbm():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic():
    """Per-launch DRAM bytes of the profiled kernels, from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "traffic_two_cubes.txt")
    out = {}
    try:
        with open(path) as f:
            for line in f:
                parts = line.split()
                if len(parts) == 2 and not line.startswith("#"):
                    out[parts[0]] = int(parts[1])
    except (OSError, ValueError):
        pass
    return out


# --------------------------------------------------------------------------- ours
def run_ours(args):
    import torch
    import torch.distributed as dist

    from femflow_gb300 import replicas as REP
    from femflow_gb300.solver import MPMSolver
    from femflow_gb300.solvers.mpm import mls_mpm, three_d
    from femflow_gb300.solvers.mpm.particle import ParticleSet

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        dist.init_process_group("nccl", device_id=dev)

    barrier = REP.barrier

    s = scene()
    n = s["n"]
    props = torch.cuda.get_device_properties(dev)
    bus = getattr(props, "pci_bus_id", None)
    clocks = ClockSampler(bus if isinstance(bus, str) else None)

    solver = MPMSolver(torch.tensor(s["x"]), res=RES, dt=DT, gravity=GRAVITY, volume=s["vol"], mass=s["mass"],
                       mu_0=s["mu"], lambda_0=s["lam"], v=torch.tensor(s["v"]), dtype=torch.float32, device=dev,
                       sort_every=SORT_EVERY)
    info = solver.plan_info()
    solver.step(args.warmup)
    torch.cuda.synchronize(dev)
    # substeps per captured CUDA graph: a multiple of the re-sort cadence where the step count allows
    # (every call starts with a sort, so a graph of 40 re-sorts exactly every 8 substeps, a graph of
    # 10 at substeps 0 and 8 of every call)
    gsteps = next((c for c in (5 * SORT_EVERY, 2 * SORT_EVERY, SORT_EVERY, 10, 2) if args.steps % c == 0), 2)
    if args.steps % gsteps == 0:
        solver.capture(gsteps)

    stream = torch.cuda.current_stream(dev)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize(dev)
    t_wall0 = time.time()
    ev0.record(stream)
    solver.step(args.steps)
    ev1.record(stream)
    torch.cuda.synchronize(dev)
    t_wall1 = time.time()
    barrier()
    t = REP.max_over_ranks(ev0.elapsed_time(ev1) / 1e3, dev)
    status, fallbacks = solver.status()
    clocks.stop()
    value = world * n * args.steps / t
    gpu_launches = (args.steps // gsteps) * solver.kernels_per_call(gsteps) if args.steps % gsteps == 0 else \
        solver.kernels_per_call(args.steps)

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded two-cube scene)",
           "config": config({"parallelism": f"replicas{world}" if world > 1 else "single GPU",
                             "cuda_graph_substeps": gsteps, "radix_passes": info["radix_passes"],
                             "block_size": info["block_size"], "sort_every": SORT_EVERY}),
           "clocks": clocks.summary(t_wall0, t_wall1), "gpu_launches": int(gpu_launches),
           "status": {"device_status": status, "polar_fp64_fallbacks": fallbacks}}

    # ---- the same workload re-sorted by block before every substep (the fused launch before each
    # re-sort writes the keys), replayed from the same 40-substep graphs
    every = MPMSolver(torch.tensor(s["x"]), res=RES, dt=DT, gravity=GRAVITY, volume=s["vol"], mass=s["mass"],
                      mu_0=s["mu"], lambda_0=s["lam"], v=torch.tensor(s["v"]), dtype=torch.float32, device=dev,
                      sort_every=1)
    every.capture(40)
    every.step(40)
    torch.cuda.synchronize(dev)
    e_steps = 80
    barrier()
    ev0.record(stream)
    every.step(e_steps)
    ev1.record(stream)
    torch.cuda.synchronize(dev)
    te1 = REP.max_over_ranks(ev0.elapsed_time(ev1) / 1e3, dev)
    every.check()
    out["every_substep_sort"] = {"value": world * n * e_steps / te1, "unit": UNIT, "ms_per_step": 1e3 * te1 / e_steps,
                                 "steps": e_steps, "sort_every": 1, "cuda_graph_substeps": 40}
    del every

    # ---- batched 2D scenes: 256 seeded scenes (2k-64k particles, grids 64^2-256^2, E capped at
    # elastic CFL 0.5 per scene), autotuned launch shape, one 100-substep CUDA graph
    from femflow_gb300.batched import Batch2D, random_scenes, stable_variant

    bt = Batch2D(stable_variant(random_scenes(256, seed=0)), dtype=torch.float32, device=dev)
    shape, _ = bt.autotune(steps=1)
    bt.capture(100)
    bt.step(100)
    torch.cuda.synchronize(dev)
    b_steps = 300
    barrier()
    ev0.record(stream)
    bt.step(b_steps)
    ev1.record(stream)
    torch.cuda.synchronize(dev)
    tb = REP.max_over_ranks(ev0.elapsed_time(ev1) / 1e3, dev)
    out["batched_2d_256_scenes"] = {"value": world * bt.n * b_steps / tb, "unit": UNIT, "ms_per_step": 1e3 * tb / b_steps,
                                    "scenes": 256, "particles": bt.n, "steps": b_steps, "cuda_graph_substeps": 100,
                                    "launch_shape": {"threads": shape[0], "ctas_per_sm": shape[1]},
                                    "status": bt.status()}
    del bt

    # ---- per-kernel times (CUDA events around each phase, same stream) for the roofline
    pro_steps = min(args.steps, 40)
    prof = solver.profile(pro_steps)
    phase_ms = {k: v[0] / max(v[1], 1) for k, v in prof.items() if v[1]}
    # active grid nodes of the current state (dense float32 P2G on the reference-facing API)
    st = solver.sorted_state()
    R = RES + 1
    gv = torch.zeros((R, R, R, 3), device=dev)
    gm = torch.zeros((R, R, R, 1), device=dev)
    ps = ParticleSet(st["x"], torch.full((n,), s["mass"], device=dev), torch.full((n,), s["mu"], device=dev),
                     torch.full((n,), s["lam"], device=dev))
    three_d.p2g(float(RES), 1.0, 1 / RES, DT, s["vol"], gv, gm, ps, st["v"], st["F"], st["C"],
                st["Jp"].view(n, 1).contiguous())
    active = int((gm > 0).sum().item())
    del gv, gm
    # algorithmic bytes per launch: P2G reads x, v, F, C and adds 16 B per active node; G2P reads x, F,
    # ids and the node velocities and writes x, v, C, F, ids and the next key; the fused G2P + P2G reads
    # x, F, ids and the node velocities (12 B), writes x, F, ids, adds 16 B per node, and writes the
    # next key only on the launch before a re-sort (4 of the 39 fused launches of a 40-substep call
    # that re-sorts every 8)
    key_frac = ((gsteps - 2) // SORT_EVERY) / max(gsteps - 1, 1)  # fused launches that write keys
    alg = {"p2g": n * 96 + active * 16, "g2p": n * 144 + active * 12,
           "g2p2g": int(n * (104 + 4 * key_frac)) + active * 28}
    alg = {k: v for k, v in alg.items() if k in phase_ms}
    dom = max(alg, key=lambda k: phase_ms[k])
    peak, peak_kind = measured_peak_hbm()
    achieved = alg[dom] / (phase_ms[dom] / 1e3) / 1e9
    traffic = ncu_traffic().get(dom)
    out["roofline"] = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                       "frac": achieved / peak, "peak_source": f"{peak_kind} hbm_gbs", "traffic": traffic,
                       "algorithmic_bytes_per_launch": alg[dom], "active_nodes": active,
                       "phase_ms_per_launch": phase_ms,
                       "phase_gbps": {k: alg[k] / (phase_ms[k] / 1e3) / 1e9 for k in alg}}

    # ---- end to end through the reference-facing API with pinned host arrays
    e2e_steps = min(args.steps, 20)
    h = lambda a: torch.tensor(a, dtype=torch.float32).pin_memory()
    pset = ParticleSet(h(s["x"]), h(np.full(n, s["mass"])), h(np.full(n, s["mu"])), h(np.full(n, s["lam"])))
    v_h, F_h, C_h, J_h = h(s["v"]), h(np.tile(np.eye(3), (n, 1, 1))), h(np.zeros((n, 3, 3))), h(np.ones((n, 1)))
    mls_mpm.solve_mls_mpm_3d(RES, float(RES), 1.0, 1 / RES, DT, s["vol"], GRAVITY, pset, v_h, F_h, C_h, J_h)
    torch.cuda.synchronize(dev)
    barrier()
    e0 = time.perf_counter()
    for _ in range(e2e_steps):
        mls_mpm.solve_mls_mpm_3d(RES, float(RES), 1.0, 1 / RES, DT, s["vol"], GRAVITY, pset, v_h, F_h, C_h, J_h)
    torch.cuda.synchronize(dev)
    te = REP.max_over_ranks(time.perf_counter() - e0, dev)
    out["e2e"] = {"value": world * n * e2e_steps / te, "unit": UNIT, "h2d_bytes_per_step": n * (12 + 12 + 12 + 36 + 36),
                  "d2h_bytes_per_step": n * (12 + 12 + 36 + 36), "steps": e2e_steps,
                  "api": "solve_mls_mpm_3d on pinned host float32 arrays (ffmpm_substep_host: uploads, scatter, "
                         "gather and downloads pipelined over chunks of particles)"}

    # ---- position error against a float64 GPU run of the same scene
    err_steps = args.fp64_steps
    if err_steps > 0:
        kw = dict(res=RES, dt=DT, gravity=GRAVITY, volume=s["vol"], mass=s["mass"], mu_0=s["mu"], lambda_0=s["lam"],
                  v=torch.tensor(s["v"]), device=dev)
        a32 = MPMSolver(torch.tensor(s["x"]), dtype=torch.float32, **kw)
        a64 = MPMSolver(torch.tensor(s["x"]), dtype=torch.float64, **kw)
        a32.step(err_steps)
        a64.step(err_steps)
        d32, d64 = a32.diagnostics(), a64.diagnostics()
        err = (a32.positions().double() - a64.positions()).abs().max().item()
        e_tot = lambda d: d["kinetic"] + d["elastic"] + d["gravitational"]
        out["fp64_error"] = {"substeps": err_steps, "max_position_error_domain_rel": err,
                             "energy_rel_diff": abs(e_tot(d32) - e_tot(d64)) / abs(e_tot(d64))}
        del a32, a64

    # ---- CPU baseline: the float64 C port of the reference on one host core
    if rank == 0 and world == 1 and args.cpu_steps > 0:
        out["cpu_baseline"] = cpu_port_baseline(s, args.cpu_steps)
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        dist.destroy_process_group()


def cpu_port_baseline(s, steps):
    import oracle as O

    O.build()
    n = s["n"]
    x, v = s["x"].copy(), s["v"].copy()
    F = np.tile(np.eye(3), (n, 1, 1)); C = np.zeros((n, 3, 3)); Jp = np.ones((n, 1))
    mass, mu, lam = np.full(n, s["mass"]), np.full(n, s["mu"]), np.full(n, s["lam"])
    t0 = time.perf_counter()
    for _ in range(steps):
        O.substep_3d(RES, float(RES), 1.0, 1 / RES, DT, s["vol"], GRAVITY, x, mass, mu, lam, v, F, C, Jp)
    t = time.perf_counter() - t0
    return {"value": n * steps / t, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{steps} substeps of the full {n}-particle scene, float64, serial C restatement of "
                      "three_d/{p2g,grid_op,g2p}.py incl. the per-substep dense grid allocation"}


# --------------------------------------------------------------------------- reference arm
def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return
    import oracle as O

    O.build()
    threads = os.cpu_count() or 1
    s = scene()
    n = s["n"]
    grid = np.empty((RES + 1) ** 3 * 4)

    def state(idx):
        m = len(idx)
        return dict(x=s["x"][idx].copy(), v=s["v"][idx].copy(), F=np.tile(np.eye(3), (m, 1, 1)),
                    C=np.zeros((m, 3, 3)), Jp=np.ones((m, 1)), mass=np.full(m, s["mass"]), mu=np.full(m, s["mu"]),
                    lam=np.full(m, s["lam"]))

    def substep(st):
        O.substep_3d_par(RES, float(RES), 1.0, 1 / RES, DT, s["vol"], GRAVITY, st["x"], st["mass"], st["mu"],
                         st["lam"], st["v"], st["F"], st["C"], st["Jp"], nthreads=threads, grid_scratch=grid)

    full = state(np.arange(n))
    t0 = time.perf_counter()
    substep(full)
    t_full = time.perf_counter() - t0
    cap_s = 150.0  # seconds of CPU work for the whole run
    frac = min(1.0, cap_s / max(1e-9, (args.steps + args.warmup) * t_full))
    if frac < 1.0:
        rng = np.random.default_rng(1)
        idx = np.sort(rng.choice(n, size=max(1024, int(n * frac)), replace=False))
        st = state(idx)
    else:
        st = full
    m = len(st["x"])
    for _ in range(args.warmup):
        substep(st)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        substep(st)
    t = time.perf_counter() - t0
    value = m * args.steps / t
    sample = (f"{'all' if m == n else m} of the {n} particles per substep on the {RES}^3 grid, float64, OpenMP C "
              f"restatement of the reference's numba loops (three_d/{{p2g,grid_op,g2p}}.py)")
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded two-cube scene)", "config": config(),
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "gpu_launches": 0}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--fp64-steps", type=int, default=1000, help="substeps of the float32-vs-float64 error run")
    ap.add_argument("--cpu-steps", type=int, default=8, help="substeps of the serial CPU-port baseline (0: skip)")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
