"""Train the learned corrector and measure it against the plain fine-dt and plain coarse-dt forms.

    python -m femflow_gb300.learned_eval [--res 128 --dt 5e-5 --ratio 8 --horizon 50 ...]

1. Data: fine-dt rollouts of ``--scenes`` seeded two-cube scenes (E log-uniform in --E-range, nu in
   [0.2, 0.35], speeds in [0.5, 1.5], textbook fixed-corotated stress), ``--samples`` sample points
   each (one coarse step exported, k fine steps as the target).
2. Training on the tensor cores (``learned.train``), then ``onpolicy_rounds`` rounds that add samples
   taken on the trajectory of the velocity-corrected coarse step itself (``generate_on_policy``)
   and train on the union.  A network trained on fine-rollout states alone makes the closed-loop
   error worse (its corrections move the state to where it has seen no data); the on-policy
   samples teach it the states it meets when it runs.
3. Selection on a held-out validation scene (its own seed) at the evaluation horizon: the corrected
   outputs ("v": velocity only, "all": velocity and F) and the strength in {0, 1/4, 1/2, 1}; strength
   0 (the network off) is always a candidate, so the selected form is never worse than the plain
   coarse step on the validation scene.
4. Evaluation on the two-cube scene of 2 x ``--n-per-cube`` particles: plain fine rollout (the
   reference for the error), plain coarse rollout and the selected corrected rollout with the det F / energy fallback,
   each timed end to end on the GPU (synchronised wall clock), for the same simulated time.  The
   fine and the plain coarse forms are also timed on the resident block-sorted solver (all substeps in
   one call; the fastest form of each), and the corrected form runs there too when the selected
   strength is 0 (the network off).
"""
from __future__ import annotations

import argparse
import json
import time

import torch

from . import learned as L


def select(net: L.Net, spec: L.SceneSpec, res, dt, ratio, horizon) -> dict:
    st = L.Stepper(spec, res=res, dt=dt, ratio=ratio)
    b0 = st.initial_state()
    fine = b0.clone()
    L.rollout_fine(st, fine, horizon * ratio)
    trials = []
    for mode in ("v", "all"):
        for a in (0.0, 0.25, 0.5, 1.0):
            if a == 0.0 and mode == "all":
                continue
            cor = L.Corrector(net, st, a)
            if mode == "v":
                cor.out_scale[0:9] = 0.0
            b = b0.clone()
            for _ in range(horizon):
                st.coarse_step(b, cor)
            err = L.position_error(b, fine)["max"]
            # a trial whose corrections drove a particle out of the grid fails (and must not leave
            # its status bits to the next one)
            left_grid = st.ws.status()[0] != 0 or int(st.status.item()) != 0
            if left_grid:
                st.ws.clear_status()
                st.status.zero_()
            ok = err == err and not left_grid
            trials.append(dict(mode=mode, strength=a, err_max=err if ok else float("inf")))
    best = min(trials, key=lambda t: t["err_max"])
    return dict(best=best, trials=trials)


def bounded_rows(X: torch.Tensor, T: torch.Tensor, out_scale: torch.Tensor, max_target: float):
    """Samples (rows of X, T) whose targets stay within `max_target` output scales and whose
    features and targets are finite, and the number of rows dropped.  A corrected trajectory can
    blow up locally without leaving the grid; the fine rollout from such a state gives targets far
    outside what the network is meant to learn, and a few of them dominate the squared loss."""
    ts = (T / out_scale).abs().amax(dim=1)
    ok = torch.isfinite(ts) & (ts < max_target) & torch.isfinite(X.float()).all(dim=1)
    return X[ok], T[ok], int((~ok).sum())


def velocity_corrector(net, st, strength):
    cor = L.Corrector(net, st, strength)
    cor.out_scale[0:9] = 0.0
    return cor


def corrector_for(net, st, choice):
    cor = L.Corrector(net, st, choice["strength"])
    if choice["mode"] == "v":
        cor.out_scale[0:9] = 0.0
    return cor


def run(res=128, dt=5e-5, ratio=8, scenes=16, per_cube=524288, samples=4, steps=4000, batch=32768, horizon=150,
        n_per_cube=524288, E_eval=120.0, E_range=(50.0, 200.0), seed=0, onpolicy_rounds=3, onpolicy_samples=8,
        onpolicy_gap=10, round_steps=None, keep=1.0 / 16, max_target=30.0) -> dict:
    rep = dict(res=res, dt_fine=dt, ratio=ratio, dt_coarse=dt * ratio, horizon_coarse_steps=horizon,
               simulated_time=horizon * ratio * dt, E_range=E_range, E_eval=E_eval, model="fixed_corotated")
    t0 = time.perf_counter()
    specs = L.training_specs(scenes, per_cube, seed=seed, E_range=E_range)
    X, T = L.generate(specs, res=res, dt=dt, ratio=ratio, samples_per_scene=samples, warm=20, gap=40, keep=keep)
    torch.cuda.synchronize()
    rep["samples_fine_rollouts"] = int(X.shape[0])
    rep["data_seconds"] = time.perf_counter() - t0
    net = L.Net(max_batch=batch, seed=seed)
    L.fit_scales(net, X, T)
    Xs, Ts = L.scaled(net, X, T)
    nval = min(Xs.shape[0] // 10 // batch * batch, 8 * batch)
    Xv, Tv = Xs[-nval:].clone(), Ts[-nval:].clone()
    base = L.evaluate_loss(net, Xv, Tv, batch)
    t0 = time.perf_counter()
    log = L.train(net, Xs[:-nval], Ts[:-nval], steps=steps, batch=batch, lr=2e-3, seed=seed)
    del Xs, Ts
    rep["val_loss_untrained"] = base
    rep["val_loss_trained"] = L.evaluate_loss(net, Xv, Tv, batch)
    # on-policy rounds: samples on the velocity-corrected coarse trajectory, training on the union
    round_steps = round_steps or max(1, (3 * steps) // 4)
    rep["onpolicy"] = []
    for rnd in range(onpolicy_rounds):
        t1 = time.perf_counter()
        # the collecting correction grows over the rounds (0.25, 0.5, 1): a network trained on
        # fine-rollout states alone can drive every scene out of the grid at full strength
        a = min(1.0, 0.25 * 2 ** rnd)
        Xo, To, dropped = L.generate_on_policy(specs, lambda st: velocity_corrector(net, st, a), res=res, dt=dt,
                                               ratio=ratio, samples_per_scene=onpolicy_samples, warm=5,
                                               gap=onpolicy_gap, keep=keep)
        if Xo is None:  # every scene left the grid: no samples this round
            rep["onpolicy"].append(dict(round=rnd + 1, strength=a, samples=int(X.shape[0]), scenes_left_grid=dropped))
            continue
        Xo, To, rows_dropped = bounded_rows(Xo, To, net.out_scale[:12], max_target)
        X, T = torch.cat([X, Xo]), torch.cat([T, To])
        del Xo, To
        Xs, Ts = L.scaled(net, X, T)
        log += L.train(net, Xs, Ts, steps=round_steps, batch=batch, lr=2e-3, seed=seed + 1 + rnd)
        del Xs, Ts
        torch.cuda.synchronize()
        rep["onpolicy"].append(dict(round=rnd + 1, strength=a, samples=int(X.shape[0]), scenes_left_grid=dropped,
                                    rows_dropped=rows_dropped, seconds=time.perf_counter() - t1))
    del X, T
    torch.cuda.synchronize()
    rep["train_seconds"] = time.perf_counter() - t0
    rep["train_steps"], rep["batch"] = steps + onpolicy_rounds * round_steps, batch
    rep["train_loss_log"] = log[:: max(1, len(log) // 10)]
    val_spec = L.SceneSpec(n_per_cube=per_cube * 2, E=E_eval, nu=0.3, speed=1.0, seed=seed * 1000 + 777)
    sel = select(net, val_spec, res, dt, ratio, horizon)
    rep["selection"] = sel
    # evaluation scene
    spec = L.SceneSpec(n_per_cube=n_per_cube, E=E_eval, nu=0.3, speed=1.0, seed=seed * 1000 + 999)
    st = L.Stepper(spec, res=res, dt=dt, ratio=ratio)
    rep["particles"] = st.n
    b0 = st.initial_state()
    for _ in range(2):  # warm-up of every path
        w = b0.clone()
        st.fine_step(w)
        st.coarse_step(w)
        st.coarse_step(w, corrector_for(net, st, sel["best"]))
    fine = b0.clone()
    _, t_fine = L.timed(L.rollout_fine, st, fine, horizon * ratio)
    plain = b0.clone()
    info_p, t_plain = L.timed(L.rollout_coarse, st, plain, horizon, None)
    cor = corrector_for(net, st, sel["best"])
    learned = b0.clone()
    info_l, t_learned = L.timed(L.rollout_coarse, st, learned, horizon, cor)
    st.check()
    # fastest forms: the resident block-sorted solver, CUDA-graph replay, same scene and material
    from .solver import MPMSolver
    s = st.scene

    def solver(dt_):
        return MPMSolver(torch.tensor(s["x"], dtype=torch.float32), res=res, dt=dt_, gravity=-9.8, volume=s["vol"],
                         mass=s["mass"], mu_0=s["mu"], lambda_0=s["lam"], v=torch.tensor(s["v"]),
                         dtype=torch.float32, device="cuda", model="fixed_corotated")

    def fast(dt_, steps):
        solver(dt_).step(2)  # first-call set-up on a throwaway instance
        sv = solver(dt_)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sv.step(steps)
        torch.cuda.synchronize()
        t = time.perf_counter() - t0
        sv.check()
        return sv, t

    sf, t_fine_fast = fast(dt, horizon * ratio)
    sc, t_coarse_fast = fast(dt * ratio, horizon)
    xf, xc = sf.positions(), sc.positions()
    err_fast = (xc - xf).abs()
    rep["fine_fast"] = dict(seconds=t_fine_fast, substeps=horizon * ratio)
    rep["plain_coarse_fast"] = dict(seconds=t_coarse_fast, error=dict(max=float(err_fast.max()),
                                                                      mean=float(err_fast.mean())))
    rep["speedup_plain_coarse_fast_vs_fine_fast"] = t_fine_fast / t_coarse_fast
    if sel["best"]["strength"] == 0.0:
        rep["learned_fast"] = dict(note="selected strength 0: the corrected form is the plain coarse form",
                                   seconds=t_coarse_fast)
        rep["speedup_learned_fast_vs_fine_fast"] = t_fine_fast / t_coarse_fast
    rep["fine"] = dict(seconds=t_fine, substeps=horizon * ratio)
    rep["plain_coarse"] = dict(seconds=t_plain, error=L.position_error(plain, fine), **info_p)
    rep["learned"] = dict(seconds=t_learned, error=L.position_error(learned, fine), choice=sel["best"], **info_l)
    rep["speedup_learned_vs_fine"] = t_fine / t_learned
    rep["speedup_plain_coarse_vs_fine"] = t_fine / t_plain
    rep["gain_error_ratio_plain_over_learned"] = rep["plain_coarse"]["error"]["max"] / max(
        rep["learned"]["error"]["max"], 1e-30)
    return rep


def profile_case(n_per_cube: int = 524288, res: int = 128, batch: int = 65536, seed: int = 0) -> dict:
    """The corrector's tensor-core kernels on the full-size scene, for a profiler: 3 coarse steps with
    an untrained network (strength 1e-3, so the state stays near the plain coarse step), then 2 more
    (`k_corrector`: G2P fused with the 4-layer MLP), then one training forward and backward of a
    batch (`k_tc_gemm`)."""
    torch.manual_seed(seed)
    st = L.Stepper(L.SceneSpec(n_per_cube=n_per_cube, E=120.0, seed=seed), res=res)
    net = L.Net(max_batch=batch, seed=seed)
    cor = L.Corrector(net, st, strength=1e-3)
    buf = st.initial_state()
    for _ in range(3):
        st.coarse_step(buf, cor)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(2):
        st.coarse_step(buf, cor)
    e1.record()
    torch.cuda.synchronize()
    st.check()
    coarse_ms = e0.elapsed_time(e1) / 2
    X = torch.randn(batch, L.N.MLP_IN, device="cuda").to(torch.bfloat16)
    T = torch.randn(batch, 12, device="cuda")
    w = torch.tensor(L.OUT_WEIGHTS, dtype=torch.float32, device="cuda")
    loss = torch.zeros(1, dtype=torch.float64, device="cuda")
    net.forward_train(X)
    net.backward_train(T, w, loss)
    torch.cuda.synchronize()
    net.check()
    return {"particles": st.n, "coarse_steps": 5, "coarse_step_ms": coarse_ms, "train_batch": batch,
            "loss": float(loss.item())}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--res", type=int, default=128)
    ap.add_argument("--dt", type=float, default=5e-5)
    ap.add_argument("--ratio", type=int, default=8)
    ap.add_argument("--scenes", type=int, default=16)
    ap.add_argument("--per-cube", type=int, default=524288)
    ap.add_argument("--keep", type=float, default=1.0 / 16, help="fraction of each sample's particles kept")
    ap.add_argument("--samples", type=int, default=4)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--batch", type=int, default=32768)
    ap.add_argument("--horizon", type=int, default=150)
    ap.add_argument("--onpolicy-rounds", type=int, default=3)
    ap.add_argument("--n-per-cube", type=int, default=524288)
    ap.add_argument("--E", type=float, default=120.0)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--profile-case", action="store_true",
                    help="only run the corrector's tensor-core kernels on the full-size scene (for a profiler)")
    a = ap.parse_args(argv)
    if a.profile_case:
        print(json.dumps(profile_case(a.n_per_cube, a.res, seed=a.seed)))
        return
    r = run(a.res, a.dt, a.ratio, a.scenes, a.per_cube, a.samples, a.steps, a.batch, a.horizon, a.n_per_cube, a.E,
            seed=a.seed, onpolicy_rounds=a.onpolicy_rounds, keep=a.keep)
    print(json.dumps(r, indent=1, default=float))


if __name__ == "__main__":
    main()
