"""Learned (sigma_T c_R)max for noTimeCounter: data, training, evaluation.

The pipeline of the learned selection, all on the GPU through the C ABI:

1. ``collect``: run the plain method and record, after chosen steps, every
   cell that had candidates: its state (log n, log T_tr, speed ratio) and the
   largest sigma_T c_R among that step's candidates (``dsmc_learn_record``).
2. ``train``: fit the 3-64-64-1 BF16 perceptron to log maxima with the
   library's own forward/backward and Adam kernels (``dsmc_mlp_train``).
3. ``calibrate``: the margin added to the log prediction so that a given
   fraction of the recorded maxima lie below the prediction.
4. ``compare``: run the plain and the learned selection from the same state
   and report candidates per accepted collision, collision throughput, the
   collision-count error and field differences.

``python -m hystrath_gb300.learn`` runs the learned form of the benchmark
workloads (heat bath and Mach-10 channel) and prints one JSON line.
"""
from __future__ import annotations

import json
import sys
import time

import numpy as np

from . import spec as S
from .dsmc import NPARAM, DsmcCloud, Mlp

H, IN = 64, 3


def init_params(seed: int = 0) -> np.ndarray:
    """Uniform(+-1/sqrt(fan_in)) weights and biases (the usual dense-layer
    initialisation), in the flat layout of the C ABI."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAM, dtype=np.float32)
    off = 0

    def put(n, fan):
        nonlocal off
        b = 1.0 / np.sqrt(fan)
        p[off:off + n] = rng.uniform(-b, b, n)
        off += n

    put(H * IN, IN)   # W1
    put(H, IN)        # b1
    put(H * H, H)     # W2
    put(H, H)         # b2
    put(H, H)         # w3
    put(1, H)         # b3
    assert off == NPARAM
    return p


def fit_norm(X: np.ndarray, Y: np.ndarray) -> np.ndarray:
    """Standardisation of inputs and target: means, scales."""
    mu = X.mean(0)
    sd = X.std(0)
    sd = np.where(sd > 1e-6, sd, 1.0)
    return np.array([*mu, *sd, Y.mean(), max(Y.std(), 1e-6)], dtype=np.float32)


def collect(make_spec, seeds, record_steps, max_rows_per_record=2_000_000, rng_seed=0,
            keep_per_record=None, log=None):
    """Plain runs of make_spec(seed) for each seed, recording after each step
    number in record_steps (ascending).  keep_per_record: random subsample of
    each record."""
    rng = np.random.default_rng(rng_seed)
    Xs, Ys = [], []
    for seed in seeds:
        g = DsmcCloud(make_spec(seed))
        g.initialise()
        done = 0
        for s in record_steps:
            if s > done:
                g.evolve(s - done)
                done = s
            X, Y = g.learn_record(max_rows_per_record)
            if keep_per_record and len(Y) > keep_per_record:
                idx = rng.choice(len(Y), keep_per_record, replace=False)
                X, Y = X[idx], Y[idx]
            Xs.append(X)
            Ys.append(Y)
            if log:
                log(f"seed {seed} step {s}: {len(Y)} rows")
        g.close()
    return np.concatenate(Xs), np.concatenate(Ys)


def train(X, Y, steps=20000, batch=65536, lr=1e-3, seed=0, tau=0.0):
    """Returns the trained model and its loss history (tau: see Mlp.set_loss)."""
    m = Mlp()
    m.set_params(init_params(seed), fit_norm(X, Y))
    m.set_loss(tau)
    m.set_data(X, Y)
    loss = m.train(steps, batch, lr, seed + 1)
    return m, loss


def calibrate(model: Mlp, X, Y, coverage=0.99):
    """Margin (log units) that puts `coverage` of the recorded maxima below
    exp(prediction + margin)."""
    r = Y - model.predict(X)
    return float(np.quantile(r, coverage))


def _run(spec, develop, steps, model=None, every=1, margin=0.0):
    # the step is deterministic: two clouds from the same spec reach the same
    # state after the same number of steps
    g = DsmcCloud(spec)
    g.initialise()
    g.evolve(develop)
    if model is not None:
        g.set_learned(model, every, margin)
    g.reset_sampling()
    i0 = g.info()
    total_ms, phases = g.evolve_profiled(steps)
    i1 = g.info()
    out = {
        "ms_per_step": total_ms / steps,
        "collide_ms_per_step": phases["collide_sample"] / steps,
        "collisions": int(i1.collisions_total - i0.collisions_total),
        "candidates": int(i1.candidates_total - i0.candidates_total),
        "nColls": g.field("nColls"),
        "fields": {k: g.field(k) for k in ("rhoN", "Ttra", "Ux", "Trot", "Tvib")},
        "count": g.cell_array("count"),
    }
    g.close()
    return out


def _block_sums(a, n, b):
    nx, ny, nz = n
    a = a.reshape(nz, ny, nx)
    return a[:nz - nz % b, :ny - ny % b, :nx - nx % b].reshape(
        nz // b, b, ny // b, b, nx // b, b).sum(axis=(1, 3, 5))


def compare(spec, develop, steps, model, every=1, margin=0.0, block=8, plain=None):
    """Plain and learned selection from the same state (develop plain steps
    after the mesh fill).  plain: a previous plain _run of the same arguments."""
    if plain is None:
        plain = _run(spec, develop, steps)
    learned = _run(spec, develop, steps, model, every, margin)
    n = list(spec.n_cells)
    res = {}
    for name, r in (("plain", plain), ("learned", learned)):
        res[name] = {
            "ms_per_step": round(r["ms_per_step"], 4),
            "collide_ms_per_step": round(r["collide_ms_per_step"], 4),
            "collisions_per_s": r["collisions"] / (r["ms_per_step"] * steps * 1e-3),
            "collide_phase_collisions_per_s": r["collisions"] / (r["collide_ms_per_step"] * steps * 1e-3),
            "candidates_per_collision": r["candidates"] / max(r["collisions"], 1),
            "collisions": r["collisions"],
        }
    res["speedup_collisions_per_s"] = res["learned"]["collisions_per_s"] / res["plain"]["collisions_per_s"]
    res["speedup_collide_phase"] = (res["learned"]["collide_phase_collisions_per_s"]
                                    / res["plain"]["collide_phase_collisions_per_s"])
    res["total_collision_error"] = learned["collisions"] / plain["collisions"] - 1
    # per-cell counts (nColls: collisions of the cell over the sampled steps);
    # the per-cell error is judged on blocks of block^3 cells (a single cell
    # sees too few collisions for a 1% statement) and on the total
    cp = _block_sums(plain["nColls"], n, block)
    cl = _block_sums(learned["nColls"], n, block)
    ok = cp > 0
    rel = (cl[ok] - cp[ok]) / cp[ok]
    se = np.sqrt(cl[ok] + cp[ok]) / cp[ok]          # Poisson standard error of the difference
    res["block_collision_error"] = {
        "block_cells": block ** 3, "blocks": int(ok.sum()),
        "mean_abs": float(np.mean(np.abs(rel))), "mean": float(np.mean(rel)),
        "mean_abs_in_se": float(np.mean(np.abs(rel) / se)),
        "mean_se": float(np.mean(se)),
    }
    # fields: difference in units of its standard error, estimated from the
    # spread of the two runs' block means
    fd = {}
    for k in plain["fields"]:
        a = _block_sums(plain["fields"][k], n, block) / block ** 3
        b = _block_sums(learned["fields"][k], n, block) / block ** 3
        d = b - a
        fd[k] = {"mean_rel_diff": float(np.mean(d) / max(abs(np.mean(a)), 1e-300)),
                 "rms_diff_over_rms_field": float(np.sqrt(np.mean(d ** 2)) / max(np.sqrt(np.mean(a ** 2)), 1e-300))}
    res["fields"] = fd
    return res


def main():
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--train-steps", type=int, default=20000)
    ap.add_argument("--batch", type=int, default=65536)
    ap.add_argument("--rows", type=int, default=5_000_000)
    ap.add_argument("--eval-steps", type=int, default=400)
    ap.add_argument("--develop", type=int, default=600)
    ap.add_argument("--every", type=int, default=50)
    ap.add_argument("--coverage", type=float, default=0.99)
    ap.add_argument("--taus", default="0", help="comma-separated loss settings: 0 = squared error + "
                    "calibrated margin, (0,1) = pinball loss at that quantile")
    ap.add_argument("--scale", type=int, default=1, help="Mach-10 channel cells divided by scale per axis")
    args = ap.parse_args()

    def log(msg):
        print(msg, file=sys.stderr, flush=True)

    t0 = time.time()
    half = args.rows // 2
    # heat bath (config 1): the relaxation from 10^4 K
    Xa, Ya = collect(lambda sd: S.config1(seed=sd), range(5), [10, 30, 60, 100, 200, 400],
                     keep_per_record=half // 30 + 1, rng_seed=1, log=log)
    # Mach-10 channel (config 2): developing and developed flow
    Xb, Yb = collect(lambda sd: S.config2(seed=sd, scale=args.scale), range(5), [200, 400, 600],
                     keep_per_record=half // 15 + 1, rng_seed=2, log=log)
    X = np.concatenate([Xa, Xb])
    Y = np.concatenate([Ya, Yb])
    t1 = time.time()
    t_collect = t1 - t0
    log(f"collected {len(Y)} rows in {t_collect:.1f} s")
    spec = S.config2(seed=11, scale=args.scale)
    plain = _run(spec, args.develop, args.eval_steps)
    for tau in [float(v) for v in args.taus.split(",")]:
        t1 = time.time()
        model, loss = train(X, Y, args.train_steps, args.batch, 1e-3, seed=0, tau=tau)
        t2 = time.time()
        log(f"tau {tau}: trained {args.train_steps} steps in {t2 - t1:.1f} s: loss {loss[0]:.4f} -> {loss[-1]:.4f}")
        margin = calibrate(model, X, Y, args.coverage) if tau == 0 else 0.0
        res = compare(spec, args.develop, args.eval_steps, model, args.every, margin, plain=plain)
        t3 = time.time()
        line = {"workload": "learned (sigma_T c_R)max, Mach-10 N2 channel", "rows": int(len(Y)),
                "loss": "squared error" if tau == 0 else f"pinball {tau}",
                "train_steps": args.train_steps, "batch": args.batch, "loss_first": float(loss[0]),
                "loss_last": float(np.mean(loss[-100:])), "margin": margin,
                "coverage": args.coverage if tau == 0 else tau,
                "every": args.every, "eval_steps": args.eval_steps, "develop_steps": args.develop,
                "scale": args.scale,
                "seconds": {"collect": t_collect, "train": t2 - t1, "evaluate": t3 - t2}, **res}
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
