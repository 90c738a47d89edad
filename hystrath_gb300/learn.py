"""Learned (sigma_T c_R)max for noTimeCounter: data, training, evaluation.

The pipeline of the learned selection, all on the GPU through the C ABI:

1. ``collect``: run the plain method and record, after chosen steps, every
   cell that had candidates: its state (log n, log T_tr, speed ratio) and the
   largest sigma_T c_R among that step's candidates (``dsmc_learn_record``).
2. ``train``: fit the 3-64-64-1 BF16 perceptron to log maxima with the
   library's own forward/backward and Adam kernels (``dsmc_mlp_train``).
3. ``calibrate``: the margin added to the log prediction so that a given
   fraction of the recorded maxima lie below the prediction.
4. ``run_window`` / ``compare_windows``: run the plain and the learned
   selection from the same developed state (the speed comparison) and from
   independently seeded runs of the same development (the per-cell
   collision-count test and the field differences in standard errors), and
   report candidates per accepted collision, collision throughput, the
   collision-count error and the field differences.

``python -m hystrath_gb300.learn`` runs the learned form of the benchmark
workloads (heat bath and Mach-10 channel) and prints one JSON line.
"""
from __future__ import annotations

import json
import math
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


FIELDS = ("rhoN", "Ttra", "Ux", "Trot", "Tvib")


def develop(spec, steps):
    """A cloud of spec after the mesh fill and `steps` plain steps (the step is
    deterministic: two clouds of the same spec reach the same state)."""
    g = DsmcCloud(spec)
    g.initialise()
    if steps:
        g.evolve(steps)
    return g


def run_window(g, steps, batches=8, fields=FIELDS, blk=8):
    """`steps` graph-launched steps of one cloud (run_windows of one)."""
    return run_windows([g], steps, batches, fields, blk)[0]


def run_windows(clouds, steps, batches=8, fields=FIELDS, blk=8):
    """`steps` graph-launched steps of every cloud in `batches` equal batches,
    the clouds taking turns batch by batch (so a drift of the GPU's clocks
    over the window affects them alike); sampling restarts at each batch.
    Per cloud: device time, collision and candidate counts, parcel counts at
    both ends, every batch's per-cell collision counts, the per-cell mean of
    Ttra over the batches, every batch's fields as means over blocks of blk^3
    cells (batch means), and the selection audit over the window when it is
    on."""
    per = max(1, steps // batches)
    outs = []
    for g in clouds:
        c0 = g.counts()
        outs.append({"steps": per * batches, "ms": 0.0, "n_start": int(c0.n_particles), "nColls": [],
                     "Ttra": None, "blk": blk, "batches": {k: [] for k in fields}, "audit": None, "_c0": c0})
    for _ in range(batches):
        for g, out in zip(clouds, outs):
            n = list(g.spec.n_cells)
            g.reset_sampling()
            out["ms"] += g.evolve_timed(per)
            out["nColls"].append(g.field("nColls").astype(np.float32))
            for k in fields:
                f = g.field(k)
                if k == "Ttra":
                    out["Ttra"] = f / batches if out["Ttra"] is None else out["Ttra"] + f / batches
                out["batches"][k].append(_block_means(f, n, blk))
            try:
                a = g.cell_array("selectionAudit")
                out["audit"] = a if out["audit"] is None else out["audit"] + a
            except Exception:
                pass
    for g, out in zip(clouds, outs):
        c0 = out.pop("_c0")
        c1 = g.counts()
        out["n_end"] = int(c1.n_particles)
        out["collisions"] = int(c1.collisions_total - c0.collisions_total)
        out["candidates"] = int(c1.candidates_total - c0.candidates_total)
    return outs


def arm_rates(w):
    """Throughput of a run_window result."""
    t = w["ms"] * 1e-3
    n_avg = 0.5 * (w["n_start"] + w["n_end"])
    return {"ms_per_step": w["ms"] / w["steps"], "particle_steps_per_s": n_avg * w["steps"] / t,
            "collisions_per_s": w["collisions"] / t,
            "candidates_per_collision": w["candidates"] / max(w["collisions"], 1),
            "collisions": w["collisions"], "candidates": w["candidates"]}


def per_cell_count_test(batches_a, batches_b, groups=None, group_names=None):
    """Per-cell collision counts of two independent runs of the same flow,
    each given as per-batch counts (batches x cells), batch b of both runs
    covering the same steps.

    NTC counts are not Poisson (the candidate remainder is carried from step
    to step and a candidate is a Bernoulli trial of high probability), and a
    developing flow changes every cell's expected count from batch to batch
    in both runs alike.  So each cell's difference is taken batch by batch,
    d_cb = b_cb - a_cb, and its variance from the spread of d_cb over the
    batches, which the common trend does not enter.  With d_c the mean of
    d_cb and v_c its estimated variance, T = sum_c (d_c^2 - v_c) has mean
    zero when every cell has the same expected count in both runs, and
    T / sum_c m_c^2 estimates the mean square relative difference of the
    per-cell counts (weighted by m_c^2, m_c the first run's batch mean); its
    one-sided 95% upper bound uses the spread of d_c^2 - v_c over cells.
    groups: an integer label per cell (-1: none); each group's total
    relative difference with its standard error (from the paired batch
    totals) is reported as well.  The batch spread does not see variation
    slower than the window (a shock that wanders differently in the two
    runs): in a flow that has it, z grows with the window and T bounds the
    per-cell difference from above."""
    A = np.asarray(batches_a, dtype=np.float64)
    B = np.asarray(batches_b, dtype=np.float64)
    if A.shape != B.shape:
        raise ValueError("both runs need the same batches")
    k = A.shape[0]
    ma, mb = A.mean(0), B.mean(0)
    m = (ma + mb) > 0
    D = B[:, m] - A[:, m]
    d = D.mean(0)
    v = D.var(0, ddof=1) / k
    t = d * d - v
    n = int(m.sum())
    T = float(t.sum())
    sd = float(np.std(t) * math.sqrt(n)) if n > 1 else 1.0
    # sum of m_c^2 with the sampling variance of m_c removed
    w = float(np.sum(ma[m] ** 2 - A[:, m].var(0, ddof=1) / k))
    tot_a, tot_b = float(A.sum()), float(B.sum())
    res = {"cells": n, "batches": k, "statistic": T, "sd": sd, "z": T / sd if sd > 0 else 0.0,
           "mean_count_per_cell_and_batch": float(ma[m].mean()) if n else 0.0,
           "paired_variance_over_mean": float(np.sum(D.var(0, ddof=1)) / max(np.sum(ma[m] + mb[m]), 1e-300)),
           "rms_rel_diff_estimate": math.sqrt(max(T, 0.0) / w) if w > 0 else 0.0,
           "rms_rel_diff_upper95": math.sqrt(max(T + 1.645 * sd, 0.0) / w) if w > 0 else 0.0,
           "total_rel_diff": tot_b / max(tot_a, 1e-300) - 1.0}
    dt = B.sum(1) - A.sum(1)
    res["total_rel_diff_se"] = math.sqrt(dt.var(ddof=1) / k) / max(A.sum(1).mean(), 1e-300)
    if groups is not None:
        gl = []
        for gi in np.unique(groups):
            if gi < 0:
                continue   # cells without a label (no temperature: solid or empty)
            sel = groups == gi
            ga, gb = A[:, sel].sum(1), B[:, sel].sum(1)
            if ga.sum() <= 0:
                continue
            se = math.sqrt((gb - ga).var(ddof=1) / k) / ga.mean()
            gl.append({"group": group_names[int(gi)] if group_names else int(gi), "cells": int(sel.sum()),
                       "rel_diff": gb.mean() / ga.mean() - 1.0, "se": se})
        res["groups"] = gl
    return res


def audit_summary(audit, min_expected=10.0):
    """The selection audit of a run (cells x 2: summed acceptances
    sigma/max and their part above 1): per cell the expected relative
    shortfall of the collision count, y/x.  Cells with fewer than
    min_expected expected collisions are left out of the per-cell figures
    (the total includes them)."""
    a = np.asarray(audit, dtype=np.float64)
    x, y = a[:, 0], a[:, 1]
    ok = x >= min_expected
    r = y[ok] / x[ok]
    res = {"expected_shortfall_total": float(y.sum() / max(x.sum(), 1e-300)), "cells": int(ok.sum()),
           "min_expected_collisions": min_expected}
    if r.size:
        res.update({"cells_above_1pct": float(np.mean(r > 0.01)),
                    "collisions_in_cells_above_1pct": float(x[ok][r > 0.01].sum() / x[ok].sum()),
                    "p99": float(np.quantile(r, 0.99)), "p999": float(np.quantile(r, 0.999)),
                    "max": float(r.max()), "mean": float(r.mean())})
    return res


def _block_means(a, n, blk):
    nx, ny, nz = n
    a = a.reshape(nz, ny, nx)
    a = a[:nz - nz % blk, :ny - ny % blk, :nx - nx % blk]
    return a.reshape(nz // blk, blk, ny // blk, blk, nx // blk, blk).mean(axis=(1, 3, 5)).ravel()


def batch_mean_z(batches_a, batches_b):
    """Differences of time-averaged fields between two independent runs in
    units of their standard error, per block of cells (the batches hold
    block means): each run's block value is the mean of its batch means and
    its standard error the spread of the batch means / sqrt(batches) (batch
    means absorb the autocorrelation).  Blocks where a field does not vary
    (solid cells, or a temperature with no excited level) are left out."""
    A = np.array(batches_a)
    B = np.array(batches_b)
    if A.shape != B.shape:
        raise ValueError("both runs need the same batches")
    # batch b of both runs covers the same steps: the difference is taken
    # batch by batch, so a trend common to both runs (a developing flow)
    # stays out of the standard error
    k = A.shape[0]
    ma, mb = A.mean(0), B.mean(0)
    D = B - A
    se = np.sqrt(D.var(0, ddof=1) / k)
    ok = (se > 0) & np.isfinite(se) & (np.abs(ma) > 0)
    z = (mb[ok] - ma[ok]) / se[ok]
    # |z| > 2 is expected in the fraction 2 P(t_(k-1) > 2), not 4.6%, with this few batches
    return {"blocks": int(ok.sum()), "batches": k, "mean_abs_z": float(np.mean(np.abs(z))) if z.size else 0.0,
            "frac_abs_z_gt_2": float(np.mean(np.abs(z) > 2.0)) if z.size else 0.0,
            "expected_frac_abs_z_gt_2": float(np.ravel(_t_two_sided_tail(2.0, k - 1))[0]) if z.size else 0.0,
            "mean_z": float(np.mean(z)) if z.size else 0.0,
            "rel_diff_of_means": float(np.sum(mb[ok] - ma[ok]) / max(abs(np.sum(ma[ok])), 1e-300))}


def _t_two_sided_tail(t, nu):
    """P(|T| > t) for Student's t with nu degrees of freedom (array)."""
    from scipy.stats import t as student_t
    return 2.0 * student_t.sf(t, np.asarray(nu, dtype=np.float64))


def temperature_groups(ttra, k=5):
    """Cells grouped by quantiles of a temperature field (k groups; cells with
    no temperature, e.g. solid ones, in group -1)."""
    t = np.asarray(ttra)
    g = np.full(t.shape, -1, dtype=np.int64)
    ok = t > 0
    if ok.any():
        edges = np.quantile(t[ok], np.linspace(0, 1, k + 1)[1:-1])
        g[ok] = np.searchsorted(edges, t[ok], side="right")
    names = [f"Ttra quantile {i + 1}/{k}" for i in range(k)]
    return g, names


def compare_windows(spec, plain, learned, replicate=None, control=None):
    """The learned_vs_plain report.  plain and learned: run_window results
    from the same developed state (the speed comparison); replicate: a
    run_window of the learned selection from an independently seeded run of
    the same development, the per-cell count and field comparisons (which
    need independent runs) use it when given; control: the plain selection
    of that independent run, compared with plain the same way (two plain
    runs: what the statistics read when only the seeds differ)."""
    del spec
    rp, rl = arm_rates(plain), arm_rates(learned)
    res = {"window_steps": plain["steps"], "plain": rp, "learned": rl,
           "ratio_collisions_per_s": rl["collisions_per_s"] / rp["collisions_per_s"],
           "ratio_particle_steps_per_s": rl["particle_steps_per_s"] / rp["particle_steps_per_s"],
           "candidate_reduction": 1.0 - rl["candidates_per_collision"] / rp["candidates_per_collision"],
           "total_collision_error_same_state": learned["collisions"] / plain["collisions"] - 1.0}
    other = replicate if replicate is not None else learned
    tp = plain.get("Ttra")
    groups, names = temperature_groups(tp) if tp is not None else (None, None)
    res["per_cell_counts"] = per_cell_count_test(plain["nColls"], other["nColls"], groups, names)
    res["per_cell_counts"]["runs"] = "independent seeds" if replicate is not None else "same state"
    for name, w in (("plain", plain), ("learned", learned)):
        if w.get("audit") is not None:
            res.setdefault("selection_audit", {})[name] = audit_summary(w["audit"])
    res["fields_in_se"] = {k: batch_mean_z(plain["batches"][k], other["batches"][k])
                           for k in plain["batches"] if k in other["batches"]}
    res["fields_in_se"]["block_cells"] = plain["blk"] ** 3
    if control is not None:
        res["per_cell_counts_control"] = per_cell_count_test(plain["nColls"], control["nColls"], groups, names)
        res["per_cell_counts_control"]["runs"] = "independent seeds, both plain"
        res["fields_in_se_control"] = {k: batch_mean_z(plain["batches"][k], control["batches"][k])
                                       for k in plain["batches"] if k in control["batches"]}
    return res


def train_default(scale=1, seeds=range(5), rows=5_000_000, train_steps=20000, batch=65536, tau=0.95,
                  coverage=0.99, log=None):
    """The learned maximum of the benchmark: rows recorded from plain runs of
    the heat bath (the relaxation from 10^4 K) and the Mach-10 channel
    (developing and developed flow) at the given seeds, then Adam on the GPU.
    Returns (model, margin, description)."""
    t0 = time.time()
    half = rows // 2
    Xa, Ya = collect(lambda sd: S.config1(seed=sd), seeds, [10, 30, 60, 100, 200, 400],
                     keep_per_record=half // (6 * len(seeds)) + 1, rng_seed=1, log=log)
    Xb, Yb = collect(lambda sd: S.config2(seed=sd, scale=scale), seeds, [200, 400, 600],
                     keep_per_record=half // (3 * len(seeds)) + 1, rng_seed=2, log=log)
    X = np.concatenate([Xa, Xb])
    Y = np.concatenate([Ya, Yb])
    t1 = time.time()
    model, loss = train(X, Y, train_steps, batch, 1e-3, seed=0, tau=tau)
    t2 = time.time()
    margin = calibrate(model, X, Y, coverage) if tau == 0 else 0.0
    desc = {"rows": int(len(Y)), "seeds": list(seeds), "loss": "squared error" if tau == 0 else f"pinball {tau}",
            "train_steps": train_steps, "batch": batch, "lr": 1e-3, "loss_first": float(loss[0]),
            "loss_last": float(np.mean(loss[-100:])), "margin": margin,
            "seconds": {"collect": round(t1 - t0, 2), "train": round(t2 - t1, 2)}}
    return model, margin, desc


def evaluate(spec, spec_replicate, model, margin, every, develop_steps, window, batches=8, log=None):
    """Plain and learned from the same developed state, and the learned run
    of an independently seeded development, over `window` steps each."""
    p = develop(spec, develop_steps)
    lr = develop(spec, develop_steps)
    lr.set_learned(model, every, margin)
    for g in (p, lr):
        g.set_selection_audit(True)
    clouds = [p, lr]
    if spec_replicate is not None:
        # the same development and window start as the other two, learned
        # and (the control) plain
        l2 = develop(spec_replicate, develop_steps)
        l2.set_learned(model, every, margin)
        clouds.append(l2)
        clouds.append(develop(spec_replicate, develop_steps))
    ws = run_windows(clouds, window, batches)
    for g in clouds:
        g.close()
    wp, wl = ws[0], ws[1]
    rep = ws[2] if len(ws) > 2 else None
    ctl = ws[3] if len(ws) > 3 else None
    return compare_windows(spec, wp, wl, rep, ctl)


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
    ap.add_argument("--taus", default="0.95", help="comma-separated loss settings: 0 = squared error + "
                    "calibrated margin, (0,1) = pinball loss at that quantile")
    ap.add_argument("--scale", type=int, default=1, help="Mach-10 channel cells divided by scale per axis")
    args = ap.parse_args()

    def log(msg):
        print(msg, file=sys.stderr, flush=True)

    spec = S.config2(seed=11, scale=args.scale)
    rep = S.config2(seed=12, scale=args.scale)
    for tau in [float(v) for v in args.taus.split(",")]:
        t0 = time.time()
        model, margin, desc = train_default(args.scale, range(5), args.rows, args.train_steps, args.batch, tau,
                                            args.coverage, log)
        res = evaluate(spec, rep, model, margin, args.every, args.develop, args.eval_steps)
        line = {"workload": "learned (sigma_T c_R)max, Mach-10 N2 channel", "model": desc, "every": args.every,
                "develop_steps": args.develop, "scale": args.scale, "seconds": round(time.time() - t0, 1),
                **res}
        print(json.dumps(line), flush=True)
        model.close()


if __name__ == "__main__":
    main()
