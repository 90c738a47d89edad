"""Benchmark of the GB300 dsmcFoam+ step (dsmcCloud::evolve) on the N2
Larsen-Borgnakke heat bath: 64^3 cells of 1 mm, 50 parcels per cell
(13.1M parcels), T_tr = 10000 K, T_rot = T_vib = 300 K, dt = 2e-7 s, FP64
state, specular walls, noTimeCounter + LarsenBorgnakkeVariableHardSphere,
sampling every step.

One JSON line on rank 0.  ``--impl reference`` times the CPU implementation of
the same path (the oracle restatement: the reference needs OpenFOAM v1706,
which is not installable here) on all host cores.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "collisions/s & particle-steps/s on 1 GB300, learned vs plain NTC at <=1% rate error"
UNIT = "particle-steps/s"
WORKLOAD = "N2 LB heat bath, {n}^3 cells x 50 parcels, dt 2e-7 s, FP64"
CHANNEL = ("N2 Mach-10 channel past a diffuse 300 K cube, {nx}x{ny}x{nz} cells (cube of {c}^3 solid), "
           "~20 parcels per cell, freestream inflow at x=0, deletion at x=max, specular sides, dt 5e-8 s, "
           "{d} steps developed before timing, FP64")


def make_spec(args, seed):
    """The workload's case: the heat bath (default) or the Mach-10 channel."""
    from hystrath_gb300 import spec as S
    if args.workload == "channel":
        return S.config2(seed=seed, scale=args.scale)
    return S.config1(seed=seed, n=args.cells)


def workload_name(args, s):
    if args.workload == "channel":
        return CHANNEL.format(nx=s.n_cells[0], ny=s.n_cells[1], nz=s.n_cells[2], c=32 // args.scale,
                              d=args.develop)
    return WORKLOAD.format(n=args.cells)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def read_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def read_traffic(kernel):
    """dram bytes per launch from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", "traffic.md")
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch") and kernel in line:
                return float(line.strip().split()[-1])
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(gpu_index), f"--query-gpu={self.FIELDS}",
                                       "--format=csv,noheader,nounits", "-lms", "100"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        time.sleep(0.25)
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if parts[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.f.name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# parcel state: a 64-byte record (pos, U, ERot, id, species|vib) + a 4-byte cell word
STATE_BYTES = 68

# kernels of one heat-bath step (no inflow): zero_step; move, move_slow;
# sample_done, sample_finalize, sample_flushed; scan_reduce, scan_top,
# scan_down; scatter_index, gather, finish_sort; ntc_select, ntc_buckets,
# ntc_list, cell_order, cell_order_big, collide_heavy, collide_light;
# set_pending; end_step
KERNELS_PER_STEP = 21


def bytes_model(N, C, coll, cand, n_acc):
    """Algorithmic bytes per step, per phase.

    move:    read pos, U, ERot and species word (64: the step's sample of the
             post-collision state is folded into the move) + cell word (4);
             write pos (24) + cell word (4)
    sort:    stable counting sort of the state, read + write (2 x 68), plus
             the per-cell count and offset (8 B per cell)
    collide: per cell the candidate count (start, sigmaTcRMax, remainder,
             count: 36 B) and the sampling accumulators (8 B each, read and
             written every 32 samples: 0.5 B per accumulator and step); per
             parcel the id and cell word of a cell's members for the pair
             draw (8 B); per candidate the two velocities and species words
             (2 x 32 B); per collision the energies written back (2 x 64 B)
    """
    move = 96.0 * N
    sort = 2.0 * STATE_BYTES * N + 8.0 * C
    collide = (36.0 + 0.5 * n_acc) * C + 8.0 * N + 64.0 * cand + 128.0 * coll
    return move, sort, collide


def reduce_ranks(total_ms, coll, n_parcels, dist, device):
    """Whole-job figures over the replicas: the slowest rank's time, the
    summed collisions and parcels (dist None: one rank)."""
    import torch
    t = torch.tensor([total_ms, float(coll), float(n_parcels)], dtype=torch.float64, device=device)
    if dist:
        tm = t[:1].clone()
        rest = t[1:].clone()
        dist.all_reduce(tm, op=dist.ReduceOp.MAX)
        dist.all_reduce(rest, op=dist.ReduceOp.SUM)
        t = torch.cat([tm, rest])
    return float(t[0]), float(t[1]), float(t[2])


def gpu_arm(args, rank, world, local):
    import numpy as np  # noqa: F401
    from hystrath_gb300 import spec as S
    from hystrath_gb300.dsmc import DsmcCloud

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")

    s = make_spec(args, 1000 + rank)
    g = DsmcCloud(s)
    g.initialise()
    if args.workload == "channel":
        # the bow shock and wake take some hundreds of steps to form
        g.evolve(args.develop)
    C = s.n_cells[0] * s.n_cells[1] * s.n_cells[2]
    g.evolve(args.warmup)
    N = g.info().n_particles

    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clk = ClockSampler(local) if rank == 0 else None
    i0 = g.info()
    # the K timed steps: the captured step graph, CUDA events around all of them
    total_ms = g.evolve_timed(args.steps)
    i1 = g.info()
    torch.cuda.synchronize()
    clocks = clk.stop() if clk else None
    # the phase breakdown (roofline entries, not the value): K more steps
    # enqueued phase by phase with events around each phase
    _, phases = g.evolve_profiled(args.steps)
    torch.cuda.synchronize()
    coll = i1.collisions_total - i0.collisions_total
    cand = i1.candidates_total - i0.candidates_total
    max_ms, tot_coll, tot_N = reduce_ranks(total_ms, coll, N, dist, "cuda")

    # end-to-end through the C ABI with host buffers: upload the state,
    # K steps each returning the cloud totals, read a field back.
    e2e = None
    if not args.no_e2e:
        st = g.particles()
        pin = {}
        for k in ("pos", "U", "erot", "vib", "species", "id"):
            pin[k] = torch.from_numpy(st[k]).pin_memory().numpy()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g.set_particles(pin["pos"], pin["U"], pin["erot"], pin["vib"], pin["species"], pin["id"])
        for _ in range(args.steps):
            g.evolve(1)
            g.counts()      # the step's collision counters back on the host
        ttra = g.field("Ttra")
        t1 = time.perf_counter()
        nbytes_state = sum(v.nbytes for v in pin.values())
        info_bytes = 152    # the counters block read by dsmc_counts
        e2e = {"value": N * args.steps * world / (t1 - t0), "unit": UNIT,
               "h2d_bytes_per_step": nbytes_state / args.steps,
               "d2h_bytes_per_step": info_bytes + ttra.nbytes / args.steps}
        del ttra

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    mv, so, co = bytes_model(N, C, coll / args.steps, cand / args.steps, s.n_species * 7 + 2)
    peak, peak_kind = read_peaks()
    per = {k: v / args.steps for k, v in phases.items()}
    dominant = max(("move", "sort", "collide_sample"), key=lambda k: per[k])
    algo = {"move": mv, "sort": so, "collide_sample": co}
    kern = {"move": "k_move", "sort": "k_gather", "collide_sample": "k_collide_light"}

    def roof(k):
        achieved = algo[k] / (per[k] * 1e-3) / 1e9
        return {"bound": "hbm", "kernel": kern[k], "achieved": round(achieved, 1), "peak": peak,
                "unit": "GB/s", "frac": round(achieved / peak, 4),
                # the committed per-launch traffic was captured on the heat bath
                "traffic": read_traffic(kern[k]) if args.workload == "heatbath" and args.cells == 64 else None,
                "peak_source": peak_kind, "ms_per_launch": round(per[k], 4),
                "algorithmic_bytes_per_launch": algo[k]}

    ms_ms = per["move"] + per["sort"]
    line = {
        "metric": METRIC,
        "value": tot_N * args.steps / (max_ms * 1e-3),
        "unit": UNIT,
        "collisions_per_s": tot_coll / (max_ms * 1e-3),
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": max_ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": f"synthetic (dsmcMeshFill of the {args.workload} from the seed)",
        "config": {"workload": workload_name(args, s), "cells": C, "parcels": N, "parcels_total": int(tot_N),
                   "l2": f"inputs larger than L2 ({N * 68 / 1e9:.2f} GB of parcel state per buffer)",
                   "parallelism": f"{world} independent replicas" if world > 1 else "1 GPU",
                   "phase_ms_per_step": {k: round(v, 4) for k, v in per.items()}},
        "roofline": roof(dominant),
        "roofline_move_sort": {"bound": "hbm", "achieved": round((mv + so) / (ms_ms * 1e-3) / 1e9, 1),
                               "peak": peak, "unit": "GB/s",
                               "frac": round((mv + so) / (ms_ms * 1e-3) / 1e9 / peak, 4),
                               "bytes_per_parcel_step": round((mv + so) / N, 1)},
        "gpu_launches": int(args.steps * KERNELS_PER_STEP),
        "e2e": e2e,
        "clocks": clocks,
    }
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(args, sample_cells=32, steps=8)
    if args.workload == "channel":
        line["note"] = ("config-2 workload: parcels counted at the start of the timed steps; value is "
                        "parcels x steps / time")
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def cpu_baseline(args, sample_cells=32, steps=8):
    """The oracle restatement of the path on the host cores, on a sub-box of
    the same heat bath (same density, temperatures, dt and parcels per cell)."""
    from hystrath_gb300 import spec as S
    from oracle import oracle
    threads = args.cpu_threads or os.cpu_count()
    s = S.config1(seed=7, n=sample_cells)
    o = oracle.OracleCloud(s, threads=threads)
    o.initialise()
    N = o.info().n_particles
    o.evolve(1)
    t0 = time.perf_counter()
    c0 = o.info().collisions_total
    o.evolve(steps)
    t1 = time.perf_counter()
    coll = o.info().collisions_total - c0
    return {"value": N * steps / (t1 - t0), "unit": UNIT, "cores": threads, "kind": "port",
            "collisions_per_s": coll / (t1 - t0),
            "sample": f"{sample_cells}^3-cell sub-box of the heat bath ({N} parcels), {steps} steps after 1"}


def reference_arm(args, rank, world):
    if rank != 0:
        return
    cb = cpu_baseline(args, sample_cells=32, steps=max(2, min(args.steps, 10)))
    line = {"metric": METRIC, "impl": "reference", "value": cb["value"], "unit": UNIT,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (dsmcMeshFill of the heat bath from the seed)",
            "config": {"workload": WORKLOAD.format(n=args.cells), "note": "CPU restatement of dsmcCloud::evolve timed on a sub-box"},
            "collisions_per_s": cb["collisions_per_s"],
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-threads", type=int, default=0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--cells", type=int, default=64, help="heat-bath edge in cells (64 = the benchmark workload)")
    ap.add_argument("--workload", default="heatbath", choices=["heatbath", "channel"],
                    help="heatbath: the benchmark workload; channel: the Mach-10 channel past a cube")
    ap.add_argument("--scale", type=int, default=1, help="channel: cells divided by scale per axis")
    ap.add_argument("--develop", type=int, default=600, help="channel: steps run before the warm-up")
    args = ap.parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        reference_arm(args, rank, world)
        return
    from hystrath_gb300 import build
    if rank == 0:
        build.build()
    gpu_arm(args, rank, world, local)


if __name__ == "__main__":
    main()
