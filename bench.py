"""Benchmark of the GB300 dsmcFoam+ step (dsmcCloud::evolve).

Default workload: the Mach-10 N2 channel past a diffuse cube, 256x128x128
cells of 0.5 mm (a 32^3-cell solid cube at x = 48..80), n = 1e21 m^-3,
~20 parcels per cell (about 84M parcels), freestream inflow at x = 0 (200 K,
2883 m/s), deletion at x = max, specular sides, noTimeCounter +
LarsenBorgnakkeVariableHardSphere, dt = 5e-8 s, FP64 state, sampling every
step; the flow is developed for 600 steps before anything is timed.

One JSON line on rank 0:
- ``value``: particle-steps/s of the plain selection (the running maximum of
  noTimeCounter) over the K timed steps, CUDA events around K launches of the
  captured step graph; ``collisions_per_s`` beside it.
- ``learned_vs_plain``: the learned (sigma_T c_R)max, trained in this run on
  the GPU by the library's own kernels (rows recorded from plain runs of the
  heat bath and the channel at seeds 0..4; 20k Adam steps of 65536 rows,
  pinball loss at tau 0.95), against the plain selection: both arms from the
  same developed state over the same window (throughput ratio, candidates
  per collision), and the learned arm of an independently seeded run of the
  same development against the plain arm (per-cell collision-count test,
  fields in batch-mean standard errors).
- ``roofline``: the dominant kernel (move or gather), its algorithmic bytes
  over its own CUDA-event time; ``kernels``: every kernel group's time.
- ``secondary_heatbath``: the N2 heat bath (64^3 cells x 50 parcels).
- ``e2e``: the same steps through the C ABI from pinned host buffers.
- ``cpu_baseline``: the CPU restatement of the path (the oracle) on the host
  cores, from the GPU-developed state of the same channel.

``--impl reference`` times that CPU implementation (the reference dsmcFoam+
needs OpenFOAM v1706, which is not installable here) on the same channel:
the state developed on the GPU (600 steps, untimed) is handed to the CPU
restatement, which then runs a stated number of steps with OpenMP on all
host threads and one step on one thread.
"""
from __future__ import annotations

import argparse
import json
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
HEATBATH = "N2 LB heat bath, {n}^3 cells x 50 parcels, dt 2e-7 s, FP64"
CHANNEL = ("N2 Mach-10 channel past a diffuse 300 K cube, {nx}x{ny}x{nz} cells (cube of {c}^3 solid), "
           "~20 parcels per cell, freestream inflow at x=0, deletion at x=max, specular sides, dt {dt:g} s, "
           "{d} steps developed before timing, FP64")
SEED = 1000


def make_spec(args, seed):
    from hystrath_gb300 import spec as S
    if args.workload == "channel":
        return S.config2(seed=seed, scale=args.scale)
    return S.config1(seed=seed, n=args.cells)


def workload_config(args, s):
    """The workload as both arms name it (static keys only)."""
    C = s.n_cells[0] * s.n_cells[1] * s.n_cells[2]
    if args.workload == "channel":
        name = CHANNEL.format(nx=s.n_cells[0], ny=s.n_cells[1], nz=s.n_cells[2], c=32 // args.scale,
                              dt=s.delta_t, d=args.develop)
        return {"workload": name, "cells": C, "seed": SEED, "develop_steps": args.develop,
                "l2": "inputs larger than L2 (parcel state ~5.7 GB per buffer)"}
    return {"workload": HEATBATH.format(n=args.cells), "cells": C, "seed": SEED, "develop_steps": 0,
            "l2": "inputs larger than L2 (parcel state 0.89 GB per buffer)"}


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


def read_traffic(workload, kernel):
    """DRAM bytes per parcel for a kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "traffic.md")
    try:
        for line in open(path):
            parts = line.split()
            if len(parts) == 4 and parts[0] == "traffic_bytes_per_parcel" and parts[1] == workload \
                    and parts[2] == kernel:
                return float(parts[3])
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

# kernels of one step: zero_step; move, move_slow; sample_done,
# sample_finalize, sample_flushed; scan_reduce, scan_top, scan_down;
# scatter_index, gather, finish_sort; ntc_select, ntc_buckets, ntc_list,
# cell_order, cell_order_big, collide_heavy, collide_light; set_pending;
# end_step -- plus, with an inflow patch, inflow_count/scan/fill/commit and
# a second move launch (the inserted parcels move after the inflow, which
# runs beside the first), and cell_features, mlp_infer with the learned
# maximum
KERNELS_PER_STEP = 21


def kernels_per_step(has_inflow, learned):
    return KERNELS_PER_STEP + (5 if has_inflow else 0) + (2 if learned else 0)


def kernel_bytes(N, C, n_moved, coll, cand, n_acc):
    """Algorithmic bytes per step of the kernel groups.

    move:    read pos, U, ERot and species word (64: the step's sample of the
             post-collision state is folded into the move) + cell word (4);
             write the cell word (4), for the parcels moved (the parcels of
             the last step plus the inserted ones); the end point of a plain
             move is stored by the gather, which writes the record anyway,
             so only the inserted parcels' positions (24) are written here
    gather:  read and write the 68-byte state of every kept parcel, plus its
             (source index, cell word) slot entry (8) and the id copy (4)
    sort:    the gather, the index scatter (cell word in, slot entry out:
             12 B/parcel) and the per-cell count and offset (8 B per cell)
    collide: per cell the candidate count (start, sigmaTcRMax, remainder,
             count: 36 B) and the sampling accumulators (8 B each, read and
             written every 32 samples: 0.5 B per accumulator and step); per
             parcel the id and cell word of a cell's members for the pair
             draw (8 B); per candidate the two velocities and species words
             (2 x 32 B); per collision the energies written back (2 x 64 B)
    """
    move = 72.0 * n_moved + 24.0 * max(n_moved - N, 0.0)
    gather = (2.0 * STATE_BYTES + 12.0) * N
    sort = gather + 12.0 * n_moved + 8.0 * C
    collide = (36.0 + 0.5 * n_acc) * C + 8.0 * N + 64.0 * cand + 128.0 * coll
    return {"move": move, "gather": gather, "sort": sort, "collide": collide}


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


def log(msg):
    print(f"[bench {time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)


def roofline_entries(g, s, args, steps, peak, peak_kind):
    """Per-kernel-group CUDA-event times over `steps` more steps (events
    between the groups), the roofline of the move and the gather, and the
    move+sort phase fraction."""
    c0 = g.counts()
    i0 = g.info()
    tot, grp = g.evolve_kernel_profile(steps)
    c1 = g.counts()
    i1 = g.info()
    N = 0.5 * (c0.n_particles + c1.n_particles)
    n_moved = N + (i1.inserted_last_step if args.workload == "channel" else 0)
    coll = (c1.collisions_total - c0.collisions_total) / steps
    cand = (c1.candidates_total - c0.candidates_total) / steps
    C = s.n_cells[0] * s.n_cells[1] * s.n_cells[2]
    by = kernel_bytes(N, C, n_moved, coll, cand, s.n_species * 7 + 2)
    per = {k: v / steps for k, v in grp.items()}
    del i0

    def entry(kernel, key, ms):
        achieved = by[key] / (ms * 1e-3) / 1e9
        tb = read_traffic(args.workload, kernel)
        return {"bound": "hbm", "kernel": kernel, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                "traffic": round(tb * N) if tb else None,
                "ms_per_launch": round(ms, 4), "algorithmic_bytes_per_launch": round(by[key])}

    move_ms = per["move"] + per["move_slow"]
    gather_ms = per["gather"]
    cand_k = {"k_move+k_move_slow": entry("k_move+k_move_slow", "move", move_ms),
              "k_gather": entry("k_gather", "gather", gather_ms)}
    cand_k["k_move+k_move_slow"]["ms_k_move"] = round(per["move"], 4)
    cand_k["k_move+k_move_slow"]["ms_k_move_slow"] = round(per["move_slow"], 4)
    dominant = max(cand_k.values(), key=lambda e: e["ms_per_launch"])
    sort_ms = per["scan"] + per["scatter_index"] + per["gather"] + per["finish"]
    ms_ms = move_ms + per["sample"] + sort_ms
    ms_bytes = by["move"] + by["sort"]
    move_sort = {"bound": "hbm", "achieved": round(ms_bytes / (ms_ms * 1e-3) / 1e9, 1), "peak": peak,
                 "unit": "GB/s", "frac": round(ms_bytes / (ms_ms * 1e-3) / 1e9 / peak, 4),
                 "ms_per_step": round(ms_ms, 4), "bytes_per_parcel_step": round(ms_bytes / N, 1),
                 "peak_source": peak_kind}
    kernels = {k: round(v, 4) for k, v in per.items()}
    kernels["sum"] = round(sum(per.values()), 4)
    kernels["events_total_per_step"] = round(tot / steps, 4)
    return dominant, cand_k, move_sort, kernels


def train_learned(args):
    from hystrath_gb300 import learn
    seeds = list(range(args.train_seeds))
    model, margin, desc = learn.train_default(args.scale, seeds, args.train_rows, args.train_steps, 65536,
                                              args.tau, 0.99, log)
    desc["command"] = ("in this run: hystrath_gb300.learn.train_default(scale={}, seeds={}, rows={}, "
                       "train_steps={}, batch=65536, tau={})".format(args.scale, seeds, args.train_rows,
                                                                     args.train_steps, args.tau))
    return model, margin, desc


def heatbath_secondary(args, peak, peak_kind):
    """The N2 heat bath (64^3 cells x 50 parcels): K timed steps and its
    kernel roofline."""
    from hystrath_gb300 import spec as S
    from hystrath_gb300.dsmc import DsmcCloud

    class A:  # the heat bath's own arguments
        workload = "heatbath"
        cells = 64
        scale = 1
    s = S.config1(seed=SEED, n=64)
    g = DsmcCloud(s)
    g.initialise()
    g.evolve(max(3, args.warmup))
    c0 = g.counts()
    ms = g.evolve_timed(args.steps)
    c1 = g.counts()
    dom, _, ms_entry, kernels = roofline_entries(g, s, A, args.steps, peak, peak_kind)
    g.close()
    t = ms * 1e-3
    return {"workload": HEATBATH.format(n=64), "parcels": int(c0.n_particles),
            "value": c0.n_particles * args.steps / t, "unit": UNIT,
            "collisions_per_s": (c1.collisions_total - c0.collisions_total) / t,
            "ms_per_step": ms / args.steps, "roofline": dom, "roofline_move_sort": ms_entry,
            "kernels_ms_per_step": kernels}


def gpu_arm(args, rank, world, local):
    from hystrath_gb300 import learn
    from hystrath_gb300.dsmc import DsmcCloud

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")

    peak, peak_kind = read_peaks()
    channel = args.workload == "channel"
    learned = channel and not args.no_learned
    s = make_spec(args, SEED + rank)
    C = s.n_cells[0] * s.n_cells[1] * s.n_cells[2]

    model = margin = model_desc = None
    if learned:
        log("training the learned maximum")
        model, margin, model_desc = train_learned(args)

    # the plain arm (value)
    log("developing the plain arm")
    g = learn.develop(s, args.develop if channel else 0)
    g.evolve(args.warmup)
    lg = None
    if learned:
        # the learned arm from the same developed state (the step is
        # deterministic: this cloud is bit for bit the plain one here)
        log("developing the learned arm")
        lg = learn.develop(s, args.develop)
        lg.set_learned(model, args.learn_every, margin)
        lg.set_learned_forget(args.forget)
        lg.evolve(args.warmup)
        # the selection audit (per-cell expected collision shortfall) in the
        # evaluation windows; switched on after the timed steps
    c0 = g.counts()

    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clk = ClockSampler(local) if rank == 0 else None
    # the K timed steps: the captured step graph, CUDA events around all of them
    total_ms = g.evolve_timed(args.steps)
    torch.cuda.synchronize()
    clocks = clk.stop() if clk else None
    c1 = g.counts()
    coll = c1.collisions_total - c0.collisions_total
    N = 0.5 * (c0.n_particles + c1.n_particles)
    max_ms, tot_coll, tot_N = reduce_ranks(total_ms, coll, N, dist, "cuda")

    lvp = None
    if learned:
        cl0 = lg.counts()
        ms_l = lg.evolve_timed(args.steps)
        cl1 = lg.counts()
        # an independently seeded run of the same development, learned, its
        # window starting at the same step as the other two
        log("developing the independent learned run")
        rep = learn.develop(make_spec(args, SEED + 7919 + rank), args.develop)
        rep.set_learned(model, args.learn_every, margin)
        rep.set_learned_forget(args.forget)
        rep.evolve(args.warmup + args.steps)
        # the control: the same independent run with the plain selection
        ctl = learn.develop(make_spec(args, SEED + 7919 + rank), args.develop)
        ctl.evolve(args.warmup + args.steps)
        log("evaluation windows")
        for x in (g, lg):
            x.set_selection_audit(True)
        # the four clouds take turns batch by batch
        wp, wl, wr, wc = learn.run_windows([g, lg, rep, ctl], args.eval_steps, args.eval_batches)
        rep.close()
        ctl.close()
        for x in (g, lg):
            x.set_selection_audit(False)
        _, kl = lg.evolve_kernel_profile(args.steps)
        lg.close()
        lg = None
        lvp = learn.compare_windows(s, wp, wl, wr, wc)
        nl = 0.5 * (cl0.n_particles + cl1.n_particles)
        lvp["timed_steps"] = {
            "steps": args.steps,
            "plain": {"particle_steps_per_s": N * args.steps / (total_ms * 1e-3),
                      "collisions_per_s": coll / (total_ms * 1e-3), "ms_per_step": total_ms / args.steps},
            "learned": {"particle_steps_per_s": nl * args.steps / (ms_l * 1e-3),
                        "collisions_per_s": (cl1.collisions_total - cl0.collisions_total) / (ms_l * 1e-3),
                        "ms_per_step": ms_l / args.steps}}
        lvp["timed_steps"]["ratio_collisions_per_s"] = (lvp["timed_steps"]["learned"]["collisions_per_s"] /
                                                        lvp["timed_steps"]["plain"]["collisions_per_s"])
        lvp["learned_kernels_ms_per_step"] = {k: round(v / args.steps, 4) for k, v in kl.items()}
        lvp["model"] = model_desc
        lvp["every"] = args.learn_every
        lvp["forget"] = args.forget
        lvp["note"] = ("speed: both arms from the same developed state over the same steps (the learned arm's "
                       "predictions, every {} steps, inside its timed steps); per-cell counts and fields: the "
                       "plain arm against the learned arm of an independently seeded run of the same "
                       "development (the comparison needs independent runs); the *_control entries compare "
                       "the plain arm with the plain selection of that independent run, the same statistics "
                       "when only the seeds differ; Tvib is held by a few hundred excited parcels that outlive "
                       "the window, so its z values read the run-to-run spread of that population (the control "
                       "shows the same shift), not the selection".format(args.learn_every))

    # kernel groups and the roofline (not the value): K more steps with events
    log("kernel profile")
    dominant, rooflines, move_sort, kernels = roofline_entries(g, s, args, args.steps, peak, peak_kind)

    # end-to-end through the C ABI with host buffers: upload the state, K
    # steps each returning the cloud totals, read a field back
    e2e = None
    cpu_state = None
    if not args.no_e2e or (rank == 0 and world == 1 and not args.no_cpu):
        log("reading the state back")
        st = g.particles()
        cells = {k: g.cell_array(k) for k in ("sigmaTcRMax", "collisionSelectionRemainder")}
        cpu_state = (st, cells)
    if not args.no_e2e:
        st = cpu_state[0]
        pin = {}
        for k in ("pos", "U", "erot", "vib", "species", "id"):
            pin[k] = torch.from_numpy(st[k]).pin_memory().numpy()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g.set_particles(pin["pos"], pin["U"], pin["erot"], pin["vib"], pin["species"], pin["id"])
        ce0 = g.counts()
        ta = time.perf_counter()
        for _ in range(args.steps):
            g.evolve(1)
            g.counts()      # the step's collision counters back on the host
        tb = time.perf_counter()
        ttra = g.field("Ttra")
        t1 = time.perf_counter()
        ce1 = g.counts()
        nbytes_state = sum(v.nbytes for v in pin.values())
        counts_bytes = 48    # dsmc_counts_t
        ne = 0.5 * (ce0.n_particles + ce1.n_particles)
        e2e = {"value": ne * args.steps * world / (t1 - t0), "unit": UNIT,
               "collisions_per_s": (ce1.collisions_total - ce0.collisions_total) * world / (t1 - t0),
               "h2d_bytes_per_step": nbytes_state / args.steps,
               "d2h_bytes_per_step": counts_bytes + ttra.nbytes / args.steps,
               "upload_ms": round((ta - t0) * 1e3, 2), "steps_ms": round((tb - ta) * 1e3, 2),
               "field_ms": round((t1 - tb) * 1e3, 2),
               "note": f"the whole parcel state ({nbytes_state / 1e9:.2f} GB) uploaded once from pinned host "
                       f"memory and spread over the {args.steps} steps; every step's counters read back; one "
                       "field read at the end"}
        del ttra, pin
    g.close()

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    secondary = None
    if channel and not args.no_secondary:
        log("heat bath")
        secondary = heatbath_secondary(args, peak, peak_kind)

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
        "config": workload_config(args, s),
        "selection": "noTimeCounter, plain running maximum",
        "parallelism": f"{world} independent replicas" if world > 1 else "1 GPU",
        "parcels": int(N),
        "roofline": dominant,
        "roofline_kernels": rooflines,
        "roofline_move_sort": move_sort,
        "kernels_ms_per_step": kernels,
        "learned_vs_plain": lvp,
        "secondary_heatbath": secondary,
        "gpu_launches": int(args.steps * kernels_per_step(channel, False)),
        "e2e": e2e,
        "clocks": clocks,
    }
    if not args.no_cpu and world == 1 and cpu_state is not None:
        log("CPU baseline")
        line["cpu_baseline"] = cpu_run(args, s, cpu_state, omp_steps=args.cpu_steps, serial=False)
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def gpu_developed_state(args, seed):
    """The workload's state after its development, produced on the GPU
    (untimed input for the CPU arms): parcels and the per-cell selection
    state."""
    from hystrath_gb300 import build
    from hystrath_gb300 import learn
    build.build()
    g = learn.develop(make_spec(args, seed), args.develop if args.workload == "channel" else 0)
    g.evolve(args.warmup)
    st = g.particles()
    cells = {k: g.cell_array(k) for k in ("sigmaTcRMax", "collisionSelectionRemainder")}
    g.close()
    return st, cells


def cpu_run(args, s, state, omp_steps, serial):
    """The oracle restatement of the path on the host cores, started from a
    GPU-developed state of the same workload: omp_steps steps with OpenMP on
    all host threads, and with serial one step on one thread."""
    from oracle import oracle
    st, cells = state
    threads = args.cpu_threads or os.cpu_count()
    o = oracle.OracleCloud(s, threads=threads)
    o.set_particles(st["pos"], st["U"], st["erot"], st["vib"], st["species"], st["id"])
    for k, v in cells.items():
        o.set_cell_array(k, v)
    N = o.info().n_particles

    def timed(n):
        c0 = o.info()
        t0 = time.perf_counter()
        o.evolve(n)
        t1 = time.perf_counter()
        c1 = o.info()
        nn = 0.5 * (c0.n_particles + c1.n_particles)
        return nn * n / (t1 - t0), (c1.collisions_total - c0.collisions_total) / (t1 - t0), t1 - t0

    v, cps, sec = timed(omp_steps)
    out = {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "collisions_per_s": cps,
           "sample": (f"the full workload ({N} parcels) from its GPU-developed state, {omp_steps} steps with "
                      f"OpenMP on {threads} threads ({sec:.1f} s); a step costs the same at every step of the "
                      "developed flow, so the rate is the rate of the whole run")}
    if serial:
        o.set_threads(1)
        vs, cs, ss = timed(1)
        out["serial"] = {"value": vs, "unit": UNIT, "cores": 1, "collisions_per_s": cs,
                         "sample": f"1 step of the same workload on one thread ({ss:.1f} s)"}
    return out


def reference_arm(args, rank, world):
    if rank != 0:
        return
    s = make_spec(args, SEED)
    log("developing the state on the GPU (input of the CPU arm, untimed)")
    state = gpu_developed_state(args, SEED)
    log("CPU arm")
    cb = cpu_run(args, s, state, omp_steps=args.cpu_steps, serial=not args.no_serial)
    line = {"metric": METRIC, "impl": "reference", "value": cb["value"], "unit": UNIT,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": f"synthetic (dsmcMeshFill of the {args.workload} from the seed)",
            "config": workload_config(args, s),
            "selection": "noTimeCounter, plain running maximum",
            "parallelism": f"{cb['cores']} host threads (OpenMP over cells)",
            "note": ("CPU restatement of dsmcCloud::evolve (the reference needs OpenFOAM v1706, not installable "
                     "here), on the full workload from its state after the development steps, which the GPU "
                     "produced untimed; each timed step is a full step of the workload"),
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
    ap.add_argument("--workload", default="channel", choices=["channel", "heatbath"],
                    help="channel: the Mach-10 channel past a cube (the benchmark workload); "
                         "heatbath: the N2 heat bath")
    ap.add_argument("--scale", type=int, default=1, help="channel: cells divided by scale per axis")
    ap.add_argument("--cells", type=int, default=64, help="heat bath: edge in cells")
    ap.add_argument("--develop", type=int, default=600, help="channel: steps run before the warm-up")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned arm")
    ap.add_argument("--learn-every", type=int, default=100, help="learned: steps between predictions")
    ap.add_argument("--tau", type=float, default=0.95, help="learned: pinball quantile (0: squared error)")
    ap.add_argument("--forget", type=float, default=1.0,
                    help="learned: kept fraction of a cell's remembered excess at each prediction")
    ap.add_argument("--train-seeds", type=int, default=5)
    ap.add_argument("--train-rows", type=int, default=5_000_000)
    ap.add_argument("--train-steps", type=int, default=20000)
    ap.add_argument("--eval-steps", type=int, default=400, help="learned: evaluation window per arm")
    ap.add_argument("--eval-batches", type=int, default=8, help="learned: batch means in the window")
    ap.add_argument("--no-secondary", action="store_true", help="skip the heat-bath secondary line")
    ap.add_argument("--cpu-threads", type=int, default=0)
    ap.add_argument("--cpu-steps", type=int, default=2, help="CPU arms: OpenMP steps timed")
    ap.add_argument("--no-serial", action="store_true", help="reference arm: skip the one-thread step")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    args = ap.parse_args()
    if args.workload == "heatbath":
        args.develop = 0
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
