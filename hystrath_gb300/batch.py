"""Many independent heat-bath cases stepped together, and the autotuner of
their launch shapes.

``BatchCloud`` wraps ``dsmc_batch_*``: every batched step is one launch of a
CUDA graph whose children are the cases' captured steps, or, in the
persistent mode, cooperative persistent launches over all cases (four
ranges of the move and sort phases, three of the collision phases) with
per-phase (case, tile) work queues.  ``autotune`` picks,
per size class of the cases, the threads per CTA of the parcel-streaming
kernels and the cells per CTA of the lane-per-cell collision kernel by timing
batched steps (coordinate descent over the classes).

``python -m hystrath_gb300.batch`` runs the batched heat-bath workload (256
periodic cases drawn from the seed: 8^3..48^3 cells, 5..60 parcels per cell,
Ar or N2, T_tr log-uniform in 500..20000 K, T_int 300 K, n = 1e20 m^-3,
dt = 0.2 mean collision times) batched and one case at a time, and prints
one JSON line with the aggregate collision and parcel-step rates of the
persistent mode, the graph of case graphs and the cases one at a time.
"""
from __future__ import annotations

import ctypes as C
import json
import math
import sys
import time

import numpy as np

from . import spec as S
from .dsmc import DsmcCloud, DsmcError, lib

CTA_THREADS = (128, 256, 512)
CELLS_PER_CTA = (32, 64, 128)


def mean_collision_time(species: dict, T: float, n: float, tref: float = 273.0) -> float:
    """1 / (per-molecule VHS equilibrium collision rate, Bird eq. 4.64 as coded
    in dsmcVolFields.C:1722-1732)."""
    d, m, w = species["diameter"], species["mass"], species["omega"]
    nu = 2.0 * math.sqrt(math.pi) * d * d * n * (T / tref) ** (1.0 - w) * math.sqrt(2.0 * S.KB * tref / (m / 2.0))
    return 1.0 / nu


def heat_bath_cases(seed: int = 0, n_cases: int = 256, n_density: float = 1e20, cell=1e-3):
    """The batched workload: per case, drawn from the seed, an edge of
    8..48 cells, 5..60 parcels per cell, Ar or N2 (p = 0.5), T_tr log-uniform
    in 500..20000 K, T_int = 300 K, periodic sides, dt = 0.2 mean collision
    times at T_tr."""
    rng = np.random.default_rng(seed)
    specs, meta = [], []
    for i in range(n_cases):
        edge = int(rng.integers(8, 49))
        ppc = int(rng.integers(5, 61))
        diatomic = bool(rng.random() < 0.5)
        T = float(math.exp(rng.uniform(math.log(500.0), math.log(20000.0))))
        sp = S.N2 if diatomic else S.AR
        dt = 0.2 * mean_collision_time(sp, T, n_density)
        fn = n_density * cell ** 3 / ppc
        s = S.make_box_case((edge, edge, edge), cell, sp, fn=fn, dt=dt, seed=seed * 100003 + i,
                            n_density=n_density, t_tra=T,
                            t_rot=300.0 if diatomic else 0.0, t_vib=300.0 if diatomic else 0.0,
                            side_model=S.BC_SPECULAR, side_type=S.PATCH_CYCLIC,
                            collision=S.COLL_LB_VHS if diatomic else S.COLL_VHS)
        specs.append(s)
        meta.append({"edge": edge, "ppc": ppc, "species": "N2" if diatomic else "Ar", "T": T, "dt": dt})
    return specs, meta


def _bind():
    L = lib()
    if getattr(L, "_batch_bound", False):
        return L
    vp = C.c_void_p
    L.dsmc_batch_create.argtypes = [C.c_int, vp, C.POINTER(vp)]
    L.dsmc_batch_create_from_dirs.argtypes = [C.c_int, C.POINTER(C.c_char_p), C.POINTER(vp)]
    L.dsmc_batch_destroy.argtypes = [vp]
    L.dsmc_batch_destroy.restype = None
    L.dsmc_batch_last_error.argtypes = [vp]
    L.dsmc_batch_last_error.restype = C.c_char_p
    L.dsmc_batch_size.argtypes = [vp]
    L.dsmc_batch_case.argtypes = [vp, C.c_int]
    L.dsmc_batch_case.restype = vp
    L.dsmc_batch_initialise.argtypes = [vp]
    L.dsmc_batch_set_launch.argtypes = [vp, C.c_int, C.c_int, C.c_int]
    L.dsmc_batch_evolve.argtypes = [vp, C.c_longlong]
    L.dsmc_batch_evolve_timed.argtypes = [vp, C.c_longlong, C.POINTER(C.c_double)]
    L.dsmc_batch_set_persistent.argtypes = [vp, C.c_int, C.c_int]
    L.dsmc_batch_get_persistent.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.dsmc_set_launch.argtypes = [vp, C.c_int, C.c_int]
    L.dsmc_get_launch.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L._batch_bound = True
    return L


class BatchCloud:
    """Independent clouds stepped together by one graph launch per step."""

    def __init__(self, specs):
        """specs: CaseSpec objects, or OpenFOAM case directories (str)."""
        L = _bind()
        h = C.c_void_p()
        if specs and all(isinstance(x, str) for x in specs):
            arr = (C.c_char_p * len(specs))(*[x.encode() for x in specs])
            rc = L.dsmc_batch_create_from_dirs(len(specs), arr, C.byref(h))
        else:
            arr = (S.CaseSpec * len(specs))(*specs)
            rc = L.dsmc_batch_create(len(specs), C.cast(arr, C.c_void_p), C.byref(h))
        if rc != 0:
            raise DsmcError(rc, L.dsmc_batch_last_error(None).decode())
        self.h = h
        self.n = len(specs)
        self.specs = specs

    def close(self):
        if getattr(self, "h", None):
            lib().dsmc_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _chk(self, rc):
        if rc != 0:
            raise DsmcError(rc, lib().dsmc_batch_last_error(self.h).decode())

    def initialise(self):
        self._chk(lib().dsmc_batch_initialise(self.h))

    def evolve(self, n: int = 1):
        self._chk(lib().dsmc_batch_evolve(self.h, int(n)))

    def evolve_timed(self, n: int) -> float:
        ms = C.c_double()
        self._chk(lib().dsmc_batch_evolve_timed(self.h, int(n), C.byref(ms)))
        return ms.value

    def set_launch(self, i: int, cta_threads: int, cells_per_cta: int):
        self._chk(lib().dsmc_batch_set_launch(self.h, int(i), int(cta_threads), int(cells_per_cta)))

    def set_persistent(self, move_threads: int, collide_threads: int):
        """Two persistent cooperative launches per batched step over all
        cases (move and sort, then collisions); 0, 0: the graph of case
        graphs."""
        self._chk(_bind().dsmc_batch_set_persistent(self.h, int(move_threads), int(collide_threads)))

    def info(self, i: int) -> S.Info:
        inf = S.Info()
        rc = lib().dsmc_info(lib().dsmc_batch_case(self.h, int(i)), C.byref(inf))
        if rc != 0:
            raise DsmcError(rc, "case info")
        return inf

    def totals(self):
        coll = parcels = 0
        for i in range(self.n):
            inf = self.info(i)
            coll += inf.collisions_total
            parcels += inf.n_particles
        return coll, parcels


def size_classes(specs, bounds=(16, 32)):
    """Case index lists by cell-edge class: < 16, 16..31, >= 32."""
    cls = [[] for _ in range(len(bounds) + 1)]
    for i, s in enumerate(specs):
        e = s.n_cells[0]
        k = sum(e >= b for b in bounds)
        cls[k].append(i)
    return [c for c in cls if c]


def autotune(batch: BatchCloud, classes, steps=4, rounds=1, log=None):
    """Coordinate descent: for each size class in turn, the (CTA threads,
    cells per CTA) pair that gives the shortest batched step with the other
    classes fixed.  Returns the choice per class and the best time per step."""
    choice = [(256, 128)] * len(classes)

    def apply(k, cfg):
        for i in classes[k]:
            batch.set_launch(i, cfg[0], cfg[1])

    for k in range(len(classes)):
        apply(k, choice[k])
    best_ms = None
    for _ in range(rounds):
        for k in range(len(classes)):
            trial = []
            for t in CTA_THREADS:
                for c in CELLS_PER_CTA:
                    apply(k, (t, c))
                    batch.evolve(1)                      # capture and warm
                    ms = batch.evolve_timed(steps) / steps
                    trial.append((ms, (t, c)))
            ms, cfg = min(trial)
            choice[k] = cfg
            apply(k, cfg)
            best_ms = ms
            if log:
                log(f"class {k} ({len(classes[k])} cases): {cfg} {ms:.3f} ms/step")
    return choice, best_ms


MOVE_THREADS = (128, 256, 512)
COLLIDE_THREADS = (64, 128)


def autotune_persistent(batch: BatchCloud, steps=4, log=None):
    """The (move CTA threads, collision CTA threads = light cells per CTA)
    pair of the persistent mode with the shortest batched step."""
    trial = []
    for t in MOVE_THREADS:
        for c in COLLIDE_THREADS:
            batch.set_persistent(t, c)
            batch.evolve(1)                      # capture and warm
            ms = batch.evolve_timed(steps) / steps
            trial.append((ms, (t, c)))
            if log:
                log(f"persistent {t}/{c}: {ms:.3f} ms/step")
    ms, cfg = min(trial)
    batch.set_persistent(*cfg)
    return cfg, ms


def one_at_a_time(specs, steps, warmup, launch=None):
    """Each case on its own (its own graph launches), back to back."""
    tot_ms = 0.0
    coll = pst = 0
    for i, s in enumerate(specs):
        g = DsmcCloud(s)
        g.initialise()
        if launch is not None:
            _bind().dsmc_set_launch(g.h, *launch[i])
        g.evolve(warmup)
        i0 = g.info()
        tot_ms += g.evolve_timed(steps)
        i1 = g.info()
        coll += i1.collisions_total - i0.collisions_total
        pst += i0.n_particles * steps
        g.close()
    return tot_ms, coll, pst


def main():
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--cases", type=int, default=256)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-tune", action="store_true")
    args = ap.parse_args()

    def log(msg):
        print(msg, file=sys.stderr, flush=True)

    specs, meta = heat_bath_cases(args.seed, args.cases)
    t0 = time.time()
    classes = size_classes(specs)
    choice = [(256, 128)] * len(classes)
    pcfg = (256, 128)
    if not args.no_tune:
        # tuning steps change the state: the timed runs below start afresh
        b = BatchCloud(specs)
        b.initialise()
        choice, _ = autotune(b, classes, log=log)
        pcfg, _ = autotune_persistent(b, log=log)
        b.close()

    def timed(persistent):
        b = BatchCloud(specs)
        b.initialise()
        for k, idx in enumerate(classes):
            for i in idx:
                b.set_launch(i, *choice[k])
        if persistent:
            b.set_persistent(*pcfg)
        N = sum(b.info(i).n_particles for i in range(b.n))
        b.evolve(args.warmup)
        c0, _ = b.totals()
        ms = b.evolve_timed(args.steps)
        c1, _ = b.totals()
        b.close()
        return ms, c1 - c0, N

    ms, coll, N = timed(False)
    log(f"{len(specs)} cases, {N} parcels; graph of case graphs {ms / args.steps:.3f} ms/step "
        f"({time.time() - t0:.1f} s so far)")
    msp, collp, _ = timed(True)
    log(f"persistent {msp / args.steps:.3f} ms/step")
    launch = [None] * len(specs)
    for k, idx in enumerate(classes):
        for i in idx:
            launch[i] = choice[k]
    ms1, coll1, pst1 = one_at_a_time(specs, args.steps, args.warmup, launch)
    line = {
        "workload": f"{args.cases} periodic heat baths (8^3..48^3 cells, 5..60 parcels/cell, Ar|N2, "
                    "T_tr 500..20000 K, dt = 0.2 mean collision times)",
        "parcels": int(N), "steps": args.steps,
        "persistent": {"ms_per_step": msp / args.steps, "collisions_per_s": collp / (msp * 1e-3),
                       "particle_steps_per_s": N * args.steps / (msp * 1e-3),
                       "move_threads": pcfg[0], "collide_threads": pcfg[1],
                       "same_collisions_as_graph_mode": collp == coll},
        "batched": {"ms_per_step": ms / args.steps, "collisions_per_s": coll / (ms * 1e-3),
                    "particle_steps_per_s": N * args.steps / (ms * 1e-3)},
        "one_at_a_time": {"ms_per_step": ms1 / args.steps, "collisions_per_s": coll1 / (ms1 * 1e-3),
                          "particle_steps_per_s": pst1 / (ms1 * 1e-3)},
        "speedup": ms1 / ms,
        "speedup_persistent": ms1 / msp,
        "launch_per_class": [{"cases": len(idx), "edge_range": [min(specs[i].n_cells[0] for i in idx),
                                                               max(specs[i].n_cells[0] for i in idx)],
                              "cta_threads": choice[k][0], "cells_per_cta": choice[k][1]}
                             for k, idx in enumerate(classes)],
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
