"""Batched clouds and launch shapes: a batched step gives every case exactly
the state it reaches when stepped alone, and no launch shape changes a
result (the step is deterministic).  The workload generator draws the
batched heat-bath distribution."""
import math

import numpy as np
import pytest

from hystrath_gb300 import spec as S


def test_workload_generator_draws_the_batched_distribution():
    from hystrath_gb300.batch import heat_bath_cases, mean_collision_time, size_classes
    specs, meta = heat_bath_cases(0, 256)
    edges = np.array([m["edge"] for m in meta])
    ppc = np.array([m["ppc"] for m in meta])
    T = np.array([m["T"] for m in meta])
    assert edges.min() >= 8 and edges.max() <= 48
    assert ppc.min() >= 5 and ppc.max() <= 60
    assert T.min() >= 500 and T.max() <= 20000
    assert 0.35 < np.mean([m["species"] == "N2" for m in meta]) < 0.65
    for s, m in zip(specs, meta):
        sp = S.N2 if m["species"] == "N2" else S.AR
        assert math.isclose(s.delta_t, 0.2 * mean_collision_time(sp, m["T"], 1e20), rel_tol=1e-12)
        assert all(s.patches[s.side_patch[q]].type == S.PATCH_CYCLIC for q in range(6))
    assert sum(len(c) for c in size_classes(specs)) == 256


def _state(g):
    st = g.particles()
    order = np.argsort(st["id"])
    return {k: v[order] for k, v in st.items() if k != "cell"}


@pytest.mark.gpu
def test_batched_steps_equal_steps_alone():
    from hystrath_gb300.batch import BatchCloud, heat_bath_cases
    from hystrath_gb300.dsmc import DsmcCloud
    specs, _ = heat_bath_cases(3, 256)
    small = [s for s in specs if s.n_cells[0] <= 12][:4]
    assert len(small) >= 2
    b = BatchCloud(small)
    b.initialise()
    b.evolve(7)
    for i, s in enumerate(small):
        g = DsmcCloud(s)
        g.initialise()
        g.evolve(7)
        ib, ig = b.info(i), g.info()
        assert ib.collisions_total == ig.collisions_total
        assert ib.n_particles == ig.n_particles
        sb = _state_of_case(b, i)
        sg = _state(g)
        for k in sb:
            assert np.array_equal(sb[k], sg[k]), k
        g.close()
    b.close()


def _state_of_case(b, i):
    import ctypes as C
    from hystrath_gb300.dsmc import DsmcCloud, lib
    view = DsmcCloud.__new__(DsmcCloud)
    view.h = C.c_void_p(lib().dsmc_batch_case(b.h, i))
    view.spec = b.specs[i]
    s = view.spec
    view.n_cells = s.n_cells[0] * s.n_cells[1] * s.n_cells[2]
    try:
        return _state(view)
    finally:
        view.h = None       # owned by the batch


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(128, 32), (512, 64)])
def test_launch_shape_does_not_change_results(shape):
    from hystrath_gb300.batch import _bind
    from hystrath_gb300.dsmc import DsmcCloud
    s = S.config1(seed=4, n=16)
    ref = DsmcCloud(s)
    ref.initialise()
    ref.evolve(6)
    g = DsmcCloud(s)
    g.initialise()
    assert _bind().dsmc_set_launch(g.h, *shape) == 0
    g.evolve(6)
    assert g.info().collisions_total == ref.info().collisions_total
    a, b = _state(ref), _state(g)
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    np.testing.assert_array_equal(ref.field("Ttra"), g.field("Ttra"))


@pytest.mark.gpu
def test_batch_from_case_directories():
    """Cases given as OpenFOAM directories (each parsed and created before the
    next is parsed) step together as they step alone."""
    import os
    from hystrath_gb300.batch import BatchCloud
    from hystrath_gb300.dsmc import DsmcCloud
    here = os.path.dirname(os.path.abspath(__file__))
    dirs = [os.path.join(here, "golden", "cases", c) for c in ("couette_N2-O2", "hypersonic_corner")]
    b = BatchCloud(dirs)
    b.initialise()
    b.evolve(5)
    for i, d in enumerate(dirs):
        g = DsmcCloud(d)
        g.initialise()
        g.evolve(5)
        a, c = b.info(i), g.info()
        assert a.n_particles == c.n_particles and a.collisions_total == c.collisions_total
        # the totals are sums of FP64 atomics: equal to the last bits
        assert abs(a.linear_ke / c.linear_ke - 1.0) < 1e-12
    b.close()


def _case_view(b, i):
    import ctypes as C
    from hystrath_gb300.dsmc import DsmcCloud, lib
    view = DsmcCloud.__new__(DsmcCloud)
    view.h = C.c_void_p(lib().dsmc_batch_case(b.h, i))
    view.spec = b.specs[i]
    s = view.spec
    view.n_cells = s.n_cells[0] * s.n_cells[1] * s.n_cells[2]
    return view


@pytest.mark.gpu
def test_batch_follows_settings_changed_on_a_case():
    """Switching face tracking or the learned maximum on a batched case (which
    drops that case's step graphs) rebuilds the batch graph: the batch keeps
    giving each case the state it reaches alone with the same switches, and a
    model detached and destroyed is no longer read."""
    from hystrath_gb300.batch import BatchCloud
    from hystrath_gb300.dsmc import DsmcCloud, Mlp
    from hystrath_gb300.learn import init_params
    specs = [S.config1(seed=21, n=10), S.config1(seed=22, n=12)]
    b = BatchCloud(specs)
    b.initialise()
    b.evolve(2)
    alone = [DsmcCloud(s) for s in specs]
    for g in alone:
        g.initialise()
        g.evolve(2)
    model = Mlp()
    # inputs about (log n, log T, speed ratio) of the bath; output about the
    # log of its sigma_T c_R (~1e-15 m^3/s), so the untrained net predicts a
    # maximum of the right order
    norm = np.array([45.0, 8.0, 0.5, 1.0, 1.0, 0.5, -34.5, 0.3], dtype=np.float32)
    model.set_params(init_params(3), norm)
    views = [_case_view(b, i) for i in range(2)]
    try:
        views[0].set_face_tracking(True)
        alone[0].set_face_tracking(True)
        views[1].set_learned(model, 2, 0.5)
        alone[1].set_learned(model, 2, 0.5)
        b.evolve(3)
        for g in alone:
            g.evolve(3)
        flux_b = views[0].face_flux("parcelIdFlux")
        assert np.abs(flux_b).sum() > 0
        np.testing.assert_array_equal(flux_b, alone[0].face_flux("parcelIdFlux"))
        assert b.info(1).candidates_total == alone[1].info().candidates_total
        views[1].set_learned(None)
        alone[1].set_learned(None)
        model.close()
        b.evolve(2)
        for g in alone:
            g.evolve(2)
        for i in range(2):
            assert b.info(i).collisions_total == alone[i].info().collisions_total
            sb, sg = _state(views[i]), _state(alone[i])
            for k in sb:
                assert np.array_equal(sb[k], sg[k]), k
    finally:
        for v in views:
            v.h = None      # owned by the batch
        for g in alone:
            g.close()
        b.close()


@pytest.mark.gpu
@pytest.mark.parametrize("threads", [(256, 128), (128, 64), (512, 128)])
def test_persistent_batch_equals_steps_alone(threads):
    """The persistent mode (cooperative launches of phase ranges over all
    cases, per-phase work queues) gives every case exactly the state it
    reaches alone, Ar and N2 alike."""
    from hystrath_gb300.batch import BatchCloud, heat_bath_cases
    from hystrath_gb300.dsmc import DsmcCloud
    specs, _ = heat_bath_cases(5, 256)
    small = [s for s in specs if s.n_cells[0] <= 14][:6]
    assert len(small) >= 3
    b = BatchCloud(small)
    b.initialise()
    b.evolve(2)                         # the graph mode first, then switch
    b.set_persistent(*threads)
    b.evolve(5)
    for i, s in enumerate(small):
        g = DsmcCloud(s)
        g.initialise()
        g.evolve(7)
        ib, ig = b.info(i), g.info()
        assert ib.collisions_total == ig.collisions_total and ib.candidates_total == ig.candidates_total
        assert ib.n_particles == ig.n_particles and ib.step == ig.step
        sb, sg = _state_of_case(b, i), _state(g)
        for k in sb:
            assert np.array_equal(sb[k], sg[k]), k
        view = _case_view(b, i)
        try:
            np.testing.assert_array_equal(view.field("Ttra"), g.field("Ttra"))
        finally:
            view.h = None   # owned by the batch
        g.close()
    b.close()


@pytest.mark.gpu
def test_persistent_batch_rejects_cases_it_cannot_run():
    from hystrath_gb300.batch import BatchCloud
    from hystrath_gb300.dsmc import DsmcError
    b = BatchCloud([S.config1(seed=1, n=8), S.config2(seed=2, scale=8)])
    b.initialise()
    with pytest.raises(DsmcError) as e:
        b.set_persistent(256, 128)
    assert "case 1" in str(e.value) and "inflow" in str(e.value)
    b.evolve(2)                          # still steps in the graph mode
    b.close()


@pytest.mark.gpu
def test_destroying_a_batched_case_is_refused():
    """dsmc_destroy on a handle from dsmc_batch_case leaves the case to the
    batch (no double free when the batch is destroyed)."""
    from hystrath_gb300.batch import BatchCloud
    from hystrath_gb300.dsmc import lib
    b = BatchCloud([S.config1(seed=1, n=8), S.config1(seed=2, n=8)])
    b.initialise()
    h = lib().dsmc_batch_case(b.h, 1)
    lib().dsmc_destroy(h)
    assert b"belongs to a batch" in lib().dsmc_last_error(h)
    b.evolve(2)
    assert b.info(1).step == 2
    b.close()


@pytest.mark.gpu
def test_dense_heavy_cells_persistent_equal_alone():
    """A dense case (about 400 parcels and a few hundred candidates per cell:
    many conflict rounds of a heavy cell's warp) in the persistent batch
    reaches the state it reaches alone, bit for bit."""
    from hystrath_gb300.batch import BatchCloud
    from hystrath_gb300.dsmc import DsmcCloud

    def dense():
        s = S.config1(seed=91, n=6)
        s.n_equivalent_particles /= 8.0
        s.delta_t *= 50.0
        return s

    g = DsmcCloud(dense())
    g.initialise()
    g.evolve(1)
    assert g.counts().candidates_last_step / 216 > 128
    g.evolve(3)
    b = BatchCloud([dense(), S.config1(seed=92, n=8)])
    b.initialise()
    b.set_persistent(256, 128)
    b.evolve(4)
    ib, ig = b.info(0), g.info()
    assert ib.collisions_total == ig.collisions_total and ib.candidates_total == ig.candidates_total
    sb, sg = _state_of_case(b, 0), _state(g)
    for k in sb:
        assert np.array_equal(sb[k], sg[k]), k
    g.close()
    b.close()


class _FakeBatch:
    """Stands in for BatchCloud in the tuner tests (no GPU): the time of a
    batched step is a sum of per-class costs of the launch shapes set."""

    def __init__(self, classes, cost):
        self.classes, self.cost = classes, cost
        self.shape = {}
        self.persistent = None
        self.timed = 0

    def set_launch(self, i, t, c):
        self.shape[i] = (t, c)

    def set_persistent(self, t, c):
        self.persistent = (t, c)

    def evolve(self, n=1):
        pass

    def evolve_timed(self, n):
        self.timed += 1
        if self.persistent is not None:
            t, c = self.persistent
            return n * (10.0 + abs(t - 256) / 128.0 + (0.5 if c == 128 else 0.0))
        ms = 0.0
        for k, idx in enumerate(self.classes):
            ms += self.cost(k, self.shape[idx[0]])
        return n * ms


def test_autotune_picks_each_class_minimum():
    """Coordinate descent over size classes: every class ends on the launch
    shape of least cost (the costs are separable), and that shape is what
    the batch's cases carry."""
    from hystrath_gb300.batch import CELLS_PER_CTA, CTA_THREADS, autotune
    classes = [[0, 1], [2], [3, 4, 5]]
    best = {0: (128, 32), 1: (512, 128), 2: (256, 64)}

    def cost(k, cfg):
        return 1.0 + (0.0 if cfg == best[k] else 0.3 + 0.001 * (cfg[0] + cfg[1]))

    b = _FakeBatch(classes, cost)
    choice, ms = autotune(b, classes, steps=2)
    assert choice == [best[0], best[1], best[2]]
    assert abs(ms - 3.0) < 1e-12
    for k, idx in enumerate(classes):
        assert all(b.shape[i] == best[k] for i in idx)
    assert b.timed == len(classes) * len(CTA_THREADS) * len(CELLS_PER_CTA)


def test_autotune_persistent_picks_and_applies_the_minimum():
    from hystrath_gb300.batch import autotune_persistent
    b = _FakeBatch([[0]], lambda k, cfg: 0.0)
    cfg, ms = autotune_persistent(b, steps=3)
    assert cfg == (256, 64) and abs(ms - 10.0) < 1e-12
    assert b.persistent == (256, 64)
