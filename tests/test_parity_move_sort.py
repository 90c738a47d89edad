"""Bit-exact parity of the GPU move (with every boundary model), cell indexing
and occupancy sort against the CPU replay on the same state and the same
random stream.

The GPU leaves parcels of one cell in atomic-scatter order; both sides are
compared after ordering by (cell, particle id), which is the canonical order
the collision and sampling kernels use.  Parcels whose velocity is resampled
by a diffuse wall or that are created by the inflow go through log/sin/cos,
which differ between libm and CUDA by a few ulps: they are compared with a
relative tolerance of 1e-12; every other parcel must match bit for bit.
"""
import numpy as np
import pytest

from hystrath_gb300 import spec as S

pytestmark = pytest.mark.gpu


def _canonical(p):
    order = np.lexsort((p["id"], p["cell"]))
    return {k: v[order] for k, v in p.items()}


def _pair(spec, gpu_lib, oracle_mod, threads=4):
    from hystrath_gb300.dsmc import DsmcCloud
    g = DsmcCloud(spec)
    g.initialise()
    st = g.particles()
    o = oracle_mod.OracleCloud(spec, threads=threads)
    o.set_particles(st["pos"], st["U"], st["erot"], st["vib"], st["species"], st["id"])
    return g, o, st


def _taint():
    """Ids whose state went through a transcendental function (inflow
    creation, diffuse wall) in some step so far: compared with a tolerance."""
    return {"ids": np.empty(0, dtype=np.uint32)}


def _check_step(g, o, before, phases, allow_resampled=True, tainted=None):
    """One step on both sides.  ``tainted`` (from _taint) collects ids whose
    state went through a transcendental function in this or an earlier step;
    they are compared with a tolerance.  Vectorised: runs at 10^8 parcels."""
    g.run_phases(phases)
    o.run_phases(phases)
    a = _canonical(g.particles())
    b = _canonical(o.particles())
    assert len(a["id"]) == len(b["id"])
    np.testing.assert_array_equal(a["id"], b["id"])
    np.testing.assert_array_equal(a["cell"], b["cell"])
    np.testing.assert_array_equal(g.cell_array("count"), o.cell_array("count"))
    np.testing.assert_array_equal(g.cell_array("start"), o.cell_array("start"))
    # parcels whose velocity only changed by exact sign flips (specular, symmetry)
    order = np.argsort(before["id"], kind="stable")
    ids_sorted = before["id"][order]
    k = np.minimum(np.searchsorted(ids_sorted, b["id"]), max(len(ids_sorted) - 1, 0))
    old = ids_sorted[k] == b["id"] if len(ids_sorted) else np.zeros(len(b["id"]), bool)
    idx = order[k]
    exact = old.copy()
    exact[old] = np.all(np.abs(b["U"][old]) == np.abs(before["U"][idx[old]]), axis=1)
    if tainted is not None:
        tainted["ids"] = np.union1d(tainted["ids"], b["id"][~exact])
        exact &= ~np.isin(b["id"], tainted["ids"])
    n_exact = int(exact.sum())
    assert n_exact > 0
    for key in ("pos", "U"):
        np.testing.assert_array_equal(a[key][exact], b[key][exact])
    np.testing.assert_array_equal(a["erot"][exact], b["erot"][exact])
    np.testing.assert_array_equal(a["vib"][exact], b["vib"][exact])
    if not allow_resampled:
        assert n_exact == len(exact)
    else:
        rest = ~exact
        if rest.any():
            np.testing.assert_allclose(a["pos"][rest], b["pos"][rest], rtol=1e-12, atol=1e-15)
            np.testing.assert_allclose(a["U"][rest], b["U"][rest], rtol=1e-11, atol=1e-9)
    return a, b, exact


def test_move_sort_specular_box(gpu_lib, oracle_mod):
    g, o, st = _pair(S.config0(seed=11), gpu_lib, oracle_mod)
    before = _canonical(st)
    for _ in range(3):
        a, b, exact = _check_step(g, o, before, S.PHASE_MOVE | S.PHASE_SORT, allow_resampled=False)
        before = b
    assert g.info().wall_hits_last_step == o.info().wall_hits_last_step


def test_move_sort_cyclic_box(gpu_lib, oracle_mod):
    g, o, st = _pair(S.config0(seed=12, cyclic=True), gpu_lib, oracle_mod)
    before = _canonical(st)
    for _ in range(3):
        _, b, _ = _check_step(g, o, before, S.PHASE_MOVE | S.PHASE_SORT, allow_resampled=False)
        before = b


def test_move_sort_heat_bath_n2(gpu_lib, oracle_mod):
    g, o, st = _pair(S.config1(seed=13, n=12), gpu_lib, oracle_mod)
    before = _canonical(st)
    _check_step(g, o, before, S.PHASE_MOVE | S.PHASE_SORT, allow_resampled=False)


def test_move_sort_inflow_obstacle_diffuse(gpu_lib, oracle_mod):
    """Mach-10 channel with a diffuse cube, inflow at x=0 and deletion at
    x=max (config 2 at 1/8 scale): inflow, deletion, diffuse and specular
    crossings in one step."""
    s = S.config2(seed=14, scale=8)
    g, o, st = _pair(s, gpu_lib, oracle_mod)
    before = _canonical(st)
    tainted = _taint()
    for _ in range(4):
        a, b, exact = _check_step(g, o, before, S.PHASE_INFLOW | S.PHASE_MOVE | S.PHASE_SORT,
                                  tainted=tainted)
        before = b
    assert exact.sum() > 0.9 * len(exact)
    gi, oi = g.info(), o.info()
    assert gi.inserted_last_step == oi.inserted_last_step > 0
    assert gi.deleted_last_step == oi.deleted_last_step
    assert gi.wall_hits_last_step == oi.wall_hits_last_step > 0
    # wall flux accumulators of every boundary face
    np.testing.assert_allclose(g.wall_accumulators(), o.wall(), rtol=1e-9, atol=1e-30)


def test_mesh_fill_counts_and_positions(gpu_lib, oracle_mod):
    """dsmcMeshFill: counts per cell and positions are exact; velocities
    (Box-Muller through log/sin/cos) within 1e-12."""
    from hystrath_gb300.dsmc import DsmcCloud
    s = S.config1(seed=21, n=8)
    g = DsmcCloud(s)
    g.initialise()
    o = oracle_mod.OracleCloud(s, threads=2)
    o.initialise()
    np.testing.assert_array_equal(g.cell_array("count"), o.cell_array("count"))
    a, b = _canonical(g.particles()), _canonical(o.particles())
    np.testing.assert_array_equal(a["id"], b["id"])
    np.testing.assert_array_equal(a["pos"], b["pos"])
    np.testing.assert_allclose(a["U"], b["U"], rtol=1e-12, atol=1e-9)
    np.testing.assert_array_equal(a["vib"], b["vib"])
    np.testing.assert_allclose(a["erot"], b["erot"], rtol=1e-12, atol=0)
    np.testing.assert_array_equal(g.cell_array("sigmaTcRMax"), o.cell_array("sigmaTcRMax"))
    np.testing.assert_array_equal(g.cell_array("collisionSelectionRemainder"),
                                  o.cell_array("collisionSelectionRemainder"))


def test_sampling_matches_oracle(gpu_lib, oracle_mod):
    """One sample of identical states: the derived fields agree to 1e-12
    (sums are taken in different but fixed orders)."""
    g, o, _ = _pair(S.config1(seed=31, n=8), gpu_lib, oracle_mod)
    g.run_phases(S.PHASE_SAMPLE)
    o.run_phases(S.PHASE_SAMPLE)
    for f in ("rhoN", "rhoM", "Ux", "Uy", "Uz", "Ttra", "Trot", "Tvib", "Tov", "p", "dsmcNMean"):
        np.testing.assert_allclose(g.field(f), o.field(f), rtol=1e-10, atol=1e-9, err_msg=f)


def test_move_sort_reduced_d_couette(gpu_lib, oracle_mod):
    """The two-species Couette channel: one cell thick in z with empty front
    and back (tracked at the mesh centre with no z velocity), cyclic in x,
    diffuse walls moving at 300 m/s."""
    import os
    from hystrath_gb300.dsmc import parse_case
    s = parse_case(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "cases", "couette_N2-O2"))
    g, o, st = _pair(s, gpu_lib, oracle_mod)
    before = _canonical(st)
    tainted = _taint()
    for _ in range(3):
        a, b, exact = _check_step(g, o, before, S.PHASE_MOVE | S.PHASE_SORT, tainted=tainted)
        before = b
    assert np.all(a["pos"][:, 2] == 0.005) and np.abs(a["U"][:, 2]).max() > 100.0
    assert g.info().wall_hits_last_step == o.info().wall_hits_last_step > 0


def test_move_sort_graded_flat_plate(gpu_lib, oracle_mod):
    """The supersonic flat plate: graded cells in x and y (blockMesh
    simpleGrading), an empty z, free-stream inflow and deletion on four sides
    and a diffuse plate; cells are found in the half-node tables on both
    sides."""
    import os
    from hystrath_gb300.dsmc import parse_case
    s = parse_case(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "cases",
                                "supersonic_flat_plate"))
    g, o, st = _pair(s, gpu_lib, oracle_mod, threads=8)
    before = _canonical(st)
    tainted = _taint()
    for _ in range(3):
        a, b, exact = _check_step(g, o, before, S.PHASE_INFLOW | S.PHASE_MOVE | S.PHASE_SORT, tainted=tainted)
        before = b
    assert exact.sum() > 0.9 * len(exact)
    gi, oi = g.info(), o.info()
    assert gi.inserted_last_step == oi.inserted_last_step > 0
    assert gi.deleted_last_step == oi.deleted_last_step > 0
    assert gi.wall_hits_last_step == oi.wall_hits_last_step > 0
    np.testing.assert_allclose(g.wall_accumulators(), o.wall(), rtol=1e-9, atol=1e-30)


# ------------------------------------------------------ benchmarked sizes
def _oracle_from_gpu(spec, g, oracle_mod):
    """The oracle continuing the GPU cloud's state: parcels, the per-cell
    selection state, the inflow remainders and the step that keys the random
    streams (sampling sums restart on both sides)."""
    import os
    st = g.particles()
    o = oracle_mod.OracleCloud(spec, threads=os.cpu_count() or 4)
    o.set_particles(st["pos"], st["U"], st["erot"], st["vib"], st["species"], st["id"])
    for k in ("sigmaTcRMax", "collisionSelectionRemainder", "inflowAccumulator"):
        o.set_cell_array(k, g.cell_array(k))
    o.set_step(g.counts().step)
    g.reset_sampling()
    return o, st


def test_move_sort_heat_bath_bench_size(gpu_lib, oracle_mod):
    """The 64^3 heat bath of the benchmark (13.1M parcels) after 20 full steps
    on the GPU: one move and sort, bit for bit."""
    from hystrath_gb300.dsmc import DsmcCloud
    s = S.config1(seed=1000, n=64)
    g = DsmcCloud(s)
    g.initialise()
    g.evolve(20)
    o, st = _oracle_from_gpu(s, g, oracle_mod)
    assert len(st["id"]) > 13_000_000
    _check_step(g, o, _canonical(st), S.PHASE_MOVE | S.PHASE_SORT, allow_resampled=False)
    assert g.info().wall_hits_last_step == o.info().wall_hits_last_step > 0


def test_move_sort_channel_full_size_developed(gpu_lib, oracle_mod):
    """The Mach-10 channel of the benchmark at full size (256x128x128 cells,
    about 84M parcels) after 600 full steps on the GPU (bow shock and wake
    formed): one inflow+move+sort step compared parcel by parcel with the
    wall accumulators of every boundary face, then two more with the face
    tracker on, compared face by face."""
    from hystrath_gb300.dsmc import DsmcCloud
    s = S.config2(seed=1000, scale=1)
    g = DsmcCloud(s)
    g.initialise()
    g.evolve(600)
    o, st = _oracle_from_gpu(s, g, oracle_mod)
    assert len(st["id"]) > 80_000_000
    before = _canonical(st)
    del st
    tainted = _taint()
    phases = S.PHASE_INFLOW | S.PHASE_MOVE | S.PHASE_SORT
    a, b, exact = _check_step(g, o, before, phases, tainted=tainted)
    assert exact.sum() > 0.99 * len(exact)
    gi, oi = g.info(), o.info()
    assert gi.inserted_last_step == oi.inserted_last_step > 0
    assert gi.deleted_last_step == oi.deleted_last_step > 0
    assert gi.wall_hits_last_step == oi.wall_hits_last_step > 0
    np.testing.assert_allclose(g.wall_accumulators(), o.wall(), rtol=1e-9, atol=1e-30)
    g.set_face_tracking(True)
    o.set_face_tracking(True)
    before = b
    del a
    for _ in range(2):
        _, before, _ = _check_step(g, o, before, phases, tainted=tainted)
    for key in ("parcelIdFlux", "massIdFlux"):
        fa, fb = g.face_flux(key, 0), o.face_flux(key, 0)
        assert np.abs(fb).sum() > 0
        if key == "parcelIdFlux":
            np.testing.assert_array_equal(fa, fb)
        else:
            np.testing.assert_allclose(fa, fb, rtol=1e-12, atol=1e-40)


def test_derived_fields_match_oracle(gpu_lib, oracle_mod):
    """Mach number, the statistical error fields and the measureHeatFluxShearStress
    tensors (dsmcVolFields.C:1511-1661, 1859-1873) of the Mach-10 channel's
    initial state after one sample and one move: GPU fixed-point moments
    against the oracle's FP64 sums, within 1e-9 of each field's scale."""
    s = S.config2(seed=41, scale=8)
    s.measure_heat_flux_shear_stress = 1
    s.measure_errors = 1
    g, o, _ = _pair(s, gpu_lib, oracle_mod)
    for _ in range(2):
        g.run_phases(S.PHASE_SAMPLE)
        o.run_phases(S.PHASE_SAMPLE)
    names = ["Ma", "rhoMError", "UError", "TError", "pError"]
    names += [f"pressureTensor_{c}" for c in ("xx", "xy", "xz", "yy", "yz", "zz")]
    names += [f"shearStressTensor_{c}" for c in ("xx", "xy", "xz", "yy", "yz", "zz")]
    names += [f"heatFluxVector_{c}" for c in "xyz"]
    ma = g.field("Ma")
    assert 9.0 < np.median(ma[ma > 0]) < 11.0
    for f in names:
        a, b = g.field(f), o.field(f)
        scale = max(np.abs(b).max(), 1e-300)
        # the heat flux is a difference of terms ~1e3 times larger than itself
        # (0.5 m |U|^2 u against 0.5 m |U|^2 U at 2883 m/s): the fixed-point
        # moments and the FP64 sums agree to 1e-12 of those terms
        tol = 1e-7 if f.startswith("heatFlux") else 1e-9
        np.testing.assert_allclose(a, b, rtol=tol, atol=tol * scale, err_msg=f)


def test_heat_flux_fields_need_the_case_switch(gpu_lib):
    from hystrath_gb300.dsmc import DsmcCloud, DsmcError
    g = DsmcCloud(S.config0(seed=3))
    g.initialise()
    g.evolve(1)
    with pytest.raises(DsmcError):
        g.field("heatFluxVector_x")


def _two_species_box(seed):
    """Two argon species mixed in every cell, so the sampled keys (cell,
    species) alternate inside a cell."""
    s = S.make_box_case((12, 12, 12), 1e-3, S.AR, fn=2e9, dt=1e-6, seed=seed, n_density=5e19, t_tra=300.0,
                        side_model=S.BC_SPECULAR, side_type=S.PATCH_CYCLIC, collision=S.COLL_VHS)
    s.n_species = 2
    S.set_species(s, 1, dict(S.AR, name="Ar2"))
    s.init_number_density[1] = 5e19
    return s


@pytest.mark.parametrize("case", ["channel", "heatbath", "two_species"])
def test_move_sample_equals_sample_pass(gpu_lib, case):
    """The pending sample taken inside the move (segments of equal keys
    reduced through shared memory) against the same sample taken by the
    stand-alone pass, from identical states: the per-cell sums are exact
    integers, so every sampled field is equal bit for bit.  The channel adds
    inserted parcels (not sampled) and cells of 20 parcels around a solid
    cube, the heat bath cells of 50, the two-species box alternating keys."""
    from hystrath_gb300.dsmc import DsmcCloud
    spec = {"channel": lambda: S.config2(seed=77, scale=8),
            "heatbath": lambda: S.config1(seed=78, n=12),
            "two_species": lambda: _two_species_box(79)}[case]
    a, b = DsmcCloud(spec()), DsmcCloud(spec())
    for g in (a, b):
        g.initialise()
        g.evolve(30)
    a.run_phases(S.PHASE_SAMPLE)
    b.run_phases(S.PHASE_SAMPLE)
    b.run_phases(S.PHASE_INFLOW | S.PHASE_MOVE)
    names = ["rhoN", "rhoM", "Ux", "Uy", "Uz", "Ttra", "Trot", "Tvib", "p"] if case != "two_species" else \
        ["rhoN", "rhoM", "Ux", "Uy", "Uz", "Ttra", "p"]
    for f in names:
        for sp in range(a.spec.n_species):
            fa, fb = a.field(f, sp), b.field(f, sp)
            if f in ("rhoN", "Ttra"):
                assert np.abs(fa).sum() > 0, (case, f)
            np.testing.assert_array_equal(fa, fb, err_msg=f"{case} {f} species {sp}")


def test_captured_step_equals_sequential_step(gpu_lib):
    """The captured step runs the inflow beside the move of the last step's
    parcels and, on meshes of 2^18 cells or more, the heavy cells'
    collisions beside the light cells'; the profiled steps run every kernel
    one after the other.  From the same state, 12 steps each way on the
    Mach-10 channel at 1/2 scale (524288 cells: inflow, obstacle, dense
    cells) give the same parcels bit for bit."""
    from hystrath_gb300.dsmc import DsmcCloud
    a, b = DsmcCloud(S.config2(seed=83, scale=2)), DsmcCloud(S.config2(seed=83, scale=2))
    for g in (a, b):
        g.initialise()
        g.evolve(40)
    a.evolve(12)
    b.evolve_kernel_profile(12)
    ia, ib = a.info(), b.info()
    assert ia.collisions_total == ib.collisions_total and ia.n_particles == ib.n_particles
    assert ia.inserted_last_step > 0
    pa, pb = _canonical(a.particles()), _canonical(b.particles())
    for k in ("id", "cell", "pos", "U", "erot", "vib"):
        np.testing.assert_array_equal(pa[k], pb[k], err_msg=k)
