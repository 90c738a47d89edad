"""dsmcFaceTracker (faceTracker/dsmcFaceTracker.C:124-190, called from
dsmcParcel.C:106-111 after every face a parcel reaches and from
dsmcCloud.C:425-437 for inserted parcels): per-face parcel and mass fluxes.

Faces carry sign(U . S), S = +axis between two cells and outward on the
boundary; a wall or symmetry interaction is counted once with the velocity
after it, a deletion with the velocity before it, a cyclic crossing +1 on
the face it leaves through and an inserted parcel -1 on its inflow face.
Exact checks: per-cell parcel balance in open boxes, the signed plane count
of a periodic drift, and the GPU against the oracle face by face."""
import os

import numpy as np
import pytest

from hystrath_gb300 import spec as S

HERE = os.path.dirname(os.path.abspath(__file__))
CORNER = os.path.join(HERE, "golden", "cases", "hypersonic_corner")
PLATE = os.path.join(HERE, "golden", "cases", "supersonic_flat_plate")


def _split(F, n):
    nx, ny, nz = n
    fx = F[:(nx + 1) * ny * nz].reshape(nz, ny, nx + 1)
    o = (nx + 1) * ny * nz
    fy = F[o:o + nx * (ny + 1) * nz].reshape(nz, ny + 1, nx)
    o += nx * (ny + 1) * nz
    fz = F[o:].reshape(nz + 1, ny, nx)
    return fx, fy, fz


def _net_in(F, n):
    """Parcels that entered each cell according to the face fluxes (cells in
    x-fastest order); boundary faces are oriented outwards."""
    fx, fy, fz = (f.copy() for f in _split(F, n))
    fx[:, :, 0] *= -1
    fy[:, 0, :] *= -1
    fz[0, :, :] *= -1
    d = (fx[:, :, :-1] - fx[:, :, 1:]) + (fy[:, :-1, :] - fy[:, 1:, :]) + (fz[:-1] - fz[1:])
    return d.reshape(-1)


def _boundary_out(F, n):
    fx, fy, fz = _split(F, n)
    return (fx[:, :, 0].sum() + fx[:, :, -1].sum() + fy[:, 0, :].sum() + fy[:, -1, :].sum() +
            fz[0].sum() + fz[-1].sum())


def _open_box(seed, inflow=False):
    """A drifting argon gas in a box whose six sides delete (and, with
    inflow, also inject the same free stream): every face a parcel crosses is
    either internal or its last."""
    s = S.make_box_case((6, 5, 4), 1e-3, S.AR, fn=2e9, dt=2e-6, seed=seed, n_density=1e20,
                        t_tra=300.0, velocity=(250.0, -120.0, 60.0),
                        side_model=S.BC_DELETION, side_type=S.PATCH_PATCH)
    if inflow:
        p = s.patches[0]
        p.inflow = 1
        p.inflow_number_density[0] = 1e20
        p.inflow_t_tra = 300.0
        for a, u in enumerate((250.0, -120.0, 60.0)):
            p.inflow_velocity[a] = u
    return s


def _counts(cloud, n):
    return np.bincount(cloud.particles()["cell"], minlength=n[0] * n[1] * n[2])


def _balance_run(cloud, n, steps, phases=None):
    c0 = _counts(cloud, n)
    deleted = inserted = 0
    for _ in range(steps):
        if phases is None:
            cloud.evolve(1)
        else:
            cloud.run_phases(phases)
        i = cloud.info()
        deleted += i.deleted_last_step
        inserted += i.inserted_last_step
    c1 = _counts(cloud, n)
    F = cloud.face_flux("parcelIdFlux", 0)
    np.testing.assert_array_equal(c1 - c0, _net_in(F, n))
    assert _boundary_out(F, n) == deleted - inserted
    M = cloud.face_flux("massIdFlux", 0)
    np.testing.assert_allclose(M, F * S.AR["mass"], rtol=1e-12, atol=1e-40)
    return F, deleted, inserted


@pytest.mark.parametrize("inflow", [False, True])
def test_oracle_open_box_balance(oracle_mod, inflow):
    s = _open_box(21 + inflow, inflow)
    n = list(s.n_cells)
    o = oracle_mod.OracleCloud(s, threads=4)
    o.initialise()
    o.set_face_tracking(True)
    phases = S.PHASE_MOVE | S.PHASE_SORT | (S.PHASE_INFLOW if inflow else 0)
    F, deleted, inserted = _balance_run(o, n, 4, phases)
    assert deleted > 100 and (inserted > 100 or not inflow)
    # internal faces see both directions: the drift shows in the sign
    fx, fy, fz = _split(F, n)
    assert fx[:, :, 1:-1].sum() > 0 and fy[:, 1:-1, :].sum() < 0 and fz[1:-1].sum() > 0


def test_oracle_periodic_drift_plane_count(oracle_mod):
    """In a periodic box, internal planes plus (+exits at x=max) minus
    (+exits at x=0) count every parcel's signed number of x-planes crossed."""
    s = S.config0(seed=5, cyclic=True)
    n = list(s.n_cells)
    o = oracle_mod.OracleCloud(s, threads=4)
    o.initialise()
    st = o.particles()
    U = st["U"].copy()
    U[:, 0] += 400.0
    o.set_particles(st["pos"], U, st["erot"], st["vib"], st["species"], st["id"])
    o.set_face_tracking(True)
    o.run_phases(S.PHASE_MOVE | S.PHASE_SORT)
    fx, _, _ = _split(o.face_flux(), n)
    h = s.cell_size[0]
    x0 = st["pos"][:, 0]
    expect = (np.floor((x0 + U[:, 0] * s.delta_t) / h) - np.floor(x0 / h)).sum()
    got = fx[:, :, 1:-1].sum() + fx[:, :, -1].sum() - fx[:, :, 0].sum()
    assert got == expect
    assert fx[:, :, -1].sum() > 0 and fx[:, :, 0].sum() > 0


def test_oracle_walls_count_the_reflected_direction(oracle_mod):
    """A specular box: each wall hit is one -1 on its face (the parcel moves
    inwards after the hit)."""
    s = S.config0(seed=6)
    n = list(s.n_cells)
    o = oracle_mod.OracleCloud(s, threads=4)
    o.initialise()
    o.set_face_tracking(True)
    hits = 0
    for _ in range(3):
        o.run_phases(S.PHASE_MOVE | S.PHASE_SORT)
        hits += o.info().wall_hits_last_step
    F = o.face_flux()
    assert _boundary_out(F, n) == -hits and hits > 0


# ---------------------------------------------------------------- GPU


def _gpu_oracle_pair(spec, oracle_mod):
    from hystrath_gb300.dsmc import DsmcCloud
    g = DsmcCloud(spec)
    g.initialise()
    st = g.particles()
    o = oracle_mod.OracleCloud(spec, threads=4)
    o.set_particles(st["pos"], st["U"], st["erot"], st["vib"], st["species"], st["id"])
    g.set_face_tracking(True)
    o.set_face_tracking(True)
    return g, o


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["specular", "cyclic", "channel_cube", "corner", "graded_plate"])
def test_gpu_face_flux_matches_oracle(gpu_lib, oracle_mod, case):
    """Same parcels, same random streams: every face gets the same count on
    the GPU and in the oracle (walls, symmetry, cyclic, obstacle, inflow,
    deletion, graded cells with an empty axis)."""
    from hystrath_gb300.dsmc import parse_case
    spec = {"specular": lambda: S.config0(seed=31),
            "cyclic": lambda: S.config0(seed=32, cyclic=True),
            "channel_cube": lambda: S.config2(seed=33, scale=8),
            "corner": lambda: parse_case(CORNER),
            "graded_plate": lambda: parse_case(PLATE)}[case]()
    g, o = _gpu_oracle_pair(spec, oracle_mod)
    for _ in range(3):
        g.run_phases(S.PHASE_INFLOW | S.PHASE_MOVE | S.PHASE_SORT)
        o.run_phases(S.PHASE_INFLOW | S.PHASE_MOVE | S.PHASE_SORT)
    for m in range(spec.n_species):
        a, b = g.face_flux("parcelIdFlux", m), o.face_flux("parcelIdFlux", m)
        assert np.abs(b).sum() > 0
        np.testing.assert_array_equal(a, b)
        np.testing.assert_allclose(g.face_flux("massIdFlux", m), o.face_flux("massIdFlux", m),
                                   rtol=1e-12, atol=1e-40)


@pytest.mark.gpu
def test_gpu_open_box_balance_with_collisions(gpu_lib):
    """Whole steps (inflow, move, collisions, sampling): the per-cell parcel
    balance still closes exactly; dsmc_reset_sampling clears the sums."""
    from hystrath_gb300.dsmc import DsmcCloud
    s = _open_box(41, inflow=True)
    n = list(s.n_cells)
    g = DsmcCloud(s)
    g.initialise()
    g.set_face_tracking(True)
    _balance_run(g, n, 6)
    g.reset_sampling()
    assert not g.face_flux().any()


@pytest.mark.gpu
def test_gpu_face_tracking_is_off_by_default(gpu_lib):
    from hystrath_gb300.dsmc import DsmcCloud, DsmcError
    g = DsmcCloud(S.config0(seed=1))
    g.initialise()
    with pytest.raises(DsmcError):
        g.face_flux()
    g.set_face_tracking(True)
    with pytest.raises(DsmcError):
        g.face_flux("momentumFlux")
    g.evolve(2)
    assert g.face_flux().any()
    g.set_face_tracking(False)
    with pytest.raises(DsmcError):
        g.face_flux()
