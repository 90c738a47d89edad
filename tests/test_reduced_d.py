"""Reduced-D (empty) directions (dsmcParcel.C:70-84): along an axis whose
two sides are empty patches a parcel is tracked at the mesh centre with no
velocity, while its velocity keeps all three components for collisions and
walls.  The GPU against the stored fields of the reference's N2/O2 Couette
tutorial (couette_N2-O2/backup-5, LB-VHS, pre-2008 Zv) is in
test_couette.py."""
import os

import numpy as np
import pytest

from hystrath_gb300 import spec as S

HERE = os.path.dirname(os.path.abspath(__file__))
COUETTE = os.path.join(HERE, "golden", "cases", "couette_N2-O2")


def _flat_box(seed, nz=1):
    s = S.make_box_case((6, 6, nz), 1e-3, S.AR, fn=5e9, dt=1e-6, seed=seed, n_density=1e20,
                        t_tra=300.0, side_model=S.BC_SPECULAR)
    s.n_patches = 2
    s.patches[1].name = b"frontAndBack"
    s.patches[1].type = S.PATCH_EMPTY
    s.side_patch[4] = s.side_patch[5] = 1
    return s


def test_couette_case_parses(gpu_lib):
    from hystrath_gb300.dsmc import parse_case
    s = parse_case(COUETTE)
    assert list(s.n_cells) == [5, 100, 1]
    types = {s.patches[p].name: s.patches[p].type for p in range(s.n_patches)}
    assert types[b"frontAndBack"] == S.PATCH_EMPTY and types[b"periodicX_half0"] == S.PATCH_CYCLIC
    assert s.patches[s.side_patch[4]].type == S.PATCH_EMPTY == s.patches[s.side_patch[5]].type
    assert s.n_species == 2 and s.inv_zv_formulation == 0
    assert s.binary_collision_model == S.COLL_LB_VHS


def test_oracle_empty_axis_is_held_at_the_centre(oracle_mod):
    s = _flat_box(3)
    o = oracle_mod.OracleCloud(s, threads=4)
    o.initialise()
    p0 = o.particles()
    assert np.ptp(p0["pos"][:, 2]) > 0          # the mesh fill spreads z
    i0 = o.info()
    for _ in range(20):
        o.evolve(1)
    p1 = o.particles()
    assert np.all(p1["pos"][:, 2] == 0.5e-3)
    # z velocities are kept (and exchanged by collisions)
    assert np.abs(p1["U"][:, 2]).mean() > 100.0
    i1 = o.info()
    assert abs(i1.linear_ke / i0.linear_ke - 1.0) < 1e-12
    assert i1.collisions_total > 100


def test_oracle_empty_axis_matches_the_3d_box_in_x_and_y(oracle_mod):
    """With z untracked, x and y positions after a move are those of the
    same parcels in a box without the empty sides (z lies inside its cell)."""
    s2, s3 = _flat_box(4), _flat_box(4)
    s3.side_patch[4] = s3.side_patch[5] = 0
    a = oracle_mod.OracleCloud(s2, threads=2)
    a.initialise()
    st = a.particles()
    st["U"][:, 2] = 0.0
    b = oracle_mod.OracleCloud(s3, threads=2)
    pos = st["pos"].copy()
    pos[:, 2] = 0.5e-3
    for c in (a, b):
        c.set_particles(pos, st["U"], st["erot"], st["vib"], st["species"], st["id"])
        c.run_phases(S.PHASE_MOVE | S.PHASE_SORT)
    pa, pb = a.particles(), b.particles()
    oa, ob = np.argsort(pa["id"]), np.argsort(pb["id"])
    np.testing.assert_array_equal(pa["pos"][oa], pb["pos"][ob])


@pytest.mark.gpu
def test_gpu_empty_side_validation(gpu_lib):
    from hystrath_gb300.dsmc import DsmcCloud, DsmcError
    with pytest.raises(DsmcError, match="one cell thick"):
        DsmcCloud(_flat_box(1, nz=2))
    s = _flat_box(1)
    s.side_patch[5] = 0
    with pytest.raises(DsmcError, match="empty opposite side"):
        DsmcCloud(s)
    s = _flat_box(1)
    s.patches[1].inflow = 1
    with pytest.raises(DsmcError, match="no inflow"):
        DsmcCloud(s)


@pytest.mark.gpu
def test_gpu_empty_axis_conserves_and_holds_the_centre(gpu_lib):
    from hystrath_gb300.dsmc import DsmcCloud
    s = _flat_box(5)
    g = DsmcCloud(s)
    g.initialise()
    i0 = g.info()
    g.evolve(30)
    p = g.particles()
    assert np.all(p["pos"][:, 2] == 0.5e-3)
    i1 = g.info()
    assert abs(i1.linear_ke / i0.linear_ke - 1.0) < 1e-12
    assert i1.collisions_total > 150
