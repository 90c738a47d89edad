"""Rectilinear graded meshes (blockMesh simpleGrading): cells are found in a
table of the node and cell-midpoint coordinates of each graded axis, and
cell volumes and boundary-face areas vary cell by cell in the mesh fill,
the collision selection, the inflow, the wall fluxes and the fields.  The
GPU against the reference's supersonicFlatPlate fields is in
test_flat_plate.py; the bit-exact move and sort in test_parity_move_sort.py."""
import ctypes as C

import numpy as np
import pytest

from hystrath_gb300 import spec as S


def _graded_box(seed, collision=S.COLL_VHS, side_model=S.BC_SPECULAR, side_type=S.PATCH_WALL, fn=2e9):
    """8 x 6 x 4 argon cells whose x widths grow by 1.25 per cell and whose
    y widths shrink by 0.8; z uniform."""
    s = S.make_box_case((8, 6, 4), 1e-3, S.AR, fn=fn, dt=1e-7, seed=seed, n_density=1e20, t_tra=300.0,
                        side_model=side_model, side_type=side_type, collision=collision)
    x = np.concatenate([[0.0], np.cumsum(0.6e-3 * 1.25 ** np.arange(8))])
    y = np.concatenate([[0.0], np.cumsum(1.4e-3 * 0.8 ** np.arange(6))])
    s._keep = (np.ascontiguousarray(x), np.ascontiguousarray(y))
    s.node_coords[0] = s._keep[0].ctypes.data_as(C.POINTER(C.c_double))
    s.node_coords[1] = s._keep[1].ctypes.data_as(C.POINTER(C.c_double))
    return s, x, y


def _volumes(x, y, dz, nz):
    v = np.outer(np.diff(y), np.diff(x))          # [j, i]
    return np.broadcast_to(v * dz, (nz,) + v.shape).reshape(-1)


def test_oracle_mesh_fill_follows_cell_volume(oracle_mod):
    s, x, y = _graded_box(1)
    o = oracle_mod.OracleCloud(s, threads=4)
    o.initialise()
    p = o.particles()
    V = _volumes(x, y, 1e-3, 4)
    expect = 1e20 * V / 2e9
    cnt = np.bincount(p["cell"], minlength=V.size)
    # 12 tets per cell, each rounded at random: variance below the mean
    z = (cnt - expect) / np.sqrt(expect)
    assert abs(cnt.sum() / expect.sum() - 1.0) < 0.01
    assert np.abs(z).max() < 5 and z.var() < 1.0
    # every parcel lies in the cell it is filed under
    i = np.searchsorted(x, p["pos"][:, 0], side="right") - 1
    j = np.searchsorted(y, p["pos"][:, 1], side="right") - 1
    k = np.floor(p["pos"][:, 2] / 1e-3).astype(int)
    np.testing.assert_array_equal(p["cell"], i + 8 * (j + 6 * k))


def test_oracle_graded_box_keeps_a_uniform_gas(oracle_mod):
    """Collisions in cells of different volumes keep the gas uniform: the
    sampled density per unit volume shows no trend with the cell volume and
    the collision rate per parcel is the analytic VHS one in every cell."""
    s, x, y = _graded_box(2, fn=5e8)
    o = oracle_mod.OracleCloud(s, threads=8)
    o.initialise()
    i0 = o.info()
    o.evolve(300)
    i1 = o.info()
    assert abs(i1.linear_ke / i0.linear_ke - 1.0) < 1e-12
    rho = o.field("rhoN")
    V = _volumes(x, y, 1e-3, 4)
    small, large = V < np.quantile(V, 0.25), V > np.quantile(V, 0.75)
    assert abs(rho[small].mean() / rho[large].mean() - 1.0) < 0.03
    assert abs(rho.mean() / 1e20 - 1.0) < 0.02
    from tests.test_oracle import vhs_rate
    T = 2.0 * i1.linear_ke / (3.0 * i1.n_particles * s.n_equivalent_particles * S.KB)
    mcr = o.field("measuredCollisionRate")
    expect = 0.5 * vhs_rate(s, T, 1e20)          # collisions per parcel: half the collision frequency
    ratio = np.array([mcr[small].mean(), mcr[large].mean()]) / expect
    assert np.all(np.abs(ratio - 1.0) < 0.05), ratio


def test_oracle_graded_open_box_face_balance(oracle_mod):
    """Face fluxes on the graded grid close the per-cell parcel balance
    (the crossing planes come from the node table)."""
    from tests.test_face_tracker import _net_in, _boundary_out
    s, x, y = _graded_box(3, side_model=S.BC_DELETION, side_type=S.PATCH_PATCH)
    s.init_velocity[0] = 300.0
    s.init_velocity[1] = -200.0
    s.delta_t = 2e-6
    n = list(s.n_cells)
    o = oracle_mod.OracleCloud(s, threads=4)
    o.initialise()
    o.set_face_tracking(True)
    c0 = np.bincount(o.particles()["cell"], minlength=8 * 6 * 4)
    deleted = 0
    for _ in range(3):
        o.run_phases(S.PHASE_MOVE | S.PHASE_SORT)
        deleted += o.info().deleted_last_step
    c1 = np.bincount(o.particles()["cell"], minlength=8 * 6 * 4)
    F = o.face_flux()
    np.testing.assert_array_equal(c1 - c0, _net_in(F, n))
    assert _boundary_out(F, n) == deleted > 0


@pytest.mark.gpu
def test_gpu_graded_box_matches_the_oracle_statistically(gpu_lib, oracle_mod):
    from hystrath_gb300.dsmc import DsmcCloud
    s, x, y = _graded_box(4, fn=5e8)
    g = DsmcCloud(s)
    g.initialise()
    i0 = g.info()
    g.evolve(300)
    i1 = g.info()
    assert abs(i1.linear_ke / i0.linear_ke - 1.0) < 1e-12
    V = _volumes(x, y, 1e-3, 4)
    small, large = V < np.quantile(V, 0.25), V > np.quantile(V, 0.75)
    rho = g.field("rhoN")
    assert abs(rho[small].mean() / rho[large].mean() - 1.0) < 0.03
    from tests.test_oracle import vhs_rate
    T = 2.0 * i1.linear_ke / (3.0 * i1.n_particles * s.n_equivalent_particles * S.KB)
    mcr = g.field("measuredCollisionRate")
    ratio = np.array([mcr[small].mean(), mcr[large].mean()]) / (0.5 * vhs_rate(s, T, 1e20))
    assert np.all(np.abs(ratio - 1.0) < 0.05), ratio
