"""The reference's supersonicFlatPlate tutorial (Bird 1994, 14.3) against its
stored fields (backup-0.04: averages over t = 8e-3..4e-2 s): Mach ~4 N2 over
a diffuse 500 K plate, on two graded blocks (x: 5 cells shrinking by 0.5 then
95 growing by 2; y: 60 growing by 2), one cell thick in z with blockMesh's
empty defaultFaces, free-stream inflow and deletion on four sides.

The GPU runs the reference's own window: 10000 steps of the case as read,
whose output schedule (writeInterval 4e-4 s, resetAtOutput until 8e-3 s)
restarts the averages inside the library up to step 2000, as dsmcFoam+
does, so the last 8000 steps are sampled.
Fields are compared in bins of 10 x 10 cells and the plate's wall fields in
bins of 19 faces; the tolerances are a few times the bin noise of one such
window."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CASE = os.path.join(HERE, "golden", "cases", "supersonic_flat_plate")
GOLD = os.path.join(HERE, "golden", "supersonic_flat_plate_0.04.npz")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def plate(gpu_lib):
    from hystrath_gb300.dsmc import DsmcCloud, parse_case
    g = DsmcCloud(parse_case(CASE))
    g.initialise()
    g.evolve(10000)
    f = {k: g.field(k) for k in ("rhoN", "Ttra", "Trot", "Ux", "Uy")}
    # boundary faces: -x (60), +x (60), then -y (100): the plate is x >= 50 mm
    w = {k: g.wall_field(k)[125:220] for k in ("wallHeatFlux", "wallShearStress", "p_wall")}
    return f, w


def _bins(a):
    return np.asarray(a, dtype=np.float64).reshape(6, 10, 10, 10).mean(axis=(1, 3))


@pytest.mark.parametrize("name", ["Ttra", "Trot", "rhoN", "Ux"])
def test_field_bins(plate, name):
    f, _ = plate
    ref = np.load(GOLD)
    rel = _bins(f[name]) / _bins(ref[name]) - 1.0
    assert np.abs(rel).max() < 1.5e-2, rel
    assert abs(rel.mean()) < 3e-3


def test_shock_and_boundary_layer_shape(plate):
    """Temperature rises behind the leading edge to ~2.5 x free stream and
    the gas stays at 300 K far above the plate."""
    f, _ = plate
    T = f["Ttra"].reshape(60, 100)
    assert T[0, 8:12].mean() > 750.0 and abs(T[-1].mean() - 300.0) < 5.0


@pytest.mark.parametrize("name, ref_name", [("wallHeatFlux", "wallHeatFlux_plate"),
                                            ("wallShearStress", "wallShearStress_plate"),
                                            ("p_wall", "p_plate")])
def test_plate_wall_fields(plate, name, ref_name):
    _, w = plate
    ref = np.load(GOLD)
    a = w[name].reshape(5, 19).mean(1)
    b = ref[ref_name].reshape(5, 19).mean(1)
    assert np.all(np.abs(a / b - 1.0) < 0.03), (a, b)
