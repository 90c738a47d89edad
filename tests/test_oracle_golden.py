"""The CPU oracle itself against a stored output of the reference: the
supersonicFlatPlate tutorial (backup-0.04, averages over t = 8e-3..4e-2 s;
Mach ~4 N2 over a diffuse 500 K plate on two graded blocks, one cell thick
in z with empty defaultFaces, free-stream inflow and deletion on four
sides), run by the oracle alone on the host cores from the case directory.

The oracle develops the flow for the reference's 2000 steps before its last
restart of the averages (resetAtOutput until 8e-3 s), restarts them, and
averages the next 4000 steps (half the reference's window: the flow is
steady there, and the shorter window keeps the test to about a minute and a
half on eight cores).  Fields are compared in bins of 10 x 10 cells with the
GPU test's tolerances (a few times the bin noise of one window).  No GPU is
involved: this pins the restatement directly to the reference's numbers."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CASE = os.path.join(HERE, "golden", "cases", "supersonic_flat_plate")
GOLD = os.path.join(HERE, "golden", "supersonic_flat_plate_0.04.npz")


def _bins(a):
    return np.asarray(a, dtype=np.float64).reshape(6, 10, 10, 10).mean(axis=(1, 3))


@pytest.fixture(scope="module")
def oracle_plate(oracle_mod):
    from hystrath_gb300.dsmc import parse_case
    o = oracle_mod.OracleCloud(parse_case(CASE), threads=os.cpu_count() or 4)
    o.initialise()
    o.evolve(2000)
    o.reset_sampling()
    o.evolve(4000)
    return {k: o.field(k) for k in ("rhoN", "Ttra", "Trot", "Ux")}


@pytest.mark.parametrize("name", ["Ttra", "Trot", "rhoN", "Ux"])
def test_oracle_plate_field_bins(oracle_plate, name):
    ref = np.load(GOLD)
    rel = _bins(oracle_plate[name]) / _bins(ref[name]) - 1.0
    assert np.abs(rel).max() < 1.5e-2, rel
    assert abs(rel.mean()) < 3e-3
