"""The reference's N2/O2 Couette tutorial (run/hyStrath/dsmcFoam+/
couette_N2-O2) against its stored fields (backup-5: averages over
t = 0.5..5 s).  A 1 m channel between diffuse walls at 2000 K (still) and
3000 K (moving at 300 m/s), periodic in x, one cell thick in z with empty
front and back, Larsen-Borgnakke VHS with the pre-2008 variable Zv.

The GPU runs 0.5 s (the reference's transient) and averages the next
1.5 s.  The fields are compared as profiles across the channel, averaged
over the 5 cells of a row and over bins of 10 rows.  Tolerances are the
statistical ones of that sample (a few times the run-to-run spread seen on
the profiles), not of the reference's longer one.  The dsmcMeshFill
rounding is random per cell, so the two runs hold slightly different parcel
totals (47735 here, 47583 in the reference): number densities and the wall
pressure are compared per parcel."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CASE = os.path.join(HERE, "golden", "cases", "couette_N2-O2")
GOLD = os.path.join(HERE, "golden", "couette_N2-O2_5.npz")

pytestmark = pytest.mark.gpu

WARM, SAMPLE = 50_000, 150_000


@pytest.fixture(scope="module")
def couette(gpu_lib):
    from hystrath_gb300.dsmc import DsmcCloud, parse_case
    g = DsmcCloud(parse_case(CASE))
    g.initialise()
    g.evolve(WARM)
    g.reset_sampling()
    g.evolve(SAMPLE)
    prof = {}
    for sp, sel in (("N2", 0), ("O2", 1), ("mixture", None)):
        for f in ("Ttra", "Trot", "Tvib", "rhoN", "Ux"):
            prof[f"{f}_{sp}"] = g.field(f, sel).reshape(100, 5).mean(1)
    walls = {}
    for f in ("wallHeatFlux", "wallShearStress", "p_wall"):
        v = g.wall_field(f)
        # boundary faces: -x (100), +x (100), -y (5: lowerWall), +y (5: upperWall)
        walls[f"{f}_lowerWall"] = v[200:205]
        walls[f"{f}_upperWall"] = v[205:210]
    return prof, walls, g.info().n_particles


def _bins(a):
    return a.reshape(10, 10).mean(1)


@pytest.mark.parametrize("field", ["Ttra", "Trot", "Tvib"])
@pytest.mark.parametrize("sp", ["N2", "O2", "mixture"])
def test_temperature_profiles(couette, field, sp):
    prof, _, _ = couette
    ref = np.load(GOLD)
    a, b = prof[f"{field}_{sp}"], ref[f"{field}_{sp}"]
    rel = _bins(a) / _bins(b) - 1.0
    assert np.abs(rel).max() < 5e-3, rel
    assert abs(np.mean(a / b - 1.0)) < 1.5e-3


def test_velocity_profile(couette):
    prof, _, _ = couette
    ref = np.load(GOLD)
    d = _bins(prof["Ux_mixture"]) - _bins(ref["Ux_mixture"])
    assert np.abs(d).max() < 2.0, d            # m/s, of 15..282 m/s
    assert prof["Ux_mixture"][0] < 20.0 < 275.0 < prof["Ux_mixture"][-1]   # slip at both walls


@pytest.mark.parametrize("sp", ["N2", "O2"])
def test_density_profile_shape(couette, sp):
    prof, _, _ = couette
    ref = np.load(GOLD)
    a = prof[f"rhoN_{sp}"] / prof[f"rhoN_{sp}"].mean()
    b = ref[f"rhoN_{sp}"] / ref[f"rhoN_{sp}"].mean()
    rel = _bins(a) / _bins(b) - 1.0
    assert np.abs(rel).max() < 4e-3, rel


def test_wall_heat_flux_and_shear(couette):
    _, walls, n = couette
    ref = np.load(GOLD)
    for w in ("lowerWall", "upperWall"):
        q, qr = walls[f"wallHeatFlux_{w}"].mean(), ref[f"wallHeatFlux_{w}"].mean()
        assert abs(q / qr - 1.0) < 0.03, (w, q, qr)
        t, tr = walls[f"wallShearStress_{w}"].mean(), ref[f"wallShearStress_{w}"].mean()
        assert abs(t / tr - 1.0) < 0.04, (w, t, tr)


def test_wall_pressure_per_parcel(couette):
    """The surface pressure fD . n per parcel of the run."""
    _, walls, n = couette
    ref = np.load(GOLD)
    n_ref = 5.0 * ref["dsmcNMean_mixture"].sum()     # parcels in the reference run
    for w in ("lowerWall", "upperWall"):
        p, pr = walls[f"p_wall_{w}"].mean(), ref[f"p_{w}"].mean()
        assert abs((p / n) / (pr / n_ref) - 1.0) < 3e-3, (w, p, pr)
