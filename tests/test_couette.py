"""The reference's N2/O2 Couette tutorial (run/hyStrath/dsmcFoam+/
couette_N2-O2) against its stored fields (backup-5: averages over
t = 1..5 s: resetAtOutput restarts the averages at the first output time,
t = 1 s, the first whose t + deltaT passes resetAtOutputUntilTime = 0.5 s).  A 1 m channel between diffuse walls at 2000 K (still) and
3000 K (moving at 300 m/s), periodic in x, one cell thick in z with empty
front and back, Larsen-Borgnakke VHS with the pre-2008 variable Zv.

The GPU runs 0.5 s (the reference's transient) and averages the next
1.5 s in 10 batches of 0.15 s.  The fields are compared as profiles across
the channel, averaged over the 5 cells of a row and over bins of 10 rows,
two ways: in units of the standard error of the difference (batch means give
ours; the reference's 4 s average has 3/8 of our variance), with at
most the fraction of |z| > 2 that Student's t gives plus three of its
standard deviations; and within percent bands (a few times the run-to-run
spread seen on the profiles).  The dsmcMeshFill rounding is random per cell,
so the two runs hold slightly different parcel totals (47735 here, 47583 in
the reference): number densities and the wall pressure are compared per
parcel (number densities as profiles normalised by their mean)."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CASE = os.path.join(HERE, "golden", "cases", "couette_N2-O2")
GOLD = os.path.join(HERE, "golden", "couette_N2-O2_5.npz")

pytestmark = pytest.mark.gpu

WARM, SAMPLE, BATCHES = 50_000, 150_000, 10
REF_WINDOW = 400_000          # steps of the reference's average (1 .. 5 s)
FIELDS = ("Ttra", "Trot", "Tvib", "rhoN", "Ux")


@pytest.fixture(scope="module")
def couette(gpu_lib):
    from hystrath_gb300.dsmc import DsmcCloud, parse_case
    s = parse_case(CASE)
    s.reset_at_output = 0          # the batches below restart the averages themselves
    g = DsmcCloud(s)
    g.initialise()
    g.evolve(WARM)
    batches = {}
    wall_b = {}
    for _ in range(BATCHES):
        g.reset_sampling()
        g.evolve(SAMPLE // BATCHES)
        for sp, sel in (("N2", 0), ("O2", 1), ("mixture", None)):
            for f in FIELDS:
                batches.setdefault(f"{f}_{sp}", []).append(g.field(f, sel).reshape(100, 5).mean(1))
        for f in ("wallHeatFlux", "wallShearStress", "p_wall"):
            wall_b.setdefault(f, []).append(g.wall_field(f))
    batches = {k: np.array(v) for k, v in batches.items()}
    # equal batches: the mean of the batch means is the average over the window
    prof = {k: v.mean(0) for k, v in batches.items()}
    walls = {}
    for f, v in wall_b.items():
        v = np.mean(v, axis=0)
        # boundary faces: -x (100), +x (100), -y (5: lowerWall), +y (5: upperWall)
        walls[f"{f}_lowerWall"] = v[200:205]
        walls[f"{f}_upperWall"] = v[205:210]
    return prof, walls, g.info().n_particles, batches


def _bins(a):
    return a.reshape(10, 10).mean(1)


@pytest.mark.parametrize("field", ["Ttra", "Trot", "Tvib"])
@pytest.mark.parametrize("sp", ["N2", "O2", "mixture"])
def test_temperature_profiles(couette, field, sp):
    prof, _, _, _ = couette
    ref = np.load(GOLD)
    a, b = prof[f"{field}_{sp}"], ref[f"{field}_{sp}"]
    rel = _bins(a) / _bins(b) - 1.0
    assert np.abs(rel).max() < 5e-3, rel
    assert abs(np.mean(a / b - 1.0)) < 1.5e-3


def test_velocity_profile(couette):
    prof, _, _, _ = couette
    ref = np.load(GOLD)
    d = _bins(prof["Ux_mixture"]) - _bins(ref["Ux_mixture"])
    assert np.abs(d).max() < 2.0, d            # m/s, of 15..282 m/s
    assert prof["Ux_mixture"][0] < 20.0 < 275.0 < prof["Ux_mixture"][-1]   # slip at both walls


@pytest.mark.parametrize("sp", ["N2", "O2"])
def test_density_profile_shape(couette, sp):
    prof, _, _, _ = couette
    ref = np.load(GOLD)
    a = prof[f"rhoN_{sp}"] / prof[f"rhoN_{sp}"].mean()
    b = ref[f"rhoN_{sp}"] / ref[f"rhoN_{sp}"].mean()
    rel = _bins(a) / _bins(b) - 1.0
    assert np.abs(rel).max() < 4e-3, rel


def test_wall_heat_flux_and_shear(couette):
    _, walls, n, _ = couette
    ref = np.load(GOLD)
    for w in ("lowerWall", "upperWall"):
        q, qr = walls[f"wallHeatFlux_{w}"].mean(), ref[f"wallHeatFlux_{w}"].mean()
        assert abs(q / qr - 1.0) < 0.03, (w, q, qr)
        t, tr = walls[f"wallShearStress_{w}"].mean(), ref[f"wallShearStress_{w}"].mean()
        assert abs(t / tr - 1.0) < 0.04, (w, t, tr)


def test_wall_pressure_per_parcel(couette):
    """The surface pressure fD . n per parcel of the run."""
    _, walls, n, _ = couette
    ref = np.load(GOLD)
    n_ref = 5.0 * ref["dsmcNMean_mixture"].sum()     # parcels in the reference run
    for w in ("lowerWall", "upperWall"):
        p, pr = walls[f"p_wall_{w}"].mean(), ref[f"p_{w}"].mean()
        assert abs((p / n) / (pr / n_ref) - 1.0) < 3e-3, (w, p, pr)


def test_profiles_within_their_standard_errors(couette):
    """Every species' Ttra, Trot, Tvib, Ux and normalised rhoN profile, per
    bin of 10 rows: |ours - reference| / SE."""
    from scipy.stats import t as student_t
    _, _, _, batches = couette
    ref = np.load(GOLD)
    zs, report = [], {}
    for sp in ("N2", "O2", "mixture"):
        for f in FIELDS:
            key = f"{f}_{sp}"
            b = np.array([_bins(x) for x in batches[key]])          # (batches, bins)
            r = _bins(ref[key].astype(np.float64))
            if f == "rhoN":
                b = b / b.mean(1, keepdims=True)
                r = r / r.mean()
            # widened for the lag-1 correlation of consecutive batch means
            d = b - b.mean(0)
            rho = float(np.sum(d[1:] * d[:-1]) / max(np.sum(d * d), 1e-300))
            var = b.var(0, ddof=1) * max(1.0, 1.0 + 2.0 * rho)
            se = np.sqrt(var / BATCHES + var * (SAMPLE // BATCHES) / REF_WINDOW)
            z = (b.mean(0) - r) / se
            report[key] = round(float(np.mean(np.abs(z))), 2)
            zs.append(z)
    z = np.concatenate(zs)
    p2 = float(2.0 * student_t.sf(2.0, BATCHES - 1))
    frac = float(np.mean(np.abs(z) > 2.0))
    print("mean |z| per profile:", report, "fraction |z| > 2:", frac, "expected:", p2)
    assert frac <= p2 + 3.0 * np.sqrt(p2 * (1 - p2) / z.size), (frac, p2, report)
