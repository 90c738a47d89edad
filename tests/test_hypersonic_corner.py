"""The reference's hypersonicCorner tutorial (Ar, VHS, NTC, diffuse walls at
1000 K, symmetry, freestream inflow and deletion) run through
dsmc_create(case_dir) and compared with the time-averaged fields the
reference stored in backup-0.003 (tests/golden/hypersonic_corner_0.003.npz).

The stored fields are one statistical realisation, averaged over 1500 steps
(1.5e-3 .. 3e-3 s); ours are two more (two seeds), each averaged over the
same window in 10 batches of 150 steps.  Two checks:
- statistical: per bin of 3 x 3 x 3 cells, the difference between our mean
  and the reference in units of its standard error, from batch means (the
  reference's realisation has the standard error of one of our runs; the
  batch variance is widened for the lag-1 correlation of consecutive
  batches, or by how far the two seeds' window means differ where that is
  more); at most the fraction of |z| > 2 that Student's t with the
  batches' degrees of freedom gives, plus three of its standard deviations;
- the earlier percent bands: our seeds' RMS deviation from the reference no
  larger than their spread, the mean bias below 0.3%, spanwise-averaged
  x-profiles within 1%."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
CASE = os.path.join(HERE, "golden", "cases", "hypersonic_corner")
FIELDS = ("rhoN", "Ttra", "Ux", "Uy", "Uz", "p", "Ma", "mfp")
BATCHES, PER = 10, 150


def run(seed):
    from hystrath_gb300.dsmc import DsmcCloud, parse_case
    s = parse_case(CASE)
    s.seed = seed
    g = DsmcCloud(s)
    g.initialise()
    g.evolve(1500)            # averaging restarts until 1.5e-3 s
    out = {f: [] for f in FIELDS}
    for _ in range(BATCHES):  # averaged over 1.5e-3 .. 3e-3 s, in batches
        g.reset_sampling()
        g.evolve(PER)
        for f in FIELDS:
            out[f].append(g.field(f))
    g.close()
    return {f: np.array(v) for f, v in out.items()}


def reference():
    gold = np.load(os.path.join(HERE, "golden", "hypersonic_corner_0.003.npz"))
    U = gold["U_Ar"].astype(np.float64)
    return {"rhoN": gold["rhoN_Ar"], "Ttra": gold["Ttra_Ar"], "Ux": U[:, 0], "Uy": U[:, 1], "Uz": U[:, 2],
            "p": gold["p_Ar"], "Ma": gold["Ma_Ar"], "mfp": gold["mfp_Ar"]}


def bins(a):
    """Means over bins of 3 x 3 x 3 cells (the mesh is 30 x 18 x 18)."""
    a = np.asarray(a, dtype=np.float64)
    lead = a.shape[:-1]
    return a.reshape(*lead, 6, 3, 6, 3, 10, 3).mean(axis=(-5, -3, -1)).reshape(*lead, -1)


def lag1(batch_series):
    """Lag-1 correlation of consecutive batch means, pooled over bins and
    runs (each series: batches x bins)."""
    num = den = 0.0
    for b in batch_series:
        d = b - b.mean(0)
        num += float(np.sum(d[1:] * d[:-1]))
        den += float(np.sum(d * d))
    return num / den if den > 0 else 0.0


def run_variance(batches_by_seed):
    """The variance per bin of one run's window mean (BATCHES batches), from
    the batch means, and the factor it was widened by: where consecutive
    batches are not independent by 1 + 2 rho (rho the lag-1 correlation of
    the batch means, pooled over bins and seeds), and by the seeds' own
    disagreement where that is larger: the squared differences of the seeds'
    window means, pooled over bins, against what the batch variance predicts
    for them (slow motions of the shock, longer than a batch, show up there
    and in the reference's one realisation alike)."""
    Bs = [bins(b) for b in batches_by_seed]                    # seeds x (batches, bins)
    S = len(Bs)
    means = np.array([b.mean(0) for b in Bs])                  # (seeds, bins)
    var_b = np.mean([b.var(0, ddof=1) for b in Bs], axis=0)    # pooled within-seed batch variance
    var_run = var_b / BATCHES                                  # one run's window mean, independent batches
    widen = max(1.0, 1.0 + 2.0 * lag1(Bs))
    ok = var_run > 0
    spread = np.sum((means - means.mean(0)) ** 2, axis=0) / (S - 1)
    widen = max(widen, float(np.mean(spread[ok] / var_run[ok])))
    return var_run * widen, widen, means


def z_per_bin(batches_by_seed, ref):
    """(our mean - reference) / standard error per bin, the degrees of
    freedom of the batch variance, and the factor the variance was widened
    by (run_variance)."""
    var_run, widen, means = run_variance(batches_by_seed)
    S = len(batches_by_seed)
    z = (means.mean(0) - bins(ref)) / np.sqrt(var_run / S + var_run)   # ours (S runs) and the reference's one
    dof = S * (BATCHES - 1)
    return z, dof, widen


def t_tail(t, dof):
    from scipy.stats import t as student_t
    return 2.0 * student_t.sf(t, dof)


@pytest.fixture(scope="module")
def gpu_runs(gpu_lib):
    return run(1), run(2)


def test_corner_flow_matches_reference_fields(gpu_runs):
    ref = reference()
    a, b = gpu_runs
    report = {}
    for f in FIELDS:
        z, dof, widen = z_per_bin([a[f], b[f]], ref[f])
        z = z[np.isfinite(z)]
        p2 = float(t_tail(2.0, dof))
        frac = float(np.mean(np.abs(z) > 2.0))
        report[f] = (round(frac, 4), round(p2, 4), round(float(np.mean(z)), 3), round(widen, 2))
        assert frac <= p2 + 3.0 * np.sqrt(p2 * (1 - p2) / z.size), (f, report[f])
    print("fraction of bins with |z| > 2 (ours, expected, mean z, variance widened by):", report)
    for f in ("rhoN", "Ttra", "Ux", "p"):
        r = ref[f].astype(np.float64)
        ma, mb = a[f].mean(0), b[f].mean(0)
        scale = np.abs(r).mean()
        noise = np.sqrt(np.mean((ma - mb) ** 2)) / scale           # sqrt(2) sigma
        mean = 0.5 * (ma + mb)
        dev = np.sqrt(np.mean((mean - r) ** 2)) / scale            # sqrt(3/2) sigma if unbiased
        bias = np.mean(mean - r) / scale
        assert dev < 1.1 * noise, (f, dev, noise)                  # unbiased: dev = 0.87 noise
        assert abs(bias) < 0.003, (f, bias)
        prof = mean.reshape(18, 18, 30).mean(axis=(0, 1))
        rprof = r.reshape(18, 18, 30).mean(axis=(0, 1))
        np.testing.assert_allclose(prof, rprof, rtol=0.01, err_msg=f)


ORACLE_BATCHES = 5


def test_oracle_corner_window_matches_reference_fields(gpu_runs, oracle_mod):
    """The oracle itself against the reference's stored fields.  It continues
    a GPU-developed state at 1.5e-3 s (seed 3: parcels, per-cell selection
    state, inflow remainders and the step that keys the random streams) and
    averages 5 batches of 150 steps, half the reference's window, on the host
    cores: every averaged value comes from the oracle's own moves, collisions
    and samples.  Per bin of 3 x 3 x 3 cells, its window mean minus the
    reference in units of the standard error of that difference, the variance
    of a 150-step batch taken (widened as run_variance does) from the GPU's
    two runs: at most the fraction of |z| > 2 that Student's t gives plus
    three of its standard deviations; x-profiles within 1%."""
    import os
    from hystrath_gb300.dsmc import DsmcCloud, parse_case
    ref = reference()
    s = parse_case(CASE)
    s.seed = 3
    g = DsmcCloud(s)
    g.initialise()
    g.evolve(1500)
    st = g.particles()
    o = oracle_mod.OracleCloud(s, threads=os.cpu_count() or 4)
    o.set_particles(st["pos"], st["U"], st["erot"], st["vib"], st["species"], st["id"])
    for k in ("sigmaTcRMax", "collisionSelectionRemainder", "inflowAccumulator"):
        o.set_cell_array(k, g.cell_array(k))
    o.set_step(g.counts().step)
    g.close()
    del st
    out = {f: [] for f in FIELDS}
    for _ in range(ORACLE_BATCHES):
        o.reset_sampling()
        o.evolve(PER)
        for f in FIELDS:
            out[f].append(o.field(f))
    a, b = gpu_runs
    report = {}
    for f in FIELDS:
        var_run, widen, _ = run_variance([a[f], b[f]])
        var_b = var_run * BATCHES                      # one batch, widened
        mean = bins(np.array(out[f])).mean(0)
        z = (mean - bins(ref[f])) / np.sqrt(var_b / ORACLE_BATCHES + var_b / BATCHES)
        z = z[np.isfinite(z)]
        p2 = float(t_tail(2.0, 2 * (BATCHES - 1)))
        frac = float(np.mean(np.abs(z) > 2.0))
        report[f] = (round(frac, 4), round(p2, 4), round(float(np.mean(z)), 3))
        assert frac <= p2 + 3.0 * np.sqrt(p2 * (1 - p2) / z.size), (f, report[f])
    print("oracle: fraction of bins with |z| > 2 (ours, expected, mean z):", report)
    for f in ("rhoN", "Ttra", "Ux", "p"):
        r = ref[f].astype(np.float64)
        prof = np.array(out[f]).mean(0).reshape(18, 18, 30).mean(axis=(0, 1))
        rprof = r.reshape(18, 18, 30).mean(axis=(0, 1))
        np.testing.assert_allclose(prof, rprof, rtol=0.01, err_msg=f)
