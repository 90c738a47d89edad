"""The statistics behind the learned-vs-plain report (host logic, no GPU):
the per-cell collision-count test of two independent runs and the field
differences in batch-mean standard errors.  Planted differences are planted
in synthetic counts, on the CPU."""
import numpy as np
import pytest

from hystrath_gb300 import learn


def _batches(rng, mu, k=8, p=0.57):
    """k batches of NTC-like counts per cell: a candidate count that follows
    the mean (the remainder is carried) and Bernoulli acceptances, variance
    about (1 - p) x mean, well below Poisson."""
    cand = np.maximum(np.rint(mu / p), 0).astype(np.int64)
    return np.array([rng.binomial(cand, p) for _ in range(k)], dtype=np.float64)


def _mu(seed, n=300_000):
    rng = np.random.default_rng(seed)
    return rng, rng.gamma(2.0, 8.0, size=n)


def test_equal_rates_pass_the_per_cell_test():
    rng, mu = _mu(1)
    r = learn.per_cell_count_test(_batches(rng, mu), _batches(rng, mu))
    assert abs(r["z"]) < 4.0
    assert r["paired_variance_over_mean"] < 0.6   # under-dispersed, as NTC counts are
    assert r["rms_rel_diff_upper95"] < 0.01
    assert abs(r["total_rel_diff"]) < 4 * r["total_rel_diff_se"]


@pytest.mark.parametrize("bias", [0.02, 0.04])
def test_uniform_bias_is_detected_and_sized(bias):
    rng, mu = _mu(2)
    r = learn.per_cell_count_test(_batches(rng, mu), _batches(rng, mu * (1 + bias)))
    assert r["z"] > 5.0
    assert abs(r["rms_rel_diff_estimate"] - bias) < 0.25 * bias
    assert r["rms_rel_diff_upper95"] > bias * 0.9
    assert abs(r["total_rel_diff"] - bias) < 4 * r["total_rel_diff_se"] + 0.002


def test_compensating_per_cell_biases_are_detected():
    """+-3% in alternate cells keeps the total but not the per-cell counts."""
    rng, mu = _mu(3)
    sign = np.where(np.arange(mu.size) % 2 == 0, 1.03, 0.97)
    r = learn.per_cell_count_test(_batches(rng, mu), _batches(rng, mu * sign))
    assert abs(r["total_rel_diff"]) < 0.003
    assert r["z"] > 5.0
    assert abs(r["rms_rel_diff_estimate"] - 0.03) < 0.008


def test_group_biases_are_reported_per_group():
    rng, mu = _mu(4, n=100_000)
    groups = (np.arange(mu.size) % 4).astype(np.int64)
    b = _batches(rng, mu * np.where(groups == 2, 1.05, 1.0))
    r = learn.per_cell_count_test(_batches(rng, mu), b, groups, ["g0", "g1", "g2", "g3"])
    by = {g["group"]: g for g in r["groups"]}
    assert abs(by["g2"]["rel_diff"] - 0.05) < 4 * by["g2"]["se"] + 0.002
    for k in ("g0", "g1", "g3"):
        assert abs(by[k]["rel_diff"]) < 4 * by[k]["se"] + 0.002


def test_audit_summary_reads_the_shortfall_per_cell():
    x = np.full(1000, 100.0)
    y = np.zeros(1000)
    y[:10] = 5.0             # 10 cells lose 5% of their expected collisions
    y[10:20] = 0.5           # 10 cells lose 0.5%
    x[-5:] = 1.0             # too few expected collisions: left out per cell
    y[-5:] = 1.0
    r = learn.audit_summary(np.stack([x, y], 1))
    assert r["cells"] == 995
    assert abs(r["cells_above_1pct"] - 10 / 995) < 1e-12
    assert abs(r["max"] - 0.05) < 1e-12
    assert abs(r["expected_shortfall_total"] - (50 + 5 + 5) / x.sum()) < 1e-12


def test_batch_mean_z_has_the_nominal_tail_and_sees_a_shift():
    rng = np.random.default_rng(5)
    A = [rng.normal(10.0, 1.0, 4000) for _ in range(8)]
    B = [rng.normal(10.0, 1.0, 4000) for _ in range(8)]
    r = learn.batch_mean_z(A, B)
    assert r["blocks"] == 4000
    assert abs(r["frac_abs_z_gt_2"] - r["expected_frac_abs_z_gt_2"]) < 0.025
    assert 0.06 < r["expected_frac_abs_z_gt_2"] < 0.10      # t with 7 dof, not 4.6%
    C = [x + 2.0 for x in B]                                 # 2 units: ~5.7 standard errors
    r2 = learn.batch_mean_z(A, C)
    assert r2["frac_abs_z_gt_2"] > 0.9


def test_batch_mean_z_skips_constant_blocks():
    rng = np.random.default_rng(6)
    A = [np.concatenate([np.zeros(10), rng.normal(1, 0.1, 90)]) for _ in range(6)]
    B = [np.concatenate([np.zeros(10), rng.normal(1, 0.1, 90)]) for _ in range(6)]
    assert learn.batch_mean_z(A, B)["blocks"] == 90


def test_temperature_groups_leave_solid_cells_out():
    t = np.concatenate([np.zeros(5), np.linspace(100, 1000, 100)])
    g, names = learn.temperature_groups(t, 5)
    assert np.all(g[:5] == -1)
    assert sorted(set(g[5:].tolist())) == [0, 1, 2, 3, 4]
    assert len(names) == 5


def test_a_common_trend_stays_out_of_the_standard_error():
    """Both runs follow the same development (expected counts growing batch
    by batch): the paired test still has unit-scale z and a tight bound."""
    rng, mu = _mu(7)
    trend = np.linspace(0.6, 1.4, 8)[:, None]
    a = np.array([rng.binomial(np.rint(mu * t / 0.57).astype(np.int64), 0.57) for t in trend[:, 0]], float)
    b = np.array([rng.binomial(np.rint(mu * t / 0.57).astype(np.int64), 0.57) for t in trend[:, 0]], float)
    r = learn.per_cell_count_test(a, b)
    assert abs(r["z"]) < 4.0
    assert r["paired_variance_over_mean"] < 0.6
    assert r["rms_rel_diff_upper95"] < 0.012


def _window(rng, mu, ms=100.0):
    nc = _batches(rng, mu)
    return {"steps": 400, "ms": ms, "n_start": 1000, "n_end": 1000, "collisions": int(nc.sum()),
            "candidates": int(1.7 * nc.sum()), "nColls": list(nc), "Ttra": 300.0 + mu,
            "batches": {"rhoN": [rng.normal(1.0, 0.01, 500) for _ in range(8)]}, "blk": 8, "audit": None}


def test_compare_windows_reports_the_plain_control():
    """Learned and control windows from the same distribution: the learned
    comparison and the plain-vs-plain control read alike."""
    rng, mu = _mu(8, n=50_000)
    p, l, r, c = (_window(rng, mu) for _ in range(4))
    res = learn.compare_windows(None, p, l, r, c)
    for key in ("per_cell_counts", "per_cell_counts_control"):
        assert abs(res[key]["z"]) < 4.0, key
    assert res["per_cell_counts_control"]["runs"] == "independent seeds, both plain"
    assert set(res["fields_in_se_control"]) == {"rhoN"}
    assert "per_cell_counts_control" not in learn.compare_windows(None, p, l, r)
