"""The statistics behind the learned-vs-plain report (host logic, no GPU):
the per-cell collision-count test of two independent runs and the field
differences in batch-mean standard errors.  Planted differences are planted
in synthetic counts, on the CPU."""
import numpy as np
import pytest

from hystrath_gb300 import learn


def _counts(seed, n=300_000, shape=2.0, scale=50.0):
    rng = np.random.default_rng(seed)
    return rng, rng.gamma(shape, scale, size=n)


def test_equal_rates_pass_the_per_cell_test():
    rng, mu = _counts(1)
    r = learn.per_cell_count_test(rng.poisson(mu), rng.poisson(mu))
    assert abs(r["z"]) < 4.0
    assert r["p_value_two_sided"] > 1e-4
    assert r["rms_rel_bias_upper95"] < 0.012
    assert abs(r["total_rel_diff"]) < 4 * r["total_rel_diff_se"]


@pytest.mark.parametrize("bias", [0.02, 0.04])
def test_uniform_bias_is_detected_and_sized(bias):
    rng, mu = _counts(2)
    r = learn.per_cell_count_test(rng.poisson(mu), rng.poisson(mu * (1 + bias)))
    assert r["z"] > 5.0
    assert abs(r["rms_rel_bias_estimate"] - bias) < 0.25 * bias
    assert r["rms_rel_bias_upper95"] > bias * 0.9


def test_compensating_per_cell_biases_are_detected():
    """+-3% in alternate cells keeps the total but not the per-cell counts."""
    rng, mu = _counts(3)
    sign = np.where(np.arange(mu.size) % 2 == 0, 1.03, 0.97)
    r = learn.per_cell_count_test(rng.poisson(mu), rng.poisson(mu * sign))
    assert abs(r["total_rel_diff"]) < 0.002
    assert r["z"] > 10.0
    assert abs(r["rms_rel_bias_estimate"] - 0.03) < 0.006


def test_group_biases_are_reported_per_group():
    rng, mu = _counts(4, n=100_000)
    groups = (np.arange(mu.size) % 4).astype(np.int64)
    b = rng.poisson(mu * np.where(groups == 2, 1.05, 1.0))
    r = learn.per_cell_count_test(rng.poisson(mu), b, groups, ["g0", "g1", "g2", "g3"])
    by = {g["group"]: g for g in r["groups"]}
    assert abs(by["g2"]["rel_diff"] - 0.05) < 4 * by["g2"]["se"]
    for k in ("g0", "g1", "g3"):
        assert abs(by[k]["rel_diff"]) < 4 * by[k]["se"]


def test_batch_mean_z_has_the_nominal_tail_and_sees_a_shift():
    rng = np.random.default_rng(5)
    A = [rng.normal(10.0, 1.0, 4000) for _ in range(8)]
    B = [rng.normal(10.0, 1.0, 4000) for _ in range(8)]
    r = learn.batch_mean_z(A, B)
    assert r["blocks"] == 4000
    assert abs(r["frac_abs_z_gt_2"] - r["expected_frac_abs_z_gt_2"]) < 0.02
    assert 0.05 < r["expected_frac_abs_z_gt_2"] < 0.09      # t with ~14 dof, not 4.6%
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
