"""simplifiedBernoulliTrials partner selection
(collisionPartnerSelection/derived/simplifiedBernoulliTrials/
simplifiedBernoulliTrials.C:88-190): every pair of a cell is tried with
probability FN dt / V sigma_T c_R, so the collision rate is the analytic VHS
rate without any maximum; collisions conserve energy and momentum."""
import math

import numpy as np
import pytest

from hystrath_gb300 import spec as S


def _sbt(seed):
    s = S.config0(seed=seed, cyclic=True)
    s.partner_selection_model = S.SEL_SBT
    return s


def _rate_check(cloud, s, warm=300, steps=700):
    from tests.test_oracle import vhs_rate
    i0 = cloud.info()
    N = i0.n_particles
    T = 2.0 * i0.linear_ke / (3.0 * N * s.n_equivalent_particles * S.KB)
    cloud.evolve(warm)
    c0 = cloud.info().collisions_total
    cloud.evolve(steps)
    i1 = cloud.info()
    n = N * s.n_equivalent_particles / 1e-6
    expected = 0.5 * N * vhs_rate(s, T, n) * s.delta_t * steps
    scale = math.sqrt(2 * i0.linear_ke * s.species[0].mass * s.n_equivalent_particles)
    assert np.all(np.abs(np.array(i1.momentum) - np.array(i0.momentum)) < 1e-10 * scale)
    assert abs(i1.linear_ke / i0.linear_ke - 1.0) < 1e-11
    return (i1.collisions_total - c0) / expected


def test_oracle_sbt_rate_matches_analytic(oracle_mod):
    s = _sbt(11)
    o = oracle_mod.OracleCloud(s, threads=4)
    o.initialise()
    assert abs(_rate_check(o, s) - 1.0) < 0.01


@pytest.mark.gpu
def test_gpu_sbt_rate_matches_analytic(gpu_lib):
    from hystrath_gb300.dsmc import DsmcCloud
    ratios = []
    for sd in (12, 13):
        s = _sbt(sd)
        g = DsmcCloud(s)
        g.initialise()
        ratios.append(_rate_check(g, s))
    assert abs(np.mean(ratios) - 1.0) < 0.01, ratios


@pytest.mark.gpu
def test_gpu_sbt_heat_bath_conserves_energy(gpu_lib):
    from hystrath_gb300.dsmc import DsmcCloud
    s = S.config1(seed=3, n=8)
    s.partner_selection_model = S.SEL_SBT
    g = DsmcCloud(s)
    g.initialise()
    i0 = g.info()
    g.evolve(50)
    i1 = g.info()
    e0 = i0.linear_ke + i0.rotational_e + i0.vibrational_e
    e1 = i1.linear_ke + i1.rotational_e + i1.vibrational_e
    assert i1.collisions_total > 1000
    assert abs(e1 / e0 - 1.0) < 1e-10
