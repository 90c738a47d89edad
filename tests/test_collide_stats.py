"""Statistical parity of GPU collisions and sampling with the analytic VHS
rate and with the CPU replay (collisions use pow/log/sin/cos, whose last
bits differ between CUDA and libm, so the streams diverge after the first
collisions and only statistics can agree)."""
import math

import numpy as np
import pytest

from hystrath_gb300 import spec as S
from test_oracle import vhs_rate

pytestmark = pytest.mark.gpu


def test_gpu_vhs_rate_matches_analytic(gpu_lib):
    """Config 0 (Ar VHS, relaxes to 300 K): collisions per step within 1% of
    the analytic equilibrium rate."""
    from hystrath_gb300.dsmc import DsmcCloud
    s = S.config0(seed=1)
    g = DsmcCloud(s)
    g.initialise()
    i = g.info()
    N = i.n_particles
    T = 2.0 * i.linear_ke / (3.0 * N * s.n_equivalent_particles * S.KB)
    g.evolve(300)
    c0 = g.info().collisions_total
    nsteps = 3000
    g.evolve(nsteps)
    i1 = g.info()
    c1 = i1.collisions_total
    n = N * s.n_equivalent_particles / (1000 * 1e-9)
    expected = 0.5 * N * vhs_rate(s, T, n) * s.delta_t * nsteps
    assert abs((c1 - c0) / expected - 1.0) < 0.01
    # elastic collisions and specular walls conserve energy exactly up to rounding
    assert abs(i1.linear_ke / i.linear_ke - 1.0) < 1e-11
    # sampled temperature is the equilibrium temperature
    g.reset_sampling()
    g.evolve(200)
    Tf = g.field("Ttra")
    assert abs(Tf.mean() / T - 1.0) < 0.01
    mcr = g.field("measuredCollisionRate")
    acr = g.field("meanCollisionRate")
    # dsmcVolFields counts each collision once (symmFactor TODO at :1751): x2 vs nu
    assert abs(2 * mcr.mean() / acr.mean() - 1.0) < 0.05


def _lb_energies(cloud_factory, seeds, checkpoints):
    out = []
    for sd in seeds:
        c = cloud_factory(sd)
        row = []
        last = 0
        for t in checkpoints:
            c.evolve(t - last)
            last = t
            i = c.info()
            row.append((i.linear_ke, i.rotational_e, i.vibrational_e))
        out.append(row)
    return np.array(out)   # seeds x checkpoints x 3


def test_gpu_lb_relaxation_matches_oracle(gpu_lib, oracle_mod):
    """N2 heat bath (config 1 at 8^3 cells, 16 seeds per side): the
    rotational and vibrational energy fractions of GPU and CPU at 4
    checkpoints of the relaxation from 10^4 K (the translational fraction is
    their complement, so it adds nothing).  In units of the standard error of
    the difference of the seed means, with no absolute slack: at most 2 of
    the 8 values above 2 and none above 3.5, and Hotelling's T^2 over the 8
    (the values are correlated in time) with p above 1e-3."""
    from scipy.stats import f as f_dist
    from hystrath_gb300.dsmc import DsmcCloud

    def gpu(sd):
        g = DsmcCloud(S.config1(seed=100 + sd, n=8))
        g.initialise()
        return g

    def cpu(sd):
        o = oracle_mod.OracleCloud(S.config1(seed=200 + sd, n=8), threads=8)
        o.initialise()
        return o

    checkpoints = [20, 60, 150, 300]
    seeds = range(16)
    eg = _lb_energies(gpu, seeds, checkpoints)
    ec = _lb_energies(cpu, seeds, checkpoints)
    # fractions of each run's total energy: rotational and vibrational
    xg = (eg / eg.sum(axis=2, keepdims=True))[:, :, 1:].reshape(len(seeds), -1)
    xc = (ec / ec.sum(axis=2, keepdims=True))[:, :, 1:].reshape(len(seeds), -1)
    n1, n2, p = len(xg), len(xc), xg.shape[1]
    d = xg.mean(0) - xc.mean(0)
    se = np.sqrt(xg.var(0, ddof=1) / n1 + xc.var(0, ddof=1) / n2)
    z = np.abs(d / se)
    assert np.sum(z > 2.0) <= 2 and z.max() < 3.5, np.round(z, 2)
    # Hotelling's two-sample T^2 with the pooled covariance
    Sp = ((n1 - 1) * np.cov(xg, rowvar=False) + (n2 - 1) * np.cov(xc, rowvar=False)) / (n1 + n2 - 2)
    t2 = (n1 * n2) / (n1 + n2) * d @ np.linalg.solve(Sp, d)
    F = (n1 + n2 - p - 1) / (p * (n1 + n2 - 2)) * t2
    pval = float(f_dist.sf(F, p, n1 + n2 - p - 1))
    assert pval > 1e-3, (pval, np.round(z, 2))
    # energy is conserved by LB collisions in a specular box
    tot = eg.sum(axis=2)
    assert np.all(np.abs(tot / tot[:, :1] - 1.0) < 1e-10)


def test_gpu_checkpoint_resume_is_bit_exact(gpu_lib, tmp_path):
    from hystrath_gb300.dsmc import DsmcCloud
    s = S.config1(seed=7, n=6)
    a = DsmcCloud(s)
    a.initialise()
    a.evolve(10)
    path = str(tmp_path / "ck.bin")
    a.checkpoint(path)
    a.evolve(15)
    pa = a.particles()
    b = DsmcCloud(s)
    b.restore(path)
    b.evolve(15)
    pb = b.particles()
    oa = np.lexsort((pa["id"], pa["cell"]))
    ob = np.lexsort((pb["id"], pb["cell"]))
    for k in ("pos", "U", "erot", "vib", "id", "cell"):
        np.testing.assert_array_equal(pa[k][oa], pb[k][ob])
    np.testing.assert_array_equal(a.field("Ttra"), b.field("Ttra"))


@pytest.mark.gpu
def test_counts_agree_with_info(gpu_lib):
    """dsmc_counts reads the step counters without the energy pass."""
    from hystrath_gb300 import spec as S
    from hystrath_gb300.dsmc import DsmcCloud
    g = DsmcCloud(S.config0(seed=9))
    g.initialise()
    g.evolve(3)
    c, i = g.counts(), g.info()
    assert (c.n_particles, c.step, c.collisions_total, c.candidates_total) == \
        (i.n_particles, i.step, i.collisions_total, i.candidates_total)
    assert c.collisions_last_step == i.collisions_last_step > 0


@pytest.mark.gpu
def test_evolve_counts_equal_step_by_step_counts(gpu_lib):
    """dsmc_evolve_counts returns, for every step, the counters that
    dsmc_evolve(1) followed by dsmc_counts gives on the same case."""
    from hystrath_gb300 import spec as S
    from hystrath_gb300.dsmc import DsmcCloud
    a, b = DsmcCloud(S.config0(seed=10)), DsmcCloud(S.config0(seed=10))
    a.initialise()
    b.initialise()
    got = a.evolve_counts(7)
    want = []
    for _ in range(7):
        b.evolve(1)
        want.append(b.counts())
    key = lambda c: (c.n_particles, c.step, c.collisions_last_step, c.candidates_last_step,
                     c.collisions_total, c.candidates_total)
    assert [key(c) for c in got] == [key(c) for c in want]
    assert [c.step for c in got] == list(range(got[0].step, got[0].step + 7))
    assert a.evolve_counts(0) == []
