"""VariableSoftSphere and LarsenBorgnakkeVariableSoftSphere
(collisions/derived/VariableSoftSphere/VariableSoftSphere.C:80-233,
LarsenBorgnakkeVariableSoftSphere.C:111-148): conservation, the collision
rate of the shared cross-section, the smaller momentum transfer of
forward-peaked scattering (oracle, CPU), and GPU against the oracle."""
import math

import numpy as np
import pytest

from hystrath_gb300 import spec as S


def _vss(seed, alpha, cyclic=True, model=S.COLL_VSS):
    s = S.config0(seed=seed, cyclic=cyclic)
    s.binary_collision_model = model
    s.species[0].alpha = alpha
    return s


def test_oracle_vss_conserves_and_keeps_the_vhs_rate(oracle_mod):
    s = _vss(3, 1.4)
    o = oracle_mod.OracleCloud(s, threads=4)
    o.initialise()
    i0 = o.info()
    N = i0.n_particles
    T = 2.0 * i0.linear_ke / (3.0 * N * s.n_equivalent_particles * S.KB)
    o.evolve(300)
    c0 = o.info().collisions_total
    o.evolve(700)
    i1 = o.info()
    scale = math.sqrt(2 * i0.linear_ke * s.species[0].mass * s.n_equivalent_particles)
    assert np.all(np.abs(np.array(i1.momentum) - np.array(i0.momentum)) < 1e-10 * scale)
    assert abs(i1.linear_ke / i0.linear_ke - 1.0) < 1e-12
    from tests.test_oracle import vhs_rate
    n = N * s.n_equivalent_particles / 1e-6
    expected = 0.5 * N * vhs_rate(s, T, n) * s.delta_t * 700
    assert abs((i1.collisions_total - c0) / expected - 1.0) < 0.015


def test_oracle_lb_vss_conserves_energy(oracle_mod):
    s = S.config1(seed=2, n=6)
    s.binary_collision_model = S.COLL_LB_VSS
    o = oracle_mod.OracleCloud(s, threads=4)
    o.initialise()
    i0 = o.info()
    o.evolve(200)
    i1 = o.info()
    e0 = i0.linear_ke + i0.rotational_e + i0.vibrational_e
    e1 = i1.linear_ke + i1.rotational_e + i1.vibrational_e
    assert i1.collisions_total > 10000
    assert abs(e1 / e0 - 1.0) < 1e-10


def _two_species(seed, alpha, model):
    """Two identical argon species in a periodic box, half the density each."""
    s = S.make_box_case((10, 10, 10), 1e-3, S.AR, fn=5e9, dt=1e-6, seed=seed, n_density=5e19, t_tra=300.0,
                        side_model=S.BC_SPECULAR, side_type=S.PATCH_CYCLIC, collision=model)
    s.n_species = 2
    S.set_species(s, 1, dict(S.AR, name="Ar2"))
    s.init_number_density[1] = 5e19
    s.species[0].alpha = alpha
    s.species[1].alpha = alpha
    return s


def _drift_decay(cloud, steps, du=100.0):
    """log of the relative x drift of the two species after steps, starting
    from +du / -du."""
    st = cloud.particles()
    U = st["U"].copy()
    sp = st["species"]
    U[sp == 0, 0] += du
    U[sp == 1, 0] -= du
    cloud.set_particles(st["pos"], U, st["erot"], st["vib"], sp, st["id"])
    d0 = U[sp == 0, 0].mean() - U[sp == 1, 0].mean()
    out = []
    done = 0
    for s in steps:
        cloud.evolve(s - done)
        done = s
        st = cloud.particles()
        U, sp = st["U"], st["species"]
        out.append(math.log((U[sp == 0, 0].mean() - U[sp == 1, 0].mean()) / d0))
    return out


def test_oracle_forward_scattering_transfers_less_momentum(oracle_mod):
    """The relative drift of two species decays with the diffusion
    cross-section: VSS deflection cos(chi) = 2 U^(1/alpha) - 1 gives
    1 - <cos chi> = 2 / (alpha + 1), so alpha = 2 decays at 2/3 of the
    isotropic (VHS) rate."""
    decay = {}
    for alpha, model in ((1.0, S.COLL_VHS), (2.0, S.COLL_VSS)):
        vals = []
        for sd in range(3):
            o = oracle_mod.OracleCloud(_two_species(70 + sd, alpha, model), threads=4)
            o.initialise()
            vals.append(_drift_decay(o, [30])[0])
        decay[alpha] = np.mean(vals)
    ratio = decay[2.0] / decay[1.0]
    assert 0.58 < ratio < 0.78, (decay, ratio)


@pytest.mark.gpu
def test_gpu_vss_momentum_exchange_matches_oracle(gpu_lib, oracle_mod):
    from hystrath_gb300.dsmc import DsmcCloud
    steps = [10, 30]

    def runs(make, seeds):
        out = []
        for sd in seeds:
            c = make(sd)
            c.initialise()
            out.append(_drift_decay(c, steps))
        return np.array(out)

    hg = runs(lambda sd: DsmcCloud(_two_species(500 + sd, 1.5, S.COLL_VSS)), range(6))
    hc = runs(lambda sd: oracle_mod.OracleCloud(_two_species(600 + sd, 1.5, S.COLL_VSS), threads=4), range(6))
    se = np.sqrt(hg.var(0, ddof=1) / 6 + hc.var(0, ddof=1) / 6)
    assert np.all(np.abs(hg.mean(0) - hc.mean(0)) <= 2.5 * se + 5e-3), (hg.mean(0), hc.mean(0), se)


@pytest.mark.gpu
def test_gpu_lb_vss_conserves_energy(gpu_lib):
    from hystrath_gb300.dsmc import DsmcCloud
    s = S.config1(seed=8, n=8)
    s.binary_collision_model = S.COLL_LB_VSS
    g = DsmcCloud(s)
    g.initialise()
    i0 = g.info()
    g.evolve(100)
    i1 = g.info()
    e0 = i0.linear_ke + i0.rotational_e + i0.vibrational_e
    e1 = i1.linear_ke + i1.rotational_e + i1.vibrational_e
    assert i1.collisions_total > 10000
    assert abs(e1 / e0 - 1.0) < 1e-10
