"""CPU checks of the oracle itself: the Philox known-answer vectors, exact
conservation and the analytic pins the reference's own physics gives
(Bird 1994 eqs. 4.74/1.38 as coded in dsmcVolFields.C:1722-1768, the Bird
eq. 4.22 inflow flux of dsmcFreeStreamInflowPatch.C:131-140)."""
import math

import numpy as np
import pytest

from hystrath_gb300 import spec as S

# Random123 known-answer vectors for philox4x32-10 (counter, key, output).
PHILOX_KAT = [
    ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
    ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
    ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
     [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
]


@pytest.mark.parametrize("ctr,key,out", PHILOX_KAT)
def test_philox_known_answers(oracle_mod, ctr, key, out):
    assert oracle_mod.philox(ctr, key) == out


def test_u01_open_interval(oracle_mod):
    L = oracle_mod.lib()
    assert L.oracle_u01_from(0, 0) == 2.0 ** -53
    assert L.oracle_u01_from(0xFFFFFFFF, 0xFFFFFFFF) == 1.0 - 2.0 ** -53
    assert 0.0 < L.oracle_u01_from(12345, 678) < 1.0


def vhs_rate(spec, T, n):
    """Per-molecule VHS equilibrium collision rate (dsmcVolFields.C:1722-1732)."""
    sp = spec.species[0]
    tref = spec.mfp_tref
    return (2.0 * math.sqrt(math.pi) * sp.diameter ** 2 * n * (T / tref) ** (1.0 - sp.omega) *
            math.sqrt(2.0 * S.KB * tref / (sp.mass / 2.0)))


def test_specular_box_conserves_energy_and_momentum(oracle_mod):
    s = S.config0(seed=3)
    o = oracle_mod.OracleCloud(s, threads=2)
    o.initialise()
    i0 = o.info()
    o.evolve(40)
    i1 = o.info()
    assert i1.n_particles == i0.n_particles
    assert i1.collisions_total > 0
    assert abs(i1.linear_ke / i0.linear_ke - 1.0) < 1e-12
    # collisions conserve momentum; specular walls flip it, so compare magnitude of drift per step
    assert i1.wall_hits_last_step > 0


def test_cyclic_box_conserves_momentum(oracle_mod):
    s = S.config0(seed=4, cyclic=True)
    o = oracle_mod.OracleCloud(s, threads=2)
    o.initialise()
    i0 = o.info()
    o.evolve(30)
    i1 = o.info()
    p0 = np.array(i0.momentum)
    p1 = np.array(i1.momentum)
    scale = math.sqrt(2 * i0.linear_ke * s.species[0].mass * s.n_equivalent_particles)
    assert np.all(np.abs(p1 - p0) < 1e-10 * scale)
    assert abs(i1.linear_ke / i0.linear_ke - 1.0) < 1e-12


def test_oracle_vhs_rate_matches_analytic(oracle_mod):
    """Config-0 gas relaxed to 300 K: collisions per step within 1% of
    0.5 N nu dt with the analytic VHS rate at the equilibrium temperature."""
    s = S.config0(seed=1)
    o = oracle_mod.OracleCloud(s, threads=4)
    o.initialise()
    i = o.info()
    N = i.n_particles
    T = 2.0 * i.linear_ke / (3.0 * N * s.n_equivalent_particles * S.KB)
    o.evolve(300)
    c0 = o.info().collisions_total
    nsteps = 700
    o.evolve(nsteps)
    c1 = o.info().collisions_total
    vol = 1000 * 1e-9
    n = N * s.n_equivalent_particles / vol
    expected = 0.5 * N * vhs_rate(s, T, n) * s.delta_t * nsteps
    assert abs((c1 - c0) / expected - 1.0) < 0.01


def test_oracle_inflow_number_flux(oracle_mod):
    """Parcels entering through a freestream inflow side per step match Bird
    eq. 4.22 (dsmcFreeStreamInflowPatch.C:131-140)."""
    s = S.config2(seed=2, scale=8)
    o = oracle_mod.OracleCloud(s, threads=4)
    o.initialise()
    ins = 0
    nsteps = 60
    for _ in range(nsteps):
        o.run_phases(S.PHASE_ALL)
        ins += o.info().inserted_last_step
    T = 200.0
    m = s.species[0].mass
    cmp_ = math.sqrt(2 * S.KB * T / m)
    sc = S.mach10_speed() / cmp_
    area = (s.n_cells[1] * s.cell_size[1]) * (s.n_cells[2] * s.cell_size[2])
    flux = 1e21 * cmp_ * (math.exp(-sc * sc) + math.sqrt(math.pi) * sc * (1 + math.erf(sc))) / (2 * math.sqrt(math.pi))
    expected = flux * area * s.delta_t * nsteps / s.n_equivalent_particles
    assert abs(ins / expected - 1.0) < 0.02


def test_oracle_lb_equipartition(oracle_mod):
    """Larsen-Borgnakke heat bath relaxes towards Ttra = Trot (equipartition)."""
    s = S.config1(seed=5, n=6)
    o = oracle_mod.OracleCloud(s, threads=4)
    o.initialise()
    o.evolve(1500)
    i = o.info()
    N = i.n_particles
    FN = s.n_equivalent_particles
    Ttr = 2 * i.linear_ke / (3 * N * FN * S.KB)
    Trot = i.rotational_e / (N * FN * S.KB)
    E0 = None
    assert abs(Trot / Ttr - 1.0) < 0.05, (Ttr, Trot)
    del E0


def test_oracle_reset_sampling_restarts_the_averages(oracle_mod):
    """After a restart of the averages the oracle's fields average only the
    steps sampled since: the number density averaged over steps 5..8 (a
    restart after step 4) equals twice the average over steps 1..8 minus the
    average over steps 1..4 of an identical cloud (rhoN is linear in the
    sampled counts)."""
    from hystrath_gb300 import spec as S
    a = oracle_mod.OracleCloud(S.config1(seed=4, n=6), threads=2)
    b = oracle_mod.OracleCloud(S.config1(seed=4, n=6), threads=2)
    for o in (a, b):
        o.initialise()
        o.evolve(4)
    first4 = b.field("rhoN")
    a.reset_sampling()
    assert a.info().sample_steps == 0
    a.evolve(4)
    b.evolve(4)
    assert a.info().sample_steps == 4 and b.info().sample_steps == 8
    last4 = a.field("rhoN")
    assert np.abs(last4).sum() > 0
    np.testing.assert_allclose(last4, 2.0 * b.field("rhoN") - first4, rtol=1e-12, atol=1e-3 * np.abs(last4).max() * 1e-9)
