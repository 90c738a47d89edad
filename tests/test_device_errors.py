"""The device error word, driven without a fault: loop caps, the ordered-cell
limit and the inflow capacity lowered by dsmc_set_limits make a kernel
record the condition and return; the next call reports DSMC_ERR_DEVICE or
DSMC_ERR_CAPACITY with a message, the bits are cleared once reported, and the
handle steps on with the default limits.

The reference aborts in these places (FatalError, e.g.
BinaryCollisionModel.C:72-83; the unbounded acceptance-rejection loops of
dsmcCloud.C:1354-1383 and dsmcFreeStreamInflowPatch.C:288-305)."""
import pytest

from hystrath_gb300 import spec as S


def test_limits_entry_point_is_exported(gpu_lib):
    assert hasattr(gpu_lib, "dsmc_set_limits")


def _cloud(spec, steps=0):
    from hystrath_gb300.dsmc import DsmcCloud
    g = DsmcCloud(spec)
    g.initialise()
    if steps:
        g.evolve(steps)
    return g


def _expect(g, code, words, steps=1):
    from hystrath_gb300.dsmc import DsmcError
    with pytest.raises(DsmcError) as e:
        g.evolve(steps)
    assert e.value.code == code, (e.value.code, str(e.value))
    for w in words:
        assert w in str(e.value), str(e.value)


def _steps_on(g, steps=3):
    g.set_limits()
    n0 = g.counts().step
    g.evolve(steps)           # raises if an error bit were still set
    assert g.counts().step == n0 + steps
    assert g.info().n_particles > 0


@pytest.mark.gpu
def test_rejection_cap_is_reported(gpu_lib):
    """One draw allowed in the acceptance-rejection samplers: the inflow's
    normal-speed sampler (and the vibrational level draws) run out."""
    g = _cloud(S.config2(seed=51, scale=8), 2)
    g.set_limits(max_rejection=1)
    _expect(g, S.ERR_DEVICE, ["acceptance-rejection cap"])
    _steps_on(g)


@pytest.mark.gpu
def test_crossing_cap_is_reported(gpu_lib):
    """One face crossing per move: every parcel that meets a wall needs two."""
    g = _cloud(S.config0(seed=52))
    g.set_limits(max_crossings=1)
    _expect(g, S.ERR_DEVICE, ["face-crossing cap"])
    _steps_on(g)


@pytest.mark.gpu
def test_dense_cell_limit_is_reported_and_skips_collisions(gpu_lib):
    """Cells above the ordered-cell limit skip their collisions and say so."""
    g = _cloud(S.config1(seed=53, n=8), 1)
    g.set_limits(max_cell_parcels=8)
    _expect(g, S.ERR_DEVICE, ["a cell above"])
    assert g.counts().collisions_last_step == 0
    _steps_on(g)
    assert g.counts().collisions_last_step > 0


@pytest.mark.gpu
def test_inflow_capacity_overflow_is_reported(gpu_lib):
    """An inflow that would fill more than the capacity inserts nothing and
    returns DSMC_ERR_CAPACITY."""
    g = _cloud(S.config2(seed=54, scale=8), 2)
    n = g.counts().n_particles
    g.set_limits(capacity=n + 10)
    _expect(g, S.ERR_CAPACITY, ["capacity exceeded"])
    assert g.info().inserted_last_step == 0
    _steps_on(g)
    assert g.info().inserted_last_step > 10


@pytest.mark.gpu
def test_raising_a_limit_is_rejected(gpu_lib):
    from hystrath_gb300.dsmc import DsmcError
    g = _cloud(S.config0(seed=55))
    with pytest.raises(DsmcError) as e:
        g.set_limits(max_crossings=65)
    assert e.value.code == S.ERR_INVALID
    with pytest.raises(DsmcError):
        g.set_limits(max_rejection=-1)
    g.evolve(2)
