"""Spatial decomposition: the domains of a divided case, stepping with their
migrants handed over between the two halves of every step, reach exactly
the state of the undivided case (parcels bit for bit, collision totals, the
per-cell selection state and fields of every domain's own cells).

The reference moves a parcel that reaches a processor patch to the
neighbouring processor (src/lagrangian/basic/Cloud/Cloud.C:255-466) and sums
the step's totals over the processors (noTimeCounter.C:312-314).  Checked
here: the oracle's restatement divided into slabs along x and z in one
process, two gloo ranks exchanging through torch.distributed
(TorchExchange), and on the GPU the library's divided clouds against the
undivided cloud."""
import os
import socket

import numpy as np
import pytest

from hystrath_gb300 import domain
from hystrath_gb300 import spec as S


def _state(particle_dicts):
    d = {k: np.concatenate([x[k] for x in particle_dicts]) for k in particle_dicts[0]}
    order = np.argsort(d["id"])
    return {k: v[order] for k, v in d.items()}


def _owned_mask(spec, axis, lo, hi):
    n = spec.n_cells
    c = np.arange(n[0] * n[1] * n[2])
    idx = domain.cell_index(c, axis, n)
    return (idx >= lo) & (idx < hi)


def _compare(spec, whole, parts, bounds, axis, fields=("rhoN", "Ttra", "Ux", "Trot")):
    a, b = _state([whole.particles()]), _state([p.particles() for p in parts])
    assert len(a["id"]) == len(b["id"])
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    iw, ip = whole.info(), [p.info() for p in parts]
    assert iw.collisions_total == sum(x.collisions_total for x in ip)
    assert iw.n_particles == sum(x.n_particles for x in ip)
    for r, p in enumerate(parts):
        m = _owned_mask(spec, axis, bounds[r], bounds[r + 1])
        for name in ("sigmaTcRMax", "collisionSelectionRemainder"):
            assert np.array_equal(whole.cell_array(name)[m], p.cell_array(name)[m]), (name, r)
        for f in fields:
            assert np.array_equal(whole.field(f)[m], p.field(f)[m]), (f, r)


# ------------------------------------------------------------------ helpers
def test_slab_bounds_and_owners():
    assert domain.slab_bounds(32, 3) == [0, 11, 21, 32]
    with pytest.raises(ValueError):
        domain.slab_bounds(4, 5)
    n = (8, 4, 2)
    cells = np.array([0, 7, 8, 31, 32, 63], dtype=np.int64)
    assert domain.cell_index(cells, 0, n).tolist() == [0, 7, 0, 7, 0, 7]
    assert domain.cell_index(cells, 1, n).tolist() == [0, 0, 1, 3, 0, 3]
    assert domain.cell_index(cells, 2, n).tolist() == [0, 0, 0, 0, 1, 1]
    rec = np.zeros((len(cells), domain.MIGRANT_BYTES), dtype=np.uint8)
    w = (cells.astype(np.uint32) << np.uint32(3)) | np.uint32(5)
    rec[:, 64:68] = w.view(np.uint8).reshape(-1, 4)
    assert domain.migrant_cells(rec).tolist() == cells.tolist()
    assert domain.owners(rec, [0, 3, 8], 0, n).tolist() == [0, 1, 0, 1, 0, 1]


# ------------------------------------------------------------------ oracle
def _oracle(spec, threads=4):
    from oracle import oracle
    o = oracle.OracleCloud(spec, threads=threads)
    o.initialise()
    return o


@pytest.mark.parametrize("axis,parts", [(0, 3), (2, 2)])
def test_divided_oracle_steps_as_the_undivided_case(axis, parts):
    """The Mach-10 channel at 1/8 scale (inflow, deletion, specular sides,
    the diffuse cube): slabs along x (across the flow) and along z."""
    spec = S.config2(seed=5, scale=8)
    whole = _oracle(spec)
    clouds = [_oracle(spec) for _ in range(parts)]
    bounds = domain.slab_bounds(spec.n_cells[axis], parts)
    domain.divide(clouds, bounds, axis)
    ex = domain.LocalExchange(clouds, bounds, axis, spec.n_cells)
    whole.evolve(15)
    ex.step(15)
    assert ex.migrated > 1000
    _compare(spec, whole, clouds, bounds, axis)


def test_oracle_rejects_a_migrant_for_a_foreign_cell():
    spec = S.config2(seed=6, scale=8)
    a, b = _oracle(spec), _oracle(spec)
    bounds = domain.slab_bounds(spec.n_cells[0], 2)
    domain.divide([a, b], bounds, 0)
    m = a.step_begin()
    recs = a.get_migrants(m)
    assert m > 0
    with pytest.raises(RuntimeError):
        a.add_migrants(recs)          # its own migrants belong to b


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _gloo_rank(rank, world, port, out_dir):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        spec = S.config2(seed=7, scale=8)
        cloud = _oracle(spec, threads=2)
        bounds = domain.slab_bounds(spec.n_cells[0], world)
        cloud.set_domain(0, bounds[rank], bounds[rank + 1])
        ex = domain.TorchExchange(cloud, bounds, 0, spec.n_cells)
        ex.step(12)
        tot = ex.totals([cloud.info().collisions_total, cloud.info().n_particles])
        np.savez(os.path.join(out_dir, f"rank{rank}.npz"), migrated=ex.migrated, totals=tot,
                 **cloud.particles())
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_step_as_the_undivided_case(tmp_path):
    """World size 2 on CPU: each rank an oracle domain, migrants exchanged
    with torch.distributed (gloo); the union equals the undivided run."""
    import torch.multiprocessing as mp
    world = 2
    mp.spawn(_gloo_rank, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    got = [dict(np.load(tmp_path / f"rank{r}.npz")) for r in range(world)]
    spec = S.config2(seed=7, scale=8)
    whole = _oracle(spec)
    whole.evolve(12)
    a = _state([whole.particles()])
    keys = [k for k in a]
    b = _state([{k: g[k] for k in keys} for g in got])
    for k in keys:
        assert np.array_equal(a[k], b[k]), k
    assert sum(int(g["migrated"]) for g in got) > 500
    info = whole.info()
    for g in got:   # every rank holds the summed totals
        assert g["totals"][0] == info.collisions_total and g["totals"][1] == info.n_particles


# ------------------------------------------------------------------ GPU
def _gpu(spec):
    from hystrath_gb300.dsmc import DsmcCloud
    g = DsmcCloud(spec)
    g.initialise()
    return g


@pytest.mark.gpu
@pytest.mark.parametrize("case,axis,parts", [("channel", 0, 3), ("channel", 2, 2), ("heatbath", 0, 4)])
def test_divided_gpu_clouds_step_as_the_undivided_cloud(gpu_lib, case, axis, parts):
    """The library's divided clouds (inflow over every face, migrants from
    the fast path and the boundary path, the deferred end points made when
    packed) reach the undivided cloud's state bit for bit."""
    spec = S.config2(seed=11, scale=4) if case == "channel" else S.config1(seed=12, n=24)
    whole = _gpu(spec)
    clouds = [_gpu(spec) for _ in range(parts)]
    bounds = domain.slab_bounds(spec.n_cells[axis], parts)
    domain.divide(clouds, bounds, axis)
    assert sum(c.info().n_particles for c in clouds) == whole.info().n_particles
    ex = domain.LocalExchange(clouds, bounds, axis, spec.n_cells)
    whole.evolve(20)
    ex.step(20)
    assert ex.migrated > 1000
    try:
        _compare(spec, whole, clouds, bounds, axis)
    finally:
        for c in clouds:
            c.close()
        whole.close()


@pytest.mark.gpu
def test_migrants_through_device_memory(gpu_lib):
    """Migrants read into and handed over from device buffers (the NCCL
    path's pointers) give the same state as through host memory."""
    import torch
    spec = S.config2(seed=13, scale=8)
    whole = _gpu(spec)
    clouds = [_gpu(spec) for _ in range(2)]
    bounds = domain.slab_bounds(spec.n_cells[0], 2)
    domain.divide(clouds, bounds, 0)
    whole.evolve(10)
    for _ in range(10):
        bufs = []
        for c in clouds:
            m = c.step_begin()
            t = torch.empty((m, domain.MIGRANT_BYTES), dtype=torch.uint8, device="cuda")
            if m:
                c.get_migrants(m, t.data_ptr())
            bufs.append(t)
        torch.cuda.synchronize()
        for r, c in enumerate(clouds):
            other = bufs[1 - r]
            if len(other):
                c.add_migrants(other.data_ptr(), len(other))
            c.step_end()
    _compare(spec, whole, clouds, bounds, 0)
    for c in clouds + [whole]:
        c.close()


@pytest.mark.gpu
def test_divided_cloud_refuses_whole_steps_and_foreign_migrants(gpu_lib):
    from hystrath_gb300.dsmc import DsmcError
    spec = S.config2(seed=14, scale=8)
    a, b = _gpu(spec), _gpu(spec)
    bounds = domain.slab_bounds(spec.n_cells[0], 2)
    domain.divide([a, b], bounds, 0)
    with pytest.raises(DsmcError) as e:
        a.evolve(1)
    assert e.value.code == S.ERR_INVALID and "dsmc_step_begin" in str(e.value)
    with pytest.raises(DsmcError):
        a.step_end()                       # no step between its halves
    m = a.step_begin()
    assert m > 0
    recs = a.get_migrants(m)
    a.add_migrants(recs)                   # b's cells: dropped and reported
    with pytest.raises(DsmcError) as e:
        a.step_end()
    assert "outside this domain" in str(e.value)
    a.set_domain(-1)                       # undivided again: whole steps run
    a.evolve(2)
    for c in (a, b):
        c.close()
