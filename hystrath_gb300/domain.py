"""Spatial decomposition of one case over several clouds, and the migrant
exchange between them.

The reference divides the mesh into processor domains, and ``Cloud::move``
(src/lagrangian/basic/Cloud/Cloud.C:255-466) hands a parcel that reaches a
processor patch to the neighbouring processor (a ``PstreamBuffers``
exchange of the parcels per neighbour, after which they finish their move
there); the step's totals are summed over the processors
(noTimeCounter.C:312-314, dsmcCloud.C:938-958).

Here every domain's cloud holds the whole case (its per-cell arrays too) and
owns the parcels of a slab of cells along one axis (``dsmc_set_domain``).  A
parcel's move is completed where it started, so a migrant arrives with its
move done and only joins the receiver's sort; collisions and sampling are
per cell and keyed by the global cell, so the divided case steps exactly as
the undivided one.  A step: every cloud runs ``step_begin`` (inflow, move,
the migrants packed as 68-byte records with their cell words), the migrants
are routed to the owners of their cells, every cloud takes its share with
``add_migrants`` and runs ``step_end`` (sort, collisions, sampling).

``LocalExchange`` steps the domains of one process (a GPU's clouds, or
oracle clouds in tests); ``TorchExchange`` steps one domain per process with
torch.distributed point-to-point messages (NCCL with CUDA tensors, gloo with
CPU ones): the counts per peer, then the records.
"""
from __future__ import annotations

import numpy as np

MIGRANT_BYTES = 68          # the 64-byte parcel record and the cell word
CELL_WORD = slice(64, 68)   # the cell word's bytes in a migrant


def slab_bounds(n_cells: int, parts: int):
    """Boundaries of `parts` slabs of nearly equal width over n_cells cells."""
    if not 1 <= parts <= n_cells:
        raise ValueError(f"cannot divide {n_cells} cells into {parts} slabs")
    return [round(k * n_cells / parts) for k in range(parts + 1)]


def migrant_cells(records: np.ndarray) -> np.ndarray:
    """Linear cell of every migrant (68-byte rows)."""
    w = np.ascontiguousarray(records[:, CELL_WORD]).view(np.uint32).reshape(-1)
    return ((w & np.uint32(0x7FFFFFFF)) >> np.uint32(3)).astype(np.int64)


def cell_index(cells: np.ndarray, axis: int, n_cells) -> np.ndarray:
    """Index along `axis` of linear cells c = i + n0 (j + n1 k)."""
    n0, n1 = int(n_cells[0]), int(n_cells[1])
    if axis == 0:
        return cells % n0
    if axis == 1:
        return (cells // n0) % n1
    return cells // (n0 * n1)


def owners(records: np.ndarray, bounds, axis: int, n_cells) -> np.ndarray:
    """Rank owning each migrant's cell (slab r: bounds[r] <= index < bounds[r + 1])."""
    idx = cell_index(migrant_cells(records), axis, n_cells)
    return np.searchsorted(np.asarray(bounds), idx, side="right") - 1


def divide(clouds, bounds, axis: int):
    """Gives cloud r the slab bounds[r] <= index < bounds[r + 1]."""
    for r, c in enumerate(clouds):
        c.set_domain(axis, bounds[r], bounds[r + 1])


class LocalExchange:
    """Steps the domains of one case held by one process: migrants pass
    through host memory."""

    def __init__(self, clouds, bounds, axis: int, n_cells):
        self.clouds = list(clouds)
        self.bounds = list(bounds)
        self.axis = axis
        self.n_cells = tuple(n_cells)
        self.migrated = 0          # migrants handed over so far

    def step(self, n: int = 1):
        for _ in range(n):
            out = [c.get_migrants(c.step_begin()) for c in self.clouds]
            allm = np.concatenate(out) if out else np.empty((0, MIGRANT_BYTES), np.uint8)
            self.migrated += len(allm)
            dest = owners(allm, self.bounds, self.axis, self.n_cells)
            for r, c in enumerate(self.clouds):
                mine = allm[dest == r]
                if len(mine):
                    c.add_migrants(mine)
            for c in self.clouds:
                c.step_end()


class TorchExchange:
    """Steps this process's domain with torch.distributed: per step the
    migrant counts per peer (all_gather), then the records point to point.
    With device=None the records travel as CPU tensors (gloo); with a CUDA
    device they stay on the GPU (NCCL), and the cloud must take device
    pointers (the GPU library does)."""

    def __init__(self, cloud, bounds, axis: int, n_cells, device=None, group=None):
        import torch.distributed as dist
        self.dist = dist
        self.cloud = cloud
        self.bounds = list(bounds)
        self.axis = axis
        self.n_cells = tuple(n_cells)
        self.device = device
        self.group = group
        self.rank = dist.get_rank(group)
        self.world = dist.get_world_size(group)
        if len(self.bounds) != self.world + 1:
            raise ValueError("one slab per rank")
        self.migrated = 0

    def _route(self, m):
        """This step's migrants, ordered by destination, and the count per rank."""
        import torch
        if self.device is not None:
            buf = torch.empty((m, MIGRANT_BYTES), dtype=torch.uint8, device=self.device)
            if m:
                self.cloud.get_migrants(m, buf.data_ptr())
            torch.cuda.synchronize(self.device)
            host = buf.cpu().numpy()
        else:
            host = self.cloud.get_migrants(m)
            buf = torch.from_numpy(host)
        dest = owners(host, self.bounds, self.axis, self.n_cells)
        if np.any(dest == self.rank) or np.any(dest < 0) or np.any(dest >= self.world):
            raise RuntimeError("a migrant for this domain or for no domain")
        order = np.argsort(dest, kind="stable")
        counts = np.bincount(dest, minlength=self.world).astype(np.int64)
        idx = torch.from_numpy(order)
        if self.device is not None:
            idx = idx.to(self.device)
        return buf[idx] if m else buf, counts

    def step(self, n: int = 1):
        import torch
        dist = self.dist
        for _ in range(n):
            m = self.cloud.step_begin()
            self.migrated += m
            send, counts = self._route(m)
            dev = self.device if self.device is not None else "cpu"
            mine = torch.from_numpy(counts).to(dev)
            table = [torch.zeros_like(mine) for _ in range(self.world)]
            dist.all_gather(table, mine, group=self.group)
            recv_counts = [int(t[self.rank]) for t in table]
            reqs, recv = [], []
            off = np.concatenate([[0], np.cumsum(counts)])
            for peer in range(self.world):
                if peer == self.rank:
                    continue
                if counts[peer]:
                    reqs.append(dist.isend(send[off[peer]:off[peer + 1]].contiguous(), peer, group=self.group))
                if recv_counts[peer]:
                    r = torch.empty((recv_counts[peer], MIGRANT_BYTES), dtype=torch.uint8, device=dev)
                    recv.append(r)
                    reqs.append(dist.irecv(r, peer, group=self.group))
            for q in reqs:
                q.wait()
            if recv:
                got = torch.cat(recv)
                if self.device is not None:
                    torch.cuda.synchronize(self.device)
                    self.cloud.add_migrants(got.data_ptr(), len(got))
                else:
                    self.cloud.add_migrants(got.numpy())
            self.cloud.step_end()

    def totals(self, values):
        """Sums of per-domain values over the ranks (the step's totals, as
        noTimeCounter.C:312-314 reduces the collision counts)."""
        import torch
        t = torch.tensor(np.asarray(values, dtype=np.float64),
                         device=self.device if self.device is not None else "cpu")
        self.dist.all_reduce(t, group=self.group)
        return t.cpu().numpy()
