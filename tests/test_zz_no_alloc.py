"""dsmc_cell_starts_noalloc: the occupancy scan for callers that may not
allocate device memory (a host code that hands all of HBM to its own pool, a
plugin that must not grow its footprint).  Its result must equal the starts
that the regular path (which allocates its scan scratch) reports through
dsmc_get_cell_array, on two calls in a row that share the static scratch.
This file sorts last so that a failure here comes after every other test."""
import ctypes

import numpy as np
import pytest

from hystrath_gb300 import spec as S

pytestmark = pytest.mark.gpu


def test_cell_starts_noalloc_matches_allocating_path(gpu_lib):
    import torch
    from hystrath_gb300.dsmc import DsmcCloud

    L = gpu_lib
    L.dsmc_cell_starts_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p, ctypes.c_void_p]
    L.dsmc_cell_starts_noalloc.restype = ctypes.c_int
    L.dsmc_noalloc_last_error.restype = ctypes.c_char_p

    # 24^3 = 13824 cells: four scan tiles, ragged last tile
    g = DsmcCloud(S.config1(seed=77, n=24))
    g.initialise()
    g.evolve(3)
    counts = g.cell_array("count")
    start = g.cell_array("start")
    n = counts.size
    assert n > 3 * 4096

    d_counts = torch.from_numpy(counts).to("cuda")
    for call in range(2):
        d_start = torch.full((n + 1,), -7, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        rc = L.dsmc_cell_starts_noalloc(d_counts.data_ptr(), n, d_start.data_ptr(), None)
        assert rc == 0, L.dsmc_noalloc_last_error()
        torch.cuda.synchronize()
        out = d_start.cpu().numpy()
        np.testing.assert_array_equal(out[:n], start, err_msg=f"call {call}")
        assert out[n] == int(counts.sum())

    # a different, ragged count vector on the same scratch
    rng = np.random.default_rng(5)
    c2 = rng.integers(0, 90, size=5 * 4096 + 17).astype(np.int32)
    d2 = torch.from_numpy(c2).to("cuda")
    s2 = torch.empty(c2.size + 1, dtype=torch.int32, device="cuda")
    assert L.dsmc_cell_starts_noalloc(d2.data_ptr(), c2.size, s2.data_ptr(), None) == 0
    torch.cuda.synchronize()
    ref = np.concatenate([[0], np.cumsum(c2)]).astype(np.int64)
    np.testing.assert_array_equal(s2.cpu().numpy(), ref)

    # sizes beyond the static scratch are rejected, nothing launched
    assert L.dsmc_cell_starts_noalloc(d_counts.data_ptr(), (1 << 24) + 1, d_start.data_ptr(), None) == S.ERR_INVALID
    assert b"16777216" in L.dsmc_noalloc_last_error()
