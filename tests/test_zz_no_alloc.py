"""pg_cell_order_static, the allocation-free cell ordering, against
pg_cell_order (which allocates its scratch with cudaMallocAsync).

Some callers cannot let the library allocate device memory (their own pool
owns the device, or an allocation's device synchronisation would stall their
other streams); this entry point serves them from a static device array.
The comparison is exact (integer keys and indices), on two calls in a row so
that the second call runs on scratch the first one left behind.  This file is
collected last so that a run stopping at the first failure has already run
every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LIMIT = 65536


def run(lib, fn, c, org, cell, dim):
    import torch
    n = len(c)
    dc = torch.tensor(np.ascontiguousarray(c.T), dtype=torch.float64, device="cuda")
    keys = torch.full((max(n, 1),), -1, dtype=torch.int32, device="cuda")
    order = torch.full((max(n, 1),), -1, dtype=torch.int32, device="cuda")
    o = (ctypes.c_double * 3)(*org)
    dm = (ctypes.c_int * 3)(*dim)
    st = getattr(lib, fn)(ctypes.c_void_p(dc[0].data_ptr()), ctypes.c_void_p(dc[1].data_ptr()),
                          ctypes.c_void_p(dc[2].data_ptr()), n, o, cell, dm,
                          ctypes.c_void_p(keys.data_ptr()), ctypes.c_void_p(order.data_ptr()), None)
    torch.cuda.synchronize()
    return st, keys.cpu().numpy()[:n], order.cpu().numpy()[:n]


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__
    __graft_entry__.build()
    from parmec_gb300 import abi
    return abi.load_library()


def test_static_matches_allocating_entry_point_twice(lib):
    cases = [(LIMIT, 11, (0.0, 0.0, 0.0), 0.01, (128, 128, 128)),
             (40000, 12, (-0.5, -0.5, -0.5), 0.05, (30, 40, 50))]
    for n, seed, org, cell, dim in cases:            # two calls in a row
        c = np.random.default_rng(seed).uniform(-0.6, 1.4, size=(n, 3))
        st_a, k_a, o_a = run(lib, "pg_cell_order", c, org, cell, dim)
        st_b, k_b, o_b = run(lib, "pg_cell_order_static", c, org, cell, dim)
        assert st_a == 0 and st_b == 0
        assert np.array_equal(k_a, k_b)
        assert np.array_equal(o_a, o_b)
        assert np.all(np.diff(k_b.view(np.uint32).astype(np.int64)) >= 0)


def test_static_rejects_sizes_beyond_its_limit(lib):
    from parmec_gb300 import abi
    c = np.zeros((LIMIT + 1, 3))
    st, _, _ = run(lib, "pg_cell_order_static", c, (0.0, 0.0, 0.0), 1.0, (4, 4, 4))
    assert st == abi.PG_ERR_CAPACITY
