"""pg_cell_order (the replacement of partitioning_create): Morton cell keys
and a stable radix sort, against numpy's stable argsort of the same keys."""
import ctypes

import numpy as np
import pytest


def spread3(x):
    x = x.astype(np.uint64) & 0x3ff
    x = (x | (x << 16)) & 0x030000FF
    x = (x | (x << 8)) & 0x0300F00F
    x = (x | (x << 4)) & 0x030C30C3
    x = (x | (x << 2)) & 0x09249249
    return x


def cell_keys(c, org, cell, dim):
    u = np.floor((c - np.asarray(org)) / cell)
    u = np.where(u >= 0.0, u, 0.0)
    u = np.minimum(u, np.asarray(dim) - 1).astype(np.int64)
    return (spread3(u[:, 0]) | (spread3(u[:, 1]) << 1) | (spread3(u[:, 2]) << 2)).astype(np.uint32)


def call(lib, fn, c, org, cell, dim):
    import torch
    n = len(c)
    dc = torch.tensor(np.ascontiguousarray(c.T), dtype=torch.float64, device="cuda")
    keys = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
    order = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
    o = (ctypes.c_double * 3)(*org)
    dm = (ctypes.c_int * 3)(*dim)
    st = getattr(lib, fn)(ctypes.c_void_p(dc[0].data_ptr()), ctypes.c_void_p(dc[1].data_ptr()),
                          ctypes.c_void_p(dc[2].data_ptr()), n, o, cell, dm,
                          ctypes.c_void_p(keys.data_ptr()), ctypes.c_void_p(order.data_ptr()), None)
    torch.cuda.synchronize()
    return st, keys.cpu().numpy().view(np.uint32)[:n], order.cpu().numpy()[:n]


CASES = [
    (1, 0), (2, 1), (2047, 2), (2048, 3), (2049, 4), (100000, 5), (300001, 6),
    # the last size whose histogram one block scans, the first that the grid scans, and a large one
    (65536, 7), (65537, 8), (2500000, 9),
]


@pytest.mark.gpu
@pytest.mark.parametrize("n,seed", CASES)
def test_cell_order_matches_stable_argsort(gpu_lib, n, seed):
    rng = np.random.default_rng(seed)
    c = rng.uniform(-0.1, 1.1, size=(n, 3))          # some outside the grid: clamped
    org, cell, dim = (0.0, 0.0, 0.0), 0.01, (100, 100, 100)
    st, keys, order = call(gpu_lib, "pg_cell_order", c, org, cell, dim)
    assert st == 0
    ref = cell_keys(c, org, cell, dim)
    perm = np.argsort(ref, kind="stable")
    assert np.array_equal(keys, ref[perm])
    assert np.array_equal(order, perm)


@pytest.mark.gpu
def test_cell_order_equal_keys_keep_index_order(gpu_lib):
    c = np.full((5000, 3), 0.5)
    st, keys, order = call(gpu_lib, "pg_cell_order", c, (0.0, 0.0, 0.0), 1.0, (4, 4, 4))
    assert st == 0
    assert np.array_equal(order, np.arange(5000))
    assert len(set(keys.tolist())) == 1


def test_cell_order_rejects_bad_arguments():
    """Argument checks run before any device work (callable without a GPU)."""
    import __graft_entry__
    __graft_entry__.build()
    from parmec_gb300 import abi
    lib = abi.load_library()
    o = (ctypes.c_double * 3)(0.0, 0.0, 0.0)
    for dim, cell in (((0, 4, 4), 1.0), ((4, 4, 2000), 1.0), ((4, 4, 4), 0.0), ((4, 4, 4), -1.0)):
        dm = (ctypes.c_int * 3)(*dim)
        st = lib.pg_cell_order(None, None, None, 10, o, cell, dm, None, None, None)
        assert st == abi.PG_ERR_ARGUMENT
    dm = (ctypes.c_int * 3)(4, 4, 4)
    assert lib.pg_cell_order(None, None, None, 10, o, 1.0, dm, None, None, None) == abi.PG_ERR_ARGUMENT
    assert lib.pg_cell_order(None, None, None, 0, o, 1.0, dm, None, None, None) == abi.PG_OK
