"""lkg_vecchia_sets_noalloc against lkg_vecchia_sets: the same maxmin order and neighbour sets, exactly, from
caller-owned device buffers with the intermediates in the library's fixed device array.  Collected last so that it
also runs after every other GPU test in the same process."""
import ctypes

import numpy as np
import pytest

from libkriging_gb300._lib import last_error

pytestmark = pytest.mark.gpu

SCRATCH_DOUBLES = 1 << 20
FIXED_DOUBLES = 768


def _max_n(d):
    return (SCRATCH_DOUBLES - FIXED_DOUBLES) // (2 * d + 1)


def _noalloc(lk, torch, X, m):
    """Two calls in a row on torch's current stream; outputs pre-filled with junk so that every entry is written."""
    lib = lk.load()
    n, d = X.shape
    dX = torch.from_numpy(np.ascontiguousarray(X.T)).cuda()  # (d, n) row-major == n x d column-major
    stream = torch.cuda.current_stream()
    results = []
    for _ in range(2):
        order = torch.full((n,), -7, dtype=torch.int32, device="cuda")
        nbr = torch.full((max(n * m, 1),), -7, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        rc = lib.lkg_vecchia_sets_noalloc(n, d, ctypes.c_void_p(dX.data_ptr()), m, ctypes.c_void_p(order.data_ptr()),
                                          ctypes.c_void_p(nbr.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, last_error()
        stream.synchronize()
        results.append((order.cpu().numpy().copy(), nbr.cpu().numpy()[: n * m].reshape(n, m).copy()))
    return results


@pytest.mark.parametrize("n,d,m", [(3000, 3, 30), (2048, 8, 32), (5, 2, 8), (700, 4, 0), (1, 3, 4)])
def test_noalloc_sets_match_allocating_entry(gpu_lib, n, d, m):
    import torch
    X = np.random.default_rng(n + d + m).uniform(size=(n, d))
    order_ref, nbr_ref = gpu_lib.vecchia_sets(X, m)
    for order, nbr in _noalloc(gpu_lib, torch, X, m):
        assert np.array_equal(order, np.asarray(order_ref, dtype=np.int32))
        assert np.array_equal(nbr, np.asarray(nbr_ref, dtype=np.int32).reshape(n, m))


def test_noalloc_sets_at_the_size_limit(gpu_lib):
    import torch
    d, m = 8, 16
    n = _max_n(d)
    X = np.random.default_rng(7).uniform(size=(n, d))
    order_ref, nbr_ref = gpu_lib.vecchia_sets(X, m)
    for order, nbr in _noalloc(gpu_lib, torch, X, m):
        assert np.array_equal(order, np.asarray(order_ref, dtype=np.int32))
        assert np.array_equal(nbr, np.asarray(nbr_ref, dtype=np.int32).reshape(n, m))


def test_noalloc_sets_allocate_no_device_memory(gpu_lib):
    import torch
    lib = gpu_lib.load()
    n, d, m = 4000, 3, 20
    X = np.random.default_rng(11).uniform(size=(n, d))
    dX = torch.from_numpy(np.ascontiguousarray(X.T)).cuda()
    order = torch.empty(n, dtype=torch.int32, device="cuda")
    nbr = torch.empty(n * m, dtype=torch.int32, device="cuda")
    args = (n, d, ctypes.c_void_p(dX.data_ptr()), m, ctypes.c_void_p(order.data_ptr()),
            ctypes.c_void_p(nbr.data_ptr()), ctypes.c_void_p(0))
    assert lib.lkg_vecchia_sets_noalloc(*args) == 0, last_error()  # first call resolves the scratch
    torch.cuda.synchronize()
    # cudaMemGetInfo is device-wide: another context on the same GPU can move it between the two readings, so
    # only a drop seen on every one of three attempts counts as an allocation by the entry point
    drops = []
    for _ in range(3):
        free0, _ = torch.cuda.mem_get_info()
        for _ in range(3):
            assert lib.lkg_vecchia_sets_noalloc(*args) == 0, last_error()
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
        drops.append(free0 - free1)
        if free1 >= free0:
            break
    assert min(drops) <= 0, "device free memory dropped on every attempt: %s bytes" % drops


def test_noalloc_sets_reject_before_any_work(gpu_lib):
    import torch
    lib = gpu_lib.load()
    d, m = 3, 10
    n = _max_n(d) + 1
    dX = torch.zeros((d, n), dtype=torch.float64, device="cuda")
    order = torch.empty(n, dtype=torch.int32, device="cuda")
    nbr = torch.empty(n * m, dtype=torch.int32, device="cuda")
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    assert lib.lkg_vecchia_sets_noalloc(n, d, p(dX), m, p(order), p(nbr), None) == -1
    assert "scratch" in last_error()
    assert lib.lkg_vecchia_sets_noalloc(100, 9, p(dX), m, p(order), p(nbr), None) == -1
    assert lib.lkg_vecchia_sets_noalloc(100, d, p(dX), 33, p(order), p(nbr), None) == -1
    host_X = np.zeros(100 * d)
    rc = lib.lkg_vecchia_sets_noalloc(100, d, ctypes.c_void_p(host_X.ctypes.data), m, p(order), p(nbr), None)
    assert rc == -1 and "device" in last_error()
