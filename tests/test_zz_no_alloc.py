"""GPU: the allocation-free kNN entry point (rvgp_knn_noalloc).

Some callers cannot allocate device memory at the moment they need a
neighbour search (their device-memory budget is fixed at start-up, or a host
framework owns the memory pool).  rvgp_knn_noalloc takes only inputs and
outputs and uses a fixed scratch buffer inside the library.  These checks
call it through the C ABI and compare it with rvgp_knn on two calls in a row
(the second call reuses the buffer the first one left behind), check that a
call leaves the device's free memory unchanged, and that a problem too large
for the buffer or of an unsupported dimension is refused.  The file name makes
pytest collect it last.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def core():
    from rvgp_gb300 import _core
    _core.require_cuda()
    return _core


def _noalloc(core, X, k):
    n, D = X.shape
    idx = torch.empty((n, k), dtype=torch.int32, device=X.device)
    st = core.lib().rvgp_knn_noalloc(core.ptr(X), n, D, k, core.ptr(idx), core.stream())
    return st, idx


def test_noalloc_matches_workspace_entry_point_twice(core):
    from rvgp_gb300.workloads import make_points
    cases = [(make_points("torus", 6000, seed=11), 20), (make_points("swissroll64", 2500, seed=12), 15)]
    for X_np, k in cases:  # two calls in a row, different shapes, same buffer
        X = torch.as_tensor(X_np, device="cuda")
        st, idx = _noalloc(core, X, k)
        assert st == 0, core.lib().rvgp_last_error().decode()
        ref = core.knn(X, k)  # the entry point with a caller-provided workspace
        torch.cuda.synchronize()
        assert torch.equal(idx, ref)


def test_noalloc_allocates_no_device_memory(core):
    """After a first call (which looks up the buffer's device address), a
    further call leaves the device's free memory unchanged: nothing is
    allocated on the device, by this library or through torch."""
    from rvgp_gb300.workloads import make_points
    X = torch.as_tensor(make_points("sphere", 5000, seed=3), device="cuda")
    idx = torch.empty((5000, 10), dtype=torch.int32, device="cuda")
    L = core.lib()
    assert L.rvgp_knn_noalloc(core.ptr(X), 5000, 3, 10, core.ptr(idx), core.stream()) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    assert L.rvgp_knn_noalloc(core.ptr(X), 5000, 3, 10, core.ptr(idx), core.stream()) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert torch.equal(idx, core.knn(X, 10))


def test_noalloc_rejects_unsupported_dimension(core):
    L = core.lib()
    assert L.rvgp_knn_workspace(1000, 129, 10) == 0
    X = torch.zeros((1000, 129), dtype=torch.float64, device="cuda")
    st, _ = _noalloc(core, X, 10)
    assert st == -1
    assert b"unsupported shape" in L.rvgp_last_error()


def test_noalloc_rejects_problem_larger_than_buffer(core):
    L = core.lib()
    n, D, k = 200_000, 3, 20
    assert L.rvgp_knn_workspace(n, D, k) > (32 << 20)
    X = torch.zeros((n, D), dtype=torch.float64, device="cuda")
    st, _ = _noalloc(core, X, k)
    assert st == -1
    assert b"fixed" in L.rvgp_last_error()
