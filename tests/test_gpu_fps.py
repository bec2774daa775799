"""GPU: furthest-point sampling in one cooperative launch (rvgp_fps_persistent)
against the one-launch-per-selection form (rvgp_fps) and the oracle's
restatement of RVGP/geometry.py:126-162: the same permutation and the same
FP64 lambdas bit for bit (the FP32 screen only skips distances that provably
cannot lower the running minimum), with the N and the spacing stops."""
import numpy as np
import pytest
import torch

from oracle import rvgp_oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def core():
    from rvgp_gb300 import _core
    _core.require_cuda()
    return _core


@pytest.mark.parametrize("kind,n,N", [("bumpy_sphere", 20000, 6000), ("torus", 5000, 5000), ("sphere", 3000, 100)])
def test_persistent_equals_per_launch(core, kind, n, N):
    from rvgp_gb300.workloads import make_points
    X = torch.as_tensor(make_points(kind, n, seed=5), device="cuda")
    st = {}
    p1, l1 = core.fps(X, N=N, persistent=True, stats=st)
    p0, l0 = core.fps(X, N=N, persistent=False)
    assert torch.equal(p1, p0)
    assert torch.equal(l1, l0)
    if N > 1000:  # the FP32 screen skips most exact distances once the points are dense
        assert st["exact_evals"] < 0.5 * n * N
    if n <= 5000:
        pr, lr = O.furthest_point_sampling(X.cpu().numpy(), N=N)
        np.testing.assert_array_equal(p1.cpu().numpy(), pr)
        np.testing.assert_allclose(l1.cpu().numpy(), lr, rtol=1e-12, atol=1e-14)


def test_persistent_spacing_stop(core):
    from rvgp_gb300.workloads import make_points
    X = torch.as_tensor(make_points("bumpy_sphere", 8000, seed=6), device="cuda")
    p1, l1 = core.fps(X, spacing=0.05, persistent=True)
    p0, l0 = core.fps(X, spacing=0.05, persistent=False)
    assert 1 < len(p1) < 8000
    assert torch.equal(p1, p0) and torch.equal(l1, l0)
