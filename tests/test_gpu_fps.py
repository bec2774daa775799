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


@pytest.mark.parametrize("kind,n,N,D", [("bumpy_sphere", 20000, 6000, 3), ("torus", 5000, 5000, 3),
                                        ("sphere", 3000, 100, 3), ("ties", 4000, 4000, 3), ("ties", 3000, 3000, 1),
                                        ("gauss", 6000, 2500, 7), ("gauss", 100, 1, 2),
                                        ("bumpy_sphere", 120000, 60000, 3)])
def test_spatial_equals_persistent(core, kind, n, N, D):
    """The spatially pruned form (one CTA, only the blocks the new point can
    change) selects the same points with the same FP64 lambdas as the
    persistent form, including exact distance ties (points on a coarse grid,
    duplicates), one-dimensional and seven-dimensional clouds, and N = 1."""
    from rvgp_gb300.workloads import make_points
    rng = np.random.default_rng(n + D)
    if kind == "ties":
        Xh = np.round(rng.uniform(0, 1, (n, D)), 1)  # many duplicates and equal distances
    elif kind == "gauss":
        Xh = rng.standard_normal((n, D))
    else:
        Xh = make_points(kind, n, seed=5)
    X = torch.as_tensor(Xh, device="cuda")
    st = {}
    p2, l2 = core.fps(X, N=N, method="spatial", stats=st)
    p1, l1 = core.fps(X, N=N, method="persistent")
    assert torch.equal(p2, p1)
    assert torch.equal(l2, l1)
    if N >= 5000 and kind != "ties":
        assert st["exact_evals"] < 0.2 * n * N
    if n <= 4000:
        pr, lr = O.furthest_point_sampling(Xh, N=N)
        np.testing.assert_array_equal(p2.cpu().numpy(), pr)


def test_spatial_spacing_stop(core):
    from rvgp_gb300.workloads import make_points
    X = torch.as_tensor(make_points("bumpy_sphere", 8000, seed=6), device="cuda")
    p2, l2 = core.fps(X, spacing=0.05, method="spatial")
    p1, l1 = core.fps(X, spacing=0.05, method="persistent")
    assert 1 < len(p2) < 8000
    assert torch.equal(p2, p1) and torch.equal(l2, l1)
