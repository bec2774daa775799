"""CPU: host-side logic of the GP models that needs no GPU (optimiser loop,
kernel parameters and their bounds, mesh input errors)."""
import math

import numpy as np
import pytest


def test_host_adam_is_adam_and_skips_non_finite_steps():
    from rvgp_gb300.main import _host_adam
    target = np.array([1.0, -2.0, 0.5])
    state = {"x": None, "calls": 0}

    def assign(x):
        state["x"] = np.array(x)

    def loss_and_grad():
        state["calls"] += 1
        x = state["x"]
        if state["calls"] == 3:  # one failed evaluation: the step must keep x
            return float("nan"), np.full(3, np.nan)
        return float(((x - target) ** 2).sum()), 2 * (x - target)

    x, hist = _host_adam(assign, loss_and_grad, np.zeros(3), 400, 0.05)
    assert len(hist) == 400 and math.isnan(hist[2])
    np.testing.assert_allclose(x, target, atol=1e-3)
    # the first step moves every coordinate by lr against the gradient sign (bias-corrected Adam)
    state["calls"] = 0
    x1, _ = _host_adam(assign, loss_and_grad, np.zeros(3), 1, 0.05)
    np.testing.assert_allclose(x1, -0.05 * np.sign(-target), rtol=1e-6)


def test_rbf_kernel_defaults_and_bounds():
    from rvgp_gb300.kernels import RBF, default_positive_minimum, set_default_positive_minimum
    old = default_positive_minimum()
    try:
        set_default_positive_minimum(0.0)
        k = RBF()
        assert float(k.variance) == pytest.approx(1.0) and float(k.lengthscales) == pytest.approx(1.0)
        assert k.variance.lower == 0.0 and [p.name for p in k.parameters] == ["variance", "lengthscales"]
        set_default_positive_minimum(1e-2)  # later kernels see the new bound, earlier ones keep theirs
        k2 = RBF()
        assert k2.variance.lower == 1e-2 and k.variance.lower == 0.0
        np.testing.assert_array_equal(k.K_diag(np.zeros((4, 3))), np.ones(4))
        with pytest.raises(ValueError):
            k2.lengthscales.assign(1e-3)  # below the bound
    finally:
        set_default_positive_minimum(old)


def test_load_mesh_errors(tmp_path):
    from rvgp_gb300.utils import load_mesh
    with pytest.raises(FileNotFoundError):
        load_mesh("absent", folder=str(tmp_path))
    (tmp_path / "bad.obj").write_text("v 0 0\n")
    with pytest.raises(IndexError):
        load_mesh("bad", folder=str(tmp_path))


def test_ptu_dijkstra_drop_in_errors_and_expansion():
    """The drop-in for the reference's native module raises the reference's
    errors before any device work (RVGP/lib/ptu_dijkstra.pyx:68-82,152-156)
    and expands edge indices as pyx:202-214 does."""
    import scipy.sparse as sp
    from rvgp_gb300 import ptu_dijkstra as P
    X = np.zeros((10, 3))
    A = sp.eye(10, format="csr")
    with pytest.raises(ValueError, match="less than the total number"):
        P.tangent_frames(X, A, 2, 10)
    with pytest.raises(ValueError, match="larger or equal to the embedding"):
        P.tangent_frames(X, A, 3, 2)
    with pytest.raises(ValueError, match="less or equal to the ambient"):
        P.tangent_frames(X, A, 4, 5)
    with pytest.raises(ValueError, match="less or equal to the ambient"):
        P.connections(np.zeros((10, 3, 2)), A, 4)
    with pytest.raises(ValueError, match="unit edge weights"):
        P.tangent_frames(X, 2.0 * A, 2, 5)
    ei = np.array([[0, 1, 2], [1, 2, 0]])
    # the reference's construction: every (i, j) of range(dim)², edge-major
    dim = 2
    ind = [np.array([i, j]) for i in range(dim) for j in range(dim)]
    ref = np.stack([ei * dim + i[:, None] for i in ind], axis=2).reshape(2, 3 * len(ind))
    np.testing.assert_array_equal(P.expand_edge_index(ei, dim), ref)
    np.testing.assert_array_equal(P.expand_edge_index(ei, 1), ei)
