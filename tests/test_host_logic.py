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
