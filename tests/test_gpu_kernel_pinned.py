"""GPU parity of the spectral kernel against the reference's own
``ManifoldKernel`` (RVGP/kernels.py:41-67): tests/golden/kernel.npz holds
eval_S, K(X), K(X, X2) and K_diag(X) that the reference class computed on the
eigenpairs of the geometry fixtures (tests/golden/make_kernel_golden.py), for
Matérn and squared-exponential kernels at five parameter sets.  Checked through
the C ABI (rvgp_spectral_S, rvgp_kernel_matrix, rvgp_kernel_diag) and through
the public ``ManifoldKernel``.  Tolerance: 1e-12 relative to the largest entry
(FP64, different summation order)."""
from types import SimpleNamespace

import numpy as np
import pytest
import torch

from conftest import load_golden
from oracle import rvgp_oracle as O

pytestmark = pytest.mark.gpu
CASES = ["sphere", "torus", "ellipsoid", "swissroll64"]


def cu(a):
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")


def lifted(g):
    return g["evecs_Lc"] if "evecs_Lc" in g else O.lift(g["gauges"], g["evecs_Lc_local"], g["evals_Lc"].size)


@pytest.mark.parametrize("name", CASES)
def test_device_kernel_equals_reference(name):
    from rvgp_gb300 import _core
    _core.require_cuda()
    kg, g = load_golden("kernel"), load_golden(name)
    ev = lifted(g)
    X, X2 = cu(ev[kg[f"{name}_rows"]]), cu(ev[kg[f"{name}_rows2"]])
    for c, typ in enumerate(kg["params_typ"]):
        nu, kappa, sf = kg["params"][c]
        key = f"{name}_{c}"
        S, _ = _core.spectral_S(cu(g["evals_Lc"]), cu([nu, kappa, sf, 1.0]), float(kg[f"{name}_n_rows"]), str(typ))
        np.testing.assert_allclose(S.cpu().numpy(), kg[key + "_S"], rtol=1e-12)
        for got, ref in ((_core.kernel_matrix(X, S), kg[key + "_K"]), (_core.kernel_matrix(X, S, X2), kg[key + "_K2"]),
                         (_core.kernel_diag(X, S), kg[key + "_Kdiag"])):
            np.testing.assert_allclose(got.cpu().numpy(), ref, rtol=0, atol=1e-12 * np.abs(ref).max())


@pytest.mark.parametrize("name", ["sphere", "swissroll64"])
def test_public_manifold_kernel_equals_reference(name):
    from rvgp_gb300.kernels import ManifoldKernel
    kg, g = load_golden("kernel"), load_golden(name)
    n, D = g["X"].shape
    dev = SimpleNamespace(evals_Lc=cu(g["evals_Lc"]), X=cu(g["X"]))
    data = SimpleNamespace(_dev=dev, _evecs_Lc_dev=lambda: cu(lifted(g)))
    ev = lifted(g)
    X, X2 = ev[kg[f"{name}_rows"]], ev[kg[f"{name}_rows2"]]
    for c, typ in enumerate(kg["params_typ"]):
        nu, kappa, sf = kg["params"][c]
        k = ManifoldKernel(data, nu=nu, kappa=kappa, sigma_f=sf, typ=str(typ))
        key = f"{name}_{c}"
        assert k.num_verticies == float(kg[f"{name}_n_rows"]) == n * D
        np.testing.assert_allclose(k.eval_S(typ=str(typ)), kg[key + "_S"], rtol=1e-12)
        np.testing.assert_allclose(k.K(X), kg[key + "_K"], rtol=0, atol=1e-12 * np.abs(kg[key + "_K"]).max())
        np.testing.assert_allclose(k(X, X2), kg[key + "_K2"], rtol=0, atol=1e-12 * np.abs(kg[key + "_K2"]).max())
        np.testing.assert_allclose(k(X, full_cov=False), kg[key + "_Kdiag"], rtol=1e-12)
