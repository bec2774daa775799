"""GPU: the mixed-precision Adam fit on one thread-block cluster (the m x m
capacitance algebra spread over the shared memory of up to 16 CTAs) against the
FP64 device fit (rvgp_gp_fit_adam) and the one-CTA mixed fit.  m up to 512
runs on a cluster of m/32 CTAs holding one block row each; m from 513 to 1024
on 16 CTAs holding two block rows each (the wide form).

Same tolerances as the one-CTA fit: parameters 1e-4 relative, posterior means
1e-6 relative, the returned out / state the FP64 likelihood at the returned
parameters (1e-12); the LML history to 1e-4 of its largest magnitude up to
m = 200 and 3e-4 above (the history follows the parameters, which still move
fast at the last steps, so a parameter difference of 1e-4 shows in it at
~|∂LML/∂log θ| · 1e-4), 1e-3 above 512, where the FP32 pivots lose more."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def core():
    from rvgp_gb300 import _core
    _core.require_cuda()
    return _core


def cu(a):
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")


def structured_problem(seed, N, m):
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.standard_normal((N, m)))
    Phi = Q * np.sqrt(N)
    lam = np.sort(rng.uniform(0.0, 3.0, m))
    coef = rng.standard_normal(m) / (1.0 + lam) ** 2
    y = Phi @ coef + 0.05 * rng.standard_normal(N)
    return Phi, y, lam


def fit_mixed(core, force_cluster, *args, **kw):
    old = os.environ.get("RVGP_GP_FIT_CLUSTER")
    os.environ["RVGP_GP_FIT_CLUSTER"] = "1" if force_cluster else "0"
    try:
        return core.gp_fit_adam_mixed(*args, **kw)
    finally:
        if old is None:
            del os.environ["RVGP_GP_FIT_CLUSTER"]
        else:
            os.environ["RVGP_GP_FIT_CLUSTER"] = old


@pytest.mark.parametrize("m,N,typ", [(40, 600, "matern"), (97, 1500, "se"), (200, 4000, "matern"),
                                     (300, 5000, "matern"), (500, 8000, "matern"), (700, 10000, "se"),
                                     (1000, 15000, "matern")])
def test_cluster_fit_matches_fp64_fit(core, m, N, typ):
    if m > core.gp_fit_mixed_max_m():
        pytest.skip(f"clusters for m={m} cannot be launched on this device")
    Phi, y, lam = structured_problem(21, N, m)
    C, b, yy = core.gp_prepare(cu(Phi), cu(y))
    th0 = cu([3.0, 4.0, 1.0, 1.0])
    lower, mask, steps = [0.0, 0.0, 0.0, 1e-6], [1, 1, 1, 1], 200
    n_rows = 3.0 * N
    th64, _, h64, w64 = core.gp_fit_adam(C, b, yy, N, cu(lam), n_rows, th0, lower, mask, steps, typ=typ,
                                         history=True)
    mean64, _ = core.gp_predict(cu(Phi[:300]), w64.state, m)
    th32, out32, h32, w32, ok = fit_mixed(core, True, C, b, yy, N, cu(lam), n_rows, th0, lower, mask, steps,
                                          typ=typ, history=True)
    assert ok
    np.testing.assert_allclose(th32.cpu().numpy(), th64.cpu().numpy(), rtol=1e-4)
    h64n = h64.cpu().numpy()
    htol = 1e-4 if m <= 200 else 3e-4 if m <= 512 else 1e-3
    np.testing.assert_allclose(h32.cpu().numpy(), h64n, rtol=0, atol=htol * np.abs(h64n).max())
    mean32, _ = core.gp_predict(cu(Phi[:300]), w32.state, m)
    err = (torch.linalg.vector_norm(mean32 - mean64) / torch.linalg.vector_norm(mean64)).item()
    assert err <= 1e-6
    ref, _ = core.gp_lml(C, b, yy, N, cu(lam), n_rows, th32, typ=typ)
    np.testing.assert_allclose(out32.cpu().numpy(), ref.cpu().numpy(), rtol=1e-12)


def test_cluster_fit_equals_one_cta_fit(core):
    """Both mixed kernels run the same FP32 algebra in different blockings:
    their trajectories agree to FP32 rounding."""
    m, N = 150, 3000
    Phi, y, lam = structured_problem(5, N, m)
    C, b, yy = core.gp_prepare(cu(Phi), cu(y))
    args = (C, b, yy, N, cu(lam), 3.0 * N, cu([1.5, 5.0, 1.0, 1.0]), [0.0, 0.0, 0.0, 1e-6], [1, 1, 1, 1], 100)
    a = fit_mixed(core, False, *args, history=True)
    c = fit_mixed(core, True, *args, history=True)
    assert a[4] and c[4]
    np.testing.assert_allclose(c[0].cpu().numpy(), a[0].cpu().numpy(), rtol=2e-5)
    ha = a[2].cpu().numpy()
    np.testing.assert_allclose(c[2].cpu().numpy(), ha, rtol=0, atol=2e-5 * np.abs(ha).max())


def test_cluster_fit_reports_invalid_parameters(core):
    Phi, y, lam = structured_problem(3, 600, 64)
    C, b, yy = core.gp_prepare(cu(Phi), cu(y))
    th, _, _, _, ok = fit_mixed(core, True, C, b, yy, 600, cu(lam), 1800.0, cu([1.5, 5.0, -1.0, 1e-2]),
                                [0.0, 0.0, 0.0, 1e-6], [1, 1, 1, 1], 5)
    assert not ok
