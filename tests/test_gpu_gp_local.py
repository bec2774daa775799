"""GPU parity: the GP's sums and posterior from the gauge factors of the
lifted rows (rvgp_gp_prepare_local / rvgp_gp_predict_local) against the same
quantities from the explicitly lifted rows (rvgp_lift + rvgp_gather_rows +
rvgp_gp_prepare / rvgp_gp_predict) and the dense FP64 oracle.

The lifted rows of point i are Φ_i = T_i U_i (RVGP/dataclass.py:57-59), so
ΦᵀΦ, Φᵀy and the posterior at Φ* are exact functions of T and U; the only
difference is summation order.  Tolerances: C and b 1e-12 relative (FP64),
1e-6 (mixed, FP32 products), yy 1e-13; posterior mean 1e-10, variance 1e-9
(FP64), 1e-5 (mixed)."""
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


def cu(a, dtype=np.float64):
    return torch.as_tensor(np.ascontiguousarray(a, dtype=dtype), device="cuda")


def geometry(seed, n, D, d, ld, m, ortho=True):
    rng = np.random.default_rng(seed)
    T = rng.standard_normal((n, D, ld))
    if ortho:  # gauges are orthonormal frames; the factor path also handles general ones
        for i in range(n):
            q, _ = np.linalg.qr(T[i])
            T[i] = q[:, :ld]
    U = rng.standard_normal((n * d, m))
    vec = rng.standard_normal((n, D))
    return T, U, vec


def lifted(T, U, d):
    n, D, _ = T.shape
    m = U.shape[1]
    return np.einsum("iaq,iqj->iaj", T[:, :, :d], U.reshape(n, d, m)).reshape(n * D, m)


@pytest.mark.parametrize("D,d,ld,ortho", [(3, 2, 2, True), (64, 2, 8, True), (5, 3, 3, False), (7, 1, 2, True)])
@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_prepare_local_equals_lifted_rows(core, D, d, ld, ortho, mode):
    n, m = 300, 40
    T, U, vec = geometry(1, n, D, d, ld, m, ortho)
    idx = np.sort(np.random.default_rng(2).choice(n, 120, replace=False)).astype(np.int32)
    C, b, yy = core.gp_prepare_local(cu(T), d, cu(U), cu(idx, np.int32), cu(vec), mode)
    Phi = lifted(T, U, d).reshape(n, D, m)[idx].reshape(-1, m)
    y = vec[idx].reshape(-1)
    tol = 1e-12 if mode == "fp64" else 1e-6
    Cref = Phi.T @ Phi
    np.testing.assert_allclose(C.cpu().numpy(), Cref, rtol=0, atol=tol * np.abs(Cref).max())
    np.testing.assert_allclose(b.cpu().numpy(), Phi.T @ y, rtol=0, atol=1e-12 * np.abs(Phi.T @ y).max())
    np.testing.assert_allclose(yy.cpu().numpy()[0], y @ y, rtol=1e-13)
    # the device lifted path gives the same numbers
    Phid, Phid32, yd = core.gather_rows(core.lift(cu(T), d, cu(U)), D, cu(idx, np.int32), vec=cu(vec),
                                        want32=(mode == "mixed"))
    C2, b2, yy2 = core.gp_prepare(Phid, yd, Phid32, mode)
    # (mixed: both carry their own FP32 rounding, so they may differ by twice the bound)
    np.testing.assert_allclose(C.cpu().numpy(), C2.cpu().numpy(), rtol=0, atol=2 * tol * np.abs(Cref).max())
    np.testing.assert_allclose(b.cpu().numpy(), b2.cpu().numpy(), rtol=0, atol=1e-12 * np.abs(Phi.T @ y).max())


@pytest.mark.parametrize("D,d,ld", [(3, 2, 2), (64, 2, 8), (4, 3, 3)])
@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_predict_local_equals_oracle(core, D, d, ld, mode):
    n, m = 260, 30
    T, U, vec = geometry(3, n, D, d, ld, m)
    rng = np.random.default_rng(4)
    perm = rng.permutation(n)
    tr, te = np.sort(perm[:100]).astype(np.int32), np.sort(perm[100:]).astype(np.int32)
    lam = np.sort(rng.uniform(0.0, 3.0, m))
    th = np.array([1.5, 2.0, 1.3, 0.2])
    C, b, yy = core.gp_prepare_local(cu(T), d, cu(U), cu(tr, np.int32), cu(vec), "fp64")
    out, work = core.gp_lml(C, b, yy, len(tr) * D, cu(lam), float(n * D), cu(th), "matern")
    mean, var = core.gp_predict_local(cu(T), d, cu(U), cu(te, np.int32), work.state, mode)
    Phi_all = lifted(T, U, d).reshape(n, D, m)
    Phi, Phi_te = Phi_all[tr].reshape(-1, m), Phi_all[te].reshape(-1, m)
    S = O.eval_S(lam, th[0], th[1], th[2], float(n * D), "matern")
    mref, vref = O.predict_f_lowrank(Phi, vec[tr].reshape(-1), S, th[3], Phi_te)
    mt, vt = (1e-10, 1e-9) if mode == "fp64" else (1e-10, 1e-5)
    np.testing.assert_allclose(mean.cpu().numpy().reshape(-1), mref, rtol=0, atol=mt * np.abs(mref).max())
    np.testing.assert_allclose(var.cpu().numpy().reshape(-1), vref, rtol=0, atol=vt * np.abs(vref).max())
    # and the same as the lifted-row predict of the device
    m2, v2 = core.gp_predict(cu(Phi_te), work.state, m)
    np.testing.assert_allclose(mean.cpu().numpy().reshape(-1), m2.cpu().numpy(), rtol=0,
                               atol=mt * np.abs(mref).max())


def test_local_rejects_bad_d(core):
    T, U, vec = geometry(5, 20, 3, 2, 2, 8)
    with pytest.raises((ValueError, RuntimeError)):
        core.gp_prepare_local(cu(T), 3, cu(U[:, :8]), cu(np.arange(5), np.int32), cu(vec))
