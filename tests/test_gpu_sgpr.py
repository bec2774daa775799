"""GPU parity: the sparse inducing-point GP (manifold_SGPR).

The oracle is the FP64 restatement of GPflow 2.6.5 SGPR (``sgpr_elbo``,
``sgpr_predict_f`` in oracle/rvgp_oracle.py, itself checked against the
bound's N-space definition and, with Z spanning the eigenbasis, against the
exact GPR).  Tolerances: bound 1e-9 relative; gradients against central
finite differences of the oracle 1e-5 relative to the largest component;
posterior mean 1e-8 relative (norm), variance 1e-6 relative + 1e-9."""
import numpy as np
import pytest
import torch

from conftest import load_golden
from oracle import rvgp_oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def core():
    from rvgp_gb300 import _core
    _core.require_cuda()
    return _core


def problem(seed=0, N=300, m=24, Nte=50):
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.standard_normal((N + Nte, m)))
    Phi_all = Q * np.sqrt((N + Nte) / m)
    lam = np.sort(rng.uniform(0.0, 3.0, m))
    y = rng.standard_normal(N)
    return Phi_all[:N], y, lam, Phi_all[N:]


def cu(a):
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")


def device_bound(core, Phi, y, lam, th, Z, n_rows, typ="matern", jitter=1e-6):
    C, b, yy = core.gp_prepare(cu(Phi), cu(y))
    out, work = core.sgpr_elbo(C, b, yy, Phi.shape[0], cu(Z), cu(lam), n_rows, cu(th), typ, jitter)
    torch.cuda.synchronize()
    return out.cpu().numpy(), work


def oracle_bound(Phi, y, lam, th, Z, n_rows, typ="matern", jitter=1e-6):
    S = O.eval_S(lam, th[0], th[1], th[2], n_rows, typ)
    return O.sgpr_elbo(Phi, y, S, th[3], Z, jitter)


def inducing(Phi, M, seed):
    rng = np.random.default_rng(seed)
    return Phi[rng.choice(len(Phi), M, replace=False)] + 0.05 * rng.standard_normal((M, Phi.shape[1]))


@pytest.mark.parametrize("M", [7, 24, 40, 170])  # 170: past the one-CTA Cholesky (blocked factorisation)
@pytest.mark.parametrize("typ", ["matern", "se"])
@pytest.mark.parametrize("noise", [1.0, 0.05])
def test_bound_and_hyperparameter_gradients(core, M, typ, noise):
    Phi, y, lam, _ = problem(M)
    Z = inducing(Phi, M, M + 1)
    th = np.array([1.5, 2.0, 1.3, noise])
    n_rows = 900.0
    out, _ = device_bound(core, Phi, y, lam, th, Z, n_rows, typ)
    ref = oracle_bound(Phi, y, lam, th, Z, n_rows, typ)
    assert abs(out[0] - ref) <= 1e-9 * abs(ref)
    fd = np.zeros(4)
    for k in range(4):
        if typ == "se" and k == 0:
            continue
        h = 1e-5 * th[k]
        tp, tm = th.copy(), th.copy()
        tp[k] += h
        tm[k] -= h
        fd[k] = (oracle_bound(Phi, y, lam, tp, Z, n_rows, typ) - oracle_bound(Phi, y, lam, tm, Z, n_rows, typ)) / (2 * h)
    assert np.abs(out[1:] - fd).max() <= 1e-5 * np.abs(fd).max()


@pytest.mark.parametrize("M", [6, 12, 40])
def test_inducing_input_gradient(core, M):
    """∂F/∂Z against central differences of the oracle (step 1e-4; the
    difference quotient's own noise floor there is ~1e-7 absolute).  With
    M > m the inducing rows over-span the eigenbasis and ∂F/∂Z is small."""
    Phi, y, lam, _ = problem(10 + M, N=200, m=16)
    Z = inducing(Phi, M, M)
    th = np.array([1.5, 2.0, 1.3, 0.2])
    _, work = device_bound(core, Phi, y, lam, th, Z, 600.0)
    dZ = work.dZ.cpu().numpy()
    rng = np.random.default_rng(M)
    h = 1e-4
    picks = [(int(i), int(j)) for i, j in zip(rng.integers(0, M, 12), rng.integers(0, 16, 12))]
    for i, j in picks:
        Zp, Zm = Z.copy(), Z.copy()
        Zp[i, j] += h
        Zm[i, j] -= h
        fd = (oracle_bound(Phi, y, lam, th, Zp, 600.0) - oracle_bound(Phi, y, lam, th, Zm, 600.0)) / (2 * h)
        assert abs(dZ[i, j] - fd) <= 1e-5 * np.abs(dZ).max() + 1e-7


@pytest.mark.parametrize("M", [7, 40, 170])
def test_posterior_matches_oracle(core, M):
    Phi, y, lam, Phi_te = problem(20 + M)
    Z = inducing(Phi, M, 3)
    th = np.array([1.5, 2.0, 1.3, 0.1])
    _, work = device_bound(core, Phi, y, lam, th, Z, 900.0)
    mean, var = core.sgpr_predict(cu(Phi_te), work.state, Phi.shape[1])
    S = O.eval_S(lam, 1.5, 2.0, 1.3, 900.0)
    m_ref, v_ref = O.sgpr_predict_f(Phi, y, S, 0.1, Z, Phi_te)
    mean, var = mean.cpu().numpy(), var.cpu().numpy()
    assert np.linalg.norm(mean - m_ref) <= 1e-8 * np.linalg.norm(m_ref)
    np.testing.assert_allclose(var, v_ref, rtol=1e-6, atol=1e-9)


def test_spanning_inducing_inputs_give_the_exact_gp(core):
    """Z = I (the eigenbasis itself) without jitter: the bound is the GPR LML
    and the posterior is the GPR posterior (device GPR path as the other side)."""
    Phi, y, lam, Phi_te = problem(7)
    m = Phi.shape[1]
    th = np.array([1.5, 2.0, 1.3, 0.3])
    out, work = device_bound(core, Phi, y, lam, th, np.eye(m), 900.0, jitter=0.0)
    C, b, yy = core.gp_prepare(cu(Phi), cu(y))
    lml, gwork = core.gp_lml(C, b, yy, Phi.shape[0], cu(lam), 900.0, cu(th))
    lml = lml.cpu().numpy()
    np.testing.assert_allclose(out, lml, rtol=1e-9, atol=1e-9 * np.abs(lml).max())
    mean, var = core.sgpr_predict(cu(Phi_te), work.state, m)
    gm, gv = core.gp_predict(cu(Phi_te), gwork.state, m, None, "fp64")
    np.testing.assert_allclose(mean.cpu().numpy(), gm.cpu().numpy(), rtol=1e-8, atol=1e-10)
    np.testing.assert_allclose(var.cpu().numpy(), gv.cpu().numpy(), rtol=1e-7, atol=1e-10)


def test_bad_sizes_raise(core):
    Phi, y, lam, _ = problem(1)
    C, b, yy = core.gp_prepare(cu(Phi), cu(y))
    th = cu([1.5, 2.0, 1.3, 0.1])
    with pytest.raises(RuntimeError, match="rvgp_sgpr_elbo"):
        core.sgpr_elbo(C, b, yy, Phi.shape[0], cu(np.zeros((4000, Phi.shape[1]))), cu(lam), 900.0, th)


# ------------------------------------------------------------------ public API
@pytest.fixture(scope="module")
def RVGP():
    import rvgp_gb300
    return rvgp_gb300


def _torus_field(RVGP, precision="fp64"):
    g = load_golden("torus")
    d = RVGP.create_data_object(g["X"], n_neighbors=20, n_eigenpairs=int(g["m"]), precision=precision, verbose=False)
    d.random_vector_field(seed=1)
    d.smooth_vector_field(t=20)
    return d


@pytest.mark.parametrize("M", [15, 60])
def test_fit_with_inducing_points_matches_oracle(RVGP, M):
    """RVGP.fit(n_inducing_points=M, epochs=0): inducing rows are the FPS of
    the training rows (RVGP/main.py:60-61) and the posterior is GPflow SGPR's."""
    d = _torus_field(RVGP)
    n = d.n
    train = np.arange(0, n, 2)
    test = np.arange(1, n, 2)
    gp = RVGP.fit(d, train_ind=train, n_inducing_points=M, epochs=0, verbose=False)
    assert isinstance(gp, RVGP.main.manifold_SGPR)
    mean, var = gp.transform(d, list(map(int, test)))
    ev = d.evecs_Lc.reshape(n, -1)
    m = d.evecs_Lc.shape[1]
    tr, _ = O.train_test_split_indices(len(train), 0.2, 0)
    pts = train[tr]
    Phi = ev[pts].reshape(-1, m)
    y = d.vectors[pts].reshape(-1)
    ind, _ = O.furthest_point_sampling(Phi, N=M)
    Z = Phi[ind]
    np.testing.assert_array_equal(gp.inducing_variable.numpy(), Z)
    S = O.eval_S(d.evals_Lc, 1.5, 5.0, 1.0, d.evecs_Lc.shape[0])
    m_ref, v_ref = O.sgpr_predict_f(Phi, y, S, 1.0, Z, ev[test].reshape(-1, m))
    assert np.linalg.norm(mean.ravel() - m_ref) <= 1e-8 * np.linalg.norm(m_ref)
    np.testing.assert_allclose(var.ravel(), v_ref, rtol=1e-6, atol=1e-9)
    ref = O.sgpr_elbo(Phi, y, S, 1.0, Z)
    assert abs(gp.elbo() - ref) <= 1e-9 * abs(ref)


def test_fit_with_inducing_points_optimises_the_bound(RVGP):
    d = _torus_field(RVGP, "mixed")
    gp0 = RVGP.fit(d, n_inducing_points=40, epochs=0, verbose=False)
    gp = RVGP.fit(d, n_inducing_points=40, epochs=30, verbose=False)
    assert gp.elbo() > gp0.elbo()
    assert not np.array_equal(gp.inducing_variable.numpy(), gp0.inducing_variable.numpy())  # Z is trained
    # Adam on the kernel and noise parameters with the FPS inducing rows held
    gpa = RVGP.fit(d, n_inducing_points=40, epochs=0, verbose=False)
    gpa.inducing_variable.trainable = False
    gpa.optimize(epochs=40, method="adam", lr=0.05)
    assert gpa.elbo() > gp0.elbo()
    np.testing.assert_array_equal(gpa.inducing_variable.numpy(), gp0.inducing_variable.numpy())
    assert len(gpa.lml_history) == 40 and np.isfinite(gpa.lml_history).all()
    mean, var = gp.transform(d, np.arange(10))
    assert mean.shape == (10, 3) and var.shape == (10, 3) and np.all(var >= -1e-9)
    with pytest.raises(ValueError):
        RVGP.fit(d, n_inducing_points=10 ** 7, epochs=0, verbose=False)
