"""GPU parity: the RBF-kernel GP on the scalar-Laplacian eigenbasis (fit(kernel='rbf')).

The oracle is the FP64 restatement of GPflow 2.6.5 ``kernels.RBF`` + ``GPR``
with D output columns (``rbf_K``, ``rbf_gpr_lml``, ``rbf_gpr_predict_f`` in
oracle/rvgp_oracle.py).  Tolerances: kernel matrix 1e-13 relative; LML 1e-9
relative; gradients within 1e-6 of the largest component against central
differences of the oracle; posterior mean 1e-8 relative (norm), variance 1e-7
relative + 1e-10."""
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


def cu(a):
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")


def problem(seed, N, m, D=3, Nte=40):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((N, m)) * 0.3
    Y = rng.standard_normal((N, D))
    Xs = rng.standard_normal((Nte, m)) * 0.3
    return X, Y, Xs


def test_kernel_matrix(core):
    X, _, Xs = problem(0, 70, 9)
    th = np.array([1.7, 0.6, 0.1])
    K = core.rbf_matrix(cu(Xs), cu(th), cu(X)).cpu().numpy()
    np.testing.assert_allclose(K, O.rbf_K(Xs, X, 1.7, 0.6), rtol=1e-13, atol=1e-15)


@pytest.mark.parametrize("N,m", [(60, 8), (150, 20), (300, 12)])  # 300: blocked Cholesky
@pytest.mark.parametrize("noise", [1.0, 0.01])
def test_lml_gradient_and_posterior(core, N, m, noise):
    X, Y, Xs = problem(N + m, N, m)
    th = np.array([1.3, 0.9, noise])
    out, work = core.rbf_lml(cu(X), cu(Y), cu(th))
    out = out.cpu().numpy()
    ref = O.rbf_gpr_lml(X, Y, *th)
    assert abs(out[0] - ref) <= 1e-9 * abs(ref)
    fd = np.zeros(3)
    for k in range(3):
        h = 1e-6 * th[k]
        tp, tm = th.copy(), th.copy()
        tp[k] += h
        tm[k] -= h
        fd[k] = (O.rbf_gpr_lml(X, Y, *tp) - O.rbf_gpr_lml(X, Y, *tm)) / (2 * h)
    assert np.abs(out[1:] - fd).max() <= 1e-6 * np.abs(fd).max()
    mean, var = core.rbf_predict(cu(Xs), cu(X), Y.shape[1], cu(th), work.state)
    m_ref, v_ref = O.rbf_gpr_predict_f(X, Y, *th, Xs)
    mean, var = mean.cpu().numpy(), var.cpu().numpy()
    assert np.linalg.norm(mean - m_ref) <= 1e-8 * np.linalg.norm(m_ref)
    np.testing.assert_allclose(var, v_ref, rtol=1e-7, atol=1e-10)


def test_too_many_rows_raise(core):
    X, Y, _ = problem(1, 3100, 2)
    with pytest.raises(RuntimeError, match="rvgp_rbf_lml"):
        core.rbf_lml(cu(X), cu(Y), cu([1.0, 1.0, 0.1]))


# ------------------------------------------------------------------ public API
@pytest.fixture(scope="module")
def RVGP():
    import rvgp_gb300
    return rvgp_gb300


def _sphere(RVGP):
    g = load_golden("sphere")
    d = RVGP.create_data_object(g["X"], n_neighbors=10, n_eigenpairs=int(g["m"]), precision="fp64", verbose=False)
    d.random_vector_field(seed=3)
    d.smooth_vector_field(t=20)
    return d


def test_fit_rbf_matches_oracle(RVGP):
    """fit(kernel='rbf', epochs=0): inputs are the training points' rows of the
    scalar eigenbasis, outputs their vectors (RVGP/main.py:33-37); the posterior
    at the test points is GPflow GPR's with RBF() defaults and σ² = 1."""
    d = _sphere(RVGP)
    n = d.n
    train = np.arange(0, n, 2)
    test = np.arange(1, n, 2)
    gp = RVGP.fit(d, train_ind=train, kernel="rbf", epochs=0, verbose=False)
    assert isinstance(gp, RVGP.main.rbf_GPR)
    mean, var = gp.transform(d, list(map(int, test)))
    tr, _ = O.train_test_split_indices(len(train), 0.2, 0)
    pts = train[tr]
    X = d.evecs_L[pts]
    Y = d.vectors[pts]
    m_ref, v_ref = O.rbf_gpr_predict_f(X, Y, 1.0, 1.0, 1.0, d.evecs_L[test])
    assert mean.shape == (len(test), 3) and var.shape == (len(test), 3)
    assert np.linalg.norm(mean - m_ref) <= 1e-8 * np.linalg.norm(m_ref)
    np.testing.assert_allclose(var, np.repeat(v_ref[:, None], 3, axis=1), rtol=1e-7, atol=1e-10)
    ref = O.rbf_gpr_lml(X, Y, 1.0, 1.0, 1.0)
    assert abs(gp.log_marginal_likelihood() - ref) <= 1e-9 * abs(ref)


def test_fit_rbf_optimises_and_fixes_parameters(RVGP):
    d = _sphere(RVGP)
    gp0 = RVGP.fit(d, kernel="rbf", epochs=0, verbose=False)
    gp = RVGP.fit(d, kernel="rbf", epochs=40, verbose=False)
    assert gp.log_marginal_likelihood() > gp0.log_marginal_likelihood()
    gpa = RVGP.fit(d, kernel="rbf", epochs=30, optimizer="adam", lr=0.05, verbose=False)
    assert gpa.log_marginal_likelihood() > gp0.log_marginal_likelihood()
    gpf = RVGP.fit(d, kernel="rbf", epochs=20, kernel_variance=0.7, kernel_lengthscale=0.4, verbose=False)
    assert float(gpf.kernel.variance) == pytest.approx(0.7) and float(gpf.kernel.lengthscales) == pytest.approx(0.4)
    with pytest.raises(NotImplementedError):
        RVGP.fit(d, kernel="rbf", n_inducing_points=10, epochs=0, verbose=False)
