"""GPU parity: spectral kernel, log marginal likelihood + adjoint, posterior.

The oracle is the dense FP64 restatement of GPflow GPR + ManifoldKernel
(oracle/rvgp_oracle.py); GPflow itself is absent, so this layer is checked
against the restated dense algebra and central finite differences.
Tolerances: FP64 form 1e-9 relative on LML / gradients, 1e-8 on the posterior;
mixed form (FP32 tall products) 1e-5 on LML and gradients, 1e-4 on the posterior
mean (the target the mixed form must meet)."""
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


def problem(seed=0, N=300, m=24, Nte=50):
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.standard_normal((N + Nte, m)))
    Phi_all = Q * np.sqrt(N + Nte)
    lam = np.sort(rng.uniform(0.0, 3.0, m))
    y = rng.standard_normal(N)
    return Phi_all[:N], y, lam, Phi_all[N:]


def cu(a):
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")


@pytest.mark.parametrize("typ", ["matern", "se"])
def test_spectral_S_and_derivatives(core, typ):
    _, _, lam, _ = problem()
    th = np.array([1.5, 5.0, 1.3, 0.1])
    S, dS = core.spectral_S(cu(lam), cu(th), 900.0, typ)
    ref = O.eval_S(lam, th[0], th[1], th[2], 900.0, typ)
    np.testing.assert_allclose(S.cpu().numpy(), ref, rtol=1e-13)
    for k in range(3):
        if typ == "se" and k == 0:
            continue
        h = 1e-6 * th[k]
        tp, tm = th.copy(), th.copy()
        tp[k] += h
        tm[k] -= h
        fd = (O.eval_S(lam, *tp[:3], 900.0, typ) - O.eval_S(lam, *tm[:3], 900.0, typ)) / (2 * h)
        np.testing.assert_allclose(dS.cpu().numpy()[k], fd, rtol=1e-6, atol=1e-8 * np.abs(fd).max())


def chain_grad(Phi, y, lam, th, n_rows, typ="matern"):
    """Oracle gradient w.r.t. [nu, kappa, sigma_f, noise] via dS (finite differences of S)."""
    S = O.eval_S(lam, th[0], th[1], th[2], n_rows, typ)
    gS, gn = O.lml_grad_S_noise(Phi, y, S, th[3])
    out = []
    for k in range(3):
        h = 1e-7 * th[k]
        tp, tm = th.copy(), th.copy()
        tp[k] += h
        tm[k] -= h
        dS = (O.eval_S(lam, *tp[:3], n_rows, typ) - O.eval_S(lam, *tm[:3], n_rows, typ)) / (2 * h)
        out.append(gS @ dS)
    return np.array(out + [gn])


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
@pytest.mark.parametrize("noise", [1.0, 1e-2, 1e-3])
def test_lml_and_gradient(core, mode, noise):
    Phi, y, lam, _ = problem(1)
    n_rows = 900.0
    th = np.array([1.5, 5.0, 1.0, noise])
    Phi32 = cu(Phi).float() if mode == "mixed" else None
    C, b, yy = core.gp_prepare(cu(Phi), cu(y), Phi32, mode)
    out, work = core.gp_lml(C, b, yy, len(y), cu(lam), n_rows, cu(th))
    out = out.cpu().numpy()
    S = O.eval_S(lam, th[0], th[1], th[2], n_rows)
    ref = O.lml_dense(Phi, y, S, noise)
    tol = 1e-9 if mode == "fp64" else 1e-5
    assert abs(out[0] - ref) <= tol * abs(ref)
    g_ref = chain_grad(Phi, y, lam, th, n_rows)
    np.testing.assert_allclose(out[1:], g_ref, rtol=(1e-6 if mode == "fp64" else 1e-4),
                               atol=tol * np.abs(g_ref).max())


def test_lml_gradient_central_differences_at_random_points(core):
    """The adjoint against central differences of the GPU LML itself at 5 random hyperparameter points."""
    Phi, y, lam, _ = problem(2)
    C, b, yy = core.gp_prepare(cu(Phi), cu(y))
    rng = np.random.default_rng(7)
    for _ in range(5):
        th = np.array([rng.uniform(0.6, 3.0), rng.uniform(1.0, 8.0), rng.uniform(0.3, 3.0),
                       10 ** rng.uniform(-2.5, 0)])

        def f(t):
            return core.gp_lml(C, b, yy, len(y), cu(lam), 900.0, cu(t))[0].cpu().numpy()[0]

        g = core.gp_lml(C, b, yy, len(y), cu(lam), 900.0, cu(th))[0].cpu().numpy()[1:]
        for k in range(4):
            h = 1e-5 * th[k]
            tp, tm = th.copy(), th.copy()
            tp[k] += h
            tm[k] -= h
            fd = (f(tp) - f(tm)) / (2 * h)
            assert abs(fd - g[k]) <= 1e-5 * max(1.0, abs(fd)), (k, fd, g[k])


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_predict_matches_dense_posterior(core, mode):
    Phi, y, lam, Phi_te = problem(3)
    th = np.array([1.5, 5.0, 1.0, 1e-2])
    Phi32 = cu(Phi).float() if mode == "mixed" else None
    C, b, yy = core.gp_prepare(cu(Phi), cu(y), Phi32, mode)
    out, work = core.gp_lml(C, b, yy, len(y), cu(lam), 900.0, cu(th))
    mean, var = core.gp_predict(cu(Phi_te), work.state, len(lam), None, mode)
    S = O.eval_S(lam, 1.5, 5.0, 1.0, 900.0)
    m_ref, v_ref = O.predict_f(Phi, y, S, 1e-2, Phi_te)
    tol = 1e-8 if mode == "fp64" else 1e-4
    assert np.linalg.norm(mean.cpu().numpy() - m_ref) <= tol * np.linalg.norm(m_ref)
    np.testing.assert_allclose(var.cpu().numpy(), v_ref, rtol=(1e-6 if mode == "fp64" else 1e-3),
                               atol=1e-9 * np.abs(v_ref).max())


def test_kernel_matrix_and_diag(core):
    Phi, _, lam, Phi_te = problem(4, N=130, m=20, Nte=70)
    S = O.eval_S(lam, 1.5, 5.0, 1.0, 400.0)
    K = core.kernel_matrix(cu(Phi), cu(S), cu(Phi_te)).cpu().numpy()
    np.testing.assert_allclose(K, O.kernel_K(Phi, S, Phi_te), rtol=1e-12, atol=1e-10)
    Kd = core.kernel_diag(cu(Phi), cu(S)).cpu().numpy()
    np.testing.assert_allclose(Kd, np.diag(O.kernel_K(Phi, S)), rtol=1e-12)


def test_device_adam_matches_torch_adam_on_autograd_adjoint(core):
    """rvgp_gp_fit_adam (device loop) against torch.optim.Adam driving the
    hand-written adjoint through torch.autograd (main.log_marginal_likelihood)."""
    from rvgp_gb300.main import _LML
    Phi, y, lam, _ = problem(6)
    C, b, yy = core.gp_prepare(cu(Phi), cu(y))
    th0 = np.array([1.5, 5.0, 1.0, 1.0])
    lower = [0.0, 0.0, 0.0, 1e-6]
    steps, lr = 25, 0.05
    theta_dev, out, hist, work = core.gp_fit_adam(C, b, yy, len(y), cu(lam), 900.0, cu(th0), lower, [1, 1, 1, 1],
                                                  steps, lr=lr, history=True)

    class Model:  # what _LML needs
        pass
    mdl = Model()
    mdl.C, mdl.b, mdl.yy, mdl.N = C, b, yy, len(y)
    mdl.kernel = Model()
    mdl.kernel.eigenvalues, mdl.kernel.num_verticies, mdl.kernel.typ = cu(lam), 900.0, "matern"
    mdl.work = core.LMLWorkspace(len(lam), "cuda")
    lo = torch.tensor(lower, dtype=torch.float64)
    u = torch.tensor(np.log(np.expm1(th0 - np.array(lower))), dtype=torch.float64, requires_grad=True)
    opt = torch.optim.Adam([u], lr=lr)
    for _ in range(steps):
        opt.zero_grad()
        theta = (torch.nn.functional.softplus(u) + lo).to("cuda")
        loss = -_LML.apply(theta, mdl)
        loss.backward()
        opt.step()
    ref = (torch.nn.functional.softplus(u) + lo).detach().numpy()
    np.testing.assert_allclose(theta_dev.cpu().numpy(), ref, rtol=1e-9)
    h = hist.cpu().numpy()
    assert np.all(np.isfinite(h)) and h[-1] > h[0]


def test_non_pd_reports_nan(core):
    Phi, y, lam, _ = problem(5)
    C, b, yy = core.gp_prepare(cu(Phi), cu(y))
    th = np.array([1.5, 5.0, -1.0, 1e-2])  # negative sigma_f: A is not positive definite
    out, _ = core.gp_lml(C, b, yy, len(y), cu(lam), 900.0, cu(th))
    assert np.isnan(out.cpu().numpy()[0])


def structured_problem(seed, N, m):
    """Rows of an orthonormal basis and a target with most energy in the low modes."""
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.standard_normal((N, m)))
    Phi = Q * np.sqrt(N)
    lam = np.sort(rng.uniform(0.0, 3.0, m))
    coef = rng.standard_normal(m) / (1.0 + lam) ** 2
    y = Phi @ coef + 0.05 * rng.standard_normal(N)
    return Phi, y, lam


@pytest.mark.parametrize("m,N,typ", [(24, 300, "matern"), (50, 800, "se"), (97, 1500, "matern"),
                                     (200, 4000, "matern")])
def test_mixed_fit_matches_fp64_fit(core, m, N, typ):
    """The one-launch FP32 fit (rvgp_gp_fit_adam_mixed) follows the FP64 Adam
    trajectory: 200 steps from the reference's initial values, parameters to
    1e-4 relative, the LML history to 1e-4 of its largest magnitude (the FP32
    log-determinant), posterior means to 1e-6."""
    assert m <= core.gp_fit_mixed_max_m()
    Phi, y, lam = structured_problem(11, N, m)
    C, b, yy = core.gp_prepare(cu(Phi), cu(y))
    th0 = cu([3.0, 4.0, 1.0, 1.0])
    lower, mask, steps = [0.0, 0.0, 0.0, 1e-6], [1, 1, 1, 1], 200
    n_rows = 3.0 * N
    th64, _, h64, w64 = core.gp_fit_adam(C, b, yy, N, cu(lam), n_rows, th0, lower, mask, steps, typ=typ,
                                         history=True)
    mean64, _ = core.gp_predict(cu(Phi[:200]), w64.state, m)
    th32, out32, h32, w32, ok = core.gp_fit_adam_mixed(C, b, yy, N, cu(lam), n_rows, th0, lower, mask, steps,
                                                       typ=typ, history=True)
    assert ok
    np.testing.assert_allclose(th32.cpu().numpy(), th64.cpu().numpy(), rtol=1e-4)
    h64n = h64.cpu().numpy()
    np.testing.assert_allclose(h32.cpu().numpy(), h64n, rtol=0, atol=1e-4 * np.abs(h64n).max())
    mean32, _ = core.gp_predict(cu(Phi[:200]), w32.state, m)
    err = (torch.linalg.vector_norm(mean32 - mean64) / torch.linalg.vector_norm(mean64)).item()
    assert err <= 1e-6
    # out / state are the FP64 likelihood at the returned parameters
    ref, _ = core.gp_lml(C, b, yy, N, cu(lam), n_rows, th32, typ=typ)
    np.testing.assert_allclose(out32.cpu().numpy(), ref.cpu().numpy(), rtol=1e-12)


def test_mixed_fit_reports_failed_pivot(core):
    """A start with a negative kernel variance makes the FP32 capacitance matrix
    invalid: the launch stops, reports it, and writes no parameters."""
    Phi, y, lam = structured_problem(3, 300, 24)
    C, b, yy = core.gp_prepare(cu(Phi), cu(y))
    th, _, _, _, ok = core.gp_fit_adam_mixed(C, b, yy, 300, cu(lam), 900.0, cu([1.5, 5.0, -1.0, 1e-2]),
                                             [0.0, 0.0, 0.0, 1e-6], [1, 1, 1, 1], 5)
    assert not ok
