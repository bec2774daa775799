"""GP fit / predict with the surface of RVGP/main.py.

``train_gp`` (exported as ``fit``) keeps the reference's signature and flow
(RVGP/main.py:11-84): default ``ManifoldKernel(nu=3/2, kappa=5, sigma_f=1)``,
rows = (training point, ambient coordinate), sklearn's seeded 80/20
``train_test_split`` of ``train_ind``, L-BFGS-B on the negative log marginal
likelihood for at most ``epochs`` iterations, then the "Relative l2 error"
print on the held-out 20 %.  Every likelihood evaluation, gradient and
prediction is a CUDA computation (rvgp_gp_lml / rvgp_gp_predict; with
``n_inducing_points``, the sparse GP of RVGP/main.py:59-67 through
rvgp_sgpr_elbo / rvgp_sgpr_predict); the optimiser loop itself runs on the
host, as GPflow's Scipy optimiser does.

Reference behaviours kept by default (``reference_quirks=True``): the
likelihood variance starts at 1.0 because ``noise_variance`` never reaches
GPflow (RVGP/main.py:99-100); the positive-parameter lower bound of the default
kernel is the one in force when it was created (RVGP/main.py:30,52).
``reference_quirks=False`` starts the noise at ``noise_variance``.

Extensions: ``optimizer="adam"`` (``epochs`` Adam steps at ``lr``, gradients
from the hand-written adjoint behind ``torch.autograd``), ``precision``
("mixed" or "fp64", default the data object's), and ``transform`` accepting
numpy integer arrays and boolean masks.
"""
from __future__ import annotations

import math

import numpy as np
import scipy.optimize
import torch

from rvgp_gb300 import _core
from rvgp_gb300.kernels import RBF, ManifoldKernel, Parameter, set_default_positive_minimum


def train_test_split_indices(n_samples, test_size=0.2, seed=0):
    """Index split of sklearn ``train_test_split(..., test_size, random_state=seed)``
    (ShuffleSplit: RandomState(seed).permutation, first ceil(test_size*n) are test)."""
    n_test = int(math.ceil(test_size * n_samples))
    n_train = n_samples - n_test
    perm = np.random.RandomState(seed).permutation(n_samples)
    return perm[n_test:n_test + n_train], perm[:n_test]


class _LML(torch.autograd.Function):
    """Log marginal likelihood with its hand-written adjoint (see rvgp_gp_lml)."""

    @staticmethod
    def forward(ctx, theta, model):
        out, _ = _core.gp_lml(model.C, model.b, model.yy, model.N, model.kernel.eigenvalues,
                              model.kernel.num_verticies, theta.detach().contiguous(), model.kernel.typ, model.work)
        ctx.save_for_backward(out[1:5].clone())
        return out[0].clone()

    @staticmethod
    def backward(ctx, g):
        (grad,) = ctx.saved_tensors
        return g * grad, None


def log_marginal_likelihood(theta, model):
    """Differentiable LML: theta = CUDA f64 tensor [nu, kappa, sigma_f, noise]."""
    return _LML.apply(theta, model)


def _host_adam(assign, loss_and_grad, x0, steps, lr, betas=(0.9, 0.999), eps=1e-8):
    """Adam on the unconstrained vector x (the update of the device Adam of
    rvgp_gp_fit_adam), one device evaluation per step.  Returns (x, history of
    the objective −loss); a step whose loss or gradient is not finite keeps x."""
    b1, b2 = betas
    x = np.array(x0, dtype=np.float64)
    m1 = np.zeros_like(x)
    v1 = np.zeros_like(x)
    hist = []
    for step in range(steps):
        assign(x)
        f, g = loss_and_grad()
        hist.append(-f)
        if not (np.isfinite(f) and np.isfinite(g).all()):
            continue
        m1 = b1 * m1 + (1 - b1) * g
        v1 = b2 * v1 + (1 - b2) * g * g
        x = x - lr * (m1 / (1 - b1 ** (step + 1))) / (np.sqrt(v1 / (1 - b2 ** (step + 1))) + eps)
    assign(x)
    return x, np.asarray(hist)


class manifold_GPR:
    """GPflow-GPR-like model on the manifold kernel (RVGP/main.py:99-116)."""

    def __init__(self, data, kernel, train_points, noise_variance=1.0, precision="mixed"):
        self.data_obj = data
        self.kernel = kernel
        self.precision = precision
        self.likelihood = type("Gaussian", (), {})()
        self.likelihood.variance = Parameter(noise_variance, lower=1e-6, name="noise_variance")
        dev = data._dev
        if dev.vectors is None:
            raise ValueError("the data object has no vectors to fit")
        self.D = dev.X.shape[1]
        idx = torch.as_tensor(np.asarray(train_points, dtype=np.int32), device=dev.X.device)
        # C = ΦᵀΦ, b = Φᵀy and yᵀy of the rows (training point, coordinate)
        # of RVGP/main.py:24-50, from the gauges and local eigenvectors: the
        # lifted rows Φ_i = T_i U_i are never formed (d rows per point, not D)
        geo = kernel.data
        self.C, self.b, self.yy = _core.gp_prepare_local(geo._dev.T, geo.dim_man, geo._dev.evecs_Lc_local, idx,
                                                         dev.vectors, precision)
        self.N = idx.numel() * self.D
        self.m = kernel.eigenvalues.numel()
        self.work = _core.LMLWorkspace(self.m, dev.X.device)
        self.n_evals = 0
        self._eval_key, self._eval_out = None, None  # parameters of the state held in self.work
        self._train_idx = idx

    # ------------------------------------------------------------------ parameters
    @property
    def trainable_parameters(self):
        ps = self.kernel.parameters + [self.likelihood.variance]
        return [p for p in ps if p.trainable]

    def theta(self):
        return self.kernel.theta(float(self.likelihood.variance))

    def _theta_key(self):
        return tuple(float(p) if p is not None else None for p in self._slots()) + (self.kernel.typ,)

    def _evaluate(self):
        """FP64 likelihood, gradient and posterior state (in self.work) at the
        current parameters; reused while the parameters are unchanged."""
        key = self._theta_key()
        if self._eval_key == key:
            return self._eval_out
        out, _ = _core.gp_lml(self.C, self.b, self.yy, self.N, self.kernel.eigenvalues, self.kernel.num_verticies,
                              self.theta(), self.kernel.typ, self.work)
        self.n_evals += 1
        self._eval_key, self._eval_out = key, out.cpu().numpy()
        return self._eval_out

    def log_marginal_likelihood(self):
        return float(self._evaluate()[0])

    def training_loss(self):
        return -self.log_marginal_likelihood()

    def _loss_and_grad_u(self, params):
        out = self._evaluate()
        grads = {"nu": out[1], "kappa": out[2], "sigma_f": out[3], "noise_variance": out[4]}
        g = np.array([-grads[p.name] * p.dvalue_du() for p in params])
        return -out[0], g

    # ------------------------------------------------------------------ optimisation
    def optimize(self, epochs=1000, method="l-bfgs-b", lr=0.05, disp=True):
        params = self.trainable_parameters
        if not params or epochs <= 0:
            return None
        if method.lower() in ("l-bfgs-b", "lbfgs", "scipy"):
            def fun(x):
                for p, u in zip(params, x):
                    p.unconstrained = float(u)
                f, g = self._loss_and_grad_u(params)
                if not np.isfinite(f):
                    return np.inf, np.zeros_like(g)
                return f, g
            x0 = np.array([p.unconstrained for p in params])
            res = scipy.optimize.minimize(fun, x0, jac=True, method="L-BFGS-B",
                                          options={"maxiter": epochs})
            if disp:  # scipy's L-BFGS-B no longer takes "disp": report the outcome here
                print(f"L-BFGS-B: {res.message} ({res.nit} iterations, loss {res.fun:.6g})")
            for p, u in zip(params, res.x):
                p.unconstrained = float(u)
            return res
        if method.lower() == "adam":
            return self._adam(params, epochs, lr)
        raise ValueError(f"unknown optimiser {method!r}")

    def _slots(self):
        """The four hyperparameters in theta order [nu, kappa, sigma_f, noise] (nu None for SE)."""
        return [self.kernel.nu, self.kernel.kappa, self.kernel.sigma_f, self.likelihood.variance]

    def _adam(self, params, steps, lr):
        """``steps`` Adam steps on the device (rvgp_gp_fit_adam): no host round trip per step."""
        slots = self._slots()
        lower = [p.lower if p is not None else 0.0 for p in slots]
        mask = [p is not None and p.trainable for p in slots]
        args = (self.C, self.b, self.yy, self.N, self.kernel.eigenvalues, self.kernel.num_verticies, self.theta(),
                lower, mask, steps)
        ok = False
        self.fit_form = "fp64"
        if self.precision == "mixed" and self.m <= _core.gp_fit_mixed_max_m():
            # the data object's deferred eigensolve of L runs beside the one-CTA fit
            theta, out, hist, _, ok = _core.gp_fit_adam_mixed(*args, lr=lr, typ=self.kernel.typ, work=self.work,
                                                              history=True,
                                                              on_launch=getattr(self.data_obj, "_release_eig_L", None))
            self.fit_form = "mixed" if ok else "fp64 (an FP32 pivot failed)"
        if not ok:
            theta, out, hist, _ = _core.gp_fit_adam(*args, lr=lr, typ=self.kernel.typ, work=self.work, history=True)
        vals = theta.cpu().numpy()
        for p, v in zip(slots, vals):
            if p is not None and p.trainable:
                p.assign(float(v))
        self.n_evals += steps + 1
        self.lml_history = hist
        # self.work holds the FP64 likelihood, gradient and state at the fitted parameters
        self._eval_key, self._eval_out = self._theta_key(), out.cpu().numpy()
        return vals

    # ------------------------------------------------------------------ many starts
    def _device_bounds(self):
        """Lower bounds and trainable flags of [nu, kappa, sigma_f, noise] as device tensors."""
        slots = self._slots()
        lower = torch.tensor([p.lower if p is not None else 0.0 for p in slots], dtype=torch.float64,
                             device=self.kernel.device)
        mask = torch.tensor([int(p is not None and p.trainable) for p in slots], dtype=torch.int32,
                            device=self.kernel.device)
        return lower, mask

    def restart_starts(self, n_restarts, kappa_range=(0.5, 50.0), seed=0):
        """Starting parameters of a multi-start search: the model's current
        values with log-uniform initial lengthscales kappa in kappa_range
        (seeded), as an (n_restarts, 4) device tensor."""
        rng = np.random.default_rng(seed)
        th = self.theta().cpu().numpy()
        out = np.tile(th, (int(n_restarts), 1))
        lo, hi = np.log(kappa_range[0]), np.log(kappa_range[1])
        out[:, 1] = np.exp(rng.uniform(lo, hi, int(n_restarts)))
        return torch.as_tensor(out, device=self.kernel.device)

    def fit_restarts(self, theta0s, epochs=200, lr=0.05, history=False):
        """Multi-start hyperparameter search on the device: one mixed-form
        Adam fit of ``epochs`` steps from every row of theta0s (R, 4) at once
        (rvgp_gp_fit_restarts: R CTAs or R thread-block clusters in one
        launch), the FP64 log marginal likelihood of each, and the best; the
        model takes the best fit's parameters.  Returns the dict of device
        tensors of _core.gp_fit_restarts (theta, lml, status, best, ...)."""
        if self.m > _core.gp_fit_mixed_max_m():
            raise ValueError(f"fit_restarts: m={self.m} exceeds the mixed fit's limit {_core.gp_fit_mixed_max_m()}")
        lower, mask = self._device_bounds()
        out = _core.gp_fit_restarts(self.C, self.b, self.yy, self.N, self.kernel.eigenvalues,
                                    self.kernel.num_verticies, theta0s, lower, mask, epochs, lr=lr,
                                    typ=self.kernel.typ, history=history)
        for p, v in zip(self._slots(), out["theta_best"].cpu().numpy()):
            if p is not None and p.trainable:
                p.assign(float(v))
        self.n_evals += (epochs + 1) * theta0s.shape[0]
        self.fit_form = "mixed (restarts)"
        return out

    # ------------------------------------------------------------------ prediction
    def _predict_rows(self, Phi_star):
        self._evaluate()  # posterior state at the current parameters
        mode = self.precision
        mean, var = _core.gp_predict(Phi_star, self.work.state, self.m, None, mode)
        return mean, var

    def predict_f(self, Xnew):
        """Posterior mean and marginal variance, each (rows, 1), at rows of the spectral input."""
        dev = self.kernel.device
        Xd = Xnew.to(dev, torch.float64) if isinstance(Xnew, torch.Tensor) else torch.as_tensor(
            np.ascontiguousarray(Xnew, dtype=np.float64), device=dev)
        mean, var = self._predict_rows(Xd.reshape(-1, self.m).contiguous())
        return mean.reshape(-1, 1).cpu(), var.reshape(-1, 1).cpu()

    def predict_points(self, points):
        """Posterior mean and variance at manifold points (indices), each (len, D), on the device."""
        idx = torch.as_tensor(np.asarray(points, dtype=np.int32), device=self.kernel.device)
        self._evaluate()  # posterior state at the current parameters
        geo = self.kernel.data
        return _core.gp_predict_local(geo._dev.T, geo.dim_man, geo._dev.evecs_Lc_local, idx, self.work.state,
                                      self.precision)

    def predict_fields(self, fields, points):
        """Posterior means (B, len(points), D) and log marginal likelihoods (B,)
        of B fields ``fields`` (B, n, D) observed at this model's training
        points, with this model's hyperparameters: the per-time-sample fits of
        a field sequence (RVGP's EEG use, eeg_utils.py:26-35) solved for every
        field at once (rvgp_gp_posterior_batch).  The posterior variance does
        not depend on the field: ``predict_points(points)`` gives it."""
        self._evaluate()  # posterior state at the current parameters
        dev = self.kernel.device
        F = fields.to(dev, torch.float64) if isinstance(fields, torch.Tensor) else torch.as_tensor(
            np.ascontiguousarray(fields, dtype=np.float64), device=dev)
        if F.ndim != 3 or F.shape[2] != self.D:
            raise ValueError(f"fields must be (B, n, {self.D}), got {tuple(F.shape)}")
        B = F.shape[0]
        Y = F[:, self._train_idx.long(), :].reshape(B, -1).t().contiguous()  # (N, B), rows (point, coordinate)
        Phi, _, _ = _core.gather_rows(self.kernel.eigenvectors, self.D, self._train_idx)
        idx = torch.as_tensor(np.asarray(points, dtype=np.int32), device=dev)
        Phi_star, _, _ = _core.gather_rows(self.kernel.eigenvectors, self.D, idx)
        mean, lml = _core.gp_posterior_batch(Phi, Y, self.theta(), self.work.state, Phi_star)
        return mean.t().reshape(B, len(idx), self.D), lml

    def transform(self, data, test_ind):
        """Posterior mean and variance (the reference names it f_pred_std, but it
        is the variance) at test points, as in RVGP/main.py:102-116.  Integer
        indices select manifold points; floats are spectral inputs."""
        first = test_ind[0] if len(test_ind) else 0
        arr = np.asarray(test_ind)
        if arr.dtype == bool:
            arr = np.nonzero(arr)[0]
        if np.issubdtype(np.asarray(first).dtype, np.integer) or arr.dtype == bool or np.issubdtype(arr.dtype,
                                                                                                   np.integer):
            mean, var = self.predict_points(arr)
            return mean.cpu().numpy(), var.cpu().numpy()
        mean, var = self.predict_f(np.asarray(test_ind, dtype=np.float64))
        n = len(test_ind)
        return mean.numpy().reshape(n, -1), var.numpy().reshape(n, -1)


class ManyFieldsSolve:
    """Device sequence of the many-fields workload (B time-sample fields on one
    manifold observed at the same training points, RVGP's one-fit-per-sample
    use of eeg_utils.py:26-35): R restarts of the hyperparameter fit on the
    model's own field, the FP64 posterior state at the best fit's parameters,
    and the posterior means and LMLs of all B fields with those parameters.

    ``enqueue()`` issues only stream-ordered device work: no host
    synchronisation, and no allocation after the first call (the buffers are
    kept), so the sequence can be captured in a CUDA graph (``capture()``) and
    replayed (``replay()``).  ``gp`` is a manifold_GPR fitted (or prepared with
    epochs=0) on the field the restarts optimise; ``fields`` (B, n, D) on the
    device; ``points`` the prediction points; ``theta0s`` (R, 4) the starts."""

    def __init__(self, gp, fields, points, theta0s, epochs=200, lr=0.05):
        self.gp = gp
        self.epochs, self.lr = int(epochs), float(lr)
        dev = gp.kernel.device
        F = fields.to(dev, torch.float64) if isinstance(fields, torch.Tensor) else torch.as_tensor(
            np.ascontiguousarray(fields, dtype=np.float64), device=dev)
        self.B = F.shape[0]
        self.Y = F[:, gp._train_idx.long(), :].reshape(self.B, -1).t().contiguous()
        self.Phi, _, _ = _core.gather_rows(gp.kernel.eigenvectors, gp.D, gp._train_idx)
        idx = torch.as_tensor(np.asarray(points, dtype=np.int32), device=dev)
        self.Phi_star, _, _ = _core.gather_rows(gp.kernel.eigenvectors, gp.D, idx)
        self.n_points = int(idx.numel())
        self.theta0s = theta0s.to(dev, torch.float64).contiguous()
        self.lower, self.mask = gp._device_bounds()
        self.fit = None
        self.mean = torch.empty((self.Phi_star.shape[0], self.B), dtype=torch.float64, device=dev)
        self.lml = torch.empty(self.B, dtype=torch.float64, device=dev)
        L = _core.lib()
        self.ws = _core.workspace(L.rvgp_gp_posterior_batch_workspace(gp.m, self.B), dev)
        self.graph = None

    def enqueue(self):
        gp = self.gp
        self.fit = _core.gp_fit_restarts(gp.C, gp.b, gp.yy, gp.N, gp.kernel.eigenvalues, gp.kernel.num_verticies,
                                         self.theta0s, self.lower, self.mask, self.epochs, lr=self.lr,
                                         typ=gp.kernel.typ, out=self.fit)
        _core.gp_lml(gp.C, gp.b, gp.yy, gp.N, gp.kernel.eigenvalues, gp.kernel.num_verticies, self.fit["theta_best"],
                     gp.kernel.typ, gp.work)
        L = _core.lib()
        _core.check(L.rvgp_gp_posterior_batch(_core.ptr(self.Phi), self.Phi.shape[0], gp.m, _core.ptr(self.Y), self.B,
                                              _core.ptr(self.fit["theta_best"]), _core.ptr(gp.work.state),
                                              _core.ptr(self.Phi_star), self.Phi_star.shape[0], _core.ptr(self.mean),
                                              _core.ptr(self.lml), _core.ptr(self.ws), self.ws.numel(),
                                              _core.stream()), "rvgp_gp_posterior_batch")

    def capture(self):
        """Record enqueue() in a CUDA graph (after one eager call, which sets
        up every kernel and buffer)."""
        if self.fit is None:
            self.enqueue()
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.enqueue()
        return self.graph

    def replay(self):
        self.graph.replay()

    def means(self):
        """Posterior means (B, len(points), D) of the last run."""
        return self.mean.t().reshape(self.B, self.n_points, self.gp.D)


class InducingPoints:
    """GPflow ``InducingPoints``: the M x m inducing inputs Z (CUDA f64), trainable by default."""

    def __init__(self, Z):
        self.Z = Z
        self.trainable = True

    @property
    def num_inducing(self):
        return int(self.Z.shape[0])

    def numpy(self):
        return self.Z.cpu().numpy()


class manifold_SGPR(manifold_GPR):
    """GPflow-SGPR-like sparse GP on the manifold kernel (RVGP/main.py:119-137).

    The collapsed bound of Titsias (GPflow 2.6.5 ``SGPR.elbo``, jitter 1e-6 on
    Kuu), its gradient with respect to the kernel parameters, the noise
    variance and the inducing inputs Z, and ``predict_f`` are CUDA
    computations (rvgp_sgpr_elbo / rvgp_sgpr_predict) from C = ΦᵀΦ, b = Φᵀy
    and yᵀy, which are formed once.  ``inducing_variable`` (M x m spectral
    rows) defaults to the furthest-point sample of ``n_inducing_points``
    training rows, started at row 0, as RVGP/main.py:60-61 does.  Z is
    trained with the other parameters unless ``inducing_variable.trainable``
    is set to False (GPflow trains it by default).
    """

    def __init__(self, data, kernel, train_points, inducing_variable=None, n_inducing_points=None,
                 noise_variance=1.0, precision="mixed", jitter=1e-6):
        self.data_obj = data
        self.kernel = kernel
        self.precision = precision
        self.jitter = float(jitter)
        self.likelihood = type("Gaussian", (), {})()
        self.likelihood.variance = Parameter(noise_variance, lower=1e-6, name="noise_variance")
        dev = data._dev
        if dev.vectors is None:
            raise ValueError("the data object has no vectors to fit")
        self.D = dev.X.shape[1]
        idx = torch.as_tensor(np.asarray(train_points, dtype=np.int32), device=dev.X.device)
        Phi, Phi32, y = _core.gather_rows(kernel.eigenvectors, self.D, idx, vec=dev.vectors,
                                          want32=(precision == "mixed"))
        self.C, self.b, self.yy = _core.gp_prepare(Phi, y, Phi32, precision)
        self.N = Phi.shape[0]
        self.m = kernel.eigenvalues.numel()
        if inducing_variable is None:
            if n_inducing_points is None:
                raise ValueError("manifold_SGPR needs inducing_variable or n_inducing_points")
            if not 1 <= int(n_inducing_points) <= self.N:
                raise ValueError(f"n_inducing_points={n_inducing_points} must be in [1, {self.N}]")
            perm, _ = _core.fps(Phi, N=int(n_inducing_points), start_idx=0)
            Z = Phi[perm.long()].contiguous()
        else:
            Z = inducing_variable.to(Phi.device, torch.float64) if isinstance(inducing_variable, torch.Tensor) \
                else torch.as_tensor(np.ascontiguousarray(inducing_variable, dtype=np.float64), device=Phi.device)
            Z = Z.reshape(-1, self.m).contiguous().clone()
        self.inducing_variable = InducingPoints(Z)
        self.work = _core.SGPRWorkspace(Z.shape[0], self.m, Phi.device)
        self.n_evals = 0
        self._z_version = 0
        self._eval_key, self._eval_out = None, None

    def _theta_key(self):
        return super()._theta_key() + (self._z_version,)

    def predict_fields(self, fields, points):
        raise NotImplementedError("predict_fields is implemented for the full GP (manifold_GPR)")

    def _set_Z(self, values):
        self.inducing_variable.Z.copy_(torch.as_tensor(values, dtype=torch.float64).reshape(self.inducing_variable.Z.shape))
        self._z_version += 1

    def _evaluate(self):
        """FP64 bound, gradients (work.dZ) and posterior (work.state) at the
        current parameters; reused while they are unchanged."""
        key = self._theta_key()
        if self._eval_key == key:
            return self._eval_out
        out, _ = _core.sgpr_elbo(self.C, self.b, self.yy, self.N, self.inducing_variable.Z, self.kernel.eigenvalues,
                                 self.kernel.num_verticies, self.theta(), self.kernel.typ, self.jitter, self.work)
        self.n_evals += 1
        self._eval_key, self._eval_out = key, out.cpu().numpy()
        return self._eval_out

    def elbo(self):
        """The collapsed lower bound on the log marginal likelihood (GPflow ``SGPR.elbo``)."""
        return float(self._evaluate()[0])

    def log_marginal_likelihood(self):
        return self.elbo()

    def _loss_and_grad(self, params, train_Z):
        f, g = self._loss_and_grad_u(params)
        if train_Z:
            g = np.concatenate([g, -self.work.dZ.cpu().numpy().ravel()])
        return f, g

    def optimize(self, epochs=1000, method="l-bfgs-b", lr=0.05, disp=True):
        params = self.trainable_parameters
        train_Z = self.inducing_variable.trainable
        if (not params and not train_Z) or epochs <= 0:
            return None
        n_p = len(params)

        def assign(x):
            for p, u in zip(params, x[:n_p]):
                p.unconstrained = float(u)
            if train_Z:
                self._set_Z(x[n_p:])

        x0 = np.array([p.unconstrained for p in params])
        if train_Z:
            x0 = np.concatenate([x0, self.inducing_variable.numpy().ravel()])
        if method.lower() in ("l-bfgs-b", "lbfgs", "scipy"):
            def fun(x):
                assign(x)
                f, g = self._loss_and_grad(params, train_Z)
                if not np.isfinite(f):
                    return np.inf, np.zeros_like(g)
                return f, g
            res = scipy.optimize.minimize(fun, x0, jac=True, method="L-BFGS-B",
                                          options={"maxiter": epochs})
            if disp:  # scipy's L-BFGS-B no longer takes "disp": report the outcome here
                print(f"L-BFGS-B: {res.message} ({res.nit} iterations, loss {res.fun:.6g})")
            assign(res.x)
            return res
        if method.lower() == "adam":
            x, hist = _host_adam(assign, lambda: self._loss_and_grad(params, train_Z), x0, epochs, lr)
            self.lml_history = hist
            return x
        raise ValueError(f"unknown optimiser {method!r}")

    def _predict_rows(self, Phi_star):
        self._evaluate()  # posterior state at the current parameters
        return _core.sgpr_predict(Phi_star, self.work.state, self.m)

    def predict_points(self, points):
        """Posterior mean and variance at manifold points (indices), each (len, D), on the device."""
        idx = torch.as_tensor(np.asarray(points, dtype=np.int32), device=self.kernel.device)
        Phi, _, _ = _core.gather_rows(self.kernel.eigenvectors, self.D, idx)
        mean, var = self._predict_rows(Phi)
        return mean.reshape(-1, self.D), var.reshape(-1, self.D)


class rbf_GPR(manifold_GPR):
    """GPflow GPR with ``kernels.RBF()`` on the scalar-Laplacian eigenbasis, the
    D vector components as independent outputs sharing the kernel
    (``fit(..., kernel='rbf')``, RVGP/main.py:33-37,55-58,99-116).

    The likelihood, its gradient with respect to (variance, lengthscales,
    noise) and the posterior are FP64 CUDA computations over the N training
    points (rvgp_rbf_lml / rvgp_rbf_predict; N <= 3072).  ``transform`` with
    integer indices predicts at those points' rows of the scalar eigenbasis.
    """

    max_rows = 3072

    def __init__(self, data, kernel, train_points, noise_variance=1.0):
        self.data_obj = data
        self.kernel = kernel
        self.precision = "fp64"
        self.likelihood = type("Gaussian", (), {})()
        self.likelihood.variance = Parameter(noise_variance, lower=1e-6, name="noise_variance")
        dev = data._dev
        if dev.vectors is None:
            raise ValueError("the data object has no vectors to fit")
        data.wait()  # the scalar eigenpairs may still be computed concurrently
        self.D = dev.X.shape[1]
        idx = torch.as_tensor(np.asarray(train_points, dtype=np.int64), device=dev.X.device)
        self.X = dev.evecs_L[idx].contiguous()
        self.Y = dev.vectors[idx].to(torch.float64).contiguous()
        self.N = self.X.shape[0]
        self.m = self.X.shape[1]
        if self.N > self.max_rows:
            raise ValueError(f"kernel='rbf' is a dense GP over the training points: {self.N} rows exceed "
                             f"{self.max_rows}")
        self.work = _core.RBFWorkspace(self.N, self.D, dev.X.device)
        self.n_evals = 0
        self._eval_key, self._eval_out = None, None

    def _slots(self):
        return [self.kernel.variance, self.kernel.lengthscales, self.likelihood.variance]

    def predict_fields(self, fields, points):
        raise NotImplementedError("predict_fields is implemented for the full GP (manifold_GPR)")

    def theta(self):
        return self.kernel.theta(float(self.likelihood.variance), device=self.X.device)

    def _theta_key(self):
        return tuple(float(p) for p in self._slots())

    def _evaluate(self):
        key = self._theta_key()
        if self._eval_key == key:
            return self._eval_out
        out, _ = _core.rbf_lml(self.X, self.Y, self.theta(), self.work)
        self.n_evals += 1
        self._eval_key, self._eval_out = key, out.cpu().numpy()
        return self._eval_out

    def _loss_and_grad_u(self, params):
        out = self._evaluate()
        grads = {"variance": out[1], "lengthscales": out[2], "noise_variance": out[3]}
        g = np.array([-grads[p.name] * p.dvalue_du() for p in params])
        return -out[0], g

    def _adam(self, params, steps, lr):
        def assign(x):
            for p, u in zip(params, x):
                p.unconstrained = float(u)
        x0 = np.array([p.unconstrained for p in params])
        x, self.lml_history = _host_adam(assign, lambda: self._loss_and_grad_u(params), x0, steps, lr)
        return x

    def _predict_rows(self, Xs):
        self._evaluate()  # posterior state at the current parameters
        mean, var = _core.rbf_predict(Xs, self.X, self.D, self.theta(), self.work.state)
        return mean, var[:, None].expand(-1, self.D)

    def predict_f(self, Xnew):
        """Mean and variance, each (rows, D), at rows of the scalar eigenbasis."""
        Xd = Xnew.to(self.X.device, torch.float64) if isinstance(Xnew, torch.Tensor) else torch.as_tensor(
            np.ascontiguousarray(Xnew, dtype=np.float64), device=self.X.device)
        mean, var = self._predict_rows(Xd.reshape(-1, self.m).contiguous())
        return mean.cpu(), var.cpu()

    def predict_points(self, points):
        dev = self.data_obj._dev
        idx = torch.as_tensor(np.asarray(points, dtype=np.int64), device=self.X.device)
        return self._predict_rows(dev.evecs_L[idx].contiguous())


def optimize_model_with_scipy(model, epochs):
    """RVGP/main.py:87-95: L-BFGS-B with maxiter=epochs."""
    model.optimize(epochs=epochs, method="l-bfgs-b")
    return model


def train_gp(data, train_ind=None, n_inducing_points=None, test_size=0.2, kernel=None, noise_variance=0.001,
             kernel_lengthscale=None, kernel_variance=None, epochs=1000, positivity_constraint=1e-2, seed=0, *,
             optimizer="l-bfgs-b", lr=0.05, precision=None, reference_quirks=True, verbose=True):
    """Fit a vector-field GP on the manifold (RVGP/main.py:11-84)."""
    if train_ind is None:
        train_ind = np.arange(data.n)
    train_ind = np.asarray(train_ind)
    if kernel is None:
        kernel = ManifoldKernel(data, nu=3 / 2, kappa=5, typ="matern", sigma_f=1.0)
    elif isinstance(kernel, str):
        if kernel != "rbf":
            raise NotImplementedError(f"kernel={kernel!r}: use None (the manifold kernel) or 'rbf'")
        kernel = RBF()
        if verbose:
            print("Using RBF kernel, treating vectors channel-wise.")
    tr, te = train_test_split_indices(len(train_ind), test_size, seed)
    pts_train, pts_test = train_ind[tr], train_ind[te]
    set_default_positive_minimum(positivity_constraint)
    precision = precision or getattr(data, "precision", "mixed")
    noise0 = 1.0 if reference_quirks else noise_variance
    if isinstance(kernel, RBF):
        if n_inducing_points is not None:
            raise NotImplementedError("n_inducing_points with kernel='rbf' is not implemented in rvgp_gb300")
        GP = rbf_GPR(data, kernel, pts_train, noise_variance=noise0)
    elif n_inducing_points is None:
        GP = manifold_GPR(data, kernel, pts_train, noise_variance=noise0, precision=precision)
    else:
        GP = manifold_SGPR(data, kernel, pts_train, n_inducing_points=n_inducing_points, noise_variance=noise0,
                           precision=precision)
    # RVGP/main.py:69-75 assigns kernel.variance / kernel.lengthscales: GPflow's
    # names on the RBF kernel, sigma_f / kappa on the manifold kernel
    var_p, len_p = (kernel.variance, kernel.lengthscales) if isinstance(kernel, RBF) else (kernel.sigma_f, kernel.kappa)
    if kernel_variance is not None:
        var_p.assign(kernel_variance)
        var_p.trainable = False
    if kernel_lengthscale is not None:
        len_p.assign(kernel_lengthscale)
        len_p.trainable = False
    GP.optimize(epochs=epochs, method=optimizer, lr=lr, disp=verbose)
    if len(pts_test):
        mean, _ = GP.predict_points(pts_test)
        out_test = data._dev.vectors[torch.as_tensor(pts_test, device=mean.device, dtype=torch.long)]
        l2_error = float(torch.linalg.vector_norm(out_test - mean, dim=1).mean())
        if verbose:
            print("Relative l2 error is {}".format(l2_error))
        GP.l2_error = l2_error
    return GP
