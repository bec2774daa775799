"""Spectral manifold kernel with the surface of RVGP/kernels.py.

``ManifoldKernel(data, nu=3, kappa=4, sigma_f=1, typ='matern')`` keeps the
reference's constructor, its trainable parameters ``nu``, ``kappa``,
``sigma_f`` (positive, softplus-parameterised as GPflow's ``positive()``) and
the methods ``eval_S``, ``K``, ``K_diag`` and ``__call__`` (RVGP/kernels.py:25-67).
All arithmetic runs on the GPU; inputs and outputs of the public methods are
numpy arrays (CUDA tensors are accepted too).
"""
from __future__ import annotations

import math

import numpy as np
import torch

from rvgp_gb300 import _core

# GPflow's process-global default lower bound for positive parameters
# (gpflow.config.set_default_positive_minimum).  RVGP/main.py:52 sets it after
# the default kernel was created, so that kernel keeps the bound of its
# creation time; later kernels see the new value.
_DEFAULT_POSITIVE_MINIMUM = [0.0]


def set_default_positive_minimum(value):
    _DEFAULT_POSITIVE_MINIMUM[0] = float(value)


def default_positive_minimum():
    return _DEFAULT_POSITIVE_MINIMUM[0]


def _softplus(u):
    return u + math.log1p(math.exp(-u)) if u > 0 else math.log1p(math.exp(u))


def _inv_softplus(v):
    return v + math.log(-math.expm1(-v)) if v > 0 else float("-inf")


class Parameter:
    """A positive parameter: value = softplus(u) + lower, u unconstrained (GPflow ``positive()``)."""

    def __init__(self, value, lower=None, name=None, trainable=True):
        self.lower = default_positive_minimum() if lower is None else float(lower)
        self.name = name
        self.trainable = trainable
        self.assign(value)

    def assign(self, value):
        value = float(value)
        if value <= self.lower:
            raise ValueError(f"{self.name}: value {value} must exceed the lower bound {self.lower}")
        self.unconstrained = _inv_softplus(value - self.lower)

    def numpy(self):
        return np.float64(_softplus(self.unconstrained) + self.lower)

    def __float__(self):
        return float(self.numpy())

    def dvalue_du(self):
        """d value / d unconstrained = sigmoid(u)."""
        u = self.unconstrained
        return 1.0 / (1.0 + math.exp(-u)) if u >= 0 else math.exp(u) / (1.0 + math.exp(u))

    def __repr__(self):
        return f"Parameter({self.name}={float(self):.6g}, trainable={self.trainable})"


def _to_dev(X, device):
    if isinstance(X, torch.Tensor):
        return X.to(device=device, dtype=torch.float64).contiguous()
    return torch.as_tensor(np.ascontiguousarray(X, dtype=np.float64), device=device)


class ManifoldKernel:
    """Matérn / squared-exponential kernel on the connection-Laplacian eigenbasis."""

    def __init__(self, data, nu=3, kappa=4, sigma_f=1, typ="matern", dtype=np.float64):
        dev = data._dev
        self.data = data
        self.eigenvalues = dev.evals_Lc        # (m,) CUDA f64
        self.num_verticies = float(dev.X.shape[0] * dev.X.shape[1])  # rows of evecs_Lc: n * D
        self.dtype = dtype
        self.typ = typ
        if typ not in ("se", "matern"):
            raise NotImplementedError(f"kernel type {typ!r} (use 'matern' or 'se')")
        self.nu = Parameter(nu, name="nu") if typ == "matern" else None
        self.kappa = Parameter(kappa, name="kappa")
        self.sigma_f = Parameter(sigma_f, name="sigma_f")
        self.device = self.eigenvalues.device

    @property
    def eigenvectors(self):
        """The lifted eigenvectors evecs_Lc, (n*D, m) CUDA f64 (formed on first use)."""
        return self.data._evecs_Lc_dev()

    @property
    def parameters(self):
        return [p for p in (self.kappa, self.nu, self.sigma_f) if p is not None]

    def theta(self, noise=1.0):
        nu = float(self.nu) if self.nu is not None else 0.0
        return torch.tensor([nu, float(self.kappa), float(self.sigma_f), noise], dtype=torch.float64,
                            device=self.device)

    def _S(self):
        S, _ = _core.spectral_S(self.eigenvalues, self.theta(), self.num_verticies, self.typ, want_grad=False)
        return S

    def eval_S(self, typ="matern"):
        """Spectral weights S (RVGP/kernels.py:41-53)."""
        if typ != self.typ:
            k = ManifoldKernel.__new__(ManifoldKernel)
            k.__dict__.update(self.__dict__)
            k.typ = typ
            return k.eval_S(typ)
        return self._S().cpu().numpy()

    def K(self, X, X2=None):
        """(X S) X2ᵀ (RVGP/kernels.py:55-61)."""
        Xd = _to_dev(X, self.device)
        X2d = None if X2 is None else _to_dev(X2, self.device)
        return _core.kernel_matrix(Xd, self._S(), X2d).cpu().numpy()

    def K_diag(self, X):
        """diag((X S) Xᵀ) without forming the matrix (RVGP/kernels.py:63-67)."""
        return _core.kernel_diag(_to_dev(X, self.device), self._S()).cpu().numpy()

    def __call__(self, X, X2=None, full_cov=True):
        if not full_cov and X2 is None:
            return self.K_diag(X)
        return self.K(X, X2)


class RBF:
    """Squared-exponential kernel with GPflow ``kernels.RBF()``'s parameters and
    defaults (``variance`` = 1, ``lengthscales`` = 1, both positive), used by
    ``fit(..., kernel='rbf')`` on the scalar-Laplacian eigenbasis
    (RVGP/main.py:33-37):  K(x, x') = variance · exp(−½ |x − x'|² / lengthscales²)."""

    def __init__(self, variance=1.0, lengthscales=1.0):
        self.variance = Parameter(variance, name="variance")
        self.lengthscales = Parameter(lengthscales, name="lengthscales")

    @property
    def parameters(self):
        return [self.variance, self.lengthscales]

    def theta(self, noise=1.0, device="cuda"):
        return torch.tensor([float(self.variance), float(self.lengthscales), noise], dtype=torch.float64,
                            device=device)

    def K(self, X, X2=None):
        Xd = _to_dev(X, "cuda")
        X2d = None if X2 is None else _to_dev(X2, "cuda")
        return _core.rbf_matrix(Xd, self.theta(), X2d).cpu().numpy()

    def K_diag(self, X):
        return np.full(len(X), float(self.variance))

    def __call__(self, X, X2=None, full_cov=True):
        if not full_cov and X2 is None:
            return self.K_diag(X)
        return self.K(X, X2)
