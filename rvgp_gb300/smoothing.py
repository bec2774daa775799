"""Diffusion with the names of RVGP/smoothing.py, computed on the GPU.

``method="matrix_exp"`` applies exp(-t A) exactly (Chebyshev–Bessel expansion
of the action; the reference forms the dense expm).  ``method="spectral"``
takes ``par = (evals, evecs)`` (orthonormal or scaled by sqrt(rows)) and
applies Φ e^{-tΛ} Φᵀ, the branch the reference intends at smoothing.py:17-32.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import torch

from rvgp_gb300 import _core
from rvgp_gb300.geometry import _dev_array


def _bound(A):
    return float(abs(A).sum(axis=1).max()) * (1.0 + 1e-12)


def scalar_diffusion(x, t, method="matrix_exp", par=None):
    x = np.asarray(x, dtype=np.float64)
    if x.ndim == 1:
        x = x[:, None]
    if method == "matrix_exp":
        A = sp.csr_matrix(par)
        A.sort_indices()
        out = []
        for c0 in range(0, x.shape[1], 4):
            out.append(_core.expm_action(_dev_array(A.indptr, torch.int32), _dev_array(A.indices, torch.int32),
                                         _dev_array(A.data), _dev_array(x[:, c0:c0 + 4]), t, _bound(A)))
        return torch.cat(out, dim=1).cpu().numpy()
    if method == "spectral":
        assert isinstance(par, (list, tuple)) and len(par) == 2, \
            "For spectral method, par must be a tuple of eigenvalues, eigenvectors!"
        evals, evecs = par
        Phi = _dev_array(evecs)
        Phi = Phi / torch.linalg.vector_norm(Phi, dim=0, keepdim=True)
        return _core.spectral_diffusion(Phi, _dev_array(evals), _dev_array(x), t).cpu().numpy()
    raise NotImplementedError


def vector_diffusion(x, t, Lc, L=None, method="spectral", normalise=True):
    """RVGP/smoothing.py:37-63."""
    x = np.asarray(x, dtype=np.float64)
    n, d = x.shape[0], x.shape[1]
    nd = Lc[1].shape[0] if method == "spectral" else Lc.shape[0]
    assert (n * d % nd) == 0, "Data dimension must be an integer multiple of the dimensions of the connection Laplacian!"
    out = scalar_diffusion(x.reshape(nd, -1), t, method, Lc).reshape(x.shape)
    if normalise:
        assert L is not None, "Need Laplacian for normalised diffusion!"
        x_abs = np.linalg.norm(x, axis=-1, keepdims=True)
        both = scalar_diffusion(np.concatenate([x_abs, np.ones((n, 1))], axis=1), t, method, L)
        out = out * both[:, :1] / (both[:, 1:] * np.linalg.norm(out, axis=-1, keepdims=True))
    return out
