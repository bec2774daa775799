"""Seeded synthetic point clouds and fields for the benchmark workloads.

Host-side numpy only (no GPU).  The shapes follow the five workloads the
benchmark is defined on:

* ``sphere``          uniform on the unit sphere S² in R³;
* ``torus``           torus R=1, r=0.35 in R³ with N(0, 0.01²) ambient jitter;
* ``swissroll64``     Swiss roll t∈[1.5π, 4.5π], height∈[0, 20], embedded in
                      R⁶⁴ by a seeded random orthogonal map + N(0, 0.02²) noise;
* ``half_ellipsoid``  upper half of the ellipsoid with semi-axes (1.0, 0.85, 1.1);
* ``bumpy_sphere``    S² with radius 1 + Σ of 32 Gaussian bumps (amplitude 0.1,
                      width 0.3) at seeded centres.
"""
from __future__ import annotations

import numpy as np


def _unit(rng, n, D=3):
    v = rng.standard_normal((n, D))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def make_points(kind: str, n: int, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    if kind == "sphere":
        return _unit(rng, n)
    if kind == "torus":
        R, r = 1.0, 0.35
        th, ph = rng.uniform(0, 2 * np.pi, size=(2, n))
        X = np.stack([(R + r * np.cos(th)) * np.cos(ph),
                      (R + r * np.cos(th)) * np.sin(ph),
                      r * np.sin(th)], axis=1)
        return X + 0.01 * rng.standard_normal(X.shape)
    if kind == "swissroll64":
        t = rng.uniform(1.5 * np.pi, 4.5 * np.pi, size=n)
        h = rng.uniform(0.0, 20.0, size=n)
        Y = np.stack([t * np.cos(t), h, t * np.sin(t)], axis=1)
        Q, _ = np.linalg.qr(rng.standard_normal((64, 64)))
        return Y @ Q[:3] + 0.02 * rng.standard_normal((n, 64))
    if kind == "half_ellipsoid":
        u = _unit(rng, n)
        u[:, 2] = np.abs(u[:, 2])
        return u * np.array([1.0, 0.85, 1.1])
    if kind == "bumpy_sphere":
        u = _unit(rng, n)
        c = _unit(rng, 32)
        d2 = ((u[:, None, :] - c[None, :, :]) ** 2).sum(-1)
        rad = 1.0 + 0.1 * np.exp(-d2 / (2 * 0.3 ** 2)).sum(1)
        return u * rad[:, None]
    raise ValueError(f"unknown point cloud kind {kind!r}")


def rotational_field(X: np.ndarray) -> np.ndarray:
    """∂/∂φ about the z axis, (-y, x, 0): the torus's rotational field."""
    return np.stack([-X[:, 1], X[:, 0], np.zeros(len(X))], axis=1)


def split(n: int, frac_train: float, seed: int = 0):
    """Seeded split into train / test point indices (a permutation, no repeats)."""
    perm = np.random.default_rng(seed).permutation(n)
    n_tr = int(round(frac_train * n))
    return np.sort(perm[:n_tr]), np.sort(perm[n_tr:])
