"""Vector-field features on a point cloud (examples/eeg_example/eeg_utils.py:37-80).

``compute_vectorfield_features(positions, vectors, k=5)`` estimates the
divergence and curl of a 3-d field from each point's k nearest neighbours
(exact kNN on the GPU, as the reference's KD-tree query);
``compute_vectorfield_features_time`` does every time sample of a field
sequence in one launch.  With ``reference_quirks=True`` (default) the
difference vectors are taken against the unit vector of point 0 for every
point, as the reference computes them (``normalized_vectors[0]``,
eeg_utils.py:67); ``False`` uses each point's own vector.
"""
from __future__ import annotations

import numpy as np
import torch

from rvgp_gb300 import _core


def _dev(x):
    if isinstance(x, torch.Tensor):
        return x.to(device="cuda", dtype=torch.float64).contiguous()
    return torch.as_tensor(np.ascontiguousarray(x, dtype=np.float64), device="cuda")


def _features(positions, fields, k, reference_quirks):
    _core.require_cuda()
    P = _dev(positions)
    if P.ndim != 2 or P.shape[1] != 3:
        raise ValueError("positions must be (n, 3): the curl estimate is a 3-d cross product")
    V = _dev(fields)
    if V.shape[1:] != P.shape:
        raise ValueError(f"vectors must be (..., {P.shape[0]}, 3), got {tuple(V.shape)}")
    nbr = _core.knn(P, k)
    div, curl = _core.vectorfield_features(P, V, nbr, ref_first=reference_quirks)
    return div.cpu().numpy(), curl.cpu().numpy()


def compute_vectorfield_features(positions, vectors, k=5, reference_quirks=True):
    """div (n,), curl (n, 3) of the field ``vectors`` (n, 3) at ``positions`` (n, 3)."""
    div, curl = _features(positions, _dev(vectors)[None], k, reference_quirks)
    return div[0], curl[0]


def compute_vectorfield_features_time(timepoints, positions, vectors, k=5, reference_quirks=True):
    """div (T, n), curl (T, n, 3) of vectors[t] (vectors: (times, n, 3)) for t in
    ``timepoints``, all in one launch."""
    V = _dev(vectors)[torch.as_tensor(np.asarray(timepoints, dtype=np.int64), device="cuda")]
    return _features(positions, V.contiguous(), k, reference_quirks)
