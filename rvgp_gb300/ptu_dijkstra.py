"""Drop-in for the reference's native module ``ptu_dijkstra``
(RVGP/lib/ptu_dijkstra.pyx, imported by RVGP/dataclass.py:8 and called at
RVGP/dataclass.py:35,41): the same two functions with the same arguments,
return types and errors, computed by the CUDA kernels of this package.

    tangent_frames(X, G, d, K) -> (tangents (N, D, d) float64, Sigma (N, d) float64)
    connections(tangents, G, d) -> scipy.sparse.coo_matrix (N*d x N*d)

``G`` is the proximity graph as the reference receives it (a networkx graph,
read with ``nx.adjacency_matrix(G, weight='weight')`` as pyx:84/162 do) or
directly its scipy sparse adjacency matrix.  The graph is symmetrised as
pyx:96-101 does.  Its weights must be 1 (the reference's graphs come from
``kneighbors_graph(mode='connectivity')``, RVGP/geometry.py:103-112): the
device search counts hops, which is the reference's Dijkstra on unit weights.

A user of the reference switches with ``import rvgp_gb300.ptu_dijkstra as
ptu_dijkstra`` (or by putting this module first on the path under the name
``ptu_dijkstra``).  Inputs and outputs are host numpy / scipy objects, as the
Cython module's; the work runs on the current CUDA device.  Without a GPU the
functions raise (there is no CPU fallback).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

__all__ = ["tangent_frames", "connections", "expand_edge_index"]


def _symmetrised_csr(G):
    """CSR (indptr, indices) int32 of max(A, Aᵀ) for the graph G, as
    pyx:84-101 build it; raises if a weight is not 1."""
    if sp.issparse(G):
        A = sp.csr_matrix(G, dtype=np.float64)
    else:
        import networkx as nx
        A = sp.csr_matrix(nx.adjacency_matrix(G, weight="weight"), dtype=np.float64)
    if A.shape[0] != A.shape[1]:
        raise ValueError(f"the adjacency matrix must be square, got {A.shape}")
    if np.any(A.data < 0):
        raise ValueError("Graph has negative weights: negative distances are not allowed.")
    S = A.maximum(A.T.tocsr()).tocsr()
    S.sort_indices()
    S.eliminate_zeros()
    if S.nnz and not np.all(S.data == 1.0):
        raise ValueError("rvgp_gb300.ptu_dijkstra: only unit edge weights (hop distances) are supported, as the "
                         "reference's kneighbors_graph(mode='connectivity') graphs have")
    return S.indptr.astype(np.int32), S.indices.astype(np.int32)


def tangent_frames(X, G, d, K):
    """Local tangent frames from geodesic neighbourhoods (pyx:33-125).

    X (N, D); G the proximity graph; d the manifold dimension; K the
    neighbourhood size (K+1 nodes, truncated to an integer as the Cython
    signature does).  Returns the first d left singular vectors of every
    centred neighbourhood, (N, D, d), and its d largest singular values,
    (N, d).  Singular vectors are signed so that their largest entry is
    positive (the reference's carry LAPACK's arbitrary signs)."""
    import torch
    from rvgp_gb300 import _core
    X = np.ascontiguousarray(X, dtype=np.float64)
    N, D = X.shape
    K = int(K)
    d = int(d)
    if K >= N:
        raise ValueError("Geodesic neighborhood size must be less than the total number of samples")
    if K < d:
        raise ValueError("Geodesic neighborhood size must be larger or equal to the embedding dimension")
    if D < d:
        raise ValueError("Embedding dimension must be less or equal to the ambient dimension of input data")
    indptr, indices = _symmetrised_csr(G)
    if indptr.size != N + 1:
        raise ValueError(f"the graph has {indptr.size - 1} nodes, X has {N} points")
    _core.require_cuda()
    maxdeg = int(max(1, np.diff(indptr).max()))  # bounds the search's node pool (self-loops included)
    dev = torch.device("cuda", torch.cuda.current_device())
    T, S, _ = _core.gauges(torch.as_tensor(X, device=dev), torch.as_tensor(indptr, device=dev),
                           torch.as_tensor(indices, device=dev), K, maxdeg, d)
    Sigma = S[:, :d].cpu().numpy()
    if np.any(Sigma < 1e-10):
        raise RuntimeError("Local tangent space approximation failed, at least one geodesic neighborhood does not "
                           "span d-dimensional space")
    return np.ascontiguousarray(T.cpu().numpy()), np.ascontiguousarray(Sigma)


def expand_edge_index(edge_index, dim=1):
    """Rows / columns of the d x d blocks of every edge (pyx:202-214): edge
    (i, j) becomes entries (i*dim + p, j*dim + q), p, q < dim, edge-major with
    (p, q) row-major."""
    edge_index = np.asarray(edge_index)
    if dim == 1:
        return edge_index
    p, q = np.meshgrid(np.arange(dim), np.arange(dim), indexing="ij")
    rows = (edge_index[0][:, None] * dim + p.ravel()[None, :]).ravel()
    cols = (edge_index[1][:, None] * dim + q.ravel()[None, :]).ravel()
    return np.stack([rows, cols])


def connections(tangents, G, d):
    """Parallel transports between the frames of adjacent points (pyx:128-199):
    for every stored edge (i, j) of the symmetrised graph the orthogonal
    polar factor R_ij = U Vᵀ of T_iᵀ T_j, returned as the reference's sparse
    COO matrix of N*d x N*d with the blocks expanded by expand_edge_index."""
    import torch
    from rvgp_gb300 import _core
    T = np.ascontiguousarray(tangents, dtype=np.float64)
    if T.ndim != 3:
        raise ValueError(f"tangents must be (N, D, d), got shape {T.shape}")
    N, D, ld = T.shape
    d = int(d)
    if D < d:
        raise ValueError("Embedding dimension must be less or equal to the ambient dimension of input data")
    if ld < d:
        raise ValueError(f"tangents hold {ld} frame vectors, fewer than d={d}")
    indptr, indices = _symmetrised_csr(G)
    if indptr.size != N + 1:
        raise ValueError(f"the graph has {indptr.size - 1} nodes, tangents has {N} frames")
    _core.require_cuda()
    dev = torch.device("cuda", torch.cuda.current_device())
    R, _, _ = _core.connections(torch.as_tensor(T, device=dev), d, torch.as_tensor(indptr, device=dev),
                                torch.as_tensor(indices, device=dev), want_R=True, want64=False, want32=False)
    rows = np.repeat(np.arange(N), np.diff(indptr))
    edge_index = expand_edge_index(np.vstack([rows, indices]), dim=d)
    return sp.coo_matrix((R.cpu().numpy().ravel(), (edge_index[0], edge_index[1])))
