"""Geometry functions with the names of RVGP/geometry.py, computed on the GPU.

Inputs and outputs are numpy / scipy.sparse as in the reference.  The graph
returned by ``manifold_graph`` is a :class:`Graph` holding the symmetrised CSR
on the device (``to_networkx()`` gives the reference's networkx object).
"""
from __future__ import annotations

import math

import numpy as np
import scipy.sparse as sp
import torch

from rvgp_gb300 import _core


def _dev_array(x, dtype=torch.float64):
    _core.require_cuda()
    if isinstance(x, torch.Tensor):
        return x.to(device="cuda", dtype=dtype).contiguous()
    return torch.as_tensor(np.ascontiguousarray(x), device="cuda").to(dtype)


class Graph:
    """kNN graph + self-loops, symmetrised, as device CSR (RVGP/geometry.py:100-123)."""

    def __init__(self, X, indptr, indices, maxdeg):
        self.X, self.indptr, self.indices, self.maxdeg = X, indptr, indices, maxdeg

    def __len__(self):
        return self.indptr.numel() - 1

    def adjacency(self):
        n = len(self)
        ix = self.indices.cpu().numpy()
        return sp.csr_matrix((np.ones(ix.size), ix, self.indptr.cpu().numpy()), shape=(n, n))

    def to_networkx(self):
        import networkx as nx
        G = nx.from_scipy_sparse_array(self.adjacency())
        X = self.X.cpu().numpy()
        nx.set_node_attributes(G, {i: X[i] for i in G.nodes}, "pos")
        return G


def manifold_graph(X, typ="knn", n_neighbors=5):
    if typ != "knn":
        raise NotImplementedError("only typ='knn' graphs are built on the GPU")
    Xd = _dev_array(X)
    idx = _core.knn(Xd, n_neighbors)
    indptr, indices, maxdeg = _core.graph_build(idx)
    return Graph(Xd, indptr, indices, maxdeg)


def compute_laplacian(G, normalization=False):
    """L = D - A of the graph (RVGP/geometry.py:55-63), as scipy CSR."""
    if normalization:
        raise NotImplementedError("normalised Laplacian")
    vals = _core.laplacian_values(G.indptr, G.indices)
    n = len(G)
    return sp.csr_matrix((vals.cpu().numpy(), G.indices.cpu().numpy(), G.indptr.cpu().numpy()), shape=(n, n))


def compute_spectrum(laplacian, n_eigenpairs=None, dtype=None, precision="fp64"):
    """m smallest eigenpairs, eigenvectors scaled by sqrt(N) (RVGP/geometry.py:66-80)."""
    A = sp.csr_matrix(laplacian)
    A.sort_indices()
    N = A.shape[0]
    m = N if n_eigenpairs is None or n_eigenpairs >= N else int(n_eigenpairs)
    ev, V, _ = _core.eigsh(_dev_array(A.indptr, torch.int32), _dev_array(A.indices, torch.int32),
                           _dev_array(A.data), m=m, mode=precision, scale=math.sqrt(N))
    return ev.cpu().numpy(), V.cpu().numpy()


def manifold_dimension(Sigma, frac_explained=0.9):
    """RVGP/geometry.py:83-97 (prints the explained variance like the reference)."""
    if frac_explained == 1.0:
        return Sigma.shape[1]
    dim, var = _core.manifold_dimension(_dev_array(Sigma), frac_explained)
    print("Fraction of variance explained: ", var.cpu().numpy())
    if dim < 0:
        raise IndexError("no number of dimensions explains the requested fraction of variance")
    return int(dim)


def furthest_point_sampling(x, N=None, spacing=0.1, start_idx=0):
    """Greedy FPS (RVGP/geometry.py:126-162): (perm int32, lambdas)."""
    if spacing == 0.0:
        return np.arange(len(x)), None
    perm, lam = _core.fps(_dev_array(x), N=N, spacing=spacing, start_idx=start_idx)
    return perm.cpu().numpy(), lam.cpu().numpy()


def _frame(x, gauges, mode):
    g = _dev_array(gauges)
    out = _core.frame_map(g, g.shape[2], _dev_array(x), mode)
    return out.cpu().numpy()


def project_to_manifold(x, gauges):
    """RVGP/geometry.py:165-168."""
    return _frame(x, gauges, "project")


def express_in_local_frame(x, gauges, reverse=False):
    """RVGP/geometry.py:171-175."""
    return _frame(x, gauges, "from_local" if reverse else "to_local")
