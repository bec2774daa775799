"""Oracle: FP64 CPU restatement of the RVGP numerical core (test infrastructure).

This module is the checker for the CUDA path.  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg import it; the
product package ``rvgp_gb300`` never does.

Each function cites the reference code it restates (paths inside the
agosztolai/RVGP checkout).  Third-party arithmetic the reference delegates to
(sklearn ``kneighbors_graph`` / ``train_test_split`` / ``pairwise_distances``,
networkx Laplacians, scipy ARPACK, LAPACK ``dgesvd``, GPflow ``GPR`` and ``SGPR``)
is restated from its published semantics.  GPflow 2.6.5 and TensorFlow are absent here, so
the GP functions below are "parity unpinned" against GPflow itself: they are
pinned only by their internal consistency (dense vs low-rank algebra, finite
differences).  Everything up to and including the eigenpairs and the vector
diffusion is pinned against the reference's own code by the fixtures under
``tests/golden/``.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess

import numpy as np
import scipy.linalg
import scipy.sparse as sp
import scipy.sparse.linalg as spla

HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(HERE, "_build")
_LIB = None


# ----------------------------------------------------------------------------- build
def build_c(quiet=True):
    """Compile oracle/geonbh.c into oracle/_build/libgeonbh.so (gcc, portable flags)."""
    os.makedirs(_BUILD, exist_ok=True)
    src = os.path.join(HERE, "geonbh.c")
    so = os.path.join(_BUILD, "libgeonbh.so")
    if not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-O2", "-shared", "-fPIC", "-std=c99", src, "-o", so])
    return so


def _lib():
    global _LIB
    if _LIB is None:
        _LIB = ctypes.CDLL(build_c())
        f = _LIB.oracle_geodesic_neighbourhoods
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                      ctypes.c_int, ctypes.c_void_p]
    return _LIB


# ----------------------------------------------------------------------------- graph
def sq_dist_rows(A, B):
    """Exact FP64 squared distances, summed over coordinates in order 0..D-1.

    The per-coordinate terms are added left to right without fused
    multiply-add, which is the order a plain loop (and sklearn's kd-tree
    ``rdist``) uses.  Shape (len(A), len(B)).
    """
    out = np.zeros((A.shape[0], B.shape[0]))
    for j in range(A.shape[1]):
        diff = A[:, j, None] - B[None, :, j]
        out += diff * diff
    return out


def knn(X, k, chunk=2048):
    """k nearest neighbours of every point, excluding the point itself.

    Restates ``kneighbors_graph(X, k, mode='connectivity', include_self=False)``
    (RVGP/geometry.py:103-110) as an exact FP64 brute-force search.  Ties in
    distance are broken by the lower index.  Returns int32 (n, k), each row in
    ascending (distance, index) order.
    """
    X = np.ascontiguousarray(X, dtype=np.float64)
    n = X.shape[0]
    if k >= n:
        raise ValueError(f"Expected n_neighbors < n_samples, got {k} >= {n}")
    out = np.empty((n, k), dtype=np.int32)
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        d2 = sq_dist_rows(X[s:e], X)
        d2[np.arange(e - s), np.arange(s, e)] = np.inf
        part = np.argpartition(d2, k, axis=1)[:, : k + 1]
        for r in range(e - s):
            cand = part[r]
            dv = d2[r, cand]
            kth = np.sort(dv)[k - 1]
            # every point at the k-th distance competes, lowest index first
            sel = np.nonzero(d2[r] <= kth)[0]
            order = np.lexsort((sel, d2[r, sel]))
            out[s + r] = sel[order[:k]]
    return out


def knn_kdtree(X, k):
    """The k nearest neighbours by scipy's KD-tree, the tree search sklearn's
    ``kneighbors_graph`` uses for low-dimensional points (RVGP/geometry.py:103-110).
    The same lists as ``knn`` when distances do not tie; the timing form of the
    CPU baseline."""
    from scipy.spatial import KDTree
    X = np.ascontiguousarray(X, dtype=np.float64)
    idx = KDTree(X).query(X, k + 1)[1]
    out = np.empty((len(X), k), dtype=np.int32)
    for r in range(len(X)):  # drop the point itself wherever the tree returned it
        row = idx[r][idx[r] != r]
        out[r] = row[:k]
    return out


def knn_gemm(X, k, rows=None, chunk=2000, threads=None):
    """k nearest neighbours by brute force with the squared distances from
    the expansion |x|² + |y|² - 2 x·y (one matrix product per chunk of
    queries), the method sklearn's ``kneighbors_graph`` uses for
    high-dimensional points (RVGP/geometry.py:103-110; sklearn's 'auto' picks
    brute force above 15 dimensions).  The timing form of the CPU baseline at
    D = 64; ties may order differently from ``knn`` (FP64 rounding of the
    expansion).  ``rows``: query subset (default all points); chunks run on
    ``threads`` host threads (default all cores).  Returns int32 (len(rows), k)."""
    import os
    from concurrent.futures import ThreadPoolExecutor
    X = np.ascontiguousarray(X, dtype=np.float64)
    n = X.shape[0]
    if k >= n:
        raise ValueError(f"Expected n_neighbors < n_samples, got {k} >= {n}")
    q = np.arange(n) if rows is None else np.asarray(rows)
    xx = np.einsum("ij,ij->i", X, X)

    def one(s):
        r = q[s:s + chunk]
        D2 = xx[r, None] + xx[None, :] - 2.0 * (X[r] @ X.T)
        D2[np.arange(len(r)), r] = np.inf
        part = np.argpartition(D2, k, axis=1)[:, :k]
        o = np.argsort(np.take_along_axis(D2, part, 1), axis=1, kind="stable")
        return np.take_along_axis(part, o, 1)

    with ThreadPoolExecutor(threads or os.cpu_count()) as ex:
        return np.concatenate(list(ex.map(one, range(0, len(q), chunk)))).astype(np.int32)


def symmetrised_csr(knn_idx, n):
    """CSR (indptr, indices) of max(A, Aᵀ) with A = kNN connectivity + I.

    Restates RVGP/geometry.py:111-112 (``A += I``; undirected networkx graph)
    followed by ``nx.adjacency_matrix`` and the symmetrisation in
    RVGP/lib/ptu_dijkstra.pyx:84-103.  Column indices are sorted within each
    row; every stored weight is 1.0.
    """
    k = knn_idx.shape[1]
    rows = np.concatenate([np.repeat(np.arange(n), k), knn_idx.ravel(), np.arange(n)])
    cols = np.concatenate([knn_idx.ravel(), np.repeat(np.arange(n), k), np.arange(n)])
    A = sp.csr_matrix((np.ones(rows.size), (rows, cols)), shape=(n, n))
    A.sum_duplicates()
    A.sort_indices()
    return A.indptr.astype(np.int32), A.indices.astype(np.int32)


def laplacian(indptr, indices, n):
    """Combinatorial Laplacian L = D - A of the symmetrised graph.

    Restates ``nx.laplacian_matrix`` as used by RVGP/geometry.py:55-63: the
    self-loop adds 1 to both D and A, so the diagonal is the number of
    distinct neighbours and every off-diagonal stored entry is -1.
    """
    data = -np.ones(indices.size)
    rows = np.repeat(np.arange(n), np.diff(indptr))
    diag = rows == indices
    deg = np.diff(indptr) - 1
    data[diag] = deg
    return sp.csr_matrix((data, indices.copy(), indptr.copy()), shape=(n, n))


# ----------------------------------------------------------------------------- gauges
def geodesic_neighbourhoods(indptr, indices, K, weights=None):
    """First K+1 nodes scanned by the heap-based Dijkstra from every node.

    Restates RVGP/lib/ptu_dijkstra.pyx:361-394 with its Fibonacci heap
    (pyx:444-690), in C (oracle/geonbh.c).  Returns int32 (n, K+1) in scan order.
    """
    n = indptr.size - 1
    indptr = np.ascontiguousarray(indptr, dtype=np.int32)
    indices = np.ascontiguousarray(indices, dtype=np.int32)
    w = np.ones(indices.size) if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
    out = np.empty((n, K + 1), dtype=np.int32)
    st = _lib().oracle_geodesic_neighbourhoods(n, indptr.ctypes.data, indices.ctypes.data,
                                               w.ctypes.data, int(K), out.ctypes.data)
    if st != 0:
        raise RuntimeError(f"geodesic neighbourhood of point {st - 1} has fewer than K+1 nodes")
    return out


def tangent_frames(X, nbh, d):
    """Local PCA gauges: centred SVD of each geodesic neighbourhood.

    Restates RVGP/lib/ptu_dijkstra.pyx:396-434: centre the D x (K+1) block of
    neighbourhood coordinates, take its SVD, keep the first d left singular
    vectors (tangents, (n, D, d)) and singular values (Sigma, (n, d)).  Raises
    like pyx:119-123 when one of the d leading singular values is below 1e-10.
    Singular vectors carry LAPACK's arbitrary signs.
    """
    Y = X[nbh]                                      # (n, K+1, D)
    Y = Y - Y.mean(axis=1, keepdims=True)
    U, S, _ = np.linalg.svd(np.transpose(Y, (0, 2, 1)), full_matrices=False)
    if np.any(S[:, :d] < 1e-10):
        raise RuntimeError("Local tangent space approximation failed, at least one geodesic "
                           "neighborhood does not span d-dimensional space")
    return np.ascontiguousarray(U[:, :, :d]), np.ascontiguousarray(S[:, :d])


def manifold_dimension(Sigma, frac_explained=0.9):
    """RVGP/geometry.py:83-97 (without the in-place mutation of Sigma)."""
    if frac_explained == 1.0:
        return Sigma.shape[1]
    S = Sigma ** 2
    S = S / S.sum(1, keepdims=True)
    S = S.cumsum(1)
    var_exp = S.mean(0) - S.std(0)
    return int(np.where(var_exp >= frac_explained)[0][0] + 1)


def connections(gauges, indptr, indices):
    """Per stored edge (i, j) in CSR order: R_ij = U Vᵀ with U S Vᵀ = T_iᵀ T_j.

    Restates RVGP/lib/ptu_dijkstra.pyx:258-293.  Returns (E, d, d).
    """
    n = indptr.size - 1
    rows = np.repeat(np.arange(n), np.diff(indptr))
    M = np.einsum("eki,ekj->eij", gauges[rows], gauges[indices])
    U, _, Vt = np.linalg.svd(M)
    return U @ Vt


def connection_laplacian(L, R, indptr, indices, d):
    """Lc = kron(L, 1_{dxd}) ⊙ R as a CSR matrix of size nd x nd.

    Restates RVGP/geometry.py:14-52 (normalization=None): block (i, j) is
    L_ij R_ij, so the diagonal blocks are deg_i R_ii and the off-diagonal
    blocks -R_ij.
    """
    n = indptr.size - 1
    blocks = L.data[:, None, None] * R
    B = sp.bsr_matrix((blocks, indices, indptr), shape=(n * d, n * d))
    return B.tocsr()


def spectrum(M, m):
    """m smallest-magnitude eigenpairs, eigenvectors scaled by sqrt(rows).

    Restates RVGP/geometry.py:66-80 (``eigsh(which="SM")``); eigenvalues ascending.
    """
    N = M.shape[0]
    if m is None or m >= N:
        m = N
    evals, evecs = spla.eigsh(M, k=m, which="SM")
    order = np.argsort(evals)
    evals, evecs = evals[order], evecs[:, order]
    return evals, evecs * np.sqrt(len(evecs))


def spectrum_shift_invert(M, m, sigma=-1e-3):
    """Same eigenpairs as ``spectrum`` via shift-invert Lanczos (faster at large n)."""
    evals, evecs = spla.eigsh(M.tocsc(), k=m, sigma=sigma, which="LM")
    order = np.argsort(evals)
    evals, evecs = evals[order], evecs[:, order]
    return evals, evecs * np.sqrt(len(evecs))


def lift(gauges, evecs, m):
    """RVGP/dataclass.py:57-59: evecs_Lc[i] = T_i U_i, reshaped to (n*D, m)."""
    n, D, d = gauges.shape
    U = evecs.reshape(n, d, m)
    return np.einsum("bij,bjk->bik", gauges, U).reshape(n * D, m)


def data_object(X, n_neighbors=10, frac_geodesic_neighbours=1.5, explained_variance=0.8,
                n_eigenpairs=50, dim_man=None, eig="sm"):
    """The pipeline of RVGP/dataclass.py:22-89 as a dict of arrays."""
    n, D = X.shape
    K = int(n_neighbors * frac_geodesic_neighbours)
    nn = knn(X, n_neighbors)
    indptr, indices = symmetrised_csr(nn, n)
    nbh = geodesic_neighbourhoods(indptr, indices, K)
    d_req = min(D, K + 1)
    T, Sigma = tangent_frames(X, nbh, d_req)
    d = manifold_dimension(Sigma, explained_variance) if dim_man is None else dim_man
    T = np.ascontiguousarray(T[:, :, :d])
    R = connections(T, indptr, indices)
    L = laplacian(indptr, indices, n)
    Lc = connection_laplacian(L, R, indptr, indices, d)
    solve = spectrum if eig == "sm" else spectrum_shift_invert
    evals_L, evecs_L = solve(L, n_eigenpairs)
    evals_Lc, evecs = solve(Lc, n_eigenpairs)
    return dict(knn=nn, indptr=indptr, indices=indices, nbh=nbh, gauges=T, Sigma=Sigma,
                dim_man=d, R=R, L=L, Lc=Lc, evals_L=evals_L, evecs_L=evecs_L,
                evals_Lc=evals_Lc, evecs_Lc=lift(T, evecs, evecs.shape[1]))


# ----------------------------------------------------------------------------- fields
def project_to_manifold(x, gauges):
    """RVGP/geometry.py:165-168."""
    coeffs = np.einsum("bij,bi->bj", gauges, x)
    return np.einsum("bj,bij->bi", coeffs, gauges)


def express_in_local_frame(x, gauges, reverse=False):
    """RVGP/geometry.py:171-175."""
    if reverse:
        return np.einsum("bji,bi->bj", gauges, x)
    return np.einsum("bij,bi->bj", gauges, x)


def random_vector_field(X, gauges, seed=0):
    """RVGP/dataclass.py:91-103 (legacy numpy global RNG, as the reference)."""
    rs = np.random.RandomState(seed)
    v = rs.uniform(low=-0.5, high=0.5, size=X.shape)
    v = project_to_manifold(v, gauges)
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def vector_diffusion(x_local, t, L, Lc, exact="expm"):
    """RVGP/smoothing.py:37-63 with ``method="matrix_exp"``, ``normalise=True``.

    ``exact="expm"`` forms the dense exponential as the reference does
    (smoothing.py:13-15); ``exact="action"`` uses scipy's ``expm_multiply``,
    the same operator applied without forming it (for n beyond a few thousand).
    """
    n, d = x_local.shape

    def act(M, v):
        if exact == "expm":
            return scipy.linalg.expm(-t * M.toarray()) @ v
        return spla.expm_multiply(-t * M.tocsc(), v)

    out = act(Lc, x_local.reshape(n * d, 1)).reshape(n, d)
    x_abs = np.linalg.norm(x_local, axis=-1, keepdims=True)
    out_abs = act(L, x_abs)
    ind = act(L, np.ones((n, 1)))
    return out * out_abs / (ind * np.linalg.norm(out, axis=-1, keepdims=True))


def smooth_vector_field(vectors, gauges, L, Lc, t, exact="expm"):
    """RVGP/dataclass.py:105-120."""
    loc = express_in_local_frame(vectors, gauges)
    loc = vector_diffusion(loc, t, L, Lc, exact=exact)
    return express_in_local_frame(loc, gauges, reverse=True)


def spectral_diffusion(x_local, t, evals_L, evecs_L, evals_Lc, evecs_Lc_local):
    """Truncated spectral form Φ e^{-tΛ} Φᵀ x of the same diffusion (the
    ``method="spectral"`` branch of RVGP/smoothing.py:17-32, written as intended).
    Eigenvectors are expected orthonormal (not scaled by sqrt(rows))."""
    n, d = x_local.shape

    def act(lam, phi, v):
        return phi @ (np.exp(-t * lam)[:, None] * (phi.T @ v))

    out = act(evals_Lc, evecs_Lc_local, x_local.reshape(n * d, 1)).reshape(n, d)
    x_abs = np.linalg.norm(x_local, axis=-1, keepdims=True)
    out_abs = act(evals_L, evecs_L, x_abs)
    ind = act(evals_L, evecs_L, np.ones((n, 1)))
    return out * out_abs / (ind * np.linalg.norm(out, axis=-1, keepdims=True))


# ----------------------------------------------------------------------------- sampling
def furthest_point_sampling(x, N=None, spacing=0.1, start_idx=0):
    """RVGP/geometry.py:126-162 with exact FP64 direct-difference distances.

    Greedy: argmax (first index on ties) of the running minimum distance.
    Row distances are computed on the fly instead of as an n x n matrix.
    """
    if spacing == 0.0:
        return np.arange(len(x)), None
    x = np.asarray(x, dtype=np.float64)
    n_pts = len(x)
    diam = None
    if N is None:
        diam = 0.0
        for s in range(0, n_pts, 1024):
            diam = max(diam, float(np.sqrt(sq_dist_rows(x[s:s + 1024], x).max())))
    n = n_pts if N is None else N
    perm = np.zeros(n, dtype=np.int32)
    perm[0] = start_idx
    lambdas = np.zeros(n)
    ds = np.sqrt(sq_dist_rows(x[start_idx:start_idx + 1], x)[0])
    for i in range(1, n):
        idx = int(np.argmax(ds))
        perm[i] = idx
        lambdas[i] = ds[idx]
        ds = np.minimum(ds, np.sqrt(sq_dist_rows(x[idx:idx + 1], x)[0]))
        if N is None and lambdas[i] / diam < spacing:
            perm = perm[:i]
            lambdas = lambdas[:i]
            break
    return perm, lambdas


# ----------------------------------------------------------------------------- GP
def train_test_split_indices(n_samples, test_size=0.2, seed=0):
    """Index split of sklearn ``train_test_split(..., test_size, random_state)``
    as called at RVGP/main.py:40-45: ShuffleSplit with a RandomState(seed)
    permutation; the first ceil(test_size*n) entries are the test part."""
    n_test = int(math.ceil(test_size * n_samples))
    n_train = n_samples - n_test
    perm = np.random.RandomState(seed).permutation(n_samples)
    return perm[n_test:n_test + n_train], perm[:n_test]


def eval_S(evals, nu, kappa, sigma_f, n_rows, typ="matern"):
    """RVGP/kernels.py:41-53: s = (λ + 2ν/κ²)^(-ν) (Matérn) or exp(-λκ²/2) (SE),
    normalised to sum n_rows, times sigma_f."""
    if typ == "matern":
        s = (evals + 2.0 * nu / kappa ** 2) ** (-nu)
    else:
        s = np.exp(-0.5 * evals * kappa ** 2)
    return s * (n_rows / s.sum()) * sigma_f


def kernel_K(X, S, X2=None):
    """RVGP/kernels.py:55-61."""
    X2 = X if X2 is None else X2
    return (X * S) @ X2.T


def softplus(u):
    return np.logaddexp(0.0, u)


def inv_softplus(v):
    return v + np.log(-np.expm1(-v))


def lml_dense(Phi, y, S, noise):
    """log N(y | 0, Φ diag(S) Φᵀ + σ² I) by a dense Cholesky (GPflow GPR)."""
    N = Phi.shape[0]
    Ky = kernel_K(Phi, S) + noise * np.eye(N)
    Lc = np.linalg.cholesky(Ky)
    a = scipy.linalg.solve_triangular(Lc, y, lower=True)
    return float(-0.5 * a @ a - np.log(np.diag(Lc)).sum() - 0.5 * N * np.log(2 * np.pi))


def lml_lowrank(Phi, y, S, noise):
    """Same quantity through the rank-m Woodbury identity and determinant lemma."""
    N, m = Phi.shape
    r = np.sqrt(S)
    C = Phi.T @ Phi
    A = np.eye(m) + (r[:, None] * C * r[None, :]) / noise
    LA = np.linalg.cholesky(A)
    b = r * (Phi.T @ y)
    z = scipy.linalg.solve_triangular(LA, b, lower=True)
    quad = (y @ y - z @ z / noise) / noise
    logdet = N * np.log(noise) + 2.0 * np.log(np.diag(LA)).sum()
    return float(-0.5 * quad - 0.5 * logdet - 0.5 * N * np.log(2 * np.pi))


def lml_grad_S_noise(Phi, y, S, noise):
    """∂LML/∂S (m,) and ∂LML/∂σ² from the dense formulas:
    g_l = ½[(Φᵀα)_l² − (Φᵀ K_y⁻¹ Φ)_ll],  ∂/∂σ² = ½(αᵀα − tr K_y⁻¹)."""
    N = Phi.shape[0]
    Ky = kernel_K(Phi, S) + noise * np.eye(N)
    Kinv = np.linalg.inv(Ky)
    alpha = Kinv @ y
    pa = Phi.T @ alpha
    gS = 0.5 * (pa ** 2 - ((Kinv @ Phi) * Phi).sum(0))
    gn = 0.5 * (alpha @ alpha - np.trace(Kinv))
    return gS, gn


def predict_f(Phi, y, S, noise, Phi_new):
    """GPflow ``GPR.predict_f(full_cov=False)``: mean K*ᵀK_y⁻¹y and the marginal
    variance diag K** − diag(K*ᵀK_y⁻¹K*) (no noise), dense Cholesky."""
    N = Phi.shape[0]
    Ky = kernel_K(Phi, S) + noise * np.eye(N)
    Lc = np.linalg.cholesky(Ky)
    Ks = kernel_K(Phi, S, Phi_new)
    A = scipy.linalg.solve_triangular(Lc, Ks, lower=True)
    v = scipy.linalg.solve_triangular(Lc, y, lower=True)
    mean = A.T @ v
    var = np.einsum("ij,ij->i", Phi_new * S, Phi_new) - (A * A).sum(0)
    return mean, var


def predict_f_lowrank(Phi, y, S, noise, Phi_new):
    """Same posterior in weight space: w = S^½ A⁻¹ S^½ Φᵀy/σ², cov = S^½ A⁻¹ S^½."""
    m = Phi.shape[1]
    r = np.sqrt(S)
    A = np.eye(m) + (r[:, None] * (Phi.T @ Phi) * r[None, :]) / noise
    LA = np.linalg.cholesky(A)
    b = r * (Phi.T @ y) / noise
    w = r * scipy.linalg.cho_solve((LA, True), b)
    mean = Phi_new @ w
    B = scipy.linalg.solve_triangular(LA, (Phi_new * r).T, lower=True)
    return mean, (B * B).sum(0)


# ----------------------------------------------------------------------------- sparse GP (SGPR)
SGPR_JITTER = 1e-6  # gpflow.config.default_jitter(), added to Kuu


def sgpr_elbo(Phi, y, S, noise, Z, jitter=SGPR_JITTER):
    """Collapsed variational bound of GPflow 2.6.5 ``SGPR.elbo`` (Titsias 2009)
    for the manifold kernel, as built at RVGP/main.py:59-67,119-121.

    Kuu = K(Z, Z) + jitter I = L Lᵀ,  A = L⁻¹ K(Z, X) / σ,  B = I + A Aᵀ = L_B L_Bᵀ,
    c = L_B⁻¹ A y / σ;
    bound = −½N log 2π − Σ log diag L_B − ½N log σ² − ½ yᵀy/σ² + ½ cᵀc
            − ½ Σ diag K(X, X)/σ² + ½ tr(A Aᵀ).
    """
    N = Phi.shape[0]
    M = Z.shape[0]
    Kuu = kernel_K(Z, S) + jitter * np.eye(M)
    Kuf = kernel_K(Z, S, Phi)
    L = np.linalg.cholesky(Kuu)
    sigma = np.sqrt(noise)
    A = scipy.linalg.solve_triangular(L, Kuf, lower=True) / sigma
    AAT = A @ A.T
    LB = np.linalg.cholesky(np.eye(M) + AAT)
    c = scipy.linalg.solve_triangular(LB, A @ y, lower=True) / sigma
    kdiag = (Phi * Phi) @ S
    bound = -0.5 * N * np.log(2 * np.pi) - np.log(np.diag(LB)).sum() - 0.5 * N * np.log(noise)
    bound += -0.5 * (y @ y) / noise + 0.5 * (c @ c)
    bound += -0.5 * kdiag.sum() / noise + 0.5 * np.trace(AAT)
    return float(bound)


def sgpr_elbo_dense(Phi, y, S, noise, Z, jitter=SGPR_JITTER):
    """The same bound in its defining N-space form:
    log N(y | 0, Q + σ² I) − ½ tr(K − Q)/σ²,  Q = K(X, Z) Kuu⁻¹ K(Z, X)."""
    N = Phi.shape[0]
    M = Z.shape[0]
    Kuu = kernel_K(Z, S) + jitter * np.eye(M)
    Kuf = kernel_K(Z, S, Phi)
    Q = Kuf.T @ np.linalg.solve(Kuu, Kuf)
    Lc = np.linalg.cholesky(Q + noise * np.eye(N))
    a = scipy.linalg.solve_triangular(Lc, y, lower=True)
    lml = -0.5 * a @ a - np.log(np.diag(Lc)).sum() - 0.5 * N * np.log(2 * np.pi)
    return float(lml - 0.5 * (np.einsum("ij,ij->i", Phi * S, Phi).sum() - np.trace(Q)) / noise)


def sgpr_predict_f(Phi, y, S, noise, Z, Phi_new, jitter=SGPR_JITTER):
    """GPflow 2.6.5 ``SGPR.predict_f(full_cov=False)``: mean tmp2ᵀ c and the
    marginal variance diag K** + colsum(tmp2²) − colsum(tmp1²), with
    tmp1 = L⁻¹ K(Z, X*), tmp2 = L_B⁻¹ tmp1."""
    M = Z.shape[0]
    Kuu = kernel_K(Z, S) + jitter * np.eye(M)
    Kuf = kernel_K(Z, S, Phi)
    Kus = kernel_K(Z, S, Phi_new)
    sigma = np.sqrt(noise)
    L = np.linalg.cholesky(Kuu)
    A = scipy.linalg.solve_triangular(L, Kuf, lower=True) / sigma
    LB = np.linalg.cholesky(A @ A.T + np.eye(M))
    c = scipy.linalg.solve_triangular(LB, A @ y, lower=True) / sigma
    tmp1 = scipy.linalg.solve_triangular(L, Kus, lower=True)
    tmp2 = scipy.linalg.solve_triangular(LB, tmp1, lower=True)
    mean = tmp2.T @ c
    var = np.einsum("ij,ij->i", Phi_new * S, Phi_new) + (tmp2 * tmp2).sum(0) - (tmp1 * tmp1).sum(0)
    return mean, var


# ----------------------------------------------------------------------------- RBF GP (kernel='rbf')
def rbf_K(X, X2, variance, lengthscale):
    """GPflow 2.6.5 ``kernels.RBF`` as used at RVGP/main.py:33-37:
    variance · exp(−½ |x − x'|² / lengthscale²)."""
    d2 = ((X[:, None, :] - X2[None, :, :]) ** 2).sum(-1)
    return variance * np.exp(-0.5 * d2 / lengthscale ** 2)


def rbf_gpr_lml(X, Y, variance, lengthscale, noise):
    """GPflow ``GPR.log_marginal_likelihood`` with D output columns sharing the
    kernel (RVGP/main.py:36,55-58): Σ_c log N(y_c | 0, K + σ² I)."""
    N, D = Y.shape
    Lc = np.linalg.cholesky(rbf_K(X, X, variance, lengthscale) + noise * np.eye(N))
    a = scipy.linalg.solve_triangular(Lc, Y, lower=True)
    return float(-0.5 * (a * a).sum() - D * np.log(np.diag(Lc)).sum() - 0.5 * N * D * np.log(2 * np.pi))


def rbf_gpr_predict_f(X, Y, variance, lengthscale, noise, Xs):
    """GPflow ``GPR.predict_f(full_cov=False)``: mean (Nte, D) and the marginal
    variance (Nte,), the same for every output column."""
    N = X.shape[0]
    Lc = np.linalg.cholesky(rbf_K(X, X, variance, lengthscale) + noise * np.eye(N))
    Ks = rbf_K(X, Xs, variance, lengthscale)
    A = scipy.linalg.solve_triangular(Lc, Ks, lower=True)
    V = scipy.linalg.solve_triangular(Lc, Y, lower=True)
    return A.T @ V, variance - (A * A).sum(0)


# ----------------------------------------------------------------------------- vector-field features
def vectorfield_features(positions, vectors, k=5, reference_quirks=True, kdtree=False):
    """Divergence and curl estimates of examples/eeg_example/eeg_utils.py:46-80:
    unit vectors u; for each neighbour i of point j (the k nearest, exact
    search, lower index first on ties) Δp = p_i − p_j, Δu = u_i − u_ref,
    div_j = mean (Δu·Δp)/|Δp|², curl_j = mean (Δu × Δp)/|Δp|²; u_ref = u_0 for
    every j as the reference computes it (eeg_utils.py:67), u_j otherwise.
    ``kdtree=True`` finds the neighbours with scipy's KD-tree, as the reference
    does (eeg_utils.py:54-60; the same neighbours when distances do not tie),
    which is the fast CPU form used as the timing baseline."""
    P = np.asarray(positions, dtype=np.float64)
    U = vectors / np.linalg.norm(vectors, axis=1)[:, None]
    if kdtree:
        from scipy.spatial import KDTree
        nbr = KDTree(P).query(P, k + 1)[1][:, 1:]
    else:
        nbr = knn(P, k)
    dp = P[nbr] - P[:, None, :]                       # (n, k, 3)
    ref = U[0][None, None, :] if reference_quirks else U[:, None, :]
    du = U[nbr] - ref
    r2 = np.linalg.norm(dp, axis=2) ** 2
    div = ((du * dp).sum(2) / r2).sum(1) / k
    curl = (np.cross(du, dp) / r2[:, :, None]).sum(1) / k
    return div, curl
