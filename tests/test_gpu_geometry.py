"""GPU parity: graph, gauges, connections and the sparse products against the
oracle and the reference's golden fixtures (all through the C ABI)."""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

from conftest import load_golden, projector_distance
from oracle import rvgp_oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def core():
    from rvgp_gb300 import _core
    _core.require_cuda()
    return _core


def cu(a, dtype=torch.float64):
    return torch.as_tensor(np.ascontiguousarray(a)).to("cuda", dtype)


@pytest.mark.parametrize("name", ["sphere", "torus", "ellipsoid", "swissroll64"])
def test_knn_and_graph_match_reference(core, name):
    g = load_golden(name)
    X, k = g["X"], int(g["k"])
    idx = core.knn(cu(X), k).cpu().numpy()
    assert np.array_equal(idx, O.knn(X, k))
    indptr, indices, maxdeg = core.graph_build(torch.as_tensor(idx).cuda())
    assert np.array_equal(indptr.cpu().numpy(), g["indptr"])
    assert np.array_equal(indices.cpu().numpy(), g["indices"])
    assert maxdeg == int(np.diff(g["indptr"]).max() - 1)
    vals = core.laplacian_values(indptr, indices).cpu().numpy()
    assert np.array_equal(vals, g["L_data"])


@pytest.mark.parametrize("kind,n,k", [("sphere", 5000, 10), ("torus", 6000, 20), ("swissroll64", 3000, 15),
                                      ("bumpy_sphere", 4000, 20)])
def test_knn_random_clouds(core, kind, n, k):
    from rvgp_gb300.workloads import make_points
    X = make_points(kind, n, seed=3)
    idx = core.knn(cu(X), k).cpu().numpy()
    assert np.array_equal(idx, O.knn(X, k))


def test_knn_exact_ties_and_fallback(core):
    """A lattice: FP32 cannot separate the many exactly tied distances, so rows
    go to the exact FP64 scan; ties resolve to the lower index."""
    g = np.stack(np.meshgrid(np.arange(9), np.arange(9), np.arange(9), indexing="ij"), -1)
    X = g.reshape(-1, 3).astype(float) * 0.37 + 5.0
    for k in (6, 18, 7):
        idx = core.knn(cu(X), k).cpu().numpy()
        assert np.array_equal(idx, O.knn(X, k))
    # k = 7 cuts the 12-point shell at distance sqrt(2) spacing: FP32 cannot certify it
    assert core.lib().rvgp_knn_fallback_rows(len(X), 3, 7, core.ptr(core.knn.last_ws), core.stream()) > 0


def test_knn_duplicates_and_small(core):
    rng = np.random.default_rng(5)
    X = rng.standard_normal((40, 3))
    X[10] = X[3]
    X[11] = X[3]
    for k in (1, 5, 39):
        idx = core.knn(cu(X), k).cpu().numpy()
        assert np.array_equal(idx, O.knn(X, k))
    with pytest.raises(ValueError):
        core.knn(cu(X), 40)


@pytest.mark.parametrize("name", ["sphere", "torus", "ellipsoid", "swissroll64"])
def test_gauges_match_reference(core, name):
    g = load_golden(name)
    X, K, d = g["X"], int(g["K"]), int(g["dim_man"])
    n, D = X.shape
    ip, ix = cu(g["indptr"], torch.int32), cu(g["indices"], torch.int32)
    maxdeg = int(np.diff(g["indptr"]).max() - 1)
    c = min(D, K + 1)
    T, S, nbh = core.gauges(cu(X), ip, ix, K, maxdeg, d_out=min(c, 4), return_nbh=True)
    nbh = nbh.cpu().numpy()
    # exact neighbourhood sets and scan order of the reference's heap
    assert np.array_equal(nbh, O.geodesic_neighbourhoods(g["indptr"], g["indices"], K))
    Sg = g["Sigma"]
    np.testing.assert_allclose(S.cpu().numpy()[:, :Sg.shape[1]], Sg, rtol=1e-11, atol=1e-13)
    T = T.cpu().numpy()
    assert projector_distance(T[:, :, :d], g["gauges"]) < 1e-11
    # orthonormal columns
    G = np.einsum("nki,nkj->nij", T, T)
    assert np.abs(G - np.eye(T.shape[2])).max() < 1e-12


def test_gauges_pool_overflow_fallback(core):
    """k = 40 (K = 60): about 40 % of the searches touch more nodes than the
    256-slot shared-memory pool holds and are redone by the global-memory
    search; every neighbourhood must still equal the oracle's heap order."""
    from rvgp_gb300.workloads import make_points
    X = make_points("sphere", 3000, seed=4)
    k, K = 40, 60
    nn = O.knn(X, k)
    ipn, ixn = O.symmetrised_csr(nn, len(X))
    maxdeg = int(np.diff(ipn).max() - 1)
    T, S, nbh = core.gauges(cu(X), cu(ipn, torch.int32), cu(ixn, torch.int32), K, maxdeg, 2, return_nbh=True)
    assert np.array_equal(nbh.cpu().numpy(), O.geodesic_neighbourhoods(ipn, ixn, K))
    Tr, Sr = O.tangent_frames(X, O.geodesic_neighbourhoods(ipn, ixn, K), 3)
    np.testing.assert_allclose(S.cpu().numpy(), Sr, rtol=1e-10, atol=1e-13)
    assert projector_distance(T.cpu().numpy(), Tr[:, :, :2]) < 1e-10


def test_gauges_component_too_small(core):
    # two far-apart clusters of 5 points each: K=6 cannot be met inside a component
    rng = np.random.default_rng(0)
    X = np.concatenate([rng.standard_normal((5, 3)), 100 + rng.standard_normal((5, 3))])
    idx = core.knn(cu(X), 3)
    ip, ix, maxdeg = core.graph_build(idx)
    with pytest.raises(RuntimeError):
        core.gauges(cu(X), ip, ix, 6, maxdeg, 2)


@pytest.mark.parametrize("name", ["sphere", "torus", "swissroll64"])
def test_connections_and_lc(core, name):
    g = load_golden(name)
    d = int(g["dim_man"])
    ip, ix = cu(g["indptr"], torch.int32), cu(g["indices"], torch.int32)
    # with the reference's own gauges the transports must equal the reference's R
    R, v64, v32 = core.connections(cu(g["gauges"]), d, ip, ix)
    np.testing.assert_allclose(R.cpu().numpy(), g["R"], atol=1e-13)
    n = len(g["X"])
    L = O.laplacian(g["indptr"], g["indices"], n)
    Lc = O.connection_laplacian(L, g["R"], g["indptr"], g["indices"], d)
    Lc_gpu = sp.bsr_matrix((v64.cpu().numpy(), g["indices"], g["indptr"]), shape=Lc.shape).tocsr()
    assert abs(Lc_gpu - Lc).max() < 1e-12
    np.testing.assert_allclose(v32.cpu().numpy(), v64.cpu().numpy().astype(np.float32), rtol=0, atol=0)


@pytest.mark.parametrize("d,dtype,b", [(1, torch.float64, 6), (2, torch.float64, 40), (2, torch.float32, 64),
                                       (3, torch.float32, 8), (1, torch.float32, 12), (1, torch.float32, 4),
                                       (2, torch.float32, 228), (2, torch.float64, 228), (4, torch.float32, 20),
                                       (3, torch.float64, 130), (1, torch.float32, 1040), (2, torch.float32, 564),
                                       (2, torch.float64, 564), (1, torch.float32, 564), (2, torch.float32, 132)])
def test_bspmm(core, d, dtype, b):
    # widths above 32 column groups (128 FP32 / 64 FP64 columns) run the
    # column-chunked kernel, narrower ones the row-per-warp kernel
    rng = np.random.default_rng(d * 100 + b)
    n = 700
    A = sp.random(n, n, density=0.02, random_state=1, format="csr") + sp.eye(n)
    A.sort_indices()
    blocks = rng.standard_normal((A.nnz, d, d))
    M = sp.bsr_matrix((blocks, A.indices, A.indptr), shape=(n * d, n * d))
    X = rng.standard_normal((n * d, b))
    Z = rng.standard_normal((n * d, b))
    ref = 0.7 * (M @ X) - 0.3 * X + 1.9 * Z
    vals = cu(blocks if d > 1 else blocks[:, 0, 0], dtype)
    Y = core.bspmm(cu(A.indptr, torch.int32), cu(A.indices, torch.int32), vals, cu(X, dtype), Z=cu(Z, dtype),
                   alpha=0.7, beta=-0.3, gamma=1.9)
    tol = 1e-12 if dtype == torch.float64 else 2e-5
    np.testing.assert_allclose(Y.cpu().double().numpy(), ref, atol=tol * np.abs(ref).max())


@pytest.mark.parametrize("d,dtype,b", [(1, torch.float32, 564), (2, torch.float32, 564), (2, torch.float64, 130),
                                       (3, torch.float32, 40), (4, torch.float64, 8), (1, torch.float64, 6),
                                       (2, torch.float32, 4)])
@pytest.mark.parametrize("variant", [None, "8", "9", "10"])
def test_bspmm_planned_same_bits(core, d, dtype, b, variant, monkeypatch):
    """The planned product (tuned, or forced: 8 = tiled with halo rows staged
    in shared memory, 9 / 10 = grouped, merged neighbour lists of 4 rows)
    gives the bits of the plain product: tiles of 32 rows with ragged last
    column chunks, empty rows, a tile whose halo exceeds the shared-memory
    budget and one with more than 2048 entries (both gather from global
    memory), a last tile of fewer than 32 rows and a last group of one row,
    a hub row longer than the merge's look-ahead, and rows whose entries are
    in shuffled (conflicting) orders."""
    if variant is not None:
        monkeypatch.setenv("RVGP_SPMM_VARIANT", variant)
    rng = np.random.default_rng(7 * d + b)
    n = 1000 + 17
    A = sp.random(n, n, density=0.012, random_state=3, format="lil")
    A[40:72, :] = 0.0                      # tile 1: rows 40..63 empty, ...
    A[70, rng.choice(n, 900, replace=False)] = 1.0   # ... tile 2: halo above every budget
    A[128:160, :] = sp.random(32, n, density=0.08, random_state=4).tolil()  # tile 4: > 2048 entries
    A = (A.tocsr() + sp.eye(n)).tocsr()
    A.sort_indices()
    ind = A.indices.copy()
    for i in range(200, 240):  # rows 200..239 in shuffled orders
        s0, s1 = A.indptr[i], A.indptr[i + 1]
        ind[s0:s1] = rng.permutation(ind[s0:s1])
    A = sp.csr_matrix((A.data, ind, A.indptr), shape=A.shape)
    blocks = rng.standard_normal((A.nnz, d, d))
    X = rng.standard_normal((n * d, b))
    Z = rng.standard_normal((n * d, b))
    vals = cu(blocks if d > 1 else blocks[:, 0, 0], dtype)
    ip, ix = cu(A.indptr, torch.int32), cu(A.indices, torch.int32)
    plan = core.spmm_plan(ip, ix, d)
    for beta, Zt in ((-0.3, cu(Z, dtype)), (0.0, None)):
        monkeypatch.delenv("RVGP_SPMM_VARIANT", raising=False)
        ref = core.bspmm(ip, ix, vals, cu(X, dtype), Z=Zt, alpha=0.7, beta=beta, gamma=1.9)
        if variant is not None:
            monkeypatch.setenv("RVGP_SPMM_VARIANT", variant)
        got = core.bspmm(ip, ix, vals, cu(X, dtype), Z=Zt, alpha=0.7, beta=beta, gamma=1.9, plan=plan)
        torch.cuda.synchronize()
        assert torch.equal(got, ref)
    M = sp.bsr_matrix((blocks, ind, A.indptr), shape=(n * d, n * d))
    want = 0.7 * (M @ X) - 0.3 * X + 1.9 * Z
    got = core.bspmm(ip, ix, vals, cu(X, dtype), Z=cu(Z, dtype), alpha=0.7, beta=-0.3, gamma=1.9, plan=plan)
    tol = 1e-12 if dtype == torch.float64 else 2e-5
    np.testing.assert_allclose(got.cpu().double().numpy(), want, atol=tol * np.abs(want).max())


@pytest.mark.parametrize("D,n,k", [(20, 3001, 10), (33, 2500, 15), (64, 4100, 15), (64, 700, 1), (48, 1500, 60),
                                   (40, 50, 5), (17, 129, 8), (64, 129, 20)])
def test_knn_tensor_core_screen(core, D, n, k):
    """The tensor-core screen (16 < D <= 64: block-centred split-TF32
    distances, certified bound) gives the oracle's exact neighbour lists and
    the SIMT screen's (RVGP_KNN_TC=0): a cloud near a 3-dimensional manifold
    embedded in D dimensions, tiles cut short (n not a multiple of 128, a
    single partial block, a full block and one more point, the smallest D
    routed to the tensor cores), two duplicated points and a pair at exactly
    equal distances."""
    import os
    rng = np.random.default_rng(D * 1000 + n)
    t = rng.uniform(0, 3, (n, 3))
    Q, _ = np.linalg.qr(rng.standard_normal((D, D)))
    X = np.concatenate([np.sin(t), np.cos(t)], axis=1) @ Q[:6] + 0.01 * rng.standard_normal((n, D))
    X[5] = X[17]
    X[40] = X[17]
    X[41] = 2 * X[42] - X[43]  # 42 is the midpoint of 41 and 43
    idx = core.knn(cu(X), k).cpu().numpy()
    old = os.environ.get("RVGP_KNN_TC")
    os.environ["RVGP_KNN_TC"] = "0"
    try:
        idx0 = core.knn(cu(X), k).cpu().numpy()
    finally:
        if old is None:
            del os.environ["RVGP_KNN_TC"]
        else:
            os.environ["RVGP_KNN_TC"] = old
    assert np.array_equal(idx, idx0)
    assert np.array_equal(idx, O.knn(X, k))


@pytest.mark.parametrize("kind", ["clusters", "manifold_and_clusters"])
def test_knn_tensor_core_rescreen_lists(core, kind):
    """Rows the tensor-core certificate cannot settle go to the SIMT re-screen
    as a list (its partial lists indexed by list slot, splits per row sized
    on the device from the list's length).  Tight clusters far apart make a
    query block straddle clusters, so its centred norms dwarf the neighbour
    gaps and most rows (all, or a part beside a manifold) are listed; the
    result equals the oracle's and the SIMT screen's."""
    import os
    D, k = 64, 15
    rng = np.random.default_rng(11)
    cen = 100.0 * rng.standard_normal((40, D))
    Xc = cen[rng.integers(0, 40, 3000)] + 0.01 * rng.standard_normal((3000, D))
    if kind == "clusters":
        X = Xc
    else:
        t = rng.uniform(0, 3, (2000, 3))
        Q, _ = np.linalg.qr(rng.standard_normal((D, D)))
        Xm = np.concatenate([np.sin(t), np.cos(t)], axis=1) @ Q[:6] + 0.01 * rng.standard_normal((2000, D))
        X = np.concatenate([Xm, Xc])[rng.permutation(5000)]
    idx = core.knn(cu(X), k).cpu().numpy()
    old = os.environ.get("RVGP_KNN_TC")
    os.environ["RVGP_KNN_TC"] = "0"
    try:
        idx0 = core.knn(cu(X), k).cpu().numpy()
    finally:
        if old is None:
            del os.environ["RVGP_KNN_TC"]
        else:
            os.environ["RVGP_KNN_TC"] = old
    assert np.array_equal(idx, idx0)
    assert np.array_equal(idx, O.knn(X, k))


def test_knn_tensor_core_certifies_manifold_rows(core):
    """On manifold data (the Swiss roll in R^64) the tensor-core screen's
    certificate settles almost every row: at most 1 % go to the exact scan."""
    from rvgp_gb300.workloads import make_points
    X = make_points("swissroll64", 20000, seed=4)
    idx = core.knn(cu(X), 15).cpu().numpy()
    rows = core.lib().rvgp_knn_fallback_rows(len(X), 64, 15, core.ptr(core.knn.last_ws), core.stream())
    assert 0 <= rows <= 200
    sample = np.random.default_rng(0).choice(len(X), 300, replace=False)
    d = np.zeros((300, len(X)))
    for j in range(X.shape[1]):  # coordinates summed in order, as the contract states
        d += (X[sample, j, None] - X[None, :, j]) ** 2
    d[np.arange(300), sample] = np.inf
    ref = np.argsort(d, axis=1, kind="stable")[:, :15]
    assert np.array_equal(idx[sample], ref)
