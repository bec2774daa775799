"""GPU: the locality renumbering of the eigensolves' matrices — the Morton
order against a numpy restatement (bit-exact), the renumbered block-CSR
against scipy's P A Pᵀ, and eigenpairs of the renumbered solve against the
plain one."""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

from conftest import cluster_slices, load_golden, subspace_sin
from oracle import rvgp_oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def core():
    from rvgp_gb300 import _core
    _core.require_cuda()
    return _core


def cu(a, dtype=torch.float64):
    return torch.as_tensor(np.ascontiguousarray(a)).to("cuda", dtype)


def spread3(v):
    v = v.astype(np.uint64) & 0x3FF
    v = (v | (v << 16)) & 0x030000FF
    v = (v | (v << 8)) & 0x0300F00F
    v = (v | (v << 4)) & 0x030C30C3
    v = (v | (v << 2)) & 0x09249249
    return v


def morton_perm(X):
    """Stable sort of 30-bit Morton codes of the three widest coordinates."""
    lo, hi = X.min(0), X.max(0)
    dims = np.argsort(-(hi - lo), kind="stable")[:3]
    code = np.zeros(len(X), dtype=np.uint64)
    for q, j in enumerate(dims):
        t = (X[:, j] - lo[j]) / (hi[j] - lo[j]) if hi[j] > lo[j] else np.zeros(len(X))
        c = np.minimum(1023.0, np.maximum(0.0, t * 1024.0)).astype(np.uint64)
        code |= spread3(c) << np.uint64(q)
    return np.argsort(code, kind="stable")


@pytest.mark.parametrize("n,D", [(1, 3), (777, 3), (5000, 2), (3000, 64), (20000, 3)])
def test_locality_order_matches_numpy(core, n, D):
    rng = np.random.default_rng(n + D)
    X = rng.standard_normal((n, D)) * np.linspace(1.0, 3.0, D)
    X[: n // 3, 0] = X[0, 0]  # ties
    perm, rank = core.locality_order(cu(X))
    p = perm.cpu().numpy()
    np.testing.assert_array_equal(p, morton_perm(X))
    np.testing.assert_array_equal(rank.cpu().numpy()[p], np.arange(n))


@pytest.mark.parametrize("d", [1, 2, 3])
def test_permute_csr_is_PAPt(core, d):
    rng = np.random.default_rng(d)
    n = 900
    A = sp.random(n, n, density=0.01, random_state=2, format="csr") + sp.eye(n)
    A = (A + A.T).tocsr()
    A.sort_indices()
    blocks = rng.standard_normal((A.nnz, d, d))
    v64 = cu(blocks if d > 1 else blocks[:, 0, 0])
    v32 = v64.float()
    perm = rng.permutation(n).astype(np.int32)
    rank = np.empty(n, np.int32)
    rank[perm] = np.arange(n)
    ip, ix, o64, o32 = core.permute_csr(cu(A.indptr, torch.int32), cu(A.indices, torch.int32), v64, v32,
                                        cu(perm, torch.int32), cu(rank, torch.int32))
    M = sp.bsr_matrix((blocks, A.indices, A.indptr), shape=(n * d, n * d)).tocsr()
    rows = (perm[:, None] * d + np.arange(d)[None]).reshape(-1)
    ref = M[rows][:, rows]
    got = sp.bsr_matrix((o64.cpu().numpy().reshape(-1, d, d), ix.cpu().numpy(), ip.cpu().numpy()),
                        shape=(n * d, n * d)).tocsr()
    assert abs(got - ref).max() == 0
    np.testing.assert_array_equal(o32.cpu().numpy(), o64.cpu().numpy().astype(np.float32))
    # row entries keep their order: new row r lists old row perm[r]'s columns, renumbered
    ipn, ixn = ip.cpu().numpy(), ix.cpu().numpy()
    for r in (0, 17, n - 1):
        o = perm[r]
        np.testing.assert_array_equal(ixn[ipn[r]:ipn[r + 1]], rank[A.indices[A.indptr[o]:A.indptr[o + 1]]])
    src = cu(rng.standard_normal((n * d, 5)))
    back = core.unpermute_rows(src, cu(rank, torch.int32), d).cpu().numpy()
    np.testing.assert_array_equal(back[rows], src.cpu().numpy())


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_eigsh_renumbered_equals_plain(core, mode):
    g = load_golden("torus")
    n, d, m = len(g["X"]), int(g["dim_man"]), int(g["m"])
    ip, ix = cu(g["indptr"], torch.int32), cu(g["indices"], torch.int32)
    L = O.laplacian(g["indptr"], g["indices"], n)
    v64 = cu(L.data[:, None, None] * g["R"])
    perm, rank = core.locality_order(cu(g["X"]))
    pip, pix, p64, _ = core.permute_csr(ip, ix, v64, None, perm, rank)
    ev0, V0, _ = core.eigsh(ip, ix, v64, m=m, mode=mode, tol=1e-11, scale=np.sqrt(n * d))
    ev1, V1, _ = core.eigsh(pip, pix, p64, m=m, mode=mode, tol=1e-11, scale=np.sqrt(n * d), perm=perm)
    ev0, ev1, V0, V1 = ev0.cpu().numpy(), ev1.cpu().numpy(), V0.cpu().numpy(), V1.cpu().numpy()
    np.testing.assert_allclose(ev1, ev0, rtol=1e-9, atol=1e-9 * abs(ev0).max())
    for sl in cluster_slices(ev0, rtol=1e-5):
        if sl.stop < m:
            assert subspace_sin(V1[:, sl], V0[:, sl]) < 1e-6
    # and against the reference's ARPACK pairs
    np.testing.assert_allclose(ev1, g["evals_Lc"], rtol=1e-9, atol=1e-9 * abs(g["evals_Lc"]).max())
