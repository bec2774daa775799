"""GPU parity: the eigensolver against the reference's ARPACK eigenpairs
(golden fixtures) and against scipy on mid-size Laplacians, in both the plain
FP64 and the mixed FP32/FP64 form."""
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


def check_pairs(ev, V, ev_ref, V_ref, m, rtol_ev, sin_tol):
    np.testing.assert_allclose(ev, ev_ref, rtol=rtol_ev, atol=rtol_ev * max(1.0, abs(ev_ref).max()))
    for sl in cluster_slices(ev_ref, rtol=1e-5):
        if sl.stop < m:  # a cluster cut by the m-th pair is not a common subspace
            assert subspace_sin(V[:, sl], V_ref[:, sl]) < sin_tol, (sl, subspace_sin(V[:, sl], V_ref[:, sl]))


@pytest.mark.parametrize("name", ["sphere", "torus", "ellipsoid", "swissroll64"])
@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_eigsh_matches_reference(core, name, mode):
    g = load_golden(name)
    n, d, m = len(g["X"]), int(g["dim_man"]), int(g["m"])
    ip, ix = cu(g["indptr"], torch.int32), cu(g["indices"], torch.int32)
    # scalar Laplacian (evecs scaled by sqrt(n) as compute_spectrum does)
    ev, V, info = core.eigsh(ip, ix, cu(g["L_data"]), m=m, mode=mode, tol=1e-11, scale=np.sqrt(n))
    check_pairs(ev.cpu().numpy(), V.cpu().numpy(), g["evals_L"], g["evecs_L"], m, 1e-9, 1e-6)
    np.testing.assert_allclose(np.linalg.norm(V.cpu().numpy(), axis=0), np.sqrt(n), rtol=1e-10)
    # connection Laplacian from the reference's own transports
    L = O.laplacian(g["indptr"], g["indices"], n)
    blocks = L.data[:, None, None] * g["R"]
    ev, V, info = core.eigsh(ip, ix, cu(blocks), m=m, mode=mode, tol=1e-11, scale=np.sqrt(n * d))
    check_pairs(ev.cpu().numpy(), V.cpu().numpy(), g["evals_Lc"], g["evecs_Lc_local"], m, 1e-9, 1e-6)


@pytest.mark.parametrize("name", ["sphere", "torus"])
def test_eigsh_mixed_default_accuracy(core, name):
    """The mixed form's default stops at FP32-level residuals (no FP64 tall
    iterations): eigenvalues to 1e-5 relative of the reference's ARPACK values."""
    g = load_golden(name)
    n, d, m = len(g["X"]), int(g["dim_man"]), int(g["m"])
    ip, ix = cu(g["indptr"], torch.int32), cu(g["indices"], torch.int32)
    L = O.laplacian(g["indptr"], g["indices"], n)
    blocks = L.data[:, None, None] * g["R"]
    ev, V, info = core.eigsh(ip, ix, cu(blocks), m=m, mode="mixed", scale=np.sqrt(n * d))
    assert info["refine_iters"] == 0
    ref = g["evals_Lc"]
    assert np.abs(ev.cpu().numpy() - ref).max() <= 1e-5 * ref.max()


@pytest.mark.parametrize("kind,n,k,m", [("torus", 4000, 20, 60), ("sphere", 3000, 10, 40)])
def test_eigsh_midsize(core, kind, n, k, m):
    from rvgp_gb300.workloads import make_points
    X = make_points(kind, n, seed=1)
    nn = O.knn(X, k)
    ip, ix = O.symmetrised_csr(nn, n)
    L = O.laplacian(ip, ix, n)
    nbh = O.geodesic_neighbourhoods(ip, ix, int(1.5 * k))
    T, _ = O.tangent_frames(X, nbh, 3)
    R = O.connections(np.ascontiguousarray(T[:, :, :2]), ip, ix)
    Lc = O.connection_laplacian(L, R, ip, ix, 2)
    ev_ref, V_ref = O.spectrum_shift_invert(Lc, m)
    blocks = L.data[:, None, None] * R
    for mode in ("mixed", "fp64"):
        ev, V, info = core.eigsh(cu(ip, torch.int32), cu(ix, torch.int32), cu(blocks), m=m, mode=mode,
                                 tol=1e-11, scale=np.sqrt(2 * n))
        check_pairs(ev.cpu().numpy(), V.cpu().numpy(), ev_ref, V_ref, m, 1e-9, 1e-6)
        assert info["converged"] == m


def test_eigsh_rejects_too_many(core):
    ip = cu(np.arange(11) * 1, torch.int32)
    ix = cu(np.arange(10), torch.int32)
    with pytest.raises(ValueError):
        core.eigsh(ip, ix, cu(np.ones(10)), m=9)


def test_eigsh_locking(core):
    """The FP32 stage locks converged Ritz vectors (the filter, the
    orthonormalisation and the Rayleigh-Ritz step then run on the active
    columns only).  A weighted path-graph Laplacian (eigenvalues growing like
    j², so the lowest converge iterations before the m-th) locks vectors, and
    the eigenpairs agree with scipy's and with the solve without locking
    (RVGP_EIG_LOCK=0): eigenvalues, residuals against the FP64 matrix,
    orthonormality."""
    import os
    n, m = 20000, 200
    rng = np.random.default_rng(8)
    w = rng.uniform(1.0, 2.0, n - 1)
    deg = np.zeros(n)
    deg[:-1] += w
    deg[1:] += w
    L = sp.diags([-w, deg, -w], [-1, 0, 1], format="csr")
    L.sort_indices()
    ev_ref = np.sort(O.spectrum_shift_invert(L, m)[0])
    args = (cu(L.indptr, torch.int32), cu(L.indices, torch.int32), cu(L.data))

    def solve(env):
        saved = {k: os.environ.get(k) for k in env}
        os.environ.update(env)
        try:
            return core.eigsh(*args, m=m, mode="mixed", scale=1.0)
        finally:
            for k, v in saved.items():
                if v is None:
                    del os.environ[k]
                else:
                    os.environ[k] = v

    ev, V, info = solve({"RVGP_EIG_LOCK_MARGIN": "1.0"})  # lock at the tolerance itself
    ev0, V0, info0 = solve({"RVGP_EIG_LOCK": "0"})
    assert info["locked"] > 0 and info0["locked"] == 0
    assert info["converged"] == m and info0["converged"] == m
    bup = float(abs(L).sum(axis=1).max())
    for e, Vv in ((ev, V), (ev0, V0)):
        e = e.cpu().numpy()
        Vv = Vv.cpu().numpy()
        assert np.all(np.diff(e) >= 0)
        assert np.abs(e - ev_ref).max() <= 1e-5 * bup
        assert np.abs(Vv.T @ Vv - np.eye(m)).max() <= 1e-4
        assert np.linalg.norm(L @ Vv - Vv * e, axis=0).max() <= 2e-5 * bup
