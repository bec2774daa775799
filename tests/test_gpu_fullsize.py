"""GPU: the benchmark workload at full size (torus, n = 20000, k = 20, m = 200),
checked through properties that do not need an oracle run at this size:

* kNN: every row of a 256-query sample equals an exact FP64 brute-force
  search (ties by lower index); rows are sorted and exclude the query;
* graph / Laplacian: symmetric CSR with self-loops, row sums of L are zero;
* gauges: orthonormal columns;
* connection Laplacian: R_ji = R_ijᵀ, diagonal blocks deg·I;
* eigenpairs (mixed default and FP64 form): residuals ‖Lc v − λ v‖ within the
  requested tolerance of the Gershgorin bound, orthonormal vectors, ascending
  values, and the mixed eigenvalues within 1e-5 (relative to the largest) of
  the FP64 ones;
* GP: the mixed and FP64 forms reach equal prediction error against the true
  field, the condition of the benchmark metric.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

N_PTS, K_NN, M_EIG = 20000, 20, 200


@pytest.fixture(scope="module")
def core():
    from rvgp_gb300 import _core
    _core.require_cuda()
    return _core


@pytest.fixture(scope="module")
def torus():
    from rvgp_gb300.workloads import make_points
    return make_points("torus", N_PTS, seed=0)


@pytest.fixture(scope="module")
def geometry(core, torus):
    X = torch.as_tensor(torus, device="cuda")
    idx = core.knn(X, K_NN)
    ip, ix, md = core.graph_build(idx)
    K = int(1.5 * K_NN)
    T, S, _ = core.gauges(X, ip, ix, K, md, 2)
    R, v64, v32 = core.connections(T, 2, ip, ix)
    torch.cuda.synchronize()
    return dict(X=X, idx=idx, ip=ip, ix=ix, md=md, T=T, R=R, v64=v64, v32=v32)


def test_knn_sample_exact(torus, geometry):
    idx = geometry["idx"].cpu().numpy()
    rng = np.random.default_rng(5)
    for q in rng.choice(N_PTS, 256, replace=False):
        d2 = ((torus - torus[q]) ** 2).sum(1)
        d2[q] = np.inf
        order = np.lexsort((np.arange(N_PTS), d2))[:K_NN]
        assert np.array_equal(idx[q], order), q
        assert q not in idx[q]


def test_graph_and_laplacian(core, geometry):
    ip, ix = geometry["ip"].cpu().numpy(), geometry["ix"].cpu().numpy()
    n = len(ip) - 1
    rows = np.repeat(np.arange(n), np.diff(ip))
    pairs = set(zip(rows.tolist(), ix.tolist()))
    assert all((j, i) in pairs for i, j in pairs)
    assert all((i, i) in pairs for i in range(n))
    vals = core.laplacian_values(geometry["ip"], geometry["ix"]).cpu().numpy()
    sums = np.add.reduceat(vals, ip[:-1])
    assert np.abs(sums).max() == 0.0


def test_gauges_orthonormal(geometry):
    T = geometry["T"].cpu().numpy()
    G = np.einsum("nij,nik->njk", T, T)
    assert np.abs(G - np.eye(2)).max() < 1e-12


def test_connection_laplacian_structure(geometry):
    ip, ix = geometry["ip"].cpu().numpy(), geometry["ix"].cpu().numpy()
    R = geometry["R"].cpu().numpy()
    v = geometry["v64"].cpu().numpy()
    n = len(ip) - 1
    pos = {}
    for i in range(n):
        for t in range(ip[i], ip[i + 1]):
            pos[(i, ix[t])] = t
    rng = np.random.default_rng(2)
    for t in rng.choice(len(ix), 2000, replace=False):
        i = int(np.searchsorted(ip, t, side="right") - 1)
        j = int(ix[t])
        np.testing.assert_allclose(R[pos[(j, i)]], R[t].T, atol=1e-12)
        np.testing.assert_allclose(v[pos[(j, i)]], v[t].T, atol=1e-12)
    deg = np.diff(ip) - 1
    for i in rng.choice(n, 500, replace=False):
        np.testing.assert_allclose(v[pos[(i, i)]], deg[i] * np.eye(2), atol=1e-12)


@pytest.fixture(scope="module")
def eig_both(core, geometry):
    g = geometry
    out = {}
    for mode in ("mixed", "fp64"):
        ev, V, info = core.eigsh(g["ip"], g["ix"], g["v64"], g["v32"], m=M_EIG, mode=mode)
        out[mode] = (ev, V, info)
    return out


@pytest.mark.parametrize("mode", ["mixed", "fp64"])
def test_eigenpairs_residuals(core, geometry, eig_both, mode):
    g = geometry
    ev, V, info = eig_both[mode]
    assert info["converged"] == M_EIG
    lam = ev.cpu().numpy()
    assert np.all(np.diff(lam) >= -1e-12)
    Vn = V / torch.linalg.vector_norm(V, dim=0, keepdim=True)
    AV = core.bspmm(g["ip"], g["ix"], g["v64"], Vn.contiguous())
    res = torch.linalg.vector_norm(AV - Vn * ev[None, :], dim=0).cpu().numpy()
    bound = 2.0 * (np.diff(g["ip"].cpu().numpy()) - 1).max()  # Gershgorin bound of Lc
    tol = 1e-11 if mode == "fp64" else 2e-5
    assert res.max() <= 2 * tol * bound
    G = (Vn.T @ Vn).cpu().numpy()
    assert np.abs(G - np.eye(M_EIG)).max() < (1e-9 if mode == "fp64" else 1e-5)


def test_mixed_eigenvalues_match_fp64(eig_both):
    lm = eig_both["mixed"][0].cpu().numpy()
    lf = eig_both["fp64"][0].cpu().numpy()
    assert np.abs(lm - lf).max() <= 1e-5 * lf.max()


def test_mixed_prediction_matches_fp64(torus):
    """The pipeline through the public API in both forms, rotational field,
    200 Adam steps: equal prediction error against the true field (within 2 %
    of each other), the condition of the benchmark metric.  The two forms' means
    also agree to 2e-3: the optimiser's path is sensitive enough that rounding at
    the 1e-7 level can end it at a neighbouring optimum of the likelihood with
    the same error."""
    import rvgp_gb300 as RVGP
    from rvgp_gb300 import geometry
    from rvgp_gb300.workloads import rotational_field, split
    train, test = split(N_PTS, 0.3, seed=0)
    means, errs = {}, {}
    for precision in ("fp64", "mixed"):
        d = RVGP.create_data_object(torus, n_neighbors=K_NN, n_eigenpairs=M_EIG, precision=precision,
                                    verbose=False)
        d.vectors = geometry.project_to_manifold(rotational_field(torus), d.gauges)
        gp = RVGP.fit(d, train_ind=train, epochs=200, optimizer="adam", lr=0.05, verbose=False)
        mean, _ = gp.transform(d, test)
        truth = d.vectors[test]
        means[precision] = mean
        errs[precision] = np.linalg.norm(mean - truth) / np.linalg.norm(truth)
    assert abs(errs["mixed"] - errs["fp64"]) <= 0.02 * errs["fp64"]
    err = np.linalg.norm(means["mixed"] - means["fp64"]) / np.linalg.norm(means["fp64"])
    assert err <= 2e-3
