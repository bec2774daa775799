"""CPU: the oracle restatement against the reference's own outputs (golden fixtures).

The fixtures were produced by tests/golden/make_golden.py from the reference's
code (RVGP/geometry.py, RVGP/dataclass.py, the Cython RVGP/lib/ptu_dijkstra.pyx).
"""
import numpy as np
import pytest

from conftest import cluster_slices, load_golden, projector_distance, subspace_sin
from oracle import rvgp_oracle as O


def test_knn_graph_matches_reference(golden):
    X, k = golden["X"], int(golden["k"])
    nn = O.knn(X, k)
    ip, ix = O.symmetrised_csr(nn, len(X))
    assert np.array_equal(ip, golden["indptr"])
    assert np.array_equal(ix, golden["indices"])


def test_gauges_match_reference(golden):
    X, K, d = golden["X"], int(golden["K"]), int(golden["dim_man"])
    nbh = O.geodesic_neighbourhoods(golden["indptr"], golden["indices"], K)
    assert nbh.shape == (len(X), K + 1)
    assert np.array_equal(nbh[:, 0], np.arange(len(X)))
    Sg = golden["Sigma"]
    T, S = O.tangent_frames(X, nbh, Sg.shape[1])
    # singular values pin the neighbourhood set: a different set moves them by O(1e-3)
    np.testing.assert_allclose(S, Sg, rtol=1e-12, atol=1e-14)
    assert projector_distance(T[:, :, :d], golden["gauges"]) < 1e-12


def test_heap_tie_breaking_is_what_is_checked():
    """Plant a mistake in the oracle: a breadth-first search that breaks ties by
    index instead of by the reference's Fibonacci heap picks different K+1 sets,
    and the singular-value check above would catch it."""
    g = load_golden("torus")
    X, K = g["X"], int(g["K"])
    ip, ix = g["indptr"], g["indices"]
    n = len(X)
    bfs = np.empty((n, K + 1), dtype=np.int64)
    for i in range(n):
        seen, order, front = {i}, [i], [i]
        while len(order) < K + 1:
            nxt = sorted({int(u) for v in front for u in ix[ip[v]:ip[v + 1]]} - seen)
            seen.update(nxt)
            order.extend(nxt)
            front = nxt
        bfs[i] = order[: K + 1]
    _, S = O.tangent_frames(X, bfs, g["Sigma"].shape[1])
    mism = np.abs(S - g["Sigma"]).max(axis=1) > 1e-9
    assert mism.sum() > n // 10


def test_manifold_dimension(golden):
    if "tangents_full" not in golden:
        pytest.skip("reference ran with d fixed for this case")
    assert O.manifold_dimension(golden["Sigma"], 0.8) == int(golden["dim_man"])


def test_connections_match_reference(golden):
    R = O.connections(golden["gauges"], golden["indptr"], golden["indices"])
    np.testing.assert_allclose(R, golden["R"], atol=1e-13)


def test_laplacians_match_reference(golden):
    n = len(golden["X"])
    L = O.laplacian(golden["indptr"], golden["indices"], n)
    assert np.array_equal(L.indptr, golden["L_indptr"])
    assert np.array_equal(L.indices, golden["L_indices"])
    assert np.array_equal(L.data, golden["L_data"])
    Lc = O.connection_laplacian(L, golden["R"], golden["indptr"], golden["indices"],
                                int(golden["dim_man"]))
    Lc.sort_indices()
    assert np.array_equal(Lc.indices, golden["Lc_indices"])
    np.testing.assert_array_equal(Lc.data, golden["Lc_data"])


def test_spectrum_matches_reference(golden):
    n, d, m = len(golden["X"]), int(golden["dim_man"]), int(golden["m"])
    L = O.laplacian(golden["indptr"], golden["indices"], n)
    Lc = O.connection_laplacian(L, golden["R"], golden["indptr"], golden["indices"], d)
    for M, ev_g, V_g in ((L, golden["evals_L"], golden["evecs_L"]),
                         (Lc, golden["evals_Lc"], golden["evecs_Lc_local"])):
        ev, V = O.spectrum(M, m)
        np.testing.assert_allclose(ev, ev_g, rtol=1e-9, atol=1e-11)
        np.testing.assert_allclose(np.linalg.norm(V, axis=0), np.sqrt(M.shape[0]), rtol=1e-10)
        for sl in cluster_slices(ev_g):
            if sl.stop < m:  # a cluster cut by the m-th eigenpair is not a subspace of both
                assert subspace_sin(V[:, sl], V_g[:, sl]) < 1e-7


def test_lift_matches_reference(golden):
    if "evecs_Lc" not in golden:
        pytest.skip("lifted basis not stored for this case")
    m = int(golden["m"])
    np.testing.assert_allclose(O.lift(golden["gauges"], golden["evecs_Lc_local"], m),
                               golden["evecs_Lc"], atol=1e-13)


def test_vector_field_and_diffusion_match_reference(golden):
    if "field_raw" not in golden:
        pytest.skip("no field for this case")
    n, d = len(golden["X"]), int(golden["dim_man"])
    L = O.laplacian(golden["indptr"], golden["indices"], n)
    Lc = O.connection_laplacian(L, golden["R"], golden["indptr"], golden["indices"], d)
    f = O.random_vector_field(golden["X"], golden["gauges"], int(golden["field_seed"]))
    np.testing.assert_array_equal(f, golden["field_raw"])
    t = float(golden["smooth_t"])
    fs = O.smooth_vector_field(f, golden["gauges"], L, Lc, t, exact="expm")
    np.testing.assert_allclose(fs, golden["field_smooth"], atol=1e-12)
    fa = O.smooth_vector_field(f, golden["gauges"], L, Lc, t, exact="action")
    np.testing.assert_allclose(fa, golden["field_smooth"], atol=1e-10)


def test_fps_matches_reference(golden):
    X = golden["X"]
    p, lam = O.furthest_point_sampling(X, N=len(golden["fps_perm"]))
    assert np.array_equal(p, golden["fps_perm"])
    np.testing.assert_allclose(lam, golden["fps_lambdas"], rtol=1e-9, atol=1e-12)
    p2, lam2 = O.furthest_point_sampling(X, spacing=float(golden["fps_spacing"]))
    assert np.array_equal(p2, golden["fps_perm_spacing"])
    np.testing.assert_allclose(lam2, golden["fps_lambdas_spacing"], rtol=1e-9, atol=1e-12)


def test_train_test_split_matches_sklearn():
    s = load_golden("train_test_split")
    i = 0
    while f"c{i}_n" in s:
        tr, te = O.train_test_split_indices(int(s[f"c{i}_n"]), float(s[f"c{i}_test_size"]),
                                            int(s[f"c{i}_seed"]))
        assert np.array_equal(tr, s[f"c{i}_train"]) and np.array_equal(te, s[f"c{i}_test"])
        i += 1
    assert i >= 5


def test_knn_ties_lower_index_first():
    # lattice: many exactly equal distances; the oracle keeps the lowest indices
    g = np.stack(np.meshgrid(np.arange(4), np.arange(4), np.arange(3), indexing="ij"), -1)
    X = g.reshape(-1, 3).astype(float)
    nn = O.knn(X, 5)
    for i in range(len(X)):
        d2 = ((X - X[i]) ** 2).sum(1)
        d2[i] = np.inf
        order = np.lexsort((np.arange(len(X)), d2))
        assert list(nn[i]) == list(order[:5])


def _gp_problem(seed=0, N=60, m=8):
    rng = np.random.default_rng(seed)
    Phi = rng.standard_normal((N, m))
    y = rng.standard_normal(N)
    lam = np.sort(rng.uniform(0, 2, m))
    return Phi, y, lam


def test_gp_lowrank_equals_dense():
    Phi, y, lam = _gp_problem()
    S = O.eval_S(lam, 1.5, 5.0, 1.3, Phi.shape[0])
    for noise in (1.0, 1e-2, 1e-3):
        a, b = O.lml_dense(Phi, y, S, noise), O.lml_lowrank(Phi, y, S, noise)
        assert abs(a - b) < 1e-9 * abs(a)
        m1, v1 = O.predict_f(Phi, y, S, noise, Phi[:7] * 0.7)
        m2, v2 = O.predict_f_lowrank(Phi, y, S, noise, Phi[:7] * 0.7)
        np.testing.assert_allclose(m1, m2, rtol=1e-8, atol=1e-10)
        np.testing.assert_allclose(v1, v2, rtol=1e-6, atol=1e-9)


def test_gp_gradient_formula_matches_fd():
    Phi, y, lam = _gp_problem(1)
    S = O.eval_S(lam, 1.5, 5.0, 1.0, Phi.shape[0])
    gS, gn = O.lml_grad_S_noise(Phi, y, S, 0.1)
    h = 1e-4  # central difference; round-off of the Cholesky LML dominates below this
    for l in range(len(S)):
        e = np.zeros_like(S)
        e[l] = h
        fd = (O.lml_dense(Phi, y, S + e, 0.1) - O.lml_dense(Phi, y, S - e, 0.1)) / (2 * h)
        assert abs(fd - gS[l]) < 1e-6 * max(1.0, abs(fd))
    h = 1e-7  # the noise derivative is steep at σ²=0.1: a small step keeps truncation down
    fd = (O.lml_dense(Phi, y, S, 0.1 + h) - O.lml_dense(Phi, y, S, 0.1 - h)) / (2 * h)
    assert abs(fd - gn) < 1e-6 * max(1.0, abs(fd))


def test_sgpr_bound_forms_agree_and_bound_the_lml():
    """The M-space SGPR bound (GPflow's algorithm) equals its N-space definition,
    lies below the exact LML, and equals it when Z spans the eigenbasis."""
    Phi, y, lam = _gp_problem(2)
    S = O.eval_S(lam, 1.5, 5.0, 1.3, Phi.shape[0])
    rng = np.random.default_rng(5)
    for M in (5, 20, 40):
        Z = Phi[rng.choice(len(Phi), M, replace=False)]
        for noise in (1.0, 0.05):
            a, b = O.sgpr_elbo(Phi, y, S, noise, Z), O.sgpr_elbo_dense(Phi, y, S, noise, Z)
            assert abs(a - b) < 1e-9 * abs(a)
            assert a <= O.lml_dense(Phi, y, S, noise) + 1e-9 * abs(a)
    m = Phi.shape[1]
    for noise in (1.0, 0.05):
        exact = O.lml_dense(Phi, y, S, noise)
        assert abs(O.sgpr_elbo(Phi, y, S, noise, np.eye(m), jitter=0.0) - exact) < 1e-9 * abs(exact)
        m1, v1 = O.sgpr_predict_f(Phi, y, S, noise, np.eye(m), Phi[:7] * 0.7, jitter=0.0)
        m2, v2 = O.predict_f(Phi, y, S, noise, Phi[:7] * 0.7)
        np.testing.assert_allclose(m1, m2, rtol=1e-8, atol=1e-10)
        np.testing.assert_allclose(v1, v2, rtol=1e-6, atol=1e-9)


def test_rbf_gpr_oracle_matches_dense_forms():
    """The multi-output RBF GPR oracle equals the sum of per-column Gaussian log
    densities, and its posterior equals the textbook K*ᵀ K_y⁻¹ form."""
    rng = np.random.default_rng(3)
    X = rng.standard_normal((40, 5)) * 0.4
    Y = rng.standard_normal((40, 3))
    Xs = rng.standard_normal((9, 5)) * 0.4
    var, ls, noise = 1.3, 0.8, 0.05
    Ky = O.rbf_K(X, X, var, ls) + noise * np.eye(40)
    _, logdet = np.linalg.slogdet(Ky)
    Kinv = np.linalg.inv(Ky)
    ref = sum(-0.5 * Y[:, c] @ Kinv @ Y[:, c] - 0.5 * logdet - 20 * np.log(2 * np.pi) for c in range(3))
    assert abs(O.rbf_gpr_lml(X, Y, var, ls, noise) - ref) < 1e-9 * abs(ref)
    mean, v = O.rbf_gpr_predict_f(X, Y, var, ls, noise, Xs)
    Ks = O.rbf_K(Xs, X, var, ls)
    np.testing.assert_allclose(mean, Ks @ Kinv @ Y, rtol=1e-8, atol=1e-10)
    np.testing.assert_allclose(v, var - np.einsum("ij,jk,ik->i", Ks, Kinv, Ks), rtol=1e-7, atol=1e-10)


@pytest.mark.parametrize("case", ["small", "large"])
def test_vectorfield_features_match_reference(case):
    g = load_golden("features")
    div, curl = O.vectorfield_features(g[f"{case}_pos"], g[f"{case}_vec"], k=5)
    np.testing.assert_allclose(div, g[f"{case}_div"], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(curl, g[f"{case}_curl"], rtol=1e-12, atol=1e-12)


def test_load_mesh_matches_reference(tmp_path):
    from rvgp_gb300.utils import load_mesh
    g = load_golden("features")
    text = bytes(g["obj_text"]).decode()
    (tmp_path / "uvsphere.obj").write_text(text)
    v, f = load_mesh("uvsphere", folder=str(tmp_path))
    np.testing.assert_array_equal(v, g["obj_vertices"])
    np.testing.assert_array_equal(f, g["obj_faces"])
    # records the reference rejects: blank lines and 'v/vt/vn' face entries
    (tmp_path / "tolerant.obj").write_text("# c\n\nv 0 0 0\nv 1 0 0\nv 0 1 0\n\nf 1/1/1 2/2/2 3/3/3\n")
    v, f = load_mesh("tolerant", folder=str(tmp_path))
    assert v.shape == (3, 3) and f.tolist() == [[0, 1, 2]]


def test_vectorfield_features_kdtree_form_matches():
    g = load_golden("features")
    a = O.vectorfield_features(g["large_pos"], g["large_vec"], k=5)
    b = O.vectorfield_features(g["large_pos"], g["large_vec"], k=5, kdtree=True)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])


@pytest.mark.parametrize("name", ["sphere", "torus"])
def test_knn_kdtree_timing_form_matches(name):
    g = load_golden(name)
    X, k = g["X"], int(g["k"])
    np.testing.assert_array_equal(np.sort(O.knn_kdtree(X, k), 1), np.sort(O.knn(X, k), 1))


def test_spectral_kernel_pinned_to_reference_kernels_py():
    """eval_S, K and K_diag of the oracle equal the reference's own
    ManifoldKernel (RVGP/kernels.py:41-67, run through the numpy-backed
    TensorFlow stub by tests/golden/make_kernel_golden.py)."""
    from conftest import load_golden
    kg = load_golden("kernel")
    for name in ("sphere", "torus", "ellipsoid", "swissroll64"):
        g = load_golden(name)
        n_rows = float(kg[f"{name}_n_rows"])
        ev = g["evecs_Lc"] if "evecs_Lc" in g else O.lift(g["gauges"], g["evecs_Lc_local"], g["evals_Lc"].size)
        X, X2 = ev[kg[f"{name}_rows"]], ev[kg[f"{name}_rows2"]]
        for c, typ in enumerate(kg["params_typ"]):
            nu, kappa, sf = kg["params"][c]
            key = f"{name}_{c}"
            S = O.eval_S(g["evals_Lc"], nu, kappa, sf, n_rows, str(typ))
            np.testing.assert_allclose(S, kg[key + "_S"], rtol=1e-13)
            np.testing.assert_allclose(O.kernel_K(X, S), kg[key + "_K"], rtol=1e-12, atol=1e-12 * np.abs(kg[key + "_K"]).max())
            np.testing.assert_allclose(O.kernel_K(X, S, X2), kg[key + "_K2"], rtol=1e-12,
                                       atol=1e-12 * np.abs(kg[key + "_K2"]).max())
            np.testing.assert_allclose(np.einsum("ij,ij->i", X * S, X), kg[key + "_Kdiag"], rtol=1e-12)
