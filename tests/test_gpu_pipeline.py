"""GPU parity of the drop-in API end to end against the reference's golden
fixtures: create_data_object -> random_vector_field -> smooth_vector_field,
furthest_point_sampling, the field helpers, and fit/transform against the
oracle's dense GP at the same hyperparameters."""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

from conftest import cluster_slices, load_golden, subspace_sin
from oracle import rvgp_oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def RVGP():
    import rvgp_gb300
    from rvgp_gb300 import _core
    _core.require_cuda()
    return rvgp_gb300


@pytest.mark.parametrize("name", ["sphere", "torus", "ellipsoid"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_data_object_matches_reference(RVGP, name, precision):
    g = load_golden(name)
    m = int(g["m"])
    d = RVGP.create_data_object(g["X"], n_neighbors=int(g["k"]), n_eigenpairs=m, precision=precision,
                                eig_tol=1e-11, verbose=False)
    assert d.dim_man == int(g["dim_man"]) and d.n == len(g["X"])
    L = d.L
    assert np.array_equal(L.indptr, g["L_indptr"]) and np.array_equal(L.indices, g["L_indices"])
    assert np.array_equal(L.data, g["L_data"])
    np.testing.assert_allclose(d.evals_L, g["evals_L"], rtol=1e-9, atol=1e-11)
    np.testing.assert_allclose(d.evals_Lc, g["evals_Lc"], rtol=1e-9, atol=1e-11)
    # the lifted eigenbasis is gauge invariant: compare subspaces per eigenvalue cluster
    for sl in cluster_slices(g["evals_Lc"], rtol=1e-5):
        if sl.stop < m:
            assert subspace_sin(d.evecs_Lc[:, sl], g["evecs_Lc"][:, sl]) < 1e-6
    np.testing.assert_allclose(np.linalg.norm(d.evecs_Lc, axis=0), np.sqrt(2 * len(g["X"])), rtol=1e-9)
    # Lc and R are gauge dependent: Lc' = Oᵀ Lc O with O_i = T_refᵢᵀ T_i
    O_ = np.einsum("nki,nkj->nij", g["gauges"], d.gauges)
    Ob = sp.block_diag(list(O_))
    Lc_ref = O.connection_laplacian(O.laplacian(g["indptr"], g["indices"], d.n), g["R"], g["indptr"],
                                    g["indices"], d.dim_man)
    diff = (Ob.T @ Lc_ref @ Ob - d.Lc.tocsr())
    assert abs(diff).max() < 1e-10


@pytest.mark.parametrize("name", ["sphere", "torus", "ellipsoid"])
def test_random_and_smoothed_field_match_reference(RVGP, name):
    g = load_golden(name)
    d = RVGP.create_data_object(g["X"], n_neighbors=int(g["k"]), n_eigenpairs=int(g["m"]), verbose=False)
    d.random_vector_field(seed=int(g["field_seed"]))
    np.testing.assert_allclose(d.vectors, g["field_raw"], atol=1e-13)
    d.smooth_vector_field(t=float(g["smooth_t"]))
    # the smoothed ambient field is gauge invariant: compare with the reference's dense-expm result
    np.testing.assert_allclose(d.vectors, g["field_smooth"], atol=1e-10)


@pytest.mark.parametrize("name", ["sphere", "torus", "ellipsoid", "swissroll64"])
def test_fps_matches_reference(RVGP, name):
    from rvgp_gb300.geometry import furthest_point_sampling
    g = load_golden(name)
    p, lam = furthest_point_sampling(g["X"], N=len(g["fps_perm"]))
    assert np.array_equal(p, g["fps_perm"])
    np.testing.assert_allclose(lam, g["fps_lambdas"], rtol=1e-12, atol=1e-14)
    p2, lam2 = furthest_point_sampling(g["X"], spacing=float(g["fps_spacing"]))
    assert np.array_equal(p2, g["fps_perm_spacing"])
    np.testing.assert_allclose(lam2, g["fps_lambdas_spacing"], rtol=1e-12, atol=1e-14)


def test_fps_larger_cloud_against_oracle(RVGP):
    from rvgp_gb300.geometry import furthest_point_sampling
    from rvgp_gb300.workloads import make_points
    X = make_points("bumpy_sphere", 6000, seed=2)
    p, lam = furthest_point_sampling(X, N=400, start_idx=17)
    p_ref, lam_ref = O.furthest_point_sampling(X, N=400, start_idx=17)
    assert np.array_equal(p, p_ref)
    np.testing.assert_array_equal(lam, lam_ref)


def test_field_helpers(RVGP):
    from rvgp_gb300 import geometry
    rng = np.random.default_rng(0)
    T, _ = np.linalg.qr(rng.standard_normal((50, 3, 2)))
    v = rng.standard_normal((50, 3))
    np.testing.assert_allclose(geometry.project_to_manifold(v, T), O.project_to_manifold(v, T), atol=1e-14)
    loc = geometry.express_in_local_frame(v, T)
    np.testing.assert_allclose(loc, O.express_in_local_frame(v, T), atol=1e-14)
    np.testing.assert_allclose(geometry.express_in_local_frame(loc, T, reverse=True),
                               O.express_in_local_frame(loc, T, reverse=True), atol=1e-14)
    S = rng.uniform(0.1, 1, (200, 3))
    assert geometry.manifold_dimension(S.copy(), 0.5) == O.manifold_dimension(S, 0.5)


def test_expm_action_against_scipy(RVGP):
    from rvgp_gb300 import smoothing
    import scipy.sparse.linalg as spla
    g = load_golden("torus")
    L = O.laplacian(g["indptr"], g["indices"], len(g["X"]))
    rng = np.random.default_rng(1)
    x = rng.standard_normal((L.shape[0], 3))
    for t in (0.3, 5.0, 60.0):
        ref = spla.expm_multiply(-t * L.tocsc(), x)
        got = smoothing.scalar_diffusion(x, t, "matrix_exp", L)
        np.testing.assert_allclose(got, ref, atol=1e-11 * np.abs(x).max())


def test_spectral_diffusion(RVGP):
    from rvgp_gb300 import smoothing
    g = load_golden("sphere")
    rng = np.random.default_rng(2)
    V = g["evecs_L"] / np.sqrt(len(g["X"]))
    x = rng.standard_normal((len(g["X"]), 2))
    ref = V @ (np.exp(-2.0 * g["evals_L"])[:, None] * (V.T @ x))
    got = smoothing.scalar_diffusion(x, 2.0, "spectral", (g["evals_L"], g["evecs_L"]))
    np.testing.assert_allclose(got, ref, atol=1e-12)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_fit_transform_against_dense_oracle(RVGP, precision):
    """Posterior at fixed hyperparameters (epochs=0) against the dense GPflow
    restatement on the oracle's own eigenbasis (the kernel is basis invariant)."""
    g = load_golden("sphere")
    X, m = g["X"], int(g["m"])
    d = RVGP.create_data_object(X, n_neighbors=10, n_eigenpairs=m, precision=precision, verbose=False)
    d.random_vector_field(seed=3)
    d.smooth_vector_field(t=20)
    n = len(X)
    train = np.arange(0, n, 2)
    test = np.arange(1, n, 2)
    gp = RVGP.fit(d, train_ind=train, epochs=0, verbose=False)
    mean, var = gp.transform(d, list(map(int, test)))
    # oracle: same split, dense GP with the reference's eigenbasis
    tr, te = O.train_test_split_indices(len(train), 0.2, 0)
    pts = train[tr]
    Phi = g["evecs_Lc"].reshape(n, -1)[pts].reshape(-1, m)
    y = d.vectors[pts].reshape(-1)
    S = O.eval_S(g["evals_Lc"], 1.5, 5.0, 1.0, g["evecs_Lc"].shape[0])
    Phi_te = g["evecs_Lc"].reshape(n, -1)[test].reshape(-1, m)
    m_ref, v_ref = O.predict_f(Phi, y, S, 1.0, Phi_te)
    tol = 1e-7 if precision == "fp64" else 1e-4
    assert np.linalg.norm(mean.ravel() - m_ref) <= tol * np.linalg.norm(m_ref)
    np.testing.assert_allclose(var.ravel(), v_ref, rtol=(1e-5 if precision == "fp64" else 1e-3), atol=1e-8)
    lml_ref = O.lml_dense(Phi, y, S, 1.0)
    ltol = 1e-8 if precision == "fp64" else 1e-5
    assert abs(gp.log_marginal_likelihood() - lml_ref) <= ltol * abs(lml_ref)


def test_fit_optimises_likelihood(RVGP):
    g = load_golden("torus")
    d = RVGP.create_data_object(g["X"], n_neighbors=20, n_eigenpairs=int(g["m"]), verbose=False)
    d.random_vector_field(seed=1)
    d.smooth_vector_field(t=20)
    gp0 = RVGP.fit(d, epochs=0, verbose=False)
    gp = RVGP.fit(d, epochs=50, verbose=False)
    assert gp.log_marginal_likelihood() > gp0.log_marginal_likelihood()
    gpa = RVGP.fit(d, epochs=60, optimizer="adam", lr=0.05, verbose=False)
    assert gpa.log_marginal_likelihood() > gp0.log_marginal_likelihood()
    mean, var = gp.transform(d, np.arange(10))
    assert mean.shape == (10, 3) and var.shape == (10, 3) and np.all(var >= 0)


def test_deferred_eigsh_L_beside_mixed_fit(RVGP, monkeypatch):
    """The concurrent eigensolve of L, deferred to the GP fit
    (RVGP_EIG_L_START=fit): it waits for the fit and runs beside it; by
    default it starts at once.  Either way its eigenpairs equal a direct
    solve's."""
    from rvgp_gb300 import _core
    g = load_golden("torus")
    m = int(g["m"])
    d0 = RVGP.create_data_object(g["X"], n_neighbors=20, n_eigenpairs=m, precision="mixed", verbose=False)
    assert d0._eig_L["thread"] is not None  # started by create_data_object
    ev0 = d0.evals_L
    monkeypatch.setenv("RVGP_EIG_L_START", "fit")
    d = RVGP.create_data_object(g["X"], n_neighbors=20, n_eigenpairs=m, precision="mixed", verbose=False)
    assert d._eig_L["thread"] is None  # not started by create_data_object
    d.random_vector_field(seed=2)
    d.smooth_vector_field(t=20)
    st = d._eig_L
    gpa = RVGP.fit(d, epochs=30, optimizer="adam", lr=0.05, verbose=False)
    assert gpa.fit_form == "mixed"
    assert st["thread"] is not None  # released by the fit
    ev = d.evals_L
    ip = torch.as_tensor(g["L_indptr"], device="cuda", dtype=torch.int32)
    ix = torch.as_tensor(g["L_indices"], device="cuda", dtype=torch.int32)
    ev_ref, _, _ = _core.eigsh(ip, ix, torch.as_tensor(g["L_data"], device="cuda"), m=m, mode="mixed")
    # the mixed form's accuracy: 1e-5 of the largest eigenvalue
    tol = 1e-5 * abs(g["evals_L"]).max()
    np.testing.assert_allclose(ev, ev_ref.cpu().numpy(), rtol=1e-5, atol=tol)
    np.testing.assert_allclose(ev, g["evals_L"], rtol=1e-5, atol=tol)
    # a data object whose L pairs are read before any fit solves them on demand
    d2 = RVGP.create_data_object(g["X"], n_neighbors=20, n_eigenpairs=m, precision="mixed", verbose=False)
    np.testing.assert_allclose(d2.evals_L, ev, rtol=0, atol=0)
    np.testing.assert_allclose(ev0, ev, rtol=0, atol=0)


@pytest.mark.parametrize("B", [1, 6])
def test_predict_fields_matches_per_field_fits(RVGP, B):
    """Many fields at the same training points: predict_fields (one batched
    solve) equals a separate fit(epochs=0) + transform per field, and each
    field's log marginal likelihood equals that fit's."""
    g = load_golden("sphere")
    d = RVGP.create_data_object(g["X"], n_neighbors=10, n_eigenpairs=int(g["m"]), precision="fp64", verbose=False)
    fields = []
    for s in range(B):
        d.random_vector_field(seed=s)
        d.smooth_vector_field(t=10 + 5 * s)
        fields.append(d.vectors)
    fields = np.stack(fields)
    train = np.arange(0, d.n, 3)
    test = np.arange(1, d.n, 3)
    d.vectors = fields[0]
    gp = RVGP.fit(d, train_ind=train, epochs=0, verbose=False)
    means, lml = gp.predict_fields(fields, test)
    means, lml = means.cpu().numpy(), lml.cpu().numpy()
    assert means.shape == (B, len(test), 3)
    for b in range(B):
        d.vectors = fields[b]
        gb = RVGP.fit(d, train_ind=train, epochs=0, verbose=False)
        mb, _ = gb.transform(d, test)
        assert np.linalg.norm(means[b] - mb) <= 1e-10 * np.linalg.norm(mb)
        assert abs(lml[b] - gb.log_marginal_likelihood()) <= 1e-10 * abs(lml[b])
