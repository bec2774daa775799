"""GPU: vector-field features (div / curl, examples/eeg_example/eeg_utils.py:37-80)
against the reference's own outputs, and a mesh read by ``load_mesh`` run end to
end (data object, furthest-point sampling by spacing, fit, transform)."""
import numpy as np
import pytest

from conftest import load_golden
from oracle import rvgp_oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def RVGP():
    import rvgp_gb300
    return rvgp_gb300


@pytest.mark.parametrize("case", ["small", "large"])
def test_features_match_reference(RVGP, case):
    from rvgp_gb300.features import compute_vectorfield_features
    g = load_golden("features")
    div, curl = compute_vectorfield_features(g[f"{case}_pos"], g[f"{case}_vec"], k=5)
    # terms (Δu·Δp)/|Δp|² reach ~1e3 here: 1e-12 relative plus 1e-11 absolute
    np.testing.assert_allclose(div, g[f"{case}_div"], rtol=1e-12, atol=1e-11)
    np.testing.assert_allclose(curl, g[f"{case}_curl"], rtol=1e-12, atol=1e-11)
    d2, c2 = compute_vectorfield_features(g[f"{case}_pos"], g[f"{case}_vec"], k=5, reference_quirks=False)
    od, oc = O.vectorfield_features(g[f"{case}_pos"], g[f"{case}_vec"], k=5, reference_quirks=False)
    np.testing.assert_allclose(d2, od, rtol=1e-12, atol=1e-11)
    np.testing.assert_allclose(c2, oc, rtol=1e-12, atol=1e-11)


def test_features_over_time_in_one_launch(RVGP):
    from rvgp_gb300.features import compute_vectorfield_features, compute_vectorfield_features_time
    g = load_golden("features")
    P = g["large_pos"]
    rng = np.random.default_rng(1)
    V = rng.standard_normal((6, len(P), 3))
    div, curl = compute_vectorfield_features_time(range(6), P, V, k=7)
    assert div.shape == (6, len(P)) and curl.shape == (6, len(P), 3)
    for t in (0, 5):
        d1, c1 = compute_vectorfield_features(P, V[t], k=7)
        np.testing.assert_array_equal(div[t], d1)
        np.testing.assert_array_equal(curl[t], c1)
    with pytest.raises(ValueError):
        compute_vectorfield_features(P[:, :2], V[0][:, :2])


def test_mesh_end_to_end(RVGP, tmp_path):
    from rvgp_gb300.geometry import furthest_point_sampling
    from rvgp_gb300.utils import load_mesh
    g = load_golden("features")
    (tmp_path / "uvsphere.obj").write_text(bytes(g["obj_text"]).decode())
    verts, faces = load_mesh("uvsphere", folder=str(tmp_path))
    perm, lam = furthest_point_sampling(verts, spacing=0.15)
    ref_perm, ref_lam = O.furthest_point_sampling(verts, spacing=0.15)
    np.testing.assert_array_equal(perm, ref_perm)
    d = RVGP.create_data_object(verts, n_neighbors=8, n_eigenpairs=20, verbose=False)
    d.random_vector_field(seed=0)
    d.smooth_vector_field(t=10)
    gp = RVGP.fit(d, epochs=5, verbose=False)
    mean, var = gp.transform(d, np.arange(10))
    assert mean.shape == (10, 3) and np.isfinite(mean).all() and (var >= -1e-9).all()
