"""GPU: a data object written by ``save`` and restored by ``load_data_object``
gives the same attributes bit for bit and the same fits, without recomputing
the geometry."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def RVGP():
    import rvgp_gb300
    return rvgp_gb300


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_save_load_roundtrip(RVGP, tmp_path, precision):
    g = load_golden("sphere")
    d = RVGP.create_data_object(g["X"], n_neighbors=10, n_eigenpairs=int(g["m"]), precision=precision,
                                verbose=False)
    d.random_vector_field(seed=2)
    d.smooth_vector_field(t=20)
    path = str(tmp_path / "sphere.npz")
    d.save(path)
    e = RVGP.load_data_object(path)
    assert (e.n, e.dim_man, e.n_eigenpairs, e.precision) == (d.n, d.dim_man, d.n_eigenpairs, d.precision)
    for name in ("vertices", "gauges", "evals_L", "evecs_L", "evals_Lc", "evecs_Lc", "vectors"):
        np.testing.assert_array_equal(getattr(e, name), getattr(d, name), err_msg=name)
    assert (e.L != d.L).nnz == 0
    np.testing.assert_array_equal(e.Lc.toarray(), d.Lc.toarray())
    train = np.arange(0, d.n, 2)
    test = np.arange(1, d.n, 2)
    m1, v1 = RVGP.fit(d, train_ind=train, epochs=0, verbose=False).transform(d, test)
    m2, v2 = RVGP.fit(e, train_ind=train, epochs=0, verbose=False).transform(e, test)
    np.testing.assert_array_equal(m1, m2)
    np.testing.assert_array_equal(v1, v2)
    r1, _ = RVGP.fit(d, train_ind=train, kernel="rbf", epochs=0, verbose=False).transform(d, test)
    r2, _ = RVGP.fit(e, train_ind=train, kernel="rbf", epochs=0, verbose=False).transform(e, test)
    np.testing.assert_array_equal(r1, r2)
    e.smooth_vector_field(t=5)  # the restored object keeps working as a data object
    assert np.isfinite(e.vectors).all()


def test_load_rejects_other_files(RVGP, tmp_path):
    path = str(tmp_path / "other.npz")
    np.savez(path, x=np.zeros(3))
    with pytest.raises(KeyError):
        RVGP.load_data_object(path)
