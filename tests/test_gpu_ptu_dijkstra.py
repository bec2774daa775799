"""GPU parity of the drop-in for the reference's native module
(rvgp_gb300.ptu_dijkstra vs RVGP/lib/ptu_dijkstra.pyx): tangent_frames and
connections called with the reference's signatures on the graphs of the
golden fixtures, whose tangents, Sigma and transports the reference's own
compiled Cython produced (tests/golden/make_golden.py).

Tolerances: Sigma 1e-11 relative; frames by projector distance 1e-11 (signs
are LAPACK's in the reference); transports 1e-12 against the reference's R,
with the COO rows / columns (p-major expansion) equal."""
import numpy as np
import pytest
import scipy.sparse as sp

from conftest import load_golden, projector_distance

pytestmark = pytest.mark.gpu


def adjacency(g):
    n = len(g["X"])
    return sp.csr_matrix((np.ones(g["indices"].size), g["indices"], g["indptr"]), shape=(n, n))


@pytest.mark.parametrize("name", ["sphere", "torus", "ellipsoid", "swissroll64"])
def test_tangent_frames_drop_in(name):
    from rvgp_gb300 import ptu_dijkstra
    g = load_golden(name)
    X, K, d = g["X"], int(g["K"]), int(g["dim_man"])
    D = X.shape[1]
    ask = D if "tangents_full" in g else d  # what the golden asked the reference for
    T, S = ptu_dijkstra.tangent_frames(X, adjacency(g), ask, g["k"] * g["frac"])
    assert T.shape == (len(X), D, ask) and S.shape == (len(X), ask)
    Sg = g["Sigma"]
    np.testing.assert_allclose(S[:, :Sg.shape[1]], Sg, rtol=1e-11, atol=1e-13)
    assert projector_distance(T[:, :, :d], g["gauges"]) < 1e-11


@pytest.mark.parametrize("name", ["sphere", "torus", "ellipsoid", "swissroll64"])
def test_connections_drop_in(name):
    from rvgp_gb300 import ptu_dijkstra
    g = load_golden(name)
    d = int(g["dim_man"])
    R = ptu_dijkstra.connections(g["gauges"], adjacency(g), d)
    assert isinstance(R, sp.coo_matrix)
    n = len(g["X"])
    rows = np.repeat(np.arange(n), np.diff(g["indptr"]))
    p, q = np.meshgrid(np.arange(d), np.arange(d), indexing="ij")
    np.testing.assert_array_equal(R.row, (rows[:, None] * d + p.ravel()).ravel())
    np.testing.assert_array_equal(R.col, (g["indices"][:, None] * d + q.ravel()).ravel())
    np.testing.assert_allclose(R.data, g["R"].ravel(), rtol=0, atol=1e-12)


def test_networkx_graph_input():
    nx = pytest.importorskip("networkx")
    from rvgp_gb300 import ptu_dijkstra
    g = load_golden("sphere")
    G = nx.from_scipy_sparse_array(adjacency(g))
    T, S = ptu_dijkstra.tangent_frames(g["X"], G, 3, g["k"] * g["frac"])
    np.testing.assert_allclose(S, g["Sigma"], rtol=1e-11, atol=1e-13)
    R = ptu_dijkstra.connections(g["gauges"], G, int(g["dim_man"]))
    np.testing.assert_allclose(R.data, g["R"].ravel(), rtol=0, atol=1e-12)
