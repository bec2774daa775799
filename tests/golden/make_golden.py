"""Generate the golden fixtures in tests/golden/*.npz from the reference's own code.

Runs where the reference checkout, sklearn, networkx and Cython are available
(``python oracle/build_ref.py`` first).  The fixtures are committed, so the test
suite itself never needs the reference.

Every array comes from the reference: ``RVGP.geometry.manifold_graph``, the
Cython ``tangent_frames`` / ``connections`` built from
``RVGP/lib/ptu_dijkstra.pyx``, ``compute_laplacian``,
``compute_connection_laplacian``, ``compute_spectrum`` (ARPACK ``which="SM"``),
``data.random_vector_field`` / ``smooth_vector_field`` (dense ``expm``),
``furthest_point_sampling`` and sklearn's ``train_test_split``.
Inputs are seeded synthetic point clouds with the shapes of the benchmark
workloads, scaled down so the reference finishes in seconds.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from ref_harness import load_reference  # noqa: E402
from rvgp_gb300.workloads import make_points  # noqa: E402


def _sym_csr(G, ptu):
    """The symmetrised CSR the Cython routines iterate over (pyx:84-103)."""
    A = ptu.nx.adjacency_matrix(G, weight="weight")
    A = A.maximum(A.T.tocsr()).tocsr()
    A.sort_indices()
    return A.indptr.astype(np.int32), A.indices.astype(np.int32), A.data


def case(name, X, k, m, frac=1.5, d_override=None, smooth_t=None, field_seed=1):
    geometry, dataclass, ptu = load_reference()
    out = dict(X=X, k=k, m=m, frac=frac)
    n, D = X.shape
    K = int(k * frac)
    G = geometry.manifold_graph(X, n_neighbors=k)
    indptr, indices, w = _sym_csr(G, ptu)
    assert np.all(w == 1.0)
    out.update(indptr=indptr, indices=indices)
    if d_override is None:
        tang, Sigma = ptu.tangent_frames(X, G, D, k * frac)
        out.update(tangents_full=tang, Sigma=Sigma.copy())
        dim_man = geometry.manifold_dimension(Sigma.copy(), frac_explained=0.8)
        gauges = np.ascontiguousarray(tang[:, :, :dim_man])
    else:
        dim_man = d_override
        tang, Sigma = ptu.tangent_frames(X, G, dim_man, k * frac)
        out.update(Sigma=Sigma.copy())
        gauges = tang
    out.update(dim_man=dim_man, gauges=gauges, K=K)
    R = ptu.connections(gauges, G, dim_man)
    E = indices.size
    rr, cc = R.row.reshape(E, dim_man * dim_man), R.col.reshape(E, dim_man * dim_man)
    assert np.array_equal(rr[:, 0] // dim_man, np.repeat(np.arange(n), np.diff(indptr)))
    assert np.array_equal(cc[:, 0] // dim_man, indices)
    out["R"] = R.data.reshape(E, dim_man, dim_man)
    L = geometry.compute_laplacian(G)
    L.sort_indices()
    out.update(L_data=L.data, L_indptr=L.indptr.astype(np.int32), L_indices=L.indices.astype(np.int32))
    Lc = geometry.compute_connection_laplacian(G, R).tocsr()
    Lc.sort_indices()
    out.update(Lc_data=Lc.data, Lc_indptr=Lc.indptr.astype(np.int32), Lc_indices=Lc.indices.astype(np.int32))
    evals_L, evecs_L = geometry.compute_spectrum(L, m)
    evals_Lc, evecs = geometry.compute_spectrum(Lc, m)
    evecs = np.asarray(evecs).reshape(n, dim_man, m)
    evecs_Lc = np.einsum("bij,bjk->bik", gauges, evecs).reshape(n * D, m)
    out.update(evals_L=np.asarray(evals_L), evecs_L=np.asarray(evecs_L),
               evals_Lc=np.asarray(evals_Lc), evecs_Lc_local=evecs.reshape(n * dim_man, m))
    if D <= 3:  # the lifted basis is exact to recompute from gauges; keep it only where small
        out["evecs_Lc"] = evecs_Lc
    if smooth_t is not None:
        obj = dataclass.data.__new__(dataclass.data)
        obj.vertices, obj.gauges, obj.dim_man, obj.L, obj.Lc = X, gauges, dim_man, L, Lc
        obj.random_vector_field(seed=field_seed)
        out["field_raw"] = obj.vectors.copy()
        obj.smooth_vector_field(t=smooth_t)
        out.update(field_smooth=np.asarray(obj.vectors), smooth_t=smooth_t, field_seed=field_seed)
    perm, lam = geometry.furthest_point_sampling(X, N=min(60, n))
    out.update(fps_perm=perm, fps_lambdas=lam)
    perm2, lam2 = geometry.furthest_point_sampling(X, spacing=0.25)
    out.update(fps_spacing=0.25, fps_perm_spacing=perm2, fps_lambdas_spacing=lam2)
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **out)
    print(f"{name}: n={n} D={D} k={k} K={K} d={dim_man} E={E} -> {os.path.getsize(path)} B")


def split_cases():
    from sklearn.model_selection import train_test_split
    rows = []
    for n, ts, seed in [(10, 0.2, 0), (37, 0.2, 0), (800, 0.2, 0), (801, 0.25, 3), (5, 0.5, 7)]:
        a = np.arange(n)
        tr, te = train_test_split(a, a, test_size=ts, random_state=seed)[:2]
        rows.append((n, ts, seed, tr, te))
    np.savez_compressed(os.path.join(HERE, "train_test_split.npz"),
                        **{f"c{i}_{key}": val for i, r in enumerate(rows)
                           for key, val in zip(("n", "test_size", "seed", "train", "test"), r)})
    print("train_test_split: %d cases" % len(rows))


if __name__ == "__main__":
    case("sphere", make_points("sphere", 300, seed=0), k=10, m=16, smooth_t=100)
    case("torus", make_points("torus", 400, seed=0), k=20, m=16, smooth_t=50)
    case("ellipsoid", make_points("half_ellipsoid", 300, seed=0), k=12, m=12, smooth_t=20)
    case("swissroll64", make_points("swissroll64", 300, seed=0), k=15, m=12, d_override=2)
    split_cases()
