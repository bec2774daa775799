"""Generate tests/golden/kernel.npz from the reference's own ``RVGP/kernels.py``.

``ManifoldKernel.eval_S``, ``K`` and ``K_diag`` (RVGP/kernels.py:41-67) run
unchanged on the eigenpairs of the committed geometry fixtures, through the
numpy-backed TensorFlow stub of ``ref_harness`` (every operation they use is a
plain FP64 array operation there) and a ``gpflow.Parameter`` stub that returns
its value.  The data object handed to the kernel carries the fixture's
``evals_Lc`` and lifted ``evecs_Lc`` (RVGP/dataclass.py:57-59, recomputed from
the fixture's gauges and local eigenvectors where the fixture omits it).

    python tests/golden/make_kernel_golden.py
"""
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

from ref_harness import load_reference_kernels  # noqa: E402

CASES = ["sphere", "torus", "ellipsoid", "swissroll64"]
# (typ, nu, kappa, sigma_f): the default kernel of RVGP/main.py:30, the
# constructor defaults of RVGP/kernels.py:25, and values away from both
PARAMS = [("matern", 1.5, 5.0, 1.0), ("matern", 3.0, 4.0, 1.0), ("matern", 0.7, 1.3, 2.5),
          ("se", 3.0, 0.8, 1.7), ("se", 3.0, 2.2, 0.4)]


def lifted(g):
    if "evecs_Lc" in g:
        return g["evecs_Lc"]
    n, D, d = g["gauges"].shape
    m = g["evecs_Lc_local"].shape[1]
    return np.einsum("bij,bjk->bik", g["gauges"], g["evecs_Lc_local"].reshape(n, d, m)).reshape(n * D, m)


def main():
    kernels = load_reference_kernels()
    out = {}
    rng = np.random.default_rng(0)
    for name in CASES:
        g = dict(np.load(os.path.join(HERE, f"{name}.npz")))
        ev = lifted(g)
        data = types.SimpleNamespace(evecs_Lc=ev, evals_Lc=g["evals_Lc"])
        rows = np.sort(rng.choice(ev.shape[0], 40, replace=False))
        rows2 = np.sort(rng.choice(ev.shape[0], 25, replace=False))
        X, X2 = ev[rows], ev[rows2]
        out[f"{name}_rows"], out[f"{name}_rows2"] = rows, rows2
        for c, (typ, nu, kappa, sf) in enumerate(PARAMS):
            k = kernels.ManifoldKernel(data, nu=nu, kappa=kappa, sigma_f=sf, typ=typ)
            key = f"{name}_{c}"
            out[key + "_S"] = np.asarray(k.eval_S(typ=typ), dtype=np.float64)
            out[key + "_K"] = np.asarray(k.K(X), dtype=np.float64)
            out[key + "_K2"] = np.asarray(k.K(X, X2), dtype=np.float64)
            out[key + "_Kdiag"] = np.asarray(k.K_diag(X), dtype=np.float64)
        out[f"{name}_n_rows"] = np.float64(ev.shape[0])
    out["params_typ"] = np.array([p[0] for p in PARAMS])
    out["params"] = np.array([p[1:] for p in PARAMS], dtype=np.float64)
    path = os.path.join(HERE, "kernel.npz")
    np.savez_compressed(path, **out)
    print(f"kernel: {len(CASES)} fixtures x {len(PARAMS)} parameter sets -> {os.path.getsize(path)} B")


if __name__ == "__main__":
    main()
