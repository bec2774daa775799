"""Import the reference RVGP package unchanged, for generating golden fixtures.

Runs only where the reference checkout and its Python dependencies exist
(sklearn, networkx, Cython-built ``ptu_dijkstra`` from ``oracle/build_ref.py``).
TensorFlow and GPflow are absent, so three harness-side shims are installed;
no reference file is edited:

1. a stub ``tensorflow`` with ``float64`` and ``convert_to_tensor`` returning an
   ndarray subclass that has ``.numpy()`` (used by ``RVGP/geometry.py:7,77-78``),
   and numpy-backed ``pow``, ``multiply``, ``reduce_sum``, ``exp``,
   ``transpose``, ``cast``, ``shape`` and ``linalg.tensor_diag_part`` (every
   TensorFlow operation of ``RVGP/kernels.py:41-67``), so the reference's own
   ``ManifoldKernel`` runs in FP64;
2. a stub ``gpflow`` exposing the names ``RVGP/kernels.py`` and ``RVGP/main.py``
   touch at import time;
3. ``ptu_dijkstra.nx`` is wrapped so ``adjacency_matrix`` returns int32 CSR
   indices, which the Cython signature ``int[:]`` requires
   (``RVGP/lib/ptu_dijkstra.pyx:222-223``); modern scipy/networkx return int64.
"""
import os
import sys
import types

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
REFERENCE = os.environ.get("RVGP_REFERENCE", "/root/reference")


class _TFArray(np.ndarray):
    def numpy(self):
        return np.asarray(self)


def _install_stubs():
    if "tensorflow" not in sys.modules:
        tf = types.ModuleType("tensorflow")
        tf.float64 = np.float64
        tf.convert_to_tensor = lambda x, dtype=None: np.asarray(x, dtype=dtype).view(_TFArray)
        tf.pow = lambda x, y: np.power(np.asarray(x, dtype=np.float64), y)
        tf.multiply = lambda x, y: np.multiply(x, y)
        tf.reduce_sum = lambda x: np.sum(x)
        tf.exp = lambda x: np.exp(np.asarray(x, dtype=np.float64))
        tf.transpose = lambda x: np.transpose(x)
        tf.cast = lambda x, dtype=None: np.asarray(x, dtype=dtype)
        tf.shape = lambda x: np.asarray(np.shape(x))
        tf.linalg = types.SimpleNamespace(tensor_diag_part=lambda x: np.diagonal(x).copy())
        sys.modules["tensorflow"] = tf
    if "gpflow" not in sys.modules:
        gp = types.ModuleType("gpflow")

        class _Kernel:
            def __init__(self, *a, **k):
                pass

        gp.kernels = types.SimpleNamespace(Kernel=_Kernel, RBF=None)
        gp.models = types.SimpleNamespace(GPR=object, SGPR=object)
        gp.Parameter = lambda v, **k: v
        gp.utilities = types.SimpleNamespace(positive=lambda *a, **k: None)
        gp.config = types.SimpleNamespace(set_default_positive_minimum=lambda v: None)
        gp.optimizers = types.SimpleNamespace(Scipy=None)
        gp.set_trainable = lambda *a, **k: None
        sys.modules["gpflow"] = gp


def load_reference_kernels():
    """Return the reference's ``RVGP.kernels`` module (TensorFlow/GPflow stubbed)."""
    load_reference()
    from RVGP import kernels
    return kernels


def load_reference():
    """Return (geometry, dataclass, ptu_dijkstra) modules of the reference."""
    sys.dont_write_bytecode = True
    ref_dir = os.path.join(REPO, "oracle", "_ref")
    if not os.path.isdir(ref_dir):
        raise RuntimeError("build oracle/_ref first: python oracle/build_ref.py")
    _install_stubs()
    for p in (ref_dir, REFERENCE):
        if p not in sys.path:
            sys.path.insert(0, p)
    import networkx as nx
    import ptu_dijkstra

    class _NxInt32:
        def __getattr__(self, name):
            return getattr(nx, name)

        @staticmethod
        def adjacency_matrix(G, weight="weight"):
            A = nx.adjacency_matrix(G, weight=weight).tocsr()
            A.indices = A.indices.astype(np.int32)
            A.indptr = A.indptr.astype(np.int32)
            return A

    ptu_dijkstra.nx = _NxInt32()
    from RVGP import geometry, dataclass  # noqa: E402
    return geometry, dataclass, ptu_dijkstra
