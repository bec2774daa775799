"""The RVGP data object (RVGP/dataclass.py:21-120) on the GPU.

``data(vertices, vectors=None, dim_man=2, n_neighbors=10,
frac_geodesic_neighbours=1.5, explained_variance=0.8, n_eigenpairs=None)``
runs kNN graph -> geodesic-neighbourhood gauges -> manifold dimension ->
connections -> Laplacians -> eigenpairs of L and Lc -> gauge lift, all as
CUDA kernels.  The reference's attributes (``vertices, n, dim_man, G, gauges,
R, L, Lc, evals_L, evecs_L, evals_Lc, evecs_Lc, vectors``) are available as
host objects (numpy / scipy.sparse, ``G`` as networkx when installed); they are
copied off the device on first access.  The device tensors live in
``self._dev``.

Differences from the reference, each deliberate:
* the gauges keep min(D, K+1) singular values (the reference asks for D and
  therefore rejects K < D, RVGP/lib/ptu_dijkstra.pyx:73-77, e.g. every
  64-dimensional cloud with n_neighbors=15);
* ``n_eigenpairs=None`` raises the error ARPACK would raise (k must be < N - 1)
  instead of attempting a full decomposition;
* ``estimate_dim=False`` uses ``dim_man`` instead of the estimate (the reference
  always estimates and ignores ``dim_man``, RVGP/dataclass.py:37).
"""
from __future__ import annotations

import math
import os
import threading
from types import SimpleNamespace

import numpy as np
import torch

from rvgp_gb300 import _core


def _log(verbose, *a):
    if verbose:
        print(*a)


class data:
    def __init__(self, vertices, vectors=None, dim_man=2, n_neighbors=10, frac_geodesic_neighbours=1.5,
                 explained_variance=0.8, n_eigenpairs=None, *, precision="mixed", estimate_dim=True,
                 strict_rank=True, eig_tol=None, seed=0, verbose=True, timings=None, nvtx=None):
        _core.require_cuda()
        device = torch.device("cuda", torch.cuda.current_device())
        marks = []

        def mark(name):  # CUDA events between stages when a timings dict is given
            if timings is not None:
                ev = torch.cuda.Event(enable_timing=True)
                ev.record()
                marks.append((name, ev))
        mark("start")
        if isinstance(vertices, torch.Tensor):
            X = vertices.to(device=device, dtype=torch.float64).contiguous()
            self._vertices_host = None
        else:
            self._vertices_host = np.asarray(vertices)
            X = torch.as_tensor(np.ascontiguousarray(vertices, dtype=np.float64), device=device)
        n, D = X.shape
        self.precision = precision
        dev = SimpleNamespace(X=X)

        _log(verbose, "Fit graph")
        knn = _core.knn(X, n_neighbors)
        indptr, indices, maxdeg = _core.graph_build(knn)
        dev.indptr, dev.indices, dev.maxdeg = indptr, indices, maxdeg
        dev.L_vals = _core.laplacian_values(indptr, indices)
        dev.bound = 2.0 * maxdeg * (1.0 + 1e-12)  # spectral bound of L and Lc (|D| + |A|)
        # The eigensolves run on the matrices renumbered along a Morton curve
        # of the points: neighbouring rows share neighbours, so the sparse
        # products hit L1 more often.  Their eigenpairs come back in the
        # caller's order.
        dev.perm, dev.rank = _core.locality_order(X)
        dev.ord_indptr, dev.ord_indices, dev.ord_L_vals, _ = _core.permute_csr(indptr, indices, dev.L_vals, None,
                                                                               dev.perm, dev.rank)
        mark("graph")

        # The eigenpairs of L feed nothing downstream (the kernel is built on
        # those of Lc), so they are computed on a second stream by a host
        # thread, off the critical path; every reader of evals_L / evecs_L
        # waits for them (wait()).  It starts at once, beside the gauges and the
        # Lc eigensolve (their latency-bound phases leave SMs idle; measured on
        # the Swiss roll at n = 100 000: 0.638 s per step against 0.663 s when
        # deferred to the GP fit); RVGP_EIG_L_START=fit defers it to fit().
        m = n if n_eigenpairs is None else min(int(n_eigenpairs), n)
        mode = "mixed" if precision == "mixed" else "fp64"
        # nvtx: name of an NVTX range the concurrent eigensolve's host thread
        # opens around its work, so that a profiler that selects kernels by the
        # caller's range also sees the kernels of that thread
        self._eig_L = self._prepare_eig_L(dev, n, m, mode, eig_tol, seed, timings, nvtx)
        if os.environ.get("RVGP_EIG_L_START", "now") != "fit":
            self._release_eig_L()

        _log(verbose, "Fit tangent spaces")
        K = int(n_neighbors * frac_geodesic_neighbours)
        if K >= n:
            raise ValueError("Geodesic neighborhood size must be less than the total number of samples")
        c = min(D, K + 1)
        d_out = min(c, 8)
        T, Sigma, _ = _core.gauges(X, indptr, indices, K, maxdeg, d_out)
        if estimate_dim:
            if explained_variance == 1.0:
                dim = c
            else:
                dim, var_exp = _core.manifold_dimension(Sigma, explained_variance)
                _log(verbose, "Fraction of variance explained: ", var_exp.cpu().numpy())
                if dim < 0:
                    raise IndexError("no number of dimensions explains the requested fraction of variance")
        else:
            dim = int(dim_man)
        if dim > d_out:
            T, Sigma, _ = _core.gauges(X, indptr, indices, K, maxdeg, dim)
        check = c if (strict_rank and D <= K) else dim
        if bool((Sigma[:, :check] < 1e-10).any()):
            raise RuntimeError("Local tangent space approximation failed, at least one geodesic neighborhood does "
                               "not span d-dimensional space")
        dev.T, dev.Sigma = T, Sigma
        mark("gauges")
        _log(verbose, "Predicted manifold dimension is {}".format(dim))

        R, lc64, lc32 = _core.connections(T, dim, indptr, indices, want32=(precision == "mixed"))
        dev.R, dev.Lc_vals, dev.Lc_vals32 = R, lc64, lc32
        _log(verbose, "Fit connections")

        _log(verbose, "Compute Laplacians")
        mark("connections")

        _log(verbose, "Compute eigendecompositions")
        # The Lc eigensolve is on the critical path and shares the GPU with the
        # L eigensolve: it runs on a higher-priority stream, so the block
        # scheduler serves its kernels first (on the Swiss roll at n = 100 000:
        # 0.543 s per step; with equal priorities the Lc eigensolve takes
        # 398 ms instead of 333 ms and the step 0.581 s).
        caller = torch.cuda.current_stream()
        hp = torch.cuda.Stream(priority=-1)
        hp.wait_stream(caller)
        try:
            with torch.cuda.stream(hp):
                _, _, o64, o32 = _core.permute_csr(indptr, indices, lc64, lc32, dev.perm, dev.rank)
                dev.evals_Lc, U, dev.eig_info_Lc = _core.eigsh(dev.ord_indptr, dev.ord_indices, o64, o32, m=m,
                                                               mode=mode, tol=eig_tol, seed=seed + 1,
                                                               scale=math.sqrt(n * dim), perm=dev.perm)
                del o64, o32
        except BaseException:
            if self._eig_L["thread"] is not None:
                self._eig_L["thread"].join()
            raise
        caller.wait_stream(hp)
        for t_ in (dev.evals_Lc, U):
            t_.record_stream(caller)  # allocated on hp, used on the caller's stream
        # The ambient (lifted) eigenvectors evecs_Lc = T_i U_i (n*D x m) are
        # formed on first use: the GP works on U and the gauges directly.
        dev.evecs_Lc_local = U
        dev.evecs_Lc = None
        mark("eigsh_Lc")
        self._dev = dev
        if timings is not None:
            torch.cuda.synchronize()
            for (a, ea), (b, eb) in zip(marks[:-1], marks[1:]):
                timings[b] = timings.get(b, 0.0) + ea.elapsed_time(eb) / 1e3
        dev.vectors = None
        self._dev = dev
        self.n = n
        self.dim_man = dim
        self.n_eigenpairs = m
        self._host = {}
        self.vectors = vectors

    def _evecs_Lc_dev(self):
        """The lifted eigenvectors (n*D, m) on the device (RVGP/dataclass.py:57-59),
        formed on first use from the gauges and the local eigenvectors."""
        d = self._dev
        if getattr(d, "evecs_Lc", None) is None:
            d.evecs_Lc = _core.lift(d.T, self.dim_man, d.evecs_Lc_local)
        return d.evecs_Lc

    # ------------------------------------------------------------------ the concurrent eigensolve of L
    @staticmethod
    def _prepare_eig_L(dev, n, m, mode, eig_tol, seed, timings, nvtx=None):
        main = torch.cuda.current_stream()
        ready = torch.cuda.Event()
        ready.record(main)  # L's renumbered CSR and values are ready
        side = torch.cuda.Stream()
        state = {"error": None, "seconds": None, "thread": None, "stream": side, "timings": timings}
        timed = timings is not None

        def run():
            if nvtx:
                torch.cuda.nvtx.range_push(nvtx)
            try:
                with torch.cuda.device(main.device), torch.cuda.stream(side):
                    side.wait_event(ready)
                    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)] if timed else None
                    if timed:
                        ev[0].record()
                    out = _core.eigsh(dev.ord_indptr, dev.ord_indices, dev.ord_L_vals, None, m=m, mode=mode,
                                      tol=eig_tol, seed=seed, scale=math.sqrt(n), perm=dev.perm)
                    if timed:
                        ev[1].record()
                    side.synchronize()
                    dev.evals_L, dev.evecs_L, dev.eig_info_L = out
                    if timed:
                        state["seconds"] = ev[0].elapsed_time(ev[1]) / 1e3
            except BaseException as e:  # re-raised by wait()
                state["error"] = e
            finally:
                if nvtx:
                    torch.cuda.nvtx.range_pop()

        state["run"] = run
        return state

    def _release_eig_L(self):
        """Start the pending eigensolve of L (once)."""
        st = self.__dict__.get("_eig_L")
        if st is not None and st["thread"] is None:
            st["thread"] = threading.Thread(target=st["run"], name="rvgp-eigsh-L", daemon=True)
            st["thread"].start()

    def wait(self):
        """Block until the eigenpairs of L (computed concurrently) are ready; the
        caller's current stream then also waits for them on the device."""
        st = self.__dict__.get("_eig_L")
        if st is None:
            return self
        self._release_eig_L()
        st["thread"].join()
        if st["timings"] is not None and st["seconds"] is not None:
            st["timings"]["eigsh_L (concurrent)"] = st["seconds"]
        if st["error"] is not None:
            err = st["error"]
            st["error"] = None
            raise err
        torch.cuda.current_stream().wait_stream(st["stream"])
        self.__dict__["_eig_L"] = None
        return self

    # ------------------------------------------------------------------ persistence
    _SAVED = ("X", "indptr", "indices", "L_vals", "perm", "rank", "ord_indptr", "ord_indices", "ord_L_vals", "T",
              "Sigma", "R", "Lc_vals", "Lc_vals32", "evals_L", "evecs_L", "evals_Lc", "evecs_Lc", "evecs_Lc_local",
              "vectors")
    _FORMAT = 1

    def save(self, path):
        """Write the computed geometry (graph, gauges, connections, Laplacians,
        both eigendecompositions, vectors) to one ``.npz`` file, so later fits
        skip the eigensolves.  ``load_data_object(path)`` restores it on the
        current device."""
        import json
        self.wait()
        d = self._dev
        arrays = {k: getattr(d, k).cpu().numpy() for k in self._SAVED if getattr(d, k, None) is not None}
        meta = {"format": self._FORMAT, "n": self.n, "dim_man": self.dim_man, "n_eigenpairs": self.n_eigenpairs,
                "precision": self.precision, "maxdeg": int(d.maxdeg), "bound": float(d.bound),
                "eig_info_L": getattr(d, "eig_info_L", None), "eig_info_Lc": getattr(d, "eig_info_Lc", None)}
        np.savez(path, __meta__=np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8), **arrays)

    @classmethod
    def load(cls, path):
        """A data object from a file written by ``save`` (no recomputation)."""
        import json
        _core.require_cuda()
        device = torch.device("cuda", torch.cuda.current_device())
        with np.load(path) as z:
            meta = json.loads(bytes(z["__meta__"]).decode())
            if meta.get("format") != cls._FORMAT:
                raise ValueError(f"{path}: unsupported data-object format {meta.get('format')!r}")
            dev = SimpleNamespace(**{k: torch.as_tensor(z[k], device=device) for k in cls._SAVED if k in z.files})
        for k in cls._SAVED:
            if not hasattr(dev, k):
                setattr(dev, k, None)
        dev.maxdeg, dev.bound = meta["maxdeg"], meta["bound"]
        dev.eig_info_L, dev.eig_info_Lc = meta["eig_info_L"], meta["eig_info_Lc"]
        obj = cls.__new__(cls)
        obj._vertices_host = None
        obj.precision = meta["precision"]
        obj._eig_L = None
        obj._dev = dev
        obj.n, obj.dim_man, obj.n_eigenpairs = meta["n"], meta["dim_man"], meta["n_eigenpairs"]
        obj._host = {}
        return obj

    # ------------------------------------------------------------------ host views
    def _cached(self, key, fn):
        if key not in self._host:
            self._host[key] = fn()
        return self._host[key]

    @property
    def vertices(self):
        if self._vertices_host is None:
            self._vertices_host = self._dev.X.cpu().numpy()
        return self._vertices_host

    @property
    def vectors(self):
        if self._dev.vectors is None:
            return None
        return self._cached("vectors", lambda: self._dev.vectors.cpu().numpy())

    @vectors.setter
    def vectors(self, v):
        self._host.pop("vectors", None)
        if v is None:
            self._dev.vectors = None
        elif isinstance(v, torch.Tensor):
            self._dev.vectors = v.to(device=self._dev.X.device, dtype=torch.float64).contiguous()
        else:
            self._host["vectors"] = np.asarray(v)
            self._dev.vectors = torch.as_tensor(np.ascontiguousarray(v, dtype=np.float64), device=self._dev.X.device)

    @property
    def gauges(self):
        return self._cached("gauges", lambda: np.ascontiguousarray(
            self._dev.T[:, :, :self.dim_man].cpu().numpy()))

    @property
    def L(self):
        import scipy.sparse as sp
        d = self._dev
        return self._cached("L", lambda: sp.csr_matrix(
            (d.L_vals.cpu().numpy(), d.indices.cpu().numpy(), d.indptr.cpu().numpy()), shape=(self.n, self.n)))

    @property
    def Lc(self):
        import scipy.sparse as sp
        d, k = self._dev, self.dim_man
        return self._cached("Lc", lambda: sp.bsr_matrix(
            (d.Lc_vals.cpu().numpy(), d.indices.cpu().numpy(), d.indptr.cpu().numpy()),
            shape=(self.n * k, self.n * k)))

    @property
    def R(self):
        """Transports as the reference's COO nd x nd (RVGP/lib/ptu_dijkstra.pyx:194-197)."""
        import scipy.sparse as sp

        def build():
            d, k = self._dev, self.dim_man
            ip, ix = d.indptr.cpu().numpy(), d.indices.cpu().numpy()
            rows = np.repeat(np.arange(self.n), np.diff(ip))
            p, q = np.meshgrid(np.arange(k), np.arange(k), indexing="ij")
            r = (rows[:, None] * k + p.ravel()[None, :]).ravel()
            c = (ix[:, None] * k + q.ravel()[None, :]).ravel()
            return sp.coo_matrix((d.R.cpu().numpy().ravel(), (r, c)))
        return self._cached("R", build)

    @property
    def evals_L(self):
        self.wait()
        return self._cached("evals_L", lambda: self._dev.evals_L.cpu().numpy())

    @property
    def evecs_L(self):
        self.wait()
        return self._cached("evecs_L", lambda: self._dev.evecs_L.cpu().numpy())

    @property
    def evals_Lc(self):
        return self._cached("evals_Lc", lambda: self._dev.evals_Lc.cpu().numpy())

    @property
    def evecs_Lc(self):
        return self._cached("evecs_Lc", lambda: self._evecs_Lc_dev().cpu().numpy())

    @property
    def G(self):
        """The kNN graph as a networkx Graph with 'pos' node attributes (needs networkx)."""
        def build():
            import networkx as nx
            A = self.L.copy()
            A.data[:] = 1.0
            G = nx.from_scipy_sparse_array(A)
            nx.set_node_attributes(G, {i: self.vertices[i] for i in G.nodes}, "pos")
            return G
        return self._cached("G", build)

    # ------------------------------------------------------------------ fields
    def random_vector_field(self, seed=0):
        """Generate random vector field over manifold (RVGP/dataclass.py:91-103).

        The random numbers come from numpy's legacy global generator exactly as
        in the reference; projection and normalisation run on the GPU."""
        np.random.seed(seed)
        v = np.random.uniform(low=-0.5, high=0.5, size=(self.n, self._dev.X.shape[1]))
        vd = torch.as_tensor(v, device=self._dev.X.device)
        vd = _core.frame_map(self._dev.T, self.dim_man, vd, "project")
        self.vectors = _core.normalise_rows(vd)

    def smooth_vector_field(self, t=100):
        """Vector diffusion of the field (RVGP/dataclass.py:105-120) with the exact
        action of exp(-t Lc) (and exp(-t L) for the magnitude renormalisation)."""
        if self._dev.vectors is None:
            print("No vectors found. Nothing to smooth.")
            return
        d = self._dev
        loc = _core.frame_map(d.T, self.dim_man, d.vectors, "to_local")
        # the smallest eigenvalue of Lc (known from the eigensolver) keeps the
        # Chebyshev sum free of cancellation at large t
        shift = max(0.0, float(d.evals_Lc[0]) * (1.0 - 1e-9) - 1e-12)
        loc = _core.vector_diffusion(d.indptr, d.indices, d.L_vals, d.Lc_vals, loc, t, d.bound, d.bound, shift)
        self.vectors = _core.frame_map(d.T, self.dim_man, loc, "from_local")


def load_data_object(path):
    """Restore a data object written by ``data.save`` on the current CUDA device."""
    return data.load(path)
