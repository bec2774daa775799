"""ctypes bindings of librvgp_gb300.so (the C ABI in include/rvgp_gb300.h).

Every wrapper takes and returns torch tensors on the current CUDA device and
launches on torch's current stream.  There is no CPU path: without the built
library or a CUDA device these functions raise.
"""
from __future__ import annotations

import ctypes
import os

import torch

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librvgp_gb300.so")

c_int, c_size_t, c_void_p, c_double, c_float = (ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_double,
                                                ctypes.c_float)
P = c_void_p

# name -> (restype, argtypes)
SIGNATURES = {
    "rvgp_last_error": (ctypes.c_char_p, []),
    "rvgp_abi_version": (c_int, []),
    "rvgp_launch_count": (ctypes.c_longlong, []),
    "rvgp_knn_workspace": (c_size_t, [c_int, c_int, c_int]),
    "rvgp_knn": (c_int, [P, c_int, c_int, c_int, P, P, c_size_t, P]),
    "rvgp_knn_fallback_rows": (c_int, [c_int, c_int, c_int, P, P]),
    "rvgp_knn_noalloc": (c_int, [P, c_int, c_int, c_int, P, P]),
    "rvgp_graph_workspace": (c_size_t, [c_int, c_int]),
    "rvgp_graph_build": (c_int, [P, c_int, c_int, P, P, P, P, P, c_size_t, P]),
    "rvgp_laplacian_values": (c_int, [P, P, c_int, P, P]),
    "rvgp_gauges_workspace": (c_size_t, [c_int, c_int, c_int, c_int]),
    "rvgp_gauges": (c_int, [P, c_int, c_int, P, P, c_int, c_int, c_int, P, P, P, P, P, c_size_t, P]),
    "rvgp_connections": (c_int, [P, c_int, c_int, c_int, c_int, P, P, P, P, P, P]),
    "rvgp_bspmm_f32": (c_int, [c_int, c_int, P, P, P, P, P, P, c_int, c_int, c_float, c_float, c_float, P]),
    "rvgp_bspmm_f64": (c_int, [c_int, c_int, P, P, P, P, P, P, c_int, c_int, c_double, c_double, c_double, P]),
    "rvgp_eigsh_workspace": (c_size_t, [c_int, c_int, c_int, c_int, c_int]),
    "rvgp_spectral_S": (c_int, [P, c_int, P, c_double, c_int, P, P, P, P]),
    "rvgp_lift": (c_int, [P, c_int, c_int, c_int, c_int, P, c_int, P, P]),
    "rvgp_gather_rows": (c_int, [P, c_int, c_int, P, c_int, P, P, P, P, P]),
    "rvgp_gp_prepare_workspace": (c_size_t, [ctypes.c_longlong, c_int]),
    "rvgp_gp_prepare": (c_int, [P, P, P, ctypes.c_longlong, c_int, c_int, P, P, P, P, c_size_t, P]),
    "rvgp_gp_lml_workspace": (c_size_t, [c_int]),
    "rvgp_gp_state_size": (c_size_t, [c_int]),
    "rvgp_gp_lml": (c_int, [P, P, P, ctypes.c_longlong, c_int, P, c_double, c_int, P, P, P, P, c_size_t, P]),
    "rvgp_gp_fit_adam": (c_int, [P, P, P, ctypes.c_longlong, c_int, P, c_double, c_int, P, P, P, c_int, c_double,
                                 c_double, c_double, c_double, P, P, P, P, P, c_size_t, P]),
    "rvgp_gp_fit_mixed_max_m": (c_int, []),
    "rvgp_symeig_f32_workspace": (c_size_t, [c_int]),
    "rvgp_symeig_f32": (c_int, [P, c_int, P, P, c_int, c_double, P, c_int, P, c_size_t, P]),
    "rvgp_fps_spatial_max_n": (c_int, [c_int]),
    "rvgp_fps_spatial_workspace": (c_size_t, [c_int, c_int]),
    "rvgp_fps_spatial": (c_int, [P, c_int, c_int, c_int, c_int, P, c_double, P, P, P, P, P, c_size_t, P]),
    "rvgp_spmm_plan_bytes": (ctypes.c_size_t, [c_int, c_int, ctypes.c_longlong]),
    "rvgp_spmm_plan_build": (c_int, [c_int, c_int, P, P, ctypes.c_longlong, P, ctypes.c_size_t, P]),
    "rvgp_bspmm_planned_f32": (c_int, [P, ctypes.c_size_t, c_int, c_int, ctypes.c_longlong, P, P, P, P, P, P, c_int,
                                       c_int, ctypes.c_float, ctypes.c_float, ctypes.c_float, P]),
    "rvgp_bspmm_planned_f64": (c_int, [P, ctypes.c_size_t, c_int, c_int, ctypes.c_longlong, P, P, P, P, P, P, c_int,
                                       c_int, c_double, c_double, c_double, P]),
    "rvgp_gp_fit_mixed_workspace": (c_size_t, [c_int]),
    "rvgp_gp_fit_adam_mixed": (c_int, [P, P, P, ctypes.c_longlong, c_int, P, c_double, c_int, P, P, P, c_int,
                                       c_double, c_double, c_double, c_double, P, P, P, P, P, P, c_size_t, P]),
    "rvgp_gp_fit_adam_mixed_launch": (c_int, [P, P, P, ctypes.c_longlong, c_int, P, c_double, c_int, P, P, P, c_int,
                                              c_double, c_double, c_double, c_double, P, P, P, c_size_t, P]),
    "rvgp_gp_fit_adam_mixed_finish": (c_int, [P, P, P, ctypes.c_longlong, c_int, P, c_double, c_int, P, P, P, P, P,
                                              c_size_t, P]),
    "rvgp_gp_predict_workspace": (c_size_t, [ctypes.c_longlong, c_int, c_int]),
    "rvgp_gp_predict": (c_int, [P, P, ctypes.c_longlong, c_int, c_int, P, P, P, P, c_size_t, P]),
    "rvgp_fps_persistent_workspace": (c_size_t, [c_int]),
    "rvgp_fps_persistent": (c_int, [P, c_int, c_int, c_int, c_int, P, c_double, P, P, P, P, P, c_size_t, P]),
    "rvgp_autotune_cache_path": (ctypes.c_char_p, []),
    "rvgp_autotune_lookup": (c_int, [ctypes.c_char_p]),
    "rvgp_gp_fit_restarts_workspace": (c_size_t, [c_int, c_int]),
    "rvgp_gp_fit_restarts": (c_int, [P, P, P, ctypes.c_longlong, c_int, P, c_double, c_int, P, P, P, c_int, c_int,
                                     c_double, c_double, c_double, c_double, P, P, P, P, P, P, P, P, c_size_t, P]),
    "rvgp_gp_prepare_local_workspace": (c_size_t, [c_int, c_int, c_int, c_int]),
    "rvgp_gp_prepare_local": (c_int, [P, c_int, c_int, c_int, c_int, P, c_int, P, c_int, P, c_int, P, P, P, P,
                                      c_size_t, P]),
    "rvgp_gp_predict_local_workspace": (c_size_t, [c_int, c_int, c_int, c_int]),
    "rvgp_gp_predict_local": (c_int, [P, c_int, c_int, c_int, c_int, P, c_int, P, c_int, c_int, P, P, P, P, c_size_t,
                                      P]),
    "rvgp_sgpr_workspace": (c_size_t, [c_int, c_int]),
    "rvgp_sgpr_state_size": (c_size_t, [c_int]),
    "rvgp_sgpr_elbo": (c_int, [P, P, P, ctypes.c_longlong, c_int, P, c_int, P, c_double, P, c_int, c_double, P, P, P,
                               P, P, c_size_t, P]),
    "rvgp_sgpr_predict_workspace": (c_size_t, [ctypes.c_longlong, c_int]),
    "rvgp_sgpr_predict": (c_int, [P, ctypes.c_longlong, c_int, P, P, P, P, c_size_t, P]),
    "rvgp_rbf_workspace": (c_size_t, [ctypes.c_longlong, c_int]),
    "rvgp_rbf_state_size": (c_size_t, [ctypes.c_longlong, c_int]),
    "rvgp_rbf_matrix": (c_int, [P, ctypes.c_longlong, P, ctypes.c_longlong, c_int, P, P, P]),
    "rvgp_rbf_lml": (c_int, [P, ctypes.c_longlong, c_int, P, c_int, P, P, P, P, P, c_size_t, P]),
    "rvgp_rbf_predict_workspace": (c_size_t, [ctypes.c_longlong, ctypes.c_longlong]),
    "rvgp_rbf_predict": (c_int, [P, ctypes.c_longlong, P, ctypes.c_longlong, c_int, c_int, P, P, P, P, P, c_size_t,
                                 P]),
    "rvgp_vectorfield_features_workspace": (c_size_t, [c_int, c_int, c_int]),
    "rvgp_vectorfield_features": (c_int, [P, c_int, P, c_int, P, c_int, c_int, P, P, P, c_size_t, P]),
    "rvgp_gp_posterior_batch_workspace": (c_size_t, [c_int, c_int]),
    "rvgp_gp_posterior_batch": (c_int, [P, ctypes.c_longlong, c_int, P, c_int, P, P, P, ctypes.c_longlong, P, P, P,
                                        c_size_t, P]),
    "rvgp_kernel_matrix": (c_int, [P, ctypes.c_longlong, P, ctypes.c_longlong, c_int, P, P, P]),
    "rvgp_kernel_diag": (c_int, [P, ctypes.c_longlong, c_int, P, P, P]),
    "rvgp_manifold_dimension": (c_int, [P, c_int, c_int, c_double, P, P, P]),
    "rvgp_frame_map": (c_int, [P, c_int, c_int, c_int, c_int, P, c_int, P, P]),
    "rvgp_normalise_rows": (c_int, [P, c_int, c_int, P]),
    "rvgp_expm_action_workspace": (c_size_t, [c_int, c_int, c_int]),
    "rvgp_expm_action": (c_int, [P, P, P, c_int, c_int, P, c_int, c_double, c_double, c_double, P, P, c_size_t, P]),
    "rvgp_vector_diffusion_workspace": (c_size_t, [c_int, c_int]),
    "rvgp_vector_diffusion": (c_int, [P, P, P, P, c_int, c_int, P, c_double, c_double, c_double, c_double, P, P,
                                      c_size_t, P]),
    "rvgp_spectral_diffusion_workspace": (c_size_t, [ctypes.c_longlong, c_int, c_int]),
    "rvgp_spectral_diffusion": (c_int, [P, ctypes.c_longlong, c_int, P, P, c_int, c_double, P, P, c_size_t, P]),
    "rvgp_fps_workspace": (c_size_t, [c_int]),
    "rvgp_fps": (c_int, [P, c_int, c_int, c_int, c_int, P, c_double, P, P, P, P, c_size_t, P]),
    "rvgp_diameter_workspace": (c_size_t, [c_int]),
    "rvgp_diameter": (c_int, [P, c_int, c_int, P, P, c_size_t, P]),
    "rvgp_eigsh": (c_int, [P, P, P, P, c_int, c_int, c_int, c_int, c_int, c_double, c_double, c_int, ctypes.c_ulonglong,
                           P, P, c_int, c_double, P, P, c_size_t, P]),
    "rvgp_eigsh_ordered": (c_int, [P, P, P, P, c_int, c_int, c_int, c_int, c_int, c_double, c_double, c_int,
                                   ctypes.c_ulonglong, P, P, P, c_int, c_double, P, P, c_size_t, P]),
    "rvgp_tc_gram_workspace": (c_size_t, [ctypes.c_longlong, c_int, c_int]),
    "rvgp_tc_gram_f32": (c_int, [P, c_int, P, c_int, ctypes.c_longlong, c_int, c_int, P, c_int, P, c_size_t, P]),
    "rvgp_tc_gemm_workspace": (c_size_t, [c_int, c_int]),
    "rvgp_tc_gemm_f32": (c_int, [P, c_int, ctypes.c_longlong, c_int, P, c_int, c_int, P, c_int, P, c_size_t, P]),
    "rvgp_locality_order_workspace": (c_size_t, [c_int, c_int]),
    "rvgp_locality_order": (c_int, [P, c_int, c_int, P, P, P, c_size_t, P]),
    "rvgp_permute_csr_workspace": (c_size_t, [c_int]),
    "rvgp_permute_csr": (c_int, [c_int, c_int, P, P, P, P, P, P, P, P, P, P, P, c_size_t, P]),
    "rvgp_unpermute_rows": (c_int, [P, c_int, P, c_int, c_int, c_int, P, c_int, P]),
}

_LIB = None


def lib():
    """Load the library (once) and declare every exported signature."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m rvgp_gb300.build`")
        handle = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(handle, name)
            f.restype = res
            f.argtypes = args
        _LIB = handle
    return _LIB


def launch_count():
    """Kernels launched by librvgp_gb300 in this process so far."""
    return int(lib().rvgp_launch_count())


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("rvgp_gb300 runs on a CUDA GPU only (no CPU fallback) and none is available")


def ptr(t):
    return None if t is None else c_void_p(t.data_ptr())


def stream():
    return c_void_p(torch.cuda.current_stream().cuda_stream)


def check(status, what):
    if status != 0:
        msg = lib().rvgp_last_error().decode()
        if status == -1 and ("must be" in msg or "Expected" in msg):
            raise ValueError(msg)
        raise RuntimeError(f"{what} failed ({status}): {msg}")


def workspace(nbytes, device):
    return torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)


def _dev(t, dtype, name):
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor")
    if t.dtype != dtype:
        raise ValueError(f"{name} must be {dtype}, got {t.dtype}")
    return t.contiguous()


# ---------------------------------------------------------------------------- graph
def knn(X, k):
    """(n, D) f64 CUDA tensor -> (n, k) int32 neighbour indices (exact, ties to lower index)."""
    X = _dev(X, torch.float64, "X")
    n, D = X.shape
    idx = torch.empty((n, k), dtype=torch.int32, device=X.device)
    L = lib()
    ws = workspace(L.rvgp_knn_workspace(n, D, k), X.device)
    check(L.rvgp_knn(ptr(X), n, D, k, ptr(idx), ptr(ws), ws.numel(), stream()), "rvgp_knn")
    knn.last_ws = ws
    return idx


def graph_build(knn_idx):
    """kNN (n, k) int32 -> (indptr (n+1,), indices (E,), maxdeg int) of the symmetrised graph + I."""
    knn_idx = _dev(knn_idx, torch.int32, "knn")
    n, k = knn_idx.shape
    dev = knn_idx.device
    indptr = torch.empty(n + 1, dtype=torch.int32, device=dev)
    indices = torch.empty(n * (2 * k + 1), dtype=torch.int32, device=dev)
    scal = torch.empty(2, dtype=torch.int32, device=dev)
    L = lib()
    ws = workspace(L.rvgp_graph_workspace(n, k), dev)
    check(L.rvgp_graph_build(ptr(knn_idx), n, k, ptr(indptr), ptr(indices), ptr(scal[0:1]), ptr(scal[1:2]),
                             ptr(ws), ws.numel(), stream()), "rvgp_graph_build")
    E, maxdeg = (int(v) for v in scal.cpu())
    return indptr, indices[:E].clone(), maxdeg


def laplacian_values(indptr, indices):
    n = indptr.numel() - 1
    vals = torch.empty(indices.numel(), dtype=torch.float64, device=indices.device)
    check(lib().rvgp_laplacian_values(ptr(indptr), ptr(indices), n, ptr(vals), stream()), "rvgp_laplacian_values")
    return vals


# ---------------------------------------------------------------------------- gauges
def gauges(X, indptr, indices, K, maxdeg, d_out, return_nbh=False):
    """Geodesic-neighbourhood PCA: (tangents (n, D, d_out), sigma (n, min(D, K+1)), nbh or None)."""
    X = _dev(X, torch.float64, "X")
    n, D = X.shape
    if K >= n:
        raise ValueError("Geodesic neighborhood size must be less than the total number of samples")
    dev = X.device
    c = min(D, K + 1)
    T = torch.empty((n, D, d_out), dtype=torch.float64, device=dev)
    S = torch.empty((n, c), dtype=torch.float64, device=dev)
    nbh = torch.empty((n, K + 1), dtype=torch.int32, device=dev) if return_nbh else None
    status = torch.empty(3, dtype=torch.int32, device=dev)
    L = lib()
    ws = workspace(L.rvgp_gauges_workspace(n, D, K, maxdeg), dev)
    check(L.rvgp_gauges(ptr(X), n, D, ptr(indptr), ptr(indices), K, maxdeg, d_out, ptr(T), ptr(S), ptr(nbh),
                        ptr(status), ptr(ws), ws.numel(), stream()), "rvgp_gauges")
    st = status.cpu().tolist()
    if st[0] < n:
        raise RuntimeError(f"the graph component of point {st[0]} holds fewer than K+1={K + 1} points")
    if st[2] < n:
        raise RuntimeError(f"geodesic neighbourhood search overflowed its node pool at point {st[2]}")
    return T, S, nbh


def connections(T, d, indptr, indices, want_R=True, want64=True, want32=True):
    """Per-edge transports (E, d, d) and block connection-Laplacian values (f64 / f32)."""
    T = _dev(T, torch.float64, "tangents")
    n, D, ld = T.shape
    E = indices.numel()
    dev = T.device
    R = torch.empty((E, d, d), dtype=torch.float64, device=dev) if want_R else None
    v64 = torch.empty((E, d, d), dtype=torch.float64, device=dev) if want64 else None
    v32 = torch.empty((E, d, d), dtype=torch.float32, device=dev) if want32 else None
    check(lib().rvgp_connections(ptr(T), n, D, ld, d, ptr(indptr), ptr(indices), ptr(R), ptr(v64), ptr(v32),
                                 stream()), "rvgp_connections")
    return R, v64, v32


# ---------------------------------------------------------------------------- products
def spmm_plan(indptr, indices, DB=1):
    """The planned product's plan of a block-CSR matrix (a byte tensor): per
    group of 4 block rows the merged list of their columns, per tile of 32
    block rows its halo of distinct columns and every entry's position in it.
    Build once per matrix, pass to ``bspmm(..., plan=)``."""
    n = indptr.numel() - 1
    nnz = indices.numel()
    L = lib()
    nbytes = L.rvgp_spmm_plan_bytes(n, DB, nnz)
    plan = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=indptr.device)
    check(L.rvgp_spmm_plan_build(n, DB, ptr(indptr), ptr(indices), nnz, ptr(plan), nbytes, stream()),
          "rvgp_spmm_plan_build")
    return plan


def bspmm(indptr, indices, vals, X, Y=None, Z=None, alpha=1.0, beta=0.0, gamma=0.0, plan=None):
    """Y = alpha*(A X) + beta*X + gamma*Z for block-CSR A with square blocks
    (through ``plan`` when given, grouped / tiled forms included: the same
    bits)."""
    n = indptr.numel() - 1
    DB = 1 if vals.dim() == 1 else vals.shape[-1]
    rows, b = X.shape
    if rows != n * DB:
        raise ValueError("X rows must equal n * block size")
    Y = torch.empty_like(X) if Y is None else Y
    L = lib()
    if plan is not None:
        f = L.rvgp_bspmm_planned_f32 if X.dtype == torch.float32 else L.rvgp_bspmm_planned_f64
        check(f(ptr(plan), plan.numel(), n, DB, indices.numel(), ptr(indptr), ptr(indices), ptr(vals), ptr(X),
                ptr(Y), ptr(Z), b, X.stride(0), alpha, beta, gamma, stream()), "rvgp_bspmm_planned")
        return Y
    f = L.rvgp_bspmm_f32 if X.dtype == torch.float32 else L.rvgp_bspmm_f64
    check(f(n, DB, ptr(indptr), ptr(indices), ptr(vals), ptr(X), ptr(Y), ptr(Z), b, X.stride(0), alpha, beta, gamma,
            stream()), "rvgp_bspmm")
    return Y


# ---------------------------------------------------------------------------- eigensolver
def block_size(m, N):
    """Subspace block: m plus a guard of max(16, m/8) vectors, a multiple of 4, at most N."""
    p = m + max(16, m // 8)
    p = (p + 3) // 4 * 4
    return min(p, N - N % 4)


def eigsh(indptr, indices, vals64, vals32=None, m=10, mode="mixed", tol=None, tol32=None, max_iter=60, seed=0,
          scale=None, p=None, perm=None):
    """m smallest eigenpairs of the block-CSR matrix: (evals (m,), evecs (N, m), stats dict).

    evecs are orthonormal times ``scale`` (default 1).  mode: "mixed" (FP32
    bulk + FP64 refinement) or "fp64" (plain FP64).  With ``perm`` the matrix
    is a renumbered one (``permute_csr``): block row r is the caller's block
    row perm[r], and evecs come back in the caller's row order.
    """
    n = indptr.numel() - 1
    DB = 1 if vals64.dim() == 1 else vals64.shape[-1]
    N = n * DB
    if m >= N - 1:
        raise ValueError(f"k must be less than ndim(A)-1, got k={m}")
    p = block_size(m, N) if p is None else p
    imode = 1 if mode == "mixed" else 0
    if imode == 1 and vals32 is None:
        vals32 = vals64.float()
    dev = vals64.device
    evals = torch.empty(m, dtype=torch.float64, device=dev)
    evecs = torch.empty((N, m), dtype=torch.float64, device=dev)
    stats = (ctypes.c_int * 16)()
    if tol32 is None:  # the FP32 stage's residual tolerance (relative to the Gershgorin bound)
        tol32 = float(os.environ.get("RVGP_EIG_TOL32", "4e-6"))
    if tol is None:  # mixed: stop at the FP32 stage's accuracy; fp64: ARPACK-level residuals
        tol = tol32 if imode == 1 else 1e-11
    L = lib()
    # + the tiled product's plan (built inside, once per solve)
    ws = workspace(L.rvgp_eigsh_workspace(n, DB, m, p, imode) + 256 +
                   L.rvgp_spmm_plan_bytes(n, DB, indices.numel()), dev)
    sc = 1.0 if scale is None else float(scale)
    if perm is None:
        st = L.rvgp_eigsh(ptr(indptr), ptr(indices), ptr(vals64), ptr(vals32), n, DB, m, p, imode, tol, tol32,
                          max_iter, seed, ptr(evals), ptr(evecs), m, sc, stats, ptr(ws), ws.numel(), stream())
    else:
        perm = _dev(perm, torch.int32, "perm")
        st = L.rvgp_eigsh_ordered(ptr(indptr), ptr(indices), ptr(vals64), ptr(vals32), n, DB, m, p, imode, tol,
                                  tol32, max_iter, seed, ptr(perm), ptr(evals), ptr(evecs), m, sc, stats, ptr(ws),
                                  ws.numel(), stream())
    info = dict(iters=stats[0], spmm=stats[1], sweeps=stats[2], converged=stats[3], refine_iters=stats[4],
                chol_rescues=stats[5], tensor_cores=bool(stats[6]), tiled_spmm=bool(stats[7]), locked=stats[12], p=p, filter_ms=stats[8] / 1e3, orth_ms=stats[9] / 1e3,
                rr_ms=stats[10] / 1e3, jacobi_ms=stats[11] / 1e3)
    if st < 0:
        check(st, "rvgp_eigsh")
    if st > 0:
        raise RuntimeError(f"ARPACK-equivalent no convergence: {lib().rvgp_last_error().decode()}")
    return evals, evecs, info


def symeig_f32(H, max_sweeps=60, tol=4e-6, method=0):
    """Eigendecomposition of a symmetric FP32 matrix on the device by Jacobi
    (the eigensolver's Rayleigh-Ritz step): (w ascending, V by column, sweeps).
    method 0: block Jacobi for p >= 64, 1: scalar, 2: block."""
    H = _dev(H, torch.float32, "H")
    p = H.shape[0]
    w = torch.empty(p, dtype=torch.float32, device=H.device)
    V = torch.empty((p, p), dtype=torch.float32, device=H.device)
    used = ctypes.c_int(0)
    L = lib()
    ws = workspace(L.rvgp_symeig_f32_workspace(p), H.device)
    check(L.rvgp_symeig_f32(ptr(H), p, ptr(w), ptr(V), int(max_sweeps), float(tol), ctypes.byref(used), int(method),
                            ptr(ws), ws.numel(), stream()), "rvgp_symeig_f32")
    return w, V, used.value


def tc_gram(A, B=None):
    """Aᵀ B (FP64 out) on the tensor cores, split-TF32: A (N, p), B (N, q) FP32, p, q <= 2048."""
    A = _dev(A, torch.float32, "A")
    B = A if B is None else _dev(B, torch.float32, "B")
    N, p = A.shape
    q = B.shape[1]
    C = torch.empty((p, q), dtype=torch.float64, device=A.device)
    ws = workspace(lib().rvgp_tc_gram_workspace(N, p, q), A.device)
    check(lib().rvgp_tc_gram_f32(ptr(A), p, ptr(B), q, N, p, q, ptr(C), q, ptr(ws), ws.numel(), stream()),
          "rvgp_tc_gram_f32")
    return C


def tc_gemm(A, Bm):
    """A (N, K) @ Bm (K, q) in FP32 on the tensor cores, split-TF32; K, q <= 2048."""
    A = _dev(A, torch.float32, "A")
    Bm = _dev(Bm, torch.float32, "Bm")
    N, K = A.shape
    q = Bm.shape[1]
    C = torch.empty((N, q), dtype=torch.float32, device=A.device)
    ws = workspace(lib().rvgp_tc_gemm_workspace(K, q), A.device)
    check(lib().rvgp_tc_gemm_f32(ptr(A), K, N, K, ptr(Bm), q, q, ptr(C), q, ptr(ws), ws.numel(), stream()),
          "rvgp_tc_gemm_f32")
    return C


def locality_order(X):
    """Morton-curve renumbering of the points X (n, D) float64: (perm, rank),
    perm[r] = point at new position r, rank its inverse (int32, device)."""
    X = _dev(X, torch.float64, "X")
    n, D = X.shape
    perm = torch.empty(n, dtype=torch.int32, device=X.device)
    rank = torch.empty(n, dtype=torch.int32, device=X.device)
    ws = workspace(lib().rvgp_locality_order_workspace(n, D), X.device)
    check(lib().rvgp_locality_order(ptr(X), n, D, ptr(perm), ptr(rank), ptr(ws), ws.numel(), stream()),
          "rvgp_locality_order")
    return perm, rank


def permute_csr(indptr, indices, vals64, vals32, perm, rank):
    """The block-CSR matrix renumbered by perm: (indptr, indices, vals64, vals32)."""
    n = indptr.numel() - 1
    DB = 1 if vals64.dim() == 1 else vals64.shape[-1]
    dev = vals64.device
    out_ptr = torch.empty(n + 1, dtype=torch.int32, device=dev)
    out_idx = torch.empty_like(indices)
    out64 = torch.empty_like(vals64)
    out32 = None if vals32 is None else torch.empty_like(vals32)
    ws = workspace(lib().rvgp_permute_csr_workspace(n), dev)
    check(lib().rvgp_permute_csr(n, DB, ptr(indptr), ptr(indices), ptr(vals64.contiguous()),
                                 ptr(None if vals32 is None else vals32.contiguous()), ptr(perm), ptr(rank),
                                 ptr(out_ptr), ptr(out_idx), ptr(out64), ptr(out32), ptr(ws), ws.numel(), stream()),
          "rvgp_permute_csr")
    return out_ptr, out_idx, out64, out32


def unpermute_rows(src, rank, DB=1):
    """Rows of src (n*DB, m) float64 in the renumbered order -> caller's order."""
    src = _dev(src, torch.float64, "src")
    N, m = src.shape
    n = N // DB
    out = torch.empty_like(src)
    check(lib().rvgp_unpermute_rows(ptr(src), m, ptr(rank), n, DB, m, ptr(out), m, stream()), "rvgp_unpermute_rows")
    return out


# ---------------------------------------------------------------------------- GP
KERNEL_TYPES = {"matern": 0, "se": 1}


def spectral_S(evals, theta, n_rows, typ="matern", want_grad=True):
    """S (m,) and dS (3, m) for theta = [nu, kappa, sigma_f, noise] (CUDA f64)."""
    m = evals.numel()
    S = torch.empty(m, dtype=torch.float64, device=evals.device)
    dS = torch.empty((3, m), dtype=torch.float64, device=evals.device) if want_grad else None
    tmp = torch.empty(3 * m, dtype=torch.float64, device=evals.device)
    check(lib().rvgp_spectral_S(ptr(evals), m, ptr(theta), float(n_rows), KERNEL_TYPES[typ], ptr(S), ptr(dS),
                                ptr(tmp), stream()), "rvgp_spectral_S")
    return S, dS


def lift(T, d, U):
    """evecs_Lc[(i*D + a), j] = Σ_q T[i, a, q] U[(i*d + q), j]  -> (n*D, m)."""
    n, D, ld = T.shape
    m = U.shape[1]
    out = torch.empty((n * D, m), dtype=torch.float64, device=T.device)
    check(lib().rvgp_lift(ptr(T), n, D, ld, d, ptr(U.contiguous()), m, ptr(out), stream()), "rvgp_lift")
    return out


def gather_rows(src, D, idx, vec=None, want64=True, want32=False):
    """Rows (point, coordinate) of src for the points in idx: (Phi (nt*D, m), Phi32, y)."""
    m = src.shape[1]
    nt = idx.numel()
    dev = src.device
    Phi = torch.empty((nt * D, m), dtype=torch.float64, device=dev) if want64 else None
    Phi32 = torch.empty((nt * D, m), dtype=torch.float32, device=dev) if want32 else None
    y = torch.empty(nt * D, dtype=torch.float64, device=dev) if vec is not None else None
    check(lib().rvgp_gather_rows(ptr(src), m, D, ptr(idx.to(torch.int32).contiguous()), nt,
                                 ptr(None if vec is None else vec.contiguous()), ptr(Phi), ptr(Phi32), ptr(y),
                                 stream()), "rvgp_gather_rows")
    return Phi, Phi32, y


def gp_prepare(Phi, y, Phi32=None, mode="fp64"):
    N, m = Phi.shape
    dev = Phi.device
    C = torch.empty((m, m), dtype=torch.float64, device=dev)
    b = torch.empty(m, dtype=torch.float64, device=dev)
    yy = torch.empty(1, dtype=torch.float64, device=dev)
    L = lib()
    ws = workspace(L.rvgp_gp_prepare_workspace(N, m), dev)
    check(L.rvgp_gp_prepare(ptr(Phi), ptr(Phi32), ptr(y), N, m, 1 if mode == "mixed" else 0, ptr(C), ptr(b), ptr(yy),
                            ptr(ws), ws.numel(), stream()), "rvgp_gp_prepare")
    return C, b, yy


def gp_prepare_local(T, d, U, idx, vec, mode="fp64"):
    """C = ΦᵀΦ, b = Φᵀy, yy = yᵀy of the lifted rows Φ_i = T_i U_i (and y_i the
    D-vectors) of the points idx, from d rows per point (rvgp_gp_prepare_local)."""
    T = _dev(T, torch.float64, "tangents")
    U = _dev(U, torch.float64, "U")
    vec = _dev(vec, torch.float64, "vectors")
    n, D, ld = T.shape
    m = U.shape[1]
    idx = idx.to(torch.int32).contiguous()
    nt = idx.numel()
    dev = U.device
    C = torch.empty((m, m), dtype=torch.float64, device=dev)
    b = torch.empty(m, dtype=torch.float64, device=dev)
    yy = torch.empty(1, dtype=torch.float64, device=dev)
    imode = 1 if mode == "mixed" else 0
    L = lib()
    ws = workspace(L.rvgp_gp_prepare_local_workspace(nt, d, m, imode), dev)
    check(L.rvgp_gp_prepare_local(ptr(T), n, D, ld, d, ptr(U), m, ptr(idx), nt, ptr(vec), imode, ptr(C), ptr(b),
                                  ptr(yy), ptr(ws), ws.numel(), stream()), "rvgp_gp_prepare_local")
    return C, b, yy


def gp_predict_local(T, d, U, idx, state, mode="fp64"):
    """Posterior mean and variance (len(idx), D) at the points idx from the
    GP state, through the local factors of the lifted rows (rvgp_gp_predict_local)."""
    T = _dev(T, torch.float64, "tangents")
    U = _dev(U, torch.float64, "U")
    n, D, ld = T.shape
    m = U.shape[1]
    idx = idx.to(torch.int32).contiguous()
    nt = idx.numel()
    dev = U.device
    mean = torch.empty((nt, D), dtype=torch.float64, device=dev)
    var = torch.empty((nt, D), dtype=torch.float64, device=dev)
    imode = 1 if mode == "mixed" else 0
    L = lib()
    ws = workspace(L.rvgp_gp_predict_local_workspace(nt, d, m, imode), dev)
    check(L.rvgp_gp_predict_local(ptr(T), n, D, ld, d, ptr(U), m, ptr(idx), nt, imode, ptr(state), ptr(mean),
                                  ptr(var), ptr(ws), ws.numel(), stream()), "rvgp_gp_predict_local")
    return mean, var


class LMLWorkspace:
    """Device buffers reused across likelihood evaluations of one problem."""

    def __init__(self, m, device):
        L = lib()
        self.m = m
        self.ws = workspace(L.rvgp_gp_lml_workspace(m), device)
        self.state = torch.empty(int(L.rvgp_gp_state_size(m)), dtype=torch.float64, device=device)
        self.out = torch.empty(5, dtype=torch.float64, device=device)


def gp_lml(C, b, yy, N, evals, n_rows, theta, typ="matern", work=None):
    """[LML, d/dnu, d/dkappa, d/dsigma_f, d/dnoise] on the device (no host sync)."""
    m = evals.numel()
    work = work or LMLWorkspace(m, evals.device)
    check(lib().rvgp_gp_lml(ptr(C), ptr(b), ptr(yy), int(N), m, ptr(evals), float(n_rows), KERNEL_TYPES[typ],
                            ptr(theta), ptr(work.out), ptr(work.state), ptr(work.ws), work.ws.numel(), stream()),
          "rvgp_gp_lml")
    return work.out, work


def gp_fit_adam(C, b, yy, N, evals, n_rows, theta0, lower, mask, steps, lr=0.05, betas=(0.9, 0.999), eps=1e-8,
                typ="matern", work=None, history=False):
    """Device-resident Adam on the LML: returns (theta (4,), out (5,), history or None, work)."""
    m = evals.numel()
    dev = evals.device
    work = work or LMLWorkspace(m, dev)
    theta = torch.empty(4, dtype=torch.float64, device=dev)
    hist = torch.empty(max(steps, 1), dtype=torch.float64, device=dev) if history else None
    lo = (ctypes.c_double * 4)(*[float(v) for v in lower])
    mk = (ctypes.c_int * 4)(*[int(bool(v)) for v in mask])
    check(lib().rvgp_gp_fit_adam(ptr(C), ptr(b), ptr(yy), int(N), m, ptr(evals), float(n_rows), KERNEL_TYPES[typ],
                                 ptr(theta0.contiguous()), lo, mk, int(steps), float(lr), float(betas[0]),
                                 float(betas[1]), float(eps), ptr(theta), ptr(hist), ptr(work.out), ptr(work.state),
                                 ptr(work.ws), work.ws.numel(), stream()), "rvgp_gp_fit_adam")
    return theta, work.out, hist, work


class SGPRWorkspace:
    """Device buffers reused across bound evaluations of one sparse-GP problem."""

    def __init__(self, M, m, device):
        L = lib()
        self.M, self.m = M, m
        self.ws = workspace(L.rvgp_sgpr_workspace(M, m), device)
        self.state = torch.empty(int(L.rvgp_sgpr_state_size(m)), dtype=torch.float64, device=device)
        self.out = torch.empty(5, dtype=torch.float64, device=device)
        self.dZ = torch.empty((M, m), dtype=torch.float64, device=device)
        self.info = torch.zeros(2, dtype=torch.int32, device=device)


def sgpr_elbo(C, b, yy, N, Z, evals, n_rows, theta, typ="matern", jitter=1e-6, work=None, grad_Z=True, state=True):
    """[F, dF/dnu, dF/dkappa, dF/dsigma_f, dF/dnoise] of the sparse GP bound (rvgp_sgpr_elbo),
    with dF/dZ in work.dZ and the posterior in work.state; no host sync."""
    M, m = Z.shape
    work = work or SGPRWorkspace(M, m, Z.device)
    check(lib().rvgp_sgpr_elbo(ptr(C), ptr(b), ptr(yy), int(N), m, ptr(Z.contiguous()), M, ptr(evals),
                               float(n_rows), ptr(theta), KERNEL_TYPES[typ], float(jitter), ptr(work.out),
                               ptr(work.dZ if grad_Z else None), ptr(work.state if state else None), ptr(work.info),
                               ptr(work.ws), work.ws.numel(), stream()), "rvgp_sgpr_elbo")
    return work.out, work


def sgpr_predict(Phi_star, state, m):
    """Posterior mean and marginal variance at the spectral rows Phi_star (rvgp_sgpr_predict)."""
    Phi_star = _dev(Phi_star, torch.float64, "Phi_star")
    Nte = Phi_star.shape[0]
    dev = Phi_star.device
    mean = torch.empty(Nte, dtype=torch.float64, device=dev)
    var = torch.empty(Nte, dtype=torch.float64, device=dev)
    if Nte == 0:
        return mean, var
    L = lib()
    ws = workspace(L.rvgp_sgpr_predict_workspace(Nte, m), dev)
    check(L.rvgp_sgpr_predict(ptr(Phi_star), int(Nte), int(m), ptr(state), ptr(mean), ptr(var), ptr(ws), ws.numel(),
                              stream()), "rvgp_sgpr_predict")
    return mean, var


class RBFWorkspace:
    """Device buffers reused across likelihood evaluations of one RBF-GP problem."""

    def __init__(self, N, D, device):
        L = lib()
        self.N, self.D = N, D
        self.ws = workspace(L.rvgp_rbf_workspace(N, D), device)
        self.state = torch.empty(int(L.rvgp_rbf_state_size(N, D)), dtype=torch.float64, device=device)
        self.out = torch.empty(4, dtype=torch.float64, device=device)
        self.info = torch.zeros(1, dtype=torch.int32, device=device)


def rbf_matrix(X1, theta, X2=None):
    """K(X1, X2) of the RBF kernel, theta = [variance, lengthscale, noise] (CUDA f64)."""
    X1 = _dev(X1, torch.float64, "X1")
    X2 = X1 if X2 is None else _dev(X2, torch.float64, "X2")
    K = torch.empty((X1.shape[0], X2.shape[0]), dtype=torch.float64, device=X1.device)
    check(lib().rvgp_rbf_matrix(ptr(X1), X1.shape[0], ptr(X2), X2.shape[0], X1.shape[1], ptr(theta), ptr(K),
                                stream()), "rvgp_rbf_matrix")
    return K


def rbf_lml(X, Y, theta, work=None):
    """[LML, d/dvariance, d/dlengthscale, d/dnoise] of the D-output RBF GP (rvgp_rbf_lml); no host sync."""
    X = _dev(X, torch.float64, "X")
    Y = _dev(Y, torch.float64, "Y")
    N, m = X.shape
    D = Y.shape[1]
    work = work or RBFWorkspace(N, D, X.device)
    check(lib().rvgp_rbf_lml(ptr(X), N, m, ptr(Y), D, ptr(theta), ptr(work.out), ptr(work.state), ptr(work.info),
                             ptr(work.ws), work.ws.numel(), stream()), "rvgp_rbf_lml")
    return work.out, work


def rbf_predict(Xs, X, D, theta, state):
    """Posterior mean (Nte, D) and marginal variance (Nte,) of the RBF GP (rvgp_rbf_predict)."""
    Xs = _dev(Xs, torch.float64, "Xs")
    X = _dev(X, torch.float64, "X")
    Nte, m = Xs.shape
    dev = Xs.device
    mean = torch.empty((Nte, D), dtype=torch.float64, device=dev)
    var = torch.empty(Nte, dtype=torch.float64, device=dev)
    if Nte == 0:
        return mean, var
    L = lib()
    ws = workspace(L.rvgp_rbf_predict_workspace(Nte, X.shape[0]), dev)
    check(L.rvgp_rbf_predict(ptr(Xs), Nte, ptr(X), X.shape[0], m, D, ptr(theta), ptr(state), ptr(mean), ptr(var),
                             ptr(ws), ws.numel(), stream()), "rvgp_rbf_predict")
    return mean, var


def vectorfield_features(P, V, nbr, ref_first=True):
    """div (B, n) and curl (B, n, 3) of the fields V (B, n, 3) at the points P (n, 3)
    from their neighbour lists nbr (n, k) (rvgp_vectorfield_features)."""
    P = _dev(P, torch.float64, "P")
    V = _dev(V, torch.float64, "V")
    nbr = nbr.to(torch.int32).contiguous()
    B, n = V.shape[0], P.shape[0]
    div = torch.empty((B, n), dtype=torch.float64, device=P.device)
    curl = torch.empty((B, n, 3), dtype=torch.float64, device=P.device)
    L = lib()
    ws = workspace(L.rvgp_vectorfield_features_workspace(n, B, nbr.shape[1]), P.device)
    check(L.rvgp_vectorfield_features(ptr(P), n, ptr(V), B, ptr(nbr), nbr.shape[1], int(bool(ref_first)), ptr(div),
                                      ptr(curl), ptr(ws), ws.numel(), stream()), "rvgp_vectorfield_features")
    return div, curl


def gp_posterior_batch(Phi, Y, theta, state, Phi_star, want_lml=True):
    """Posterior means (Nte, B) and log marginal likelihoods (B,) of the B fields
    Y (N, B) observed at the rows Phi (rvgp_gp_posterior_batch)."""
    Phi = _dev(Phi, torch.float64, "Phi")
    Y = _dev(Y, torch.float64, "Y")
    Phi_star = _dev(Phi_star, torch.float64, "Phi_star")
    N, m = Phi.shape
    B = Y.shape[1]
    dev = Phi.device
    mean = torch.empty((Phi_star.shape[0], B), dtype=torch.float64, device=dev)
    lml = torch.empty(B, dtype=torch.float64, device=dev) if want_lml else None
    L = lib()
    ws = workspace(L.rvgp_gp_posterior_batch_workspace(m, B), dev)
    check(L.rvgp_gp_posterior_batch(ptr(Phi), N, m, ptr(Y), B, ptr(theta), ptr(state), ptr(Phi_star),
                                    Phi_star.shape[0], ptr(mean), ptr(lml), ptr(ws), ws.numel(), stream()),
          "rvgp_gp_posterior_batch")
    return mean, lml


def gp_fit_mixed_max_m():
    """Largest number of eigenpairs the one-CTA mixed-precision fit handles."""
    return int(lib().rvgp_gp_fit_mixed_max_m())


def gp_fit_adam_mixed(C, b, yy, N, evals, n_rows, theta0, lower, mask, steps, lr=0.05, betas=(0.9, 0.999),
                      eps=1e-8, typ="matern", work=None, history=False, on_launch=None):
    """Adam with the m x m algebra of every step in FP32 inside one launch
    (rvgp_gp_fit_adam_mixed).  Returns (theta, out, history, work, ok); ok is
    False when an FP32 pivot failed, and nothing was fitted.  ``on_launch``
    (optional) is called once the one-CTA fit kernel is queued on an idle
    device, before waiting for it."""
    m = evals.numel()
    dev = evals.device
    work = work or LMLWorkspace(m, dev)
    L = lib()
    ws = workspace(L.rvgp_gp_fit_mixed_workspace(m), dev)
    theta = torch.empty(4, dtype=torch.float64, device=dev)
    hist = torch.empty(max(steps, 1), dtype=torch.float64, device=dev) if history else None
    lo = (ctypes.c_double * 4)(*[float(v) for v in lower])
    mk = (ctypes.c_int * 4)(*[int(bool(v)) for v in mask])
    status = ctypes.c_int(0)
    theta0 = theta0.contiguous()
    if on_launch is not None:
        # the fit's single CTA needs most of an SM: queue it on an idle
        # device, so it is resident before the caller's other work spreads
        torch.cuda.current_stream().synchronize()
    check(L.rvgp_gp_fit_adam_mixed_launch(ptr(C), ptr(b), ptr(yy), int(N), m, ptr(evals), float(n_rows),
                                          KERNEL_TYPES[typ], ptr(theta0), lo, mk, int(steps), float(lr),
                                          float(betas[0]), float(betas[1]), float(eps), ptr(theta), ptr(hist),
                                          ptr(ws), ws.numel(), stream()), "rvgp_gp_fit_adam_mixed")
    if on_launch is not None:
        on_launch()
    check(L.rvgp_gp_fit_adam_mixed_finish(ptr(C), ptr(b), ptr(yy), int(N), m, ptr(evals), float(n_rows),
                                          KERNEL_TYPES[typ], ptr(theta), ptr(work.out), ptr(work.state),
                                          ctypes.byref(status), ptr(ws), ws.numel(), stream()),
          "rvgp_gp_fit_adam_mixed")
    return theta, work.out, hist, work, status.value == 0


def gp_fit_restarts(C, b, yy, N, evals, n_rows, theta0s, lower, mask, steps, lr=0.05, betas=(0.9, 0.999), eps=1e-8,
                    typ="matern", history=False, out=None):
    """R mixed-form Adam fits from the starts theta0s (R, 4), their FP64 LMLs
    and the best (rvgp_gp_fit_restarts); lower (4,) float64 and mask (4,)
    int32 are device tensors.  Only enqueues (capturable in a CUDA graph):
    returns a dict of device tensors theta (R, 4), lml (R,), status (R,),
    best (1,), theta_best (4,), hist (R, steps) or None.  ``out``: a dict from
    an earlier call with the same shapes, reused in place."""
    theta0s = _dev(theta0s, torch.float64, "theta0s")
    R = theta0s.shape[0]
    m = evals.numel()
    dev = evals.device
    if out is None:
        L = lib()
        out = dict(theta=torch.empty((R, 4), dtype=torch.float64, device=dev),
                   lml=torch.empty(R, dtype=torch.float64, device=dev),
                   status=torch.empty(R, dtype=torch.int32, device=dev),
                   outs=torch.empty((R, 5), dtype=torch.float64, device=dev),
                   best=torch.empty(1, dtype=torch.int32, device=dev),
                   theta_best=torch.empty(4, dtype=torch.float64, device=dev),
                   hist=torch.empty((R, max(steps, 1)), dtype=torch.float64, device=dev) if history else None,
                   ws=workspace(L.rvgp_gp_fit_restarts_workspace(m, R), dev))
    check(lib().rvgp_gp_fit_restarts(ptr(C), ptr(b), ptr(yy), int(N), m, ptr(evals), float(n_rows), KERNEL_TYPES[typ],
                                     ptr(theta0s), ptr(lower), ptr(mask), R, int(steps), float(lr), float(betas[0]),
                                     float(betas[1]), float(eps), ptr(out["theta"]), ptr(out["hist"]), ptr(out["lml"]),
                                     ptr(out["status"]), ptr(out["outs"]), ptr(out["best"]), ptr(out["theta_best"]),
                                     ptr(out["ws"]), out["ws"].numel(), stream()), "rvgp_gp_fit_restarts")
    return out


def gp_predict(Phi_star, state, m, Phi_star32=None, mode="fp64"):
    Nte = Phi_star.shape[0]
    dev = Phi_star.device
    mean = torch.empty(Nte, dtype=torch.float64, device=dev)
    var = torch.empty(Nte, dtype=torch.float64, device=dev)
    imode = 1 if mode == "mixed" else 0
    if imode == 1 and Phi_star32 is None:
        Phi_star32 = Phi_star.float()
    L = lib()
    ws = workspace(L.rvgp_gp_predict_workspace(Nte, m, imode), dev)
    check(L.rvgp_gp_predict(ptr(Phi_star), ptr(Phi_star32), Nte, m, imode, ptr(state), ptr(mean), ptr(var), ptr(ws),
                            ws.numel(), stream()), "rvgp_gp_predict")
    return mean, var


def kernel_matrix(X, S, X2=None):
    X = X.contiguous()
    X2 = X if X2 is None else X2.contiguous()
    K = torch.empty((X.shape[0], X2.shape[0]), dtype=torch.float64, device=X.device)
    check(lib().rvgp_kernel_matrix(ptr(X), X.shape[0], ptr(X2), X2.shape[0], X.shape[1], ptr(S), ptr(K), stream()),
          "rvgp_kernel_matrix")
    return K


def kernel_diag(X, S):
    X = X.contiguous()
    out = torch.empty(X.shape[0], dtype=torch.float64, device=X.device)
    check(lib().rvgp_kernel_diag(ptr(X), X.shape[0], X.shape[1], ptr(S), ptr(out), stream()), "rvgp_kernel_diag")
    return out


# ---------------------------------------------------------------------------- fields / diffusion
def manifold_dimension(sigma, frac):
    """(dim, var_exp) of RVGP/geometry.py:83-97 computed on the device."""
    n, c = sigma.shape
    var = torch.empty(c, dtype=torch.float64, device=sigma.device)
    dim = torch.empty(1, dtype=torch.int32, device=sigma.device)
    check(lib().rvgp_manifold_dimension(ptr(sigma.contiguous()), n, c, float(frac), ptr(var), ptr(dim), stream()),
          "rvgp_manifold_dimension")
    return int(dim.item()), var


FRAME_MODES = {"project": 0, "to_local": 1, "from_local": 2}


def frame_map(T, d, v, mode):
    n, D, ld = T.shape
    out_cols = d if mode == "to_local" else D
    out = torch.empty((n, out_cols), dtype=torch.float64, device=T.device)
    check(lib().rvgp_frame_map(ptr(T), n, D, ld, d, ptr(v.contiguous()), FRAME_MODES[mode], ptr(out), stream()),
          "rvgp_frame_map")
    return out


def normalise_rows(v):
    v = v.contiguous()
    check(lib().rvgp_normalise_rows(ptr(v), v.shape[0], v.shape[1], stream()), "rvgp_normalise_rows")
    return v


def expm_action(indptr, indices, vals, X, t, bound, shift=0.0):
    """exp(-t A) X for block-CSR A (spectrum in [shift, bound]); X: (N, b <= 4)."""
    n = indptr.numel() - 1
    DB = 1 if vals.dim() == 1 else vals.shape[-1]
    X = X.contiguous()
    b = X.shape[1]
    Y = torch.empty_like(X)
    L = lib()
    ws = workspace(L.rvgp_expm_action_workspace(n, DB, b), X.device)
    check(L.rvgp_expm_action(ptr(indptr), ptr(indices), ptr(vals), n, DB, ptr(X), b, float(t), float(bound),
                             float(shift), ptr(Y), ptr(ws), ws.numel(), stream()), "rvgp_expm_action")
    return Y


def vector_diffusion(indptr, indices, L_vals, Lc_vals, x_loc, t, bound_L, bound_Lc, shift_Lc=0.0):
    n, d = x_loc.shape
    out = torch.empty_like(x_loc)
    L = lib()
    ws = workspace(L.rvgp_vector_diffusion_workspace(n, d), x_loc.device)
    check(L.rvgp_vector_diffusion(ptr(indptr), ptr(indices), ptr(L_vals), ptr(Lc_vals), n, d, ptr(x_loc.contiguous()),
                                  float(t), float(bound_L), float(bound_Lc), float(shift_Lc), ptr(out), ptr(ws),
                                  ws.numel(), stream()), "rvgp_vector_diffusion")
    return out


def spectral_diffusion(Phi, lam, X, t):
    N, m = Phi.shape
    X = X.contiguous()
    b = X.shape[1]
    Y = torch.empty_like(X)
    L = lib()
    ws = workspace(L.rvgp_spectral_diffusion_workspace(N, m, b), X.device)
    check(L.rvgp_spectral_diffusion(ptr(Phi.contiguous()), N, m, ptr(lam), ptr(X), b, float(t), ptr(Y), ptr(ws),
                                    ws.numel(), stream()), "rvgp_spectral_diffusion")
    return Y


# ---------------------------------------------------------------------------- sampling
def diameter(X):
    X = _dev(X, torch.float64, "X")
    n, D = X.shape
    out = torch.empty(1, dtype=torch.float64, device=X.device)
    L = lib()
    ws = workspace(L.rvgp_diameter_workspace(n), X.device)
    check(L.rvgp_diameter(ptr(X), n, D, ptr(out), ptr(ws), ws.numel(), stream()), "rvgp_diameter")
    return out


def fps(X, N=None, spacing=0.1, start_idx=0, persistent=None, stats=None, method=None):
    """(perm int32, lambdas f64) on the device: RVGP/geometry.py:126-162.
    method: "spatial" (default for D <= 8 up to rvgp_fps_spatial_max_n: one
    CTA visits only the blocks of points the new selection can change),
    "persistent" (one cooperative launch over all points per selection) or
    "steps" (one launch per selection); the same result.  persistent=True /
    False are the older names of "persistent" / "steps".  ``stats`` (dict,
    optional) receives the number of exact FP64 distances evaluated."""
    X = _dev(X, torch.float64, "X")
    n, D = X.shape
    N_max = n if N is None else int(N)
    dev = X.device
    perm = torch.empty(N_max, dtype=torch.int32, device=dev)
    lam = torch.empty(N_max, dtype=torch.float64, device=dev)
    count = torch.empty(1, dtype=torch.int32, device=dev)
    diam = diameter(X) if N is None else None
    L = lib()
    if method is None:
        if persistent is not None:
            method = "persistent" if persistent else "steps"
        elif D <= 8 and n <= L.rvgp_fps_spatial_max_n(D):
            method = "spatial"
        else:
            method = "persistent" if D <= 8 else "steps"
    if method not in ("spatial", "persistent", "steps"):
        raise ValueError(f"fps: unknown method {method!r}")
    if method == "spatial":
        ev = torch.zeros(1, dtype=torch.int64, device=dev)
        ws = workspace(L.rvgp_fps_spatial_workspace(n, D), dev)
        check(L.rvgp_fps_spatial(ptr(X), n, D, N_max, int(start_idx), ptr(diam), float(spacing), ptr(perm),
                                 ptr(lam), ptr(count), ptr(ev), ptr(ws), ws.numel(), stream()), "rvgp_fps_spatial")
        if stats is not None:
            stats["exact_evals"] = int(ev.item())
    elif method == "persistent":
        ev = torch.zeros(1, dtype=torch.int64, device=dev)
        ws = workspace(L.rvgp_fps_persistent_workspace(n), dev)
        check(L.rvgp_fps_persistent(ptr(X), n, D, N_max, int(start_idx), ptr(diam), float(spacing), ptr(perm),
                                    ptr(lam), ptr(count), ptr(ev), ptr(ws), ws.numel(), stream()),
              "rvgp_fps_persistent")
        if stats is not None:
            stats["exact_evals"] = int(ev.item())
    else:
        ws = workspace(L.rvgp_fps_workspace(n), dev)
        check(L.rvgp_fps(ptr(X), n, D, N_max, int(start_idx), ptr(diam), float(spacing), ptr(perm), ptr(lam),
                         ptr(count), ptr(ws), ws.numel(), stream()), "rvgp_fps")
    c = int(count.item())
    if c >= 0:
        perm, lam = perm[:c], lam[:c]
    return perm, lam
