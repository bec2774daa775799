import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
CASES = ["sphere", "torus", "ellipsoid", "swissroll64"]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, f"{name}.npz")))


@pytest.fixture(params=CASES)
def golden(request):
    g = load_golden(request.param)
    g["name"] = request.param
    return g


def projector_distance(A, B):
    """max_i ||A_i A_iᵀ - B_i B_iᵀ|| for stacks of orthonormal frames (n, D, d)."""
    P = np.einsum("nij,nkj->nik", A, A) - np.einsum("nij,nkj->nik", B, B)
    return float(np.abs(P).max())


def subspace_sin(A, B):
    """Largest sine of the principal angles between column spaces of A and B."""
    qa, _ = np.linalg.qr(A)
    qb, _ = np.linalg.qr(B)
    s = np.linalg.svd(qa.T @ qb, compute_uv=False)
    return float(np.sqrt(max(0.0, 1.0 - s.min() ** 2)))


def cluster_slices(evals, rtol=1e-6):
    """Split ascending eigenvalues into clusters of (numerically) equal values."""
    out, start = [], 0
    for i in range(1, len(evals) + 1):
        if i == len(evals) or abs(evals[i] - evals[i - 1]) > rtol * max(1.0, abs(evals[i])):
            out.append(slice(start, i))
            start = i
    return out
