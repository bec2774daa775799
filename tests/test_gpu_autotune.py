"""GPU: the launch-variant autotuner (autotune.cu) on the block SpMM.

Each case runs in a fresh process (the cache file is chosen at a process's
first tuning): the first process times the variants and writes its choice to
the cache file; a second process finds the choice there before any product
runs; and the product's result is the same bits whichever variant runs (row
per warp, or column-chunked with 2 or 4 neighbours per iteration)."""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

SCRIPT = r"""
import sys, numpy as np, torch, scipy.sparse as sp
sys.path.insert(0, {root!r})
from rvgp_gb300 import _core
rng = np.random.default_rng(0)
n, d, b = 3000, 2, {b}
A = sp.random(n, n, density=0.006, random_state=1, format="csr") + sp.eye(n)
A.sort_indices()
blocks = rng.standard_normal((A.nnz, d, d)).astype(np.float32)
cu = lambda a, t=torch.float32: torch.as_tensor(a, dtype=t, device="cuda")
X = cu(rng.standard_normal((n * d, b)))
Z = cu(rng.standard_normal((n * d, b)))
key = "bspmm f32 DB2 b{b} n2^11".encode()
before = _core.lib().rvgp_autotune_lookup(key)
Y = _core.bspmm(cu(A.indptr, torch.int32), cu(A.indices, torch.int32), cu(blocks), X, Z=Z, alpha=0.7, beta=-0.3,
                gamma=1.9)
torch.cuda.synchronize()
np.save({out!r}, Y.cpu().numpy())
print(before, _core.lib().rvgp_autotune_lookup(key), _core.lib().rvgp_autotune_cache_path().decode())
"""


def run(tmp_path, tag, b, env_extra):
    out = str(tmp_path / f"{tag}.npy")
    env = dict(os.environ, **env_extra)
    r = subprocess.run([sys.executable, "-c", SCRIPT.format(root=ROOT, b=b, out=out)], env=env, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    before, after, path = r.stdout.split()
    return int(before), int(after), path, np.load(out)


@pytest.mark.parametrize("b", [564, 96])
def test_autotune_cache_and_identical_variants(tmp_path, b):
    cache = str(tmp_path / "tune.txt")
    b1, a1, path, y1 = run(tmp_path, "first", b, {"RVGP_AUTOTUNE_CACHE": cache})
    assert path == cache and b1 == -1 and a1 in range(8)
    assert any(line.startswith(f"bspmm f32 DB2 b{b} n2^11 # ") for line in open(cache))
    b2, a2, _, y2 = run(tmp_path, "second", b, {"RVGP_AUTOTUNE_CACHE": cache})
    assert b2 == a1 and a2 == a1  # the second process starts from the cached choice
    # the same bits from every variant (chunked forced, row kernel forced)
    _, _, _, yc = run(tmp_path, "chunked", b, {"RVGP_AUTOTUNE_CACHE": cache, "RVGP_SPMM_CHUNK_MIN": "0"})
    _, _, _, yr = run(tmp_path, "rows", b, {"RVGP_AUTOTUNE_CACHE": cache, "RVGP_SPMM_CHUNK_MIN": "100000"})
    forced = [run(tmp_path, f"v{v}", b, {"RVGP_AUTOTUNE_CACHE": cache, "RVGP_SPMM_VARIANT": str(v)})[3]
              for v in range(8)]
    for y in [y2, yc, yr] + forced:
        assert np.array_equal(y, y1)
