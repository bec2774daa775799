"""CPU: the C-ABI library builds, loads without a GPU and exports every symbol
declared in include/rvgp_gb300.h (no compute calls here)."""
import ctypes
import os
import re

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "rvgp_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rvgp_[A-Za-z0-9_]+)\s*\(", text)))


def test_library_exports_header():
    from rvgp_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(path)
    names = declared_symbols()
    assert len(names) >= 10
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_bindings_cover_header():
    from rvgp_gb300 import _core
    names = declared_symbols()
    assert sorted(_core.SIGNATURES) == names


def test_abi_version_and_error_string():
    from rvgp_gb300 import _core
    lib = _core.lib()
    assert lib.rvgp_abi_version() >= 1
    assert isinstance(lib.rvgp_last_error(), bytes)


def test_argument_errors_without_gpu():
    """Argument validation runs before any device work, so it is testable here."""
    from rvgp_gb300 import _core
    lib = _core.lib()
    st = lib.rvgp_knn(None, 10, 3, 20, None, None, 0, None)
    assert st == -1
    assert b"" != lib.rvgp_last_error()
    assert lib.rvgp_knn_workspace(100, 3, 10) > 100 * 3 * 4
    # unsupported shapes report no workspace (rvgp_knn itself rejects them)
    assert lib.rvgp_knn_workspace(100, 129, 10) == 0
    assert lib.rvgp_knn_workspace(100, 3, 100) == 0
