"""Build recipe for the reference's own native module, used only as a test oracle.

Compiles ``RVGP/lib/ptu_dijkstra.pyx`` of the reference checkout, unchanged, with
Cython + gcc into ``oracle/_ref/`` (git-ignored).  Nothing is copied into the
repository: the generated C file and the extension module are build outputs.

The product never imports this module.  Only ``tests/golden/make_golden.py``
(fixture generation) and the parity tests use it, as the checker.

Usage::

    python oracle/build_ref.py [REFERENCE_ROOT]

REFERENCE_ROOT defaults to the environment variable ``RVGP_REFERENCE`` or
``/root/reference``.  When the reference or Cython is absent (for example on a
machine that only runs the GPU tests) the script prints why and exits 0.
"""
import os
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")


def build(ref_root=None, quiet=False):
    ref_root = ref_root or os.environ.get("RVGP_REFERENCE", "/root/reference")
    pyx = os.path.join(ref_root, "RVGP", "lib", "ptu_dijkstra.pyx")
    if not os.path.exists(pyx):
        if not quiet:
            print(f"reference source not found at {pyx}; skipping oracle/_ref build")
        return None
    try:
        import Cython  # noqa: F401
        import numpy
    except ImportError as e:  # pragma: no cover - depends on the machine
        if not quiet:
            print(f"cannot build oracle/_ref: {e}")
        return None
    os.makedirs(OUT, exist_ok=True)
    c_file = os.path.join(OUT, "ptu_dijkstra.c")
    so_file = os.path.join(OUT, "ptu_dijkstra" + sysconfig.get_config_var("EXT_SUFFIX"))
    if os.path.exists(so_file) and os.path.getmtime(so_file) >= os.path.getmtime(pyx):
        return so_file
    subprocess.check_call([sys.executable, "-m", "cython", "-3", "--fast-fail", pyx, "-o", c_file],
                          stdout=subprocess.DEVNULL if quiet else None)
    cmd = ["gcc", "-shared", "-fPIC", "-O2", "-w",
           "-DNPY_NO_DEPRECATED_API=NPY_1_7_API_VERSION",
           "-I", sysconfig.get_paths()["include"], "-I", numpy.get_include(),
           c_file, "-o", so_file]
    subprocess.check_call(cmd)
    return so_file


if __name__ == "__main__":
    out = build(sys.argv[1] if len(sys.argv) > 1 else None)
    if out:
        print(out)
