"""Generate tests/golden/features.npz from the reference's own code.

* ``compute_vectorfield_features`` (examples/eeg_example/eeg_utils.py:46-80):
  its module imports packages that are absent here (pandas, mne), so the
  function's own source is taken out of the file with ``ast`` and run as
  written, with numpy and scipy's ``KDTree`` in its namespace.
* ``load_mesh`` (RVGP/utils.py:7-47), the reference module file loaded on its
  own (the package ``__init__`` needs TensorFlow), on a synthetic OBJ file (a
  UV sphere written below; no reference data file is used).

    python tests/golden/make_features_golden.py
"""
import ast
import os
import tempfile

import numpy as np
from scipy.spatial import KDTree

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("RVGP_REFERENCE", "/root/reference")


def reference_features():
    path = os.path.join(REF, "examples", "eeg_example", "eeg_utils.py")
    tree = ast.parse(open(path).read())
    fn = next(n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name == "compute_vectorfield_features")
    ns = {"np": np, "KDTree": KDTree}
    exec(compile(ast.Module(body=[fn], type_ignores=[]), path, "exec"), ns)
    return ns["compute_vectorfield_features"]


def uv_sphere_obj(n_lat=12, n_lon=20):
    """OBJ text of a UV sphere: comment lines, 'v x y z' vertices, 'f a b c' faces (1-based)."""
    lines = ["# synthetic UV sphere", "o sphere"]
    verts = [(0.0, 0.0, 1.0)]
    for i in range(1, n_lat):
        th = np.pi * i / n_lat
        for j in range(n_lon):
            ph = 2 * np.pi * j / n_lon
            verts.append((np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)))
    verts.append((0.0, 0.0, -1.0))
    lines += ["v {:.9f} {:.9f} {:.9f}".format(*v) for v in verts]
    faces = []
    for j in range(n_lon):
        faces.append((1, 2 + j, 2 + (j + 1) % n_lon))
    for i in range(n_lat - 2):
        a0, b0 = 2 + i * n_lon, 2 + (i + 1) * n_lon
        for j in range(n_lon):
            j1 = (j + 1) % n_lon
            faces.append((a0 + j, b0 + j, b0 + j1))
            faces.append((a0 + j, b0 + j1, a0 + j1))
    last = len(verts)
    base = 2 + (n_lat - 2) * n_lon
    for j in range(n_lon):
        faces.append((base + j, last, base + (j + 1) % n_lon))
    lines += ["f {} {} {}".format(*f) for f in faces]
    return "\n".join(lines) + "\n"


def main():
    import importlib.util
    # RVGP/utils.py needs only os and numpy: load the file itself, not the package
    spec = importlib.util.spec_from_file_location("rvgp_reference_utils", os.path.join(REF, "RVGP", "utils.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    load_mesh = mod.load_mesh
    out = {}
    rng = np.random.default_rng(0)
    feats = reference_features()
    # EEG-like: 64 positions on a half sphere, 3-d vectors; and a larger cloud
    for name, n in (("small", 64), ("large", 1500)):
        P = rng.standard_normal((n, 3))
        P /= np.linalg.norm(P, axis=1, keepdims=True)
        P[:, 2] = np.abs(P[:, 2])
        V = rng.standard_normal((n, 3))
        div, curl = feats(P, V, k=5)
        out[f"{name}_pos"], out[f"{name}_vec"] = P, V
        out[f"{name}_div"], out[f"{name}_curl"] = div, curl
    text = uv_sphere_obj()
    with tempfile.TemporaryDirectory() as tmp:
        with open(os.path.join(tmp, "uvsphere.obj"), "w") as f:
            f.write(text)
        v, fa = load_mesh(data="uvsphere", folder=tmp)
    out["obj_text"] = np.frombuffer(text.encode(), dtype=np.uint8)
    out["obj_vertices"], out["obj_faces"] = v, fa
    np.savez_compressed(os.path.join(HERE, "features.npz"), **out)
    print({k: a.shape for k, a in out.items()})


if __name__ == "__main__":
    main()
