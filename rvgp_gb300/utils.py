"""Mesh input (RVGP/utils.py:7-47)."""
from __future__ import annotations

import os

import numpy as np


def load_mesh(data="bunny", folder=None):
    """Vertices (float64, (V, 3)) and triangular faces (int, (F, 3), 0-based) of
    ``<folder>/<data>.obj``.

    Reads 'v x y z' and 'f a b c' records as RVGP/utils.py:7-47 does, skipping
    '#' comments.  Deliberately more tolerant than the reference, which fails
    on these: blank lines are skipped and face entries of the form
    'a/b/c' use the vertex index before the first '/'.  With ``folder=None`` the
    file is looked up in ``examples/data`` beside the package, as in the
    reference.
    """
    if folder is None:
        folder = os.path.join(os.path.dirname(os.path.realpath(__file__)), "..", "examples", "data")
    vertices, faces = [], []
    with open(os.path.join(folder, f"{data}.obj"), "r") as f:
        for line in f:
            if line.startswith("#"):
                continue
            words = line.split()
            if not words:
                continue
            if words[0] == "v":
                vertices.append([float(words[1]), float(words[2]), float(words[3])])
            elif words[0] == "f":
                faces.append([int(w.split("/")[0]) for w in words[1:4]])
    return np.array(vertices), np.array(faces) - 1
