"""Wavefront OBJ reading and writing for the command line (the reference loads and exports meshes with trimesh,
example.py:24-40).

``load_obj`` reads vertex positions (``v``) and faces (``f``, 1-based or negative indices, ``i/t/n`` entries
reduced to the position index) in file order and splits polygons into fans (0, k, k+1), which is what
``trimesh.load(..., process=False)`` does for plain position meshes. Texture and normal data are ignored: a file
whose faces reference different texture coordinates at one position therefore keeps one vertex there (trimesh
would split it).
"""

from __future__ import annotations

import numpy as np


def load_obj(path: str):
    """(vertices float64 [n,3], faces int32 [m,3])."""
    verts = []
    faces = []
    with open(path, "r", errors="replace") as fh:
        for line in fh:
            if line.startswith("v "):
                p = line.split()
                verts.append((float(p[1]), float(p[2]), float(p[3])))
            elif line.startswith("f "):
                idx = []
                for tok in line.split()[1:]:
                    k = int(tok.split("/")[0])
                    idx.append(k - 1 if k > 0 else len(verts) + k)
                for j in range(1, len(idx) - 1):
                    faces.append((idx[0], idx[j], idx[j + 1]))
    V = np.asarray(verts, np.float64).reshape(-1, 3)
    F = np.asarray(faces, np.int64).reshape(-1, 3)
    if F.size and (F.min() < 0 or F.max() >= len(V)):
        raise ValueError(f"{path}: a face references a vertex that does not exist")
    return V, F.astype(np.int32)


def save_obj(path: str, vertices, faces) -> None:
    """Positions with 17 significant digits (float64 round trip), faces 1-based."""
    V = np.asarray(vertices, np.float64).reshape(-1, 3)
    F = np.asarray(faces, np.int64).reshape(-1, 3)
    with open(path, "w") as fh:
        fh.write("".join(f"v {x:.17g} {y:.17g} {z:.17g}\n" for x, y, z in V))
        fh.write("".join(f"f {a + 1} {b + 1} {c + 1}\n" for a, b, c in F))
