"""Loads the PV2013 golden fixtures (tests/golden) and rebuilds the reference's
boundary-point VTK text (GeometryWriter.cpp:35-69) from grid indices."""
import hashlib
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
KEYS = ["inlet"] + [f"outlet{k}" for k in range(1, 7)] + ["wall"]


def load():
    meta = json.load(open(os.path.join(GOLDEN, "pv2013_vtk.json")))
    tris = np.load(os.path.join(GOLDEN, "pv2013_tris.npz"))["tris"]
    d = np.load(os.path.join(GOLDEN, "pv2013_lists.npz"))
    lists = {k: np.cumsum(d[k]) for k in KEYS}
    return meta, tris, lists


def vtk_text(idx, dims, bbox, spacing):
    """Text of Writer::writePointsToFile for points min + ijk*spacing (ostream
    default: 6 significant digits, %g style)."""
    Nx, Ny, Nz = dims
    idx = np.asarray(idx, dtype=np.int64)
    i, j, k = idx // (Ny * Nz), (idx // Nz) % Ny, idx % Nz
    x = bbox[0] + i * spacing
    y = bbox[2] + j * spacing
    z = bbox[4] + k * spacing
    n = len(idx)
    out = ["# vtk DataFile Version 2.0", "Points Inside Complex Geometry", "ASCII", "DATASET UNSTRUCTURED_GRID",
           f"POINTS {n} double"]
    out += ["%g %g %g" % (a, b, c) for a, b, c in zip(x.tolist(), y.tolist(), z.tolist())]
    out.append(f"CELLS {n} {2 * n}")
    out += [f"1 {m}" for m in range(n)]
    out.append(f"CELL_TYPES {n}")
    out += ["1"] * n
    return "\n".join(out) + "\n"


def sha256(text):
    return hashlib.sha256(text.encode()).hexdigest()


NAN = float("nan")
# getInOutBP predicates (ComplexGeometry.cpp:587-633): list id, axis, plane
# literal (long double), open ranges on the other axes (x, y, z order)
PREDICATES = [
    (0, 1, "-175.275", (-9.9, NAN, -129.979), (-3.3, NAN, -124.799)),
    (1, 1, "-164.075", (NAN, NAN, NAN), (NAN, NAN, NAN)),
    (2, 1, "-174.475", (-5.4, NAN, -101.379), (-5, NAN, -100.979)),
    (3, 0, "-28.3", (NAN, -179.975, -97.2794), (NAN, -178.875, -96.2794)),
    (4, 0, "-25.5", (NAN, -180.675, -100.779), (NAN, -179.875, -100.379)),
    (5, 0, "-37.0", (NAN, NAN, NAN), (NAN, NAN, NAN)),
    (6, 2, "-108.379", (-29.7, -196.375, NAN), (-28.1, -194.575, NAN)),
]


def oracle_tuples():
    return [(lid, (axis, plane, 1e-2, lo, hi)) for lid, axis, plane, lo, hi in PREDICATES]
