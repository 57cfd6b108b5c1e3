#!/usr/bin/env python3
"""Generates the PV2013 golden fixtures from the reference checkout.

Inputs (read from the reference checkout given as argv[1], or else by the
PV2013_REF_DIR environment variable):
  PV2013.stl                                  the vessel surface (ASCII STL)
  InboundaryPointsFromGeometry.vtk,
  OutboundaryPointsFromGeometry{1..6}.vtk,
  WallboundaryPointsFromGeometry.vtk          boundary-point lists written by
                                              the reference (ComplexGeometry.cpp:23-31)
Outputs (this directory):
  pv2013_tris.npz     the STL's triangles as float64 (n, 12), parsed with the
                      reference's grammar (strtod-exact)
  pv2013_lists.npz    each golden list as x-major grid indices of the tight
                      grid at spacing 0.1 (delta-encoded), plus the grid
  pv2013_vtk.json     point count and SHA-256 of every golden file

The tests rebuild the VTK text from indices with the reference writer's
format (GeometryWriter.cpp:35-69, 6 significant digits) and compare hashes,
so the fixtures pin the lists byte for byte without carrying 8.6 MB of text.
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

NAMES = ["InboundaryPointsFromGeometry.vtk"] + [f"OutboundaryPointsFromGeometry{k}.vtk" for k in range(1, 7)] + \
        ["WallboundaryPointsFromGeometry.vtk"]
KEYS = ["inlet"] + [f"outlet{k}" for k in range(1, 7)] + ["wall"]


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PV2013_REF_DIR")
    if not ref:
        raise SystemExit("usage: make_golden.py REFERENCE_DIR (or set PV2013_REF_DIR)")
    from oracle import oracle as O
    tris = O.read_stl_ascii(os.path.join(ref, "PV2013.stl"))
    np.savez_compressed(os.path.join(HERE, "pv2013_tris.npz"), tris=tris)
    bb, dims = O.tight_grid(tris, 0.1)
    Nx, Ny, Nz = (int(v) for v in dims)
    meta = {"spacing": 0.1, "dims": [Nx, Ny, Nz], "bbox": [float(v) for v in bb], "files": {}}
    lists = {}
    for name, key in zip(NAMES, KEYS):
        raw = open(os.path.join(ref, name), "rb").read()
        lines = raw.decode().splitlines()
        n = int(lines[4].split()[1])
        pts = np.array([[float(v) for v in ln.split()] for ln in lines[5:5 + n]]).reshape(-1, 3)
        ijk = np.rint((pts - bb[[0, 2, 4]]) / 0.1).astype(np.int64)
        idx = (ijk[:, 0] * Ny + ijk[:, 1]) * Nz + ijk[:, 2]
        lists[key] = np.diff(idx, prepend=0)
        meta["files"][key] = {"name": name, "points": n, "sha256": hashlib.sha256(raw).hexdigest()}
    np.savez_compressed(os.path.join(HERE, "pv2013_lists.npz"), **lists)
    with open(os.path.join(HERE, "pv2013_vtk.json"), "w") as fh:
        json.dump(meta, fh, indent=1)
    print(json.dumps({k: v["points"] for k, v in meta["files"].items()}))


if __name__ == "__main__":
    main()
