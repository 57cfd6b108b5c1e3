#!/usr/bin/env python3
"""Writes tree_inlet_section.npz: the bounded sample of the vascular-tree
workload that the reference's own step loop is timed on (bench.py's reference
arm and its CPU baseline).  TEST INFRASTRUCTURE ONLY.

The sample is the 96 x 40 x 96-point block of the 512 x 1024 x 512 tree grid
(pv2013_gb300.cases.vascular_tree, seed 5) just below the inlet face, its node
types computed by the CPU oracle's column voxelizer on the full grid's rays
(the reference's own O(points x triangles) voxelizer would take days on the
tree's 2.07 M triangles).  Stored with it: the block's origin and size, the
inlet plane and centre, tau.  With the fixture the timing run needs neither
the tree's mesh nor this package's library.  tests/test_tree_section_cpu.py
regenerates the block and compares it with the fixture.

    python oracle/fixtures/make_tree_section.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "tree_inlet_section.npz")


def section(case, width=96, height=40):
    """(flags (width, height, width) uint8, origin, dims) below the inlet face."""
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    bb, dims = O.explicit_grid(case.grid, 1.0)
    cx, cz = int(case.inlet.center[0]), int(case.inlet.center[1])
    x0, z0 = cx - width // 2, cz - width // 2
    y1 = int(case.inlet.plane) + 2
    y0 = y1 - height
    block = O.voxelize_columns(case.triangles, bb, 1.0, dims, x0, x0 + width, y0, y1)
    sub = block[:, :, z0:z0 + width].copy()
    return sub, (float(x0), float(y0), float(z0)), (width, y1 - y0, width)


def main():
    sys.path.insert(0, ROOT)
    from pv2013_gb300 import cases
    case = cases.vascular_tree(h=2.2)
    flags, origin, dims = section(case)
    np.savez_compressed(OUT, flags=flags, origin=np.array(origin), dims=np.array(dims, dtype=np.int32),
                        inlet_plane=float(case.inlet.plane), inlet_center=np.array(case.inlet.center, dtype=np.float64),
                        tau=float(case.tau))
    print(OUT, flags.shape, int(flags.sum()), "fluid points")


if __name__ == "__main__":
    main()
