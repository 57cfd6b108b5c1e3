"""Host-side checks of the C ABI that need no GPU: the library loads and
exports every entry point declared in include/*.h, STL I/O follows the
reference reader's grammar, the synthetic meshes are closed surfaces and the
PV2013 predicate preset holds the reference's constants."""
import glob
import os
import re
from collections import Counter
from decimal import Decimal

import numpy as np
import pytest

import pv2013_gb300
from pv2013_gb300 import Reader, _capi, cases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(lbm_[a-z0-9_]+)\s*\(", text))
    return names


def test_library_exports_every_declared_symbol():
    lib = pv2013_gb300.load()
    names = declared_symbols()
    assert len(names) >= 25
    for n in sorted(names):
        assert hasattr(lib, n), n
    assert set(_capi.PROTOTYPES) == names
    assert lib.lbm_abi_version() == 3


def test_status_strings():
    lib = pv2013_gb300.load()
    assert lib.lbm_status_string(0) == b"LBM_OK"
    assert lib.lbm_status_string(5) == b"LBM_ERR_DIVERGED"


def test_stl_roundtrip_exact(tmp_path):
    c = cases.vessel(4002, h=2.5)
    p = tmp_path / "v.stl"
    Reader.writeSTLASCII(p, c.triangles)
    assert np.array_equal(Reader.readSTLASCII(p), c.triangles)


def test_stl_reader_grammar_matches_oracle(tmp_path, oracle_mod):
    """Malformed facets are skipped exactly as Reader::readSTLASCII does
    (GeometryReader.cpp:127-193), including a bad third vertex that makes the
    following line be read as 'endloop'."""
    text = """solid x
facet normal 0 0 1
outer loop
vertex 0 0 0
vertex 1 0 0
vertex 0 1 0
endloop
endfacet
facet normal 0 0 1
outer loop
vertex 0 0 1
vertex 1 0 1
vertex oops 1 1
endloop
endfacet
facet normal 1 nan 0
outer loop
vertex 0 0 2
vertex 1 0 2
vertex 0 1 2
endloop
endfacet
facet normal 0 0 -1
  outer    loop
vertex 0 0 3
vertex 2.5e-1 0 3
vertex 0 1e+0 3
endloop
endfacet
facet normal 0 0 -1
outer loop
vertex 1 1 4
vertex 2 1 4
vertex 1 2 4
endloop
endfacet
endsolid x
"""
    p = tmp_path / "g.stl"
    p.write_text(text)
    mine = Reader.readSTLASCII(p)
    ref = oracle_mod.read_stl_ascii(p)
    assert mine.shape == ref.shape
    assert np.array_equal(mine, ref)


def test_stl_missing_file_reports_io_error():
    with pytest.raises(_capi.LbmError) as e:
        Reader.readSTLASCII("/nonexistent/file.stl")
    assert e.value.status == 1


def test_binary_stl_reader(tmp_path):
    tris = cases.pipe().triangles.astype(np.float32)
    p = tmp_path / "b.stl"
    with open(p, "wb") as fh:
        fh.write(b"\0" * 80)
        fh.write(np.uint32(len(tris)).tobytes())
        for t in tris:
            fh.write(t[9:12].tobytes() + t[0:9].tobytes() + b"\0\0")
    got = Reader.readSTLBinary(p)
    assert np.array_equal(got[:, :9], tris[:, :9].astype(np.float64))
    n = tris[:, 9:12]
    norm = np.sqrt((n[:, 0] * n[:, 0] + n[:, 1] * n[:, 1]) + n[:, 2] * n[:, 2]).astype(np.float32)
    assert np.array_equal(got[:, 9:12], (n / norm[:, None]).astype(np.float64))   # float arithmetic, exact


def _open_edges(t):
    cnt = Counter()
    v = t[:, :9].reshape(-1, 3, 3)
    for tri in v:
        for a, b in ((0, 1), (1, 2), (2, 0)):
            cnt[tuple(sorted((tuple(tri[a]), tuple(tri[b]))))] += 1
    return sum(1 for c in cnt.values() if c != 2)


@pytest.mark.parametrize("make", [lambda: cases.pipe(), lambda: cases.vessel(4000, h=2.0),
                                  lambda: cases.bifurcation(nx=96, ny=192, nz=96, r_parent=10, r_child=8, h=2.0)])
def test_synthetic_meshes_are_closed(make):
    c = make()
    assert len(c.triangles) > 0
    assert _open_edges(c.triangles) == 0
    n = c.triangles[:, 9:12]
    assert np.allclose(np.linalg.norm(n, axis=1), 1.0)


def test_benchmark_tree_is_reproducible():
    """The seeded benchmark workload is the same mesh on every build: the
    tree's triangle count and an order-dependent checksum of its bytes are
    stable across calls (the bench's grid, fluid-node count and outlet lists
    follow from it)."""
    import hashlib
    a, b = cases.vascular_tree(h=2.2), cases.vascular_tree(h=2.2)
    assert len(a.triangles) == len(b.triangles) == 2066396
    ha = hashlib.sha256(np.ascontiguousarray(a.triangles).tobytes()).hexdigest()
    hb = hashlib.sha256(np.ascontiguousarray(b.triangles).tobytes()).hexdigest()
    assert ha == hb
    assert a.triangles.shape[1] == 12


def test_pv2013_predicates_hold_reference_constants():
    preds = pv2013_gb300.pv2013_predicates()
    planes = ["-175.275", "-164.075", "-174.475", "-28.3", "-25.5", "-37.0", "-108.379"]
    axes = [1, 1, 1, 0, 0, 0, 2]
    for p, s, ax in zip(preds, planes, axes):
        assert p.axis == ax and p.tol == 1e-2
        exact = Decimal(p.plane_hi) + Decimal(p.plane_lo)
        # the long double literal is within 2^-63 relative of the decimal constant
        assert abs(exact - Decimal(s)) <= abs(Decimal(s)) * Decimal(2) ** -60


def test_geometry_without_device_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    c = cases.pipe()
    with pytest.raises(_capi.LbmError) as e:
        c.geometry()
    assert e.value.status == 9


def test_device_stl_reader_without_device_fails_cleanly(tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    p = tmp_path / "t.stl"
    Reader.writeSTLASCII(p, cases.pipe().triangles[:3])
    with pytest.raises(_capi.LbmError) as e:
        Reader.readSTLASCIIDevice(p)
    assert e.value.status == 9


def test_prototypes_have_the_header_argument_counts():
    """Each ctypes prototype takes as many arguments as the header declares."""
    decl = {}
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        for m in re.finditer(r"\b(lbm_[a-z0-9_]+)\s*\(([^()]*)\)\s*;", text):
            params = m.group(2).strip()
            decl[m.group(1)] = 0 if params in ("", "void") else params.count(",") + 1
    assert len(decl) >= 25
    for name, n in decl.items():
        assert len(_capi.PROTOTYPES[name][1]) == n, name
