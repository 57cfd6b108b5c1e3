"""ASCII STL parsing on the GPU (lbm_stl_read_ascii_device) against the host
reader (the reference's grammar, GeometryReader.cpp:33-117, with correctly
rounded numbers): same triangles bit for bit, on the GPU path for files in
the canonical facet layout and through the host grammar otherwise."""
import time

import numpy as np
import pytest

from pv2013_gb300 import Reader, cases

pytestmark = pytest.mark.gpu

CANON = """solid odd formatting\r
facet normal 0 0 1\r
  outer   loop\r
\tvertex 0 0 0\r
vertex +.5 5. 1.e3\r
vertex -7.25E+02 1e-0 -0.000\r
endloop\r
endfacet\r

facet normal -1.2246467991473532e-16 6.123233995736766e-17 -1
outer loop extra words are ignored
vertex 1.0000000000000002 9007199254740993 123456789012345678e-27
vertex 1e-60 9999999999999999999e41 0.1
vertex 3.1415926535897932 2.5e-1 7
endloop
endfacet trailing
endsolid odd formatting"""


def _both(path):
    host = Reader.readSTLASCII(path)
    dev, on_device = Reader.readSTLASCIIDevice(path)
    return host, dev, on_device


def test_canonical_files_parse_on_the_device(tmp_path):
    p = tmp_path / "canon.stl"
    p.write_bytes(CANON.encode())
    host, dev, on_device = _both(p)
    assert on_device
    assert host.shape == (2, 12)
    assert np.array_equal(host.view(np.uint64), dev.view(np.uint64))     # bits, signed zeros included


def _pv2013_tris():
    import golden_pv2013 as G
    return G.load()[1]


@pytest.mark.parametrize("make", [lambda: cases.pipe().triangles, lambda: cases.vessel(4007).triangles, _pv2013_tris])
def test_written_meshes_match_host_reader(tmp_path, make):
    tris = np.asarray(make())
    p = tmp_path / "mesh.stl"
    Reader.writeSTLASCII(p, tris)
    host, dev, on_device = _both(p)
    assert on_device
    assert np.array_equal(host.view(np.uint64), dev.view(np.uint64))
    assert np.array_equal(dev, tris)                                      # %.17g round trip


@pytest.mark.parametrize("text,why", [
    (CANON.replace("outer   loop", "outer lop", 1), "broken facet"),
    (CANON.replace("2.5e-1 7", "2.5e-1x 7", 1), "a number the host tokenizer rejects"),
    (CANON.replace("0.1", "0.12345678901234567890123", 1), "more than 19 significant digits"),
    (CANON.replace("1e-60", "1e-400", 1), "exponent outside the exact scope"),
    (CANON.replace("vertex 1e-60", "vertex 1e400", 1), "overflow: the host reader drops the facet"),
    (CANON + "\nfacet normal 0 0 1\nouter loop\n", "truncated last facet"),
    (CANON.replace("vertex 0 0 0", "vertex 0 0\x00 0", 1), "NUL byte"),
])
def test_other_files_take_the_host_grammar(tmp_path, text, why):
    p = tmp_path / "odd.stl"
    p.write_bytes(text.encode())
    host, dev, on_device = _both(p)
    assert not on_device, why
    assert host.shape == dev.shape and np.array_equal(host.view(np.uint64), dev.view(np.uint64)), why


def test_empty_and_headerless_files(tmp_path):
    for text in ("", "solid empty\nendsolid empty\n", "\n\n\n"):
        p = tmp_path / "e.stl"
        p.write_bytes(text.encode())
        host, dev, on_device = _both(p)
        assert on_device and host.shape == dev.shape == (0, 12)


def test_large_mesh_timing(tmp_path):
    """The bifurcation workload's mesh (about 200 k triangles, %.17g): the
    device parse gives the host reader's bits and is timed beside it."""
    c = cases.bifurcation()
    p = tmp_path / "bif.stl"
    Reader.writeSTLASCII(p, c.triangles)
    t0 = time.perf_counter()
    host = Reader.readSTLASCII(p)
    t_host = time.perf_counter() - t0
    Reader.readSTLASCIIDevice(p)                                        # warm-up (context, allocations)
    t0 = time.perf_counter()
    dev, on_device = Reader.readSTLASCIIDevice(p)
    t_dev = time.perf_counter() - t0
    assert on_device and np.array_equal(host.view(np.uint64), dev.view(np.uint64))
    print(f"\n{len(host)} triangles, {p.stat().st_size / 1e6:.1f} MB: host {t_host * 1e3:.0f} ms, "
          f"device {t_dev * 1e3:.0f} ms")
