"""The .vtu writer (lbm_vtu_write): XML header, appended raw blocks, values."""
import struct
import xml.etree.ElementTree as ET

import numpy as np

from pv2013_gb300 import write_vtu


def _read_vtu(path):
    raw = open(path, "rb").read()
    head, rest = raw.split(b"<AppendedData encoding=\"raw\">", 1)
    data = rest[rest.index(b"_") + 1:]
    xml = head.decode() + "<AppendedData encoding=\"raw\"/></VTKFile>"
    root = ET.fromstring(xml)
    out = {}
    for da in root.iter("DataArray"):
        off = int(da.get("offset"))
        (nbytes,) = struct.unpack("<Q", data[off:off + 8])
        dt = {"Float64": "<f8", "Float32": "<f4", "Int64": "<i8", "UInt8": "u1"}[da.get("type")]
        out[da.get("Name")] = np.frombuffer(data[off + 8:off + 8 + nbytes], dtype=dt)
    piece = root.find(".//Piece")
    return root, int(piece.get("NumberOfPoints")), out


def test_vtu_roundtrip(tmp_path):
    rng = np.random.default_rng(3)
    n = 57
    pts = rng.integers(0, 100, size=(n, 3)).astype(np.float32)
    vel = rng.standard_normal((n, 3))
    rho = 1 + 0.01 * rng.standard_normal(n)
    p = tmp_path / "a.vtu"
    write_vtu(p, pts, {"Velocity": vel, "Density": rho})
    root, npts, arrs = _read_vtu(p)
    assert root.get("type") == "UnstructuredGrid" and root.get("header_type") == "UInt64"
    assert npts == n
    assert np.array_equal(arrs["Points"].reshape(-1, 3), pts)
    assert np.array_equal(arrs["Velocity"].reshape(-1, 3), vel)
    assert np.array_equal(arrs["Density"], rho)
    assert np.array_equal(arrs["connectivity"], np.arange(n))
    assert np.array_equal(arrs["offsets"], np.arange(1, n + 1))
    assert np.array_equal(arrs["types"], np.ones(n, dtype=np.uint8))   # VTK_VERTEX


def test_vtu_empty_and_bad_path(tmp_path):
    p = tmp_path / "e.vtu"
    write_vtu(p, np.zeros((0, 3)), {"WallShearStress": np.zeros(0)})
    _, npts, arrs = _read_vtu(p)
    assert npts == 0 and arrs["WallShearStress"].size == 0
    import pytest
    from pv2013_gb300 import _capi
    with pytest.raises(_capi.LbmError) as e:
        write_vtu(tmp_path / "no" / "dir" / "x.vtu", np.zeros((1, 3)), {"a": np.zeros(1)})
    assert e.value.status == 1
