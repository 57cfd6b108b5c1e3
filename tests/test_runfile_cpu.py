"""Run files: the reference's ConfigReader `key value` format (ConfigReader.cpp:13-51)
with boundary blocks, and the reference's inlet waveform as a preset."""
import math
import os

import numpy as np
import pytest

from pv2013_gb300 import runfile as R

EXAMPLE = """# a vessel run
stl vessel.stl
spacing 1.0
box 0 0 0 48 128 48
tau 0.8
steps 200
precision f16s
boundary 0
  axis y
  plane 107            # inlet plane
  tol 0.01
  box 0.5 nan nan nan 0.5 45.5
  kind vel_negy
  dir 0 -1 0
  u 0.05
  profile parabolic 23.5 23.5 20
  waveform sine 1000 0.5
end

boundary 2
  axis y
  plane 20
  kind pressure
  face +y
  rho 1.0
end
"""


def test_parse_example():
    cfg, blocks = R.parse(EXAMPLE.splitlines(True))
    assert cfg == {"stl": "vessel.stl", "spacing": 1.0, "box": "0 0 0 48 128 48", "tau": 0.8, "steps": 200,
                   "precision": "f16s"}
    assert R.grid_of(cfg) == ((0.0, 0.0, 0.0), (48, 128, 48))
    a, b = blocks
    assert (a.list_id, a.axis, a.plane, a.tol, a.kind, a.dir, a.u) == (0, 1, "107", 0.01, "vel_negy", (0.0, -1.0, 0.0), 0.05)
    assert a.lo[0] == 0.5 and math.isnan(a.hi[1]) and a.hi[2] == 45.5
    assert a.profile == ("parabolic", 23.5, 23.5, 20.0) and a.waveform == ("sine", 1000, 0.5)
    assert (b.list_id, b.kind, b.face, b.rho) == (2, "pressure", "+y", 1.0)
    t = R.amplitude_table(a)
    assert len(t) == 1000 and t[0] == 0.05 and abs(t[250] - 0.075) < 1e-15


@pytest.mark.parametrize("text,msg", [
    ("colour red\n", "unknown key"),
    ("tau\n", "expected 'key value'"),
    ("tau fast\n", "bad value"),
    ("boundary 0\n axis y\n plane 3\n kind vel_negy\n", "has no 'end'"),
    ("end\n", "outside a boundary block"),
    ("boundary 0\n axis w\nend\n", "axis must be"),
    ("boundary 0\n axis y\n plane 3\nend\n", "needs 'kind'"),
    ("boundary 0\n plane 3\n kind vel_negy\nend\n", "needs 'axis' and 'plane'"),
    ("boundary 0\n axis y\n plane 3\n kind velocity\nend\n", "needs 'face'"),
    ("boundary 0\n axis y\n plane 3\n kind swirl\nend\n", "unknown kind"),
    ("boundary 0\n axis y\n plane 3\n speed 2\n kind vel_negy\nend\n", "unknown boundary key"),
    ("boundary 0\n axis y\n plane 3\n box 1 2 3\n kind vel_negy\nend\n", "takes 6 value"),
    ("boundary 0\n axis y\n plane x3\n kind vel_negy\nend\n", "expected a number"),
    ("boundary 0\n axis y\n plane 3\n kind vel_negy\n waveform sine 0.5 1\nend\n", "whole number"),
    ("boundary 64\nend\n", "list id 0..63"),
    ("boundary 1\n axis y\n plane 3\n kind press_negy\nend\nboundary 1\n", "defined twice"),
])
def test_parse_errors_name_the_line(text, msg):
    with pytest.raises(R.RunFileError) as e:
        R.parse(text.splitlines(True), "f.run")
    assert msg in str(e.value) and "f.run:" in str(e.value)


def test_comments_and_blank_lines_are_skipped():
    cfg, blocks = R.parse(["# only a comment\n", "\n", "   \n", "steps 5  # trailing comment\n"])
    assert cfg == {"steps": 5} and blocks == []


def test_pv2013_waveform_is_the_reference_polynomials(oracle_mod):
    """The preset samples the reference's three-piece waveform: equal to the
    reference's own Pulsatile polynomials (pulsatile.h:8-31) selected as in
    Simulation.cpp:875-900, evaluated by the reference compiled here."""
    if not oracle_mod.ref_available(19):
        pytest.skip("the reference checker is not built here")
    n = 900
    ref = oracle_mod.reference_pulsatile(n)
    b = R.Block(0, "x")
    b.waveform, b.u = ("pv2013", n), 1.0
    assert np.array_equal(R.amplitude_table(b), ref)
    # the three pieces and the quiet tail
    assert ref[0] == 0.1423 and ref[-1] == 0.0 and 0.3 < ref.max() < 0.6
