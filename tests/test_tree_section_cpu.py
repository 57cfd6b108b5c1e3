"""The bounded tree sample the reference's step loop is timed on
(oracle/fixtures/tree_inlet_section.npz, bench.py's reference arm and CPU
baseline): it equals a fresh cut of the seeded tree, and the reference arm
runs the requested step count on it without this package's library."""
import json
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_fixture_is_the_tree_inlet_section():
    sys.path.insert(0, os.path.join(ROOT, "oracle", "fixtures"))
    import make_tree_section as M
    from pv2013_gb300 import cases
    case = cases.vascular_tree(h=2.2)
    flags, origin, dims = M.section(case)
    fx = np.load(os.path.join(ROOT, "oracle", "fixtures", "tree_inlet_section.npz"))
    assert np.array_equal(fx["flags"], flags)
    assert tuple(fx["origin"]) == origin and tuple(int(v) for v in fx["dims"]) == dims
    assert float(fx["inlet_plane"]) == case.inlet.plane and float(fx["tau"]) == case.tau


def test_sections_sized_to_the_step_count():
    import bench
    (flags, origin, dims), params = bench.reference_sample(bench.levels_for(4000))
    assert dims[1] == 3 and flags.shape == (96, 3, 96)
    # the inlet plane stays inside the section
    assert origin[1] <= params["inlet_plane"] < origin[1] + dims[1]
    assert bench.reference_sample(bench.levels_for(20))[0][2][1] == 40


def test_reference_arm_runs_the_requested_steps_without_the_engine():
    from oracle import oracle as O
    if not O.ref_available(19):
        import pytest
        pytest.skip("the reference checker is not built here")
    code = ("import sys, json, types, bench\n"
            "a = types.SimpleNamespace(steps=3, warmup=1)\n"
            "out = bench.reference_arm(a)\n"
            "out['engine_loaded'] = any(m.startswith('pv2013_gb300') for m in sys.modules)\n"
            "print(json.dumps(out))\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["impl"] == "reference" and out["steps"] == 3 and out["value"] > 0
    assert not out["engine_loaded"]
