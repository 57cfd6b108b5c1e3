"""Host code under AddressSanitizer and UndefinedBehaviorSanitizer.

Builds tests/sanitize_host.cpp with the library's host sources (STL reader
and writer, mesh generators, .vtu writer) and the oracle, all with
-fsanitize=address,undefined, and runs it: valid, truncated and malformed STL
files through both host readers, the generators, the writer, and the oracle's
voxelizer and FP64 time loop.  Any sanitizer finding aborts the run."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _sanitizers_available(tmp):
    src = os.path.join(tmp, "probe.cpp")
    with open(src, "w") as fh:
        fh.write("int main() { return 0; }\n")
    r = subprocess.run(["g++", "-fsanitize=address,undefined", src, "-o", os.path.join(tmp, "probe")],
                       capture_output=True)
    return r.returncode == 0


def test_host_code_under_sanitizers(tmp_path):
    if shutil.which("g++") is None or not _sanitizers_available(str(tmp_path)):
        pytest.skip("g++ with AddressSanitizer/UndefinedBehaviorSanitizer not available")
    exe = str(tmp_path / "sanitize_host")
    csrc = os.path.join(ROOT, "pv2013_gb300", "csrc")
    cmd = ["g++", "-std=c++17", "-O1", "-g", "-fno-omit-frame-pointer", "-fsanitize=address,undefined",
           "-fno-sanitize-recover=all", "-fopenmp", "-ffp-contract=off",
           "-I" + os.path.join(ROOT, "include"), "-I" + csrc,
           os.path.join(HERE, "sanitize_host.cpp"), os.path.join(csrc, "stl_io.cpp"), os.path.join(csrc, "synth.cpp"),
           os.path.join(csrc, "vtu.cpp"), os.path.join(ROOT, "oracle", "lbm_oracle.cpp"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    env = dict(os.environ, OMP_NUM_THREADS="2", ASAN_OPTIONS="detect_leaks=1:abort_on_error=1",
               UBSAN_OPTIONS="print_stacktrace=1:halt_on_error=1")
    run = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True, env=env, timeout=600)
    assert run.returncode == 0, (run.stdout[-2000:], run.stderr[-4000:])
    assert "sanitized host run ok" in run.stdout
