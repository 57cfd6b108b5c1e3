"""In-tree build of liblbm_gb300.so (nvcc, sm_103a) via csrc/Makefile."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))


def build_library(jobs=None):
    jobs = jobs or max(2, min(16, os.cpu_count() or 2))
    subprocess.run(["make", "-s", "-C", os.path.join(HERE, "csrc"), f"-j{jobs}"], check=True)
    return os.path.join(HERE, "_lib", "liblbm_gb300.so")


if __name__ == "__main__":
    print(build_library())
