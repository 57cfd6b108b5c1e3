#!/usr/bin/env python3
"""Stage the PV2013 reference sources for the CPU checker.  TEST INFRASTRUCTURE ONLY.

Copies the reference's own C++ files from the reference checkout into
``oracle/_ref/src`` (git-ignored, never committed) and applies the minimal
patches needed to compile them with g++ 13 and to drive them from a harness:

* ``Macro.h``: the lattice is chosen by ``-DD3Q27`` instead of an edit.
* ``mpi_call.h:143-145``: inner template parameter ``T`` shadows the class
  parameter (accepted by icc, an error in g++); renamed ``U``.
* ``OutputFile.h``: libvtk includes dropped (bodies replaced by
  ``OutputFile_noop.cpp``; .vtu output is not on the step path).
* ``Simulation.cpp:908``: iteration count read from ``g_oracle_steps`` so the
  constructor can run zero steps and the harness calls the step methods.
* ``Simulation.cpp:954``: outlet density read from ``g_oracle_outlet_rho``.
* ``Boundary.cpp:25-30``: ``SetInletVel`` assigns instead of appending, so a
  per-node, per-step inlet velocity can be set.
* ``LatticeModel.cpp`` D3Q27 constructor: passes the missing (empty) Zou-He
  pair list so the 4-argument ``VelocitySet`` constructor is matched.

Usage: ``stage_ref.py <reference dir> <out dir>``.
"""
import os
import re
import sys

FILES = [
    "Boundary.cpp", "Boundary.h", "ComplexGeometry.cpp", "ComplexGeometry.h", "GeometryReader.cpp",
    "GeometryReader.h", "GeometryWriter.cpp", "GeometryWriter.h", "HaloLayer.cpp", "HaloLayer.h",
    "LatticeModel.cpp", "LatticeModel.h", "Macro.h", "Node.cpp", "Node.h", "OutputFile.h",
    "Simulation.cpp", "Simulation.h", "Struct.h", "Subdomain.cpp", "Subdomain.h", "Utility.cpp", "Utility.h",
    "VelocitySet.cpp", "VelocitySet.h", "include.h", "mpi_call.h", "pulsatile.h", "typedef.h",
]


def sub_once(text, pattern, repl, name):
    new, n = re.subn(pattern, repl, text, count=1)
    if n != 1:
        raise SystemExit(f"stage_ref: patch '{name}' did not apply")
    return new


def main():
    src, out = sys.argv[1], sys.argv[2]
    os.makedirs(out, exist_ok=True)
    for f in FILES:
        with open(os.path.join(src, f), "r", encoding="utf-8-sig", newline="") as fh:
            text = fh.read()
        if f == "Macro.h":
            text = sub_once(text, r"#define D3Q19", "#if !defined(D3Q27)\n#define D3Q19\n#endif", f)
        elif f == "mpi_call.h":
            text = sub_once(
                text,
                r"template <typename T>(\s*)std::vector<T> flatten\(const std::vector<std::vector<T>>& vec\) \{(\s*)std::vector<T> result;",
                r"template <typename U>\1std::vector<U> flatten(const std::vector<std::vector<U>>& vec) {\2std::vector<U> result;",
                f)
        elif f == "OutputFile.h":
            text, n = re.subn(r"#include <vtk[^>]*>\r?\n", "", text)
            if n == 0:
                raise SystemExit("stage_ref: OutputFile.h vtk includes not found")
        elif f == "Simulation.cpp":
            text = sub_once(text, r'#include "Simulation.h"',
                            '#include "Simulation.h"\nextern int g_oracle_steps;\nextern double g_oracle_outlet_rho;', f)
            text = sub_once(text, r"while \(iter<20000\)", "while (iter<g_oracle_steps)", f)
            text = sub_once(text, r"double rho = 1\.01;", "double rho = g_oracle_outlet_rho;", f)
        elif f == "Boundary.cpp":
            text = sub_once(text, r"m_inletVel\.push_back\(ux\);", "m_inletVel.clear(); m_inletVel.push_back(ux);", f)
        elif f == "LatticeModel.cpp":
            # the D3Q27 block is the only one whose direction list is followed
            # directly by the c_s^2 argument after a run of blank lines
            text = sub_once(text, r"(//26\s*\r?\n\s*\r?\n\s*\r?\n\s*\},)(\s*)1\.0 / 3\.0", r"\1\2{},\g<2>1.0 / 3.0", f)
        with open(os.path.join(out, f), "w", newline="") as fh:
            fh.write(text)
    print(f"staged {len(FILES)} reference files into {out}")


if __name__ == "__main__":
    main()
