"""Regenerate tests/golden/leapfrog_golden.json from the reference's own leap-frog unit test.

Reads, as text, the parameter sets of LeapFrogTest.SimpleIntegration
(src/gromacs/mdlib/tests/leapfrog.cpp: atoms, time step, steps, initial velocity, constant force,
temperature-coupling groups, pressure-coupling interval) and its reference outputs (final
positions and velocities, src/gromacs/mdlib/tests/refdata/
WithParameters_LeapFrogTest_SimpleIntegration_<i>.xml), keeping the cases without temperature
or pressure coupling (the integrator this engine has).  The initial state is the test's own
construction (src/gromacs/mdlib/tests/leapfrogtestdata.cpp): x_i = ((i % 21), 6.5 - (i % 13), 0),
v_i = v0, f_i = f0, 1/m_i = 1 / (1 + i % 100).  Run it where the reference tree is available:

    python tests/golden/make_leapfrog_golden.py /path/to/gromacs-source
"""
from __future__ import annotations

import json
import os
import re
import sys
import xml.etree.ElementTree as ET

_NUM = r"[-+]?(?:\d+\.?\d*|\.\d+)(?:[eE][-+]?\d+)?"


def _parameter_sets(text: str) -> list[list[float]]:
    i = text.index("parametersSets[]")
    j = text.index("};", i)
    rows = []
    for line in text[i:j].splitlines():
        line = line.split("//")[0]
        vals = re.findall(_NUM, line)
        if len(vals) == 11:
            rows.append([float(v) for v in vals])
    return rows


def _vectors(root, name):
    for seq in root.iter("Sequence"):
        if seq.get("Name") == name:
            out = []
            for atom in seq.findall("Atom"):
                d = {r.get("Name"): float(r.text) for r in atom.findall("Real")}
                out.append([d["XX"], d["YY"], d["ZZ"]])
            return out
    raise KeyError(name)


def main(src_root: str) -> None:
    tests = os.path.join(src_root, "src", "gromacs", "mdlib", "tests")
    params = _parameter_sets(open(os.path.join(tests, "leapfrog.cpp")).read())
    cases = []
    for idx, p in enumerate(params):
        natoms, dt, nsteps = int(p[0]), p[1], int(p[2])
        v0, f0, ntc, npc = p[3:6], p[6:9], int(p[9]), int(p[10])
        if ntc != 0 or npc != 0:
            continue
        root = ET.parse(os.path.join(tests, "refdata",
                                     f"WithParameters_LeapFrogTest_SimpleIntegration_{idx}.xml")).getroot()
        cases.append({"index": idx, "num_atoms": natoms, "dt": dt, "num_steps": nsteps, "v0": v0, "f0": f0,
                      "final_x": _vectors(root, "FinalPositions"), "final_v": _vectors(root, "FinalVelocities"),
                      "tolerance": nsteps * 0.000005})
    out = {"source": "src/gromacs/mdlib/tests/leapfrog.cpp, refdata/WithParameters_LeapFrogTest_SimpleIntegration_*.xml",
           "initial_state": "x_i = (i % 21, 6.5 - (i % 13), 0), v_i = v0, f_i = f0, 1/m_i = 1/(1 + i % 100)",
           "cases": cases}
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "leapfrog_golden.json")
    with open(path, "w") as f:
        json.dump(out, f)
    print(f"wrote {path}: {len(cases)} cases")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <GROMACS source root of the reference>")
    main(sys.argv[1])
