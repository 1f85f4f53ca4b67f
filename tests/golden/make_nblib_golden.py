"""Regenerate tests/golden/nblib_golden.json from the reference's own nblib tests.

Reads, as text, the two golden force vectors of the reference
(api/nblib/tests/refdata/NBlibTest_ArgonForcesAreCorrect.xml and
NBlibTest_SpcMethanolForcesAreCorrect.xml) and the systems those tests build
(api/nblib/tests/testsystems.cpp: coordinates, box, C6/C12 library, charges,
exclusions; api/nblib/tests/nbkernelsystem.cpp:69-85,187-203: SimdNo,
CoulombType::Cutoff, default pairlistCutoff 1.0).  Run it where the
reference tree is available:

    python tests/golden/make_nblib_golden.py /path/to/gromacs-source
"""
from __future__ import annotations

import json
import os
import re
import sys
import xml.etree.ElementTree as ET


def _block(text: str, start_marker: str, field: str) -> str:
    i = text.index(start_marker)
    j = text.index(field, i)
    k = text.index("};", j)
    return text[j:k]


def _vectors(block: str) -> list[list[float]]:
    return [[float(a), float(b), float(c)] for a, b, c in
            re.findall(r"\{\s*([-0-9.eE+]+),\s*([-0-9.eE+]+),\s*([-0-9.eE+]+)\s*\}", block)]


def _xml_forces(path: str) -> list[list[float]]:
    root = ET.parse(path).getroot()
    vals = [float(r.text) for r in root.iter("Real")]
    return [vals[i:i + 3] for i in range(0, len(vals), 3)]


def main(ref_root: str) -> None:
    tdir = os.path.join(ref_root, "api", "nblib", "tests")
    text = open(os.path.join(tdir, "testsystems.cpp")).read()
    c6 = dict(re.findall(r'c6_\[(\w+)\.name\(\)\]\s*=\s*([-0-9.eE+]+);', text))
    c12 = dict(re.findall(r'c12_\[(\w+)\.name\(\)\]\s*=\s*([-0-9.eE+]+);', text))
    charges = dict(re.findall(r'\{\s*"(\w+)",\s*Charge\(([-+0-9.eE]+)\)\s*\}', text))
    argon_box = float(re.search(r"ArgonSimulationStateBuilder::ArgonSimulationStateBuilder\(\) :\s*box_\(([0-9.]+)\)", text).group(1))
    spc_box = float(re.search(r"SpcMethanolSimulationStateBuilder::SpcMethanolSimulationStateBuilder\(\) :\s*box_\(([0-9.]+)\)", text).group(1))
    argon_x = _vectors(_block(text, "ArgonSimulationStateBuilder::ArgonSimulationStateBuilder", "coordinates_"))
    spc_x = _vectors(_block(text, "SpcMethanolSimulationStateBuilder::SpcMethanolSimulationStateBuilder", "coordinates_"))
    ref = os.path.join(tdir, "refdata")
    out = {
        "source": "api/nblib/tests (testsystems.cpp, nbkernelsystem.cpp, refdata/*.xml)",
        "options": {"coulomb": "Cutoff", "pairlistCutoff": 1.0, "simd": "SimdNo"},
        "argon": {
            "box": argon_box,
            "x": argon_x,
            # one type, Ar; no charges; only self exclusions
            "type_names": ["Ar"],
            "c6": [float(c6["Ar"])],
            "c12": [float(c12["Ar"])],
            "types": [0] * len(argon_x),
            "q": [0.0] * len(argon_x),
            "molecules": [[i] for i in range(len(argon_x))],
            "forces": _xml_forces(os.path.join(ref, "NBlibTest_ArgonForcesAreCorrect.xml")),
        },
        "spc_methanol": {
            "box": spc_box,
            "x": spc_x,
            # atom order: Me1 (CMet), O2 (OMet), H3 (H), Ow, Hw1 (H), Hw2 (H)
            "type_names": ["Ow", "H", "OMet", "CMet"],
            "c6": [float(c6[k]) for k in ("Ow", "H", "OMet", "CMet")],
            "c12": [float(c12[k]) for k in ("Ow", "H", "OMet", "CMet")],
            "types": [3, 2, 1, 0, 1, 1],
            "q": [float(charges["CMet"]), float(charges["OMet"]), float(charges["HMet"]),
                  float(charges["Ow"]), float(charges["Hw"]), float(charges["Hw"])],
            "molecules": [[0, 1, 2], [3, 4, 5]],
            "forces": _xml_forces(os.path.join(ref, "NBlibTest_SpcMethanolForcesAreCorrect.xml")),
        },
    }
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "nblib_golden.json")
    with open(dst, "w") as fh:
        json.dump(out, fh, indent=1)
    print("wrote", dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <GROMACS source root of the reference>")
    main(sys.argv[1])
