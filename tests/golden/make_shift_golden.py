"""Regenerate tests/golden/shift_golden.json from the reference's PbcTest.CalcShiftsWorks.

Reads, as text, the box of the test (src/gromacs/pbcutil/tests/pbc.cpp: a triclinic box whose
entries make every one of the 45 shift vectors unique) and the reference output of calc_shifts
(src/gromacs/pbcutil/tests/refdata/PbcTest_CalcShiftsWorks.xml): the shift vectors in the
reference's shift-index order, the numbering the pair list's entries carry.  Run it where the
reference tree is available:

    python tests/golden/make_shift_golden.py /path/to/gromacs-source
"""
from __future__ import annotations

import json
import os
import re
import sys
import xml.etree.ElementTree as ET

_NUM = r"[-+]?(?:\d+\.?\d*|\.\d+)(?:[eE][-+]?\d+)?"


def main(src_root: str) -> None:
    tests = os.path.join(src_root, "src", "gromacs", "pbcutil", "tests")
    text = open(os.path.join(tests, "pbc.cpp")).read()
    i = text.index("const matrix box")
    j = text.index(";", i)
    vals = [float(v) for v in re.findall(_NUM, text[i:j])]
    assert len(vals) == 9, vals
    box = [vals[0:3], vals[3:6], vals[6:9]]
    root = ET.parse(os.path.join(tests, "refdata", "PbcTest_CalcShiftsWorks.xml")).getroot()
    shifts = []
    for vec in root.iter("Vector"):
        d = {r.get("Name"): float(r.text) for r in vec.findall("Real")}
        shifts.append([d["X"], d["Y"], d["Z"]])
    assert len(shifts) == 45
    out = {"source": "src/gromacs/pbcutil/tests/pbc.cpp, refdata/PbcTest_CalcShiftsWorks.xml",
           "box": box, "shift_vectors": shifts}
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "shift_golden.json")
    with open(path, "w") as f:
        json.dump(out, f)
    print(f"wrote {path}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <GROMACS source root of the reference>")
    main(sys.argv[1])
