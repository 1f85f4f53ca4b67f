"""Regenerate tests/golden/pme_golden.json from the reference's own PME unit tests.

Reads, as text, the inputs of the reference's PME tests (boxes, grid sizes,
coordinates, charges, sparse grids, spline data; src/gromacs/ewald/tests/
pmesplinespreadtest.cpp, pmesolvetest.cpp, pmegathertest.cpp, pmebsplinetest.cpp)
and their reference outputs (src/gromacs/ewald/tests/refdata/*.xml), keeping the
cases this engine covers: the rectangular box, pme_order 4, the Coulomb solver.
The refdata file index of a case is its position in googletest's Combine()
product (last parameter fastest).  Run it where the reference tree is available:

    python tests/golden/make_pme_golden.py /path/to/gromacs-source
"""
from __future__ import annotations

import json
import os
import re
import sys
import xml.etree.ElementTree as ET

_NUM = r"[-+]?(?:\d+\.?\d*|\.\d+)(?:[eE][-+]?\d+)?"


def _block(text: str, name: str) -> str:
    """The initializer text of the C++ variable `name` (up to the closing '};')."""
    i = text.index(name)
    j = text.index("{", i)
    depth = 0
    for k in range(j, len(text)):
        if text[k] == "{":
            depth += 1
        elif text[k] == "}":
            depth -= 1
            if depth == 0:
                return text[j:k + 1]
    raise ValueError(name)


def _floats(block: str) -> list[float]:
    block = re.sub(r"//[^\n]*", "", block)
    return [float(v.rstrip("F")) for v in re.findall(_NUM + r"F?", block)]


def _triples(block: str, conv=float) -> list[list]:
    block = re.sub(r"//[^\n]*", "", block)
    out = []
    for inner in re.findall(r"\{([^{}]*)\}", block):
        vals = re.findall(_NUM, inner)
        if len(vals) == 3:
            out.append([conv(v) for v in vals])
    return out


def _boxes(text: str) -> list[list[float]]:
    blk = _block(text, "c_sampleBoxes")
    mats = re.findall(r"Matrix3x3\{\s*\{([^{}]*)\}\s*\}", blk)
    return [[float(v.rstrip("F")) for v in re.findall(_NUM + r"F?", m)] for m in mats]


def _sparse(text: str, name: str, complex_values: bool):
    blk = re.sub(r"//[^\n]*", "", _block(text, name))
    grids = []
    for g in re.findall(r"Sparse\w+GridValuesInput\{(.*?)\n\s*\}", blk, flags=re.S):
        entries = []
        if complex_values:
            pat = r"IVec\{\s*(\d+),\s*(\d+),\s*(\d+)\s*\},\s*t_complex\{\s*(" + _NUM + r")F?,\s*(" + _NUM + r")F?\s*\}"
            for m in re.findall(pat, g):
                entries.append([[int(m[0]), int(m[1]), int(m[2])], [float(m[3]), float(m[4])]])
        else:
            pat = r"IVec\{\s*(\d+),\s*(\d+),\s*(\d+)\s*\},\s*(" + _NUM + r")F?\s*\}"
            for m in re.findall(pat, g):
                entries.append([[int(m[0]), int(m[1]), int(m[2])], float(m[3])])
        grids.append(entries)
    return grids


def _root(path):
    return ET.parse(path).getroot()


def _seq_reals(elem) -> list[float]:
    return [float(r.text) for r in elem.findall("Real")]


def _cells(elem) -> dict:
    return {r.get("Name"): float(r.text) for r in elem.findall("Real")}


def main(ref_root: str) -> None:
    tdir = os.path.join(ref_root, "src", "gromacs", "ewald", "tests")
    rdir = os.path.join(tdir, "refdata")
    out = {"source": "src/gromacs/ewald/tests (*.cpp inputs, refdata/*.xml outputs)"}

    # ---- spline moduli: Combine(grid sizes {64,32,64},{57,84,29}; orders 3..8; PME/P3M) ----
    moduli = []
    for gi, grid in enumerate([[64, 32, 64], [57, 84, 29]]):
        index = (gi * 6 + (4 - 3)) * 2 + 0  # order 4, plain PME moduli
        root = _root(os.path.join(rdir, f"SaneInput1_PmeBSplineModuliCorrectnessTest_ReproducesValues_{index}.xml"))
        seqs = {s.get("Name"): _seq_reals(s) for s in root.findall("Sequence")}
        moduli.append({"grid": grid, "file_index": index, "x": seqs["X"], "y": seqs["Y"], "z": seqs["Z"]})
    out["moduli"] = moduli

    # ---- spline + spread: Combine(boxes(2), orders 3..5, grid sizes(2), coordinates, charges) ----
    text = open(os.path.join(tdir, "pmesplinespreadtest.cpp")).read()
    boxes = _boxes(text)
    grids = _triples(_block(text, "c_sampleGridSizes"), int)
    charges = _floats(_block(text, "c_sampleChargesFull"))
    coords = _triples(_block(text, "c_sampleCoordinatesFull"))
    subsets = {"SaneInput1": (0, 1), "SaneInput2": (1, 3), "SaneInput13": (3, 16)}
    spread = []
    for name, (a, b) in subsets.items():
        for gi, grid in enumerate(grids):
            index = (0 * 3 + (4 - 3)) * 2 + gi  # rectangular box 0, order 4
            root = _root(os.path.join(rdir, f"{name}_PmeSplineAndSpreadTest_ReproducesOutputs_{index}.xml"))
            spl = {s.get("Name"): {q.get("Name"): _seq_reals(q) for q in s.findall("Sequence")}
                   for s in root.findall("Splines")}
            idx_seq = [s for s in root.findall("Sequence") if s.get("Name") == "Gridline indices"][0]
            idx = [[int(v.find(f"Int[@Name='{c}']").text) for c in "XYZ"] for v in idx_seq.findall("Vector")]
            nz = root.find("NonZeroGridValues")
            spread.append({
                "case": name, "file_index": index, "box": [boxes[0][0], boxes[0][4], boxes[0][8]], "grid": grid,
                "x": coords[a:b], "q": charges[a:b],
                "theta": [spl["Values"][c] for c in "XYZ"], "dtheta": [spl["Derivatives"][c] for c in "XYZ"],
                "idx": idx, "grid_values": _cells(nz),
            })
    out["spline_spread"] = spread

    # ---- solve: Combine(boxes, grid sizes, grids, eps_r, beta_q, beta_lj[, method]) ----
    text = open(os.path.join(tdir, "pmesolvetest.cpp")).read()
    sboxes = _boxes(text)
    sgrids = _triples(_block(text, "c_sampleGridSizes"), int)
    cgrids = _sparse(text, "c_sampleGrids", True)
    solve = []
    # (prefix, epsilon_r, beta_q, number of methods in the product)
    for prefix, eps, beta, nmeth in (("SaneInput", 1.2, 2.0, 2), ("DifferentEwaldCoeffQ", 1.2, 0.4, 1),
                                     ("DifferentEpsilonR", 1.9, 2.0, 2)):
        for gi, grid in enumerate(sgrids):
            for vi, vals in enumerate(cgrids):
                index = ((0 * 2 + gi) * 2 + vi) * nmeth + 0  # box 0, Coulomb
                root = _root(os.path.join(rdir, f"{prefix}_PmeSolveTest_ReproducesOutputs_{index}.xml"))
                energy = float(root.find("Real[@Name='Energy']").text)
                vir = _cells(root.find("Matrix[@Name='Virial']"))
                solve.append({
                    "case": prefix, "file_index": index, "box": [sboxes[0][0], sboxes[0][4], sboxes[0][8]],
                    "grid": grid, "epsilon_r": eps, "beta": beta, "input": vals,
                    "output": _cells(root.find("NonZeroGridValues")), "energy": energy, "virial": vir,
                })
    out["solve"] = solve

    # the Lennard-Jones (geometric) solver on the same inputs: method index 1 of SaneInput and
    # DifferentEpsilonR (beta_lj 0.7), every case of DifferentEwaldCoeffLJ (beta_lj 2.35)
    solve_lj = []
    for prefix, beta_lj, nmeth, meth in (("SaneInput", 0.7, 2, 1), ("DifferentEwaldCoeffLJ", 2.35, 1, 0),
                                         ("DifferentEpsilonR", 0.7, 2, 1)):
        for gi, grid in enumerate(sgrids):
            for vi, vals in enumerate(cgrids):
                index = ((0 * 2 + gi) * 2 + vi) * nmeth + meth  # box 0
                root = _root(os.path.join(rdir, f"{prefix}_PmeSolveTest_ReproducesOutputs_{index}.xml"))
                energy = float(root.find("Real[@Name='Energy']").text)
                vir = _cells(root.find("Matrix[@Name='Virial']"))
                solve_lj.append({
                    "case": prefix, "file_index": index, "box": [sboxes[0][0], sboxes[0][4], sboxes[0][8]],
                    "grid": grid, "beta_lj": beta_lj, "input": vals,
                    "output": _cells(root.find("NonZeroGridValues")), "energy": energy, "virial": vir,
                })
    out["solve_lj"] = solve_lj

    # ---- gather: Combine(boxes, orders 3..5, grid sizes, grids, atom counts 1, 2, 13) ----
    text = open(os.path.join(tdir, "pmegathertest.cpp")).read()
    gboxes = _boxes(text)
    ggrids = _triples(_block(text, "c_sampleGridSizes"), int)
    gcharges = _floats(_block(text, "c_sampleChargesFull"))
    gidx = _triples(_block(text, "c_sampleGridLineIndicesFull"), int)
    gvals = _floats(_block(text, "c_sampleSplineValuesFull"))
    gders = _floats(_block(text, "c_sampleSplineDerivativesFull"))
    rgrids = _sparse(text, "c_sampleGrids", False)
    gather = []
    for gi, grid in enumerate(ggrids):
        for vi, vals in enumerate(rgrids):
            start = 0
            for ci, count in enumerate((1, 2, 13)):
                index = (((0 * 3 + (4 - 3)) * 2 + gi) * 2 + vi) * 3 + ci
                root = _root(os.path.join(rdir, f"SaneInput_PmeGatherTest_ReproducesOutputs_{index}.xml"))
                seq = [s for s in root.findall("Sequence") if s.get("Name") == "Forces"][0]
                forces = [[float(v.find(f"Real[@Name='{c}']").text) for c in "XYZ"] for v in seq.findall("Vector")]
                dim = count * 4
                gather.append({
                    "file_index": index, "box": [gboxes[0][0], gboxes[0][4], gboxes[0][8]], "grid": grid,
                    "grid_values": vals, "idx": gidx[start:start + count], "q": gcharges[start:start + count],
                    "theta": [gvals[d * dim:(d + 1) * dim] for d in range(3)],
                    "dtheta": [gders[d * dim:(d + 1) * dim] for d in range(3)],
                    "forces": forces,
                })
                start += count
    out["gather"] = gather

    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "pme_golden.json")
    with open(dst, "w") as fh:
        json.dump(out, fh, indent=0, separators=(",", ":"))
    print(dst, os.path.getsize(dst), "bytes")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <GROMACS source root of the reference>")
    main(sys.argv[1])
