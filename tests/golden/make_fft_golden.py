"""Regenerate tests/golden/fft_golden.json from the reference's own 3D FFT unit test.

Reads, as text, the input array of the reference's FFT tests (`inputdata` in
src/gromacs/fft/tests/fft.cpp) and the reference output of its 3D real test
(FFFTest3D.Real5_6_9: src/gromacs/fft/tests/refdata/FFFTest3D_Real5_6_9.xml):

* forward: the real grid 5 x 6 x 9, stored with rows padded to 10 (the test copies
  the first 300 input values over the padded grid), transformed real -> complex;
  the reference lists the 5 x 6 x 5 half-complex result in its own transposed
  order, which this script identifies against numpy's rfftn and stores as
  [x][y][kz] (the engine's layout);
* backward: the first 300 input values as 150 complex numbers in the reference's
  transposed order, transformed complex -> real, unnormalised; the 30 rows of 9.

Both directions are checked against numpy (forward exactly as rfftn, backward as
irfftn times the number of points, which ignores the imaginary parts that a
Hermitian spectrum would not have).  Run it where the reference tree is available:

    python tests/golden/make_fft_golden.py /path/to/gromacs-source
"""
from __future__ import annotations

import itertools
import json
import os
import sys
import xml.etree.ElementTree as ET

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from make_pme_golden import _block, _floats  # noqa: E402

N = (5, 6, 9)


def _sequence(root, name):
    for seq in root.iter("Sequence"):
        if seq.get("Name") == name:
            return [float(r.text) for r in seq.findall("Real")]
    raise KeyError(name)


def main(src_root: str) -> None:
    tests = os.path.join(src_root, "src", "gromacs", "fft", "tests")
    text = open(os.path.join(tests, "fft.cpp")).read()
    data = _floats(_block(text, "const double inputdata[]"))
    root = ET.parse(os.path.join(tests, "refdata", "FFFTest3D_Real5_6_9.xml")).getroot()
    nzc = N[2] // 2 + 1
    size = N[0] * N[1] * nzc  # complex points (150)
    inp = np.array(data[: 2 * size])

    # forward: the padded real grid [5][6][10], z < 9 used
    x = inp.reshape(N[0], N[1], 2 * nzc)[:, :, : N[2]]
    want = np.fft.rfftn(x)  # [x][y][kz]
    fwd = np.array(_sequence(root, "forward")).reshape(-1, 2)
    fwd = fwd[:, 0] + 1j * fwd[:, 1]
    perm = None
    for p in itertools.permutations(range(3)):
        shape = [want.shape[a] for a in p]
        cand = fwd.reshape(shape).transpose(np.argsort(p))
        if np.allclose(cand, want, rtol=1e-9, atol=1e-9):
            perm = p
            break
    assert perm is not None, "no axis order of the reference output matches rfftn"
    shape = [want.shape[a] for a in perm]

    # backward: the input as complex numbers in the same transposed order
    cin = (inp[0::2] + 1j * inp[1::2]).reshape(shape).transpose(np.argsort(perm))  # [x][y][kz]
    bwd_rows = [_sequence(root, f"backward {i}") for i in range(N[0] * N[1])]
    bwd = np.array(bwd_rows).reshape(N)
    ref_np = np.fft.irfftn(cin, s=N, axes=(0, 1, 2)) * np.prod(N)
    assert np.allclose(bwd, ref_np, rtol=1e-9, atol=1e-9), np.abs(bwd - ref_np).max()

    out = {
        "source": "src/gromacs/fft/tests/fft.cpp (inputdata), refdata/FFFTest3D_Real5_6_9.xml",
        "grid": list(N),
        "reference_complex_axis_order": [["x", "y", "kz"][a] for a in perm],
        "forward_input": x.reshape(-1).tolist(),
        "forward_output": np.stack([want.real, want.imag], -1).reshape(-1).tolist(),
        "backward_input": np.stack([cin.real, cin.imag], -1).reshape(-1).tolist(),
        "backward_output": bwd.reshape(-1).tolist(),
    }
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "fft_golden.json")
    with open(path, "w") as f:
        json.dump(out, f)
    print(f"wrote {path}: reference complex order {out['reference_complex_axis_order']}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <GROMACS source root of the reference>")
    main(sys.argv[1])
