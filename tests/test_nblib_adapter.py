"""The C++ nblib adapter (include/nblib_gb300.hpp) over the C ABI.

A small C++ program (tests/cpp/nblib_adapter_driver.cpp) builds a Topology and
SimulationState, constructs nblib_gb300::ForceCalculator, computes forces,
updates the pair list and computes again, like nblib's own integration tests.
On the CPU the program is compiled and its error paths are checked (no device,
bad input); on a GPU its forces are compared with the reference's nblib golden
vectors and with the oracle.
"""
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from gmxapi_gb300 import _lib, systems
from tests.helpers import nblib_golden_system, rel_rms

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "nblib_adapter_driver.cpp")

needs_toolchain = pytest.mark.skipif(shutil.which("g++") is None or (
    shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc")), reason="no C++/CUDA toolchain")


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    if not os.path.exists(_lib.LIB_PATH):
        from gmxapi_gb300 import build

        build.build()
    libdir = os.path.dirname(_lib.LIB_PATH)
    exe = str(tmp_path_factory.mktemp("drv") / "nblib_adapter_driver")
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                    SRC, "-L", libdir, "-lnbnxm_gb300", f"-Wl,-rpath,{libdir}", "-o", exe], check=True)
    return exe


def _run(driver, tmp_path, s, mode, params, coulomb, rc, rlist, energy=True, box=None):
    box = s.box if box is None else box
    inp = tmp_path / "in.bin"
    out = tmp_path / "out.bin"
    with open(inp, "wb") as f:
        f.write(struct.pack("<5i", s.n, s.ntypes, mode, coulomb, int(energy)))
        f.write(struct.pack("<5f", rc, rlist, *[float(b) for b in box]))
        f.write(np.ascontiguousarray(s.x, "<f4").tobytes())
        f.write(np.ascontiguousarray(s.q, "<f4").tobytes())
        f.write(np.ascontiguousarray(s.type, "<i4").tobytes())
        f.write(np.ascontiguousarray(params, "<f4").tobytes())
        f.write(np.ascontiguousarray(s.excl_index, "<i4").tobytes())
        f.write(np.ascontiguousarray(s.excl_list, "<i4").tobytes())
    subprocess.run([driver, str(inp), str(out)], check=True, timeout=300)
    b = out.read_bytes()
    outcome, code, size_check = struct.unpack_from("<3i", b, 0)
    o = 12
    f1 = np.frombuffer(b, "<f4", 3 * s.n, o).reshape(-1, 3)
    o += 12 * s.n
    f2 = np.frombuffer(b, "<f4", 3 * s.n, o).reshape(-1, 3)
    o += 12 * s.n
    e = np.frombuffer(b, "<f8", 2, o)
    o += 16
    vir = np.frombuffer(b, "<f8", 9, o).reshape(3, 3)
    o += 72
    return dict(outcome=outcome, code=code, size_check=size_check, f=f1, f2=f2, e=e, vir=vir,
                msg=b[o:].decode(errors="replace"))


def _golden(key):
    import json

    s, ref = nblib_golden_system(key)
    d = json.load(open(os.path.join(ROOT, "tests", "golden", "nblib_golden.json")))[key]
    params = np.concatenate([np.array(d["c6"], np.float32), np.array(d["c12"], np.float32)])
    return s, ref, params


@needs_toolchain
def test_adapter_without_device_raises_gpu_exception(driver, tmp_path):
    pytest.importorskip("torch")
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    s, _ref, params = _golden("argon")
    r = _run(driver, tmp_path, s, 0, params, 1, 1.0, 1.0)
    assert r["outcome"] == 2 and r["code"] == _lib.NBX_ERR_NO_DEVICE, r["msg"]


@needs_toolchain
def test_adapter_rejects_bad_input_before_the_device(driver, tmp_path):
    s, _ref, params = _golden("argon")
    r = _run(driver, tmp_path, s, 0, params, 1, 1.0, 1.0, box=(-1.0, 1.0, 1.0))
    assert r["outcome"] == 1 and "box" in r["msg"]
    r = _run(driver, tmp_path, s, 3, params, 1, 1.0, 1.0)  # no such combination rule
    assert r["outcome"] == 1 and "Combination rule" in r["msg"]


@pytest.mark.gpu
@pytest.mark.parametrize("key", ["argon", "spc_methanol"])
def test_adapter_reproduces_nblib_golden_forces(driver, tmp_path, key):
    """Cutoff Coulomb, rc = rlist = 1.0, geometric combination from per-type C6/C12."""
    s, ref, params = _golden(key)
    r = _run(driver, tmp_path, s, 0, params, 1, 1.0, 1.0)
    assert r["outcome"] == 0, r["msg"]
    assert rel_rms(r["f"], ref) <= 1e-5
    assert np.abs(r["f"] - ref).max() <= 5e-5 * np.abs(ref).max()
    # the force kernel adds j-forces with atomics: repeat evaluations agree to rounding
    assert rel_rms(r["f2"], r["f"]) <= 1e-6
    assert r["size_check"] == 1


@pytest.mark.gpu
def test_adapter_matches_oracle_on_water(driver, tmp_path):
    """Ewald water (explicit type table): forces, energies and virial against the oracle."""
    from oracle import oracle as O

    s = systems.spc_water(300, 2.08, seed=5)
    o = O.Oracle(s, coulomb=0, rc=0.9, rlist=1.0)
    o.grid()
    o.search()
    o.force(energy=True)
    r = _run(driver, tmp_path, s, 1, s.nbfp, 0, 0.9, 1.0)
    assert r["outcome"] == 0, r["msg"]
    assert rel_rms(r["f"], o.forces()) <= 1e-5
    np.testing.assert_allclose(r["e"], o.energies(), rtol=1e-6)
    assert rel_rms(r["f2"], r["f"]) <= 1e-6
    assert r["size_check"] == 1
