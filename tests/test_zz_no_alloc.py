"""nbx_compute_noalloc: the force evaluation for callers that may not allocate.

Some callers cannot call cudaMalloc -- an engine that owns every device
allocation through its own memory pool, or code running where allocation is
not allowed.  nbx_compute_noalloc evaluates forces, energies and the virial on
a pair list the caller already holds and keeps its scratch in a fixed device
array inside the library instead of allocating.  This file is named so that
pytest collects it last; it checks that entry point, through the C ABI, against
the allocating device path (nbx_compute) on two calls in a row, with the same
tolerances as the other parity tests.
"""
import ctypes as C

import numpy as np
import pytest

from gmxapi_gb300 import _lib, nblib, systems
from tests.helpers import rel_rms

pytestmark = pytest.mark.gpu

FORCE_RTOL = 1e-5
ENERGY_RTOL = 1e-6


def test_noalloc_matches_allocating_path_twice():
    torch = pytest.importorskip("torch")
    s = systems.spc_water(1000, 3.104, seed=21)
    opts = nblib.NBKernelOptions(coulomb_type=nblib.CoulombType.Pme, pairlist_cutoff=1.0, rcoulomb=0.9,
                                 compute_virial_and_energy=True)
    calc = nblib.ForceCalculator(s, opts)
    f_ref = calc.compute(s.x).copy()
    e_ref = calc.energies.copy()
    v_ref = calc.virial.copy()

    # the atom data and list of the handle, in the exported nbnxm layouts
    g = calc.grid()
    pl = calc.pairlist()
    ai = g["atom_indices"]
    types = np.where(ai >= 0, s.type[np.maximum(ai, 0)], s.ntypes).astype(np.int32)
    nt1 = s.ntypes + 1
    nbfp = np.zeros((nt1, nt1, 2), np.float32)
    nbfp[: s.ntypes, : s.ntypes] = s.nbfp.reshape(s.ntypes, s.ntypes, 2)
    dev = torch.device("cuda:0")

    def d(a):
        return torch.from_numpy(np.ascontiguousarray(a)).to(dev)

    t = {
        "xq": d(g["xq"].astype(np.float32)), "types": d(types), "nbfp": d(nbfp.reshape(-1)),
        "cells": d(g["cells"].astype(np.int32)), "sci": d(pl["sci"].astype(np.int32)),
        "cj4": d(pl["cj4"].astype(np.int32)), "excl": d(pl["excl"].view(np.int32)),
        "ei": d(s.excl_index.astype(np.int32)), "el": d(s.excl_list.astype(np.int32)),
    }
    a = _lib.nbx_noalloc_args()
    a.num_atoms = s.n
    a.num_slots = int(g["npad"])
    a.num_sci = int(pl["sci"].shape[0])
    a.num_types = int(s.ntypes)
    a.xq, a.types, a.nbfp = t["xq"].data_ptr(), t["types"].data_ptr(), t["nbfp"].data_ptr()
    a.cells, a.sci, a.cj4, a.excl = (t["cells"].data_ptr(), t["sci"].data_ptr(), t["cj4"].data_ptr(),
                                     t["excl"].data_ptr())
    a.excl_index, a.excl_list = t["ei"].data_ptr(), t["el"].data_ptr()
    for k in range(3):
        a.box[k] = float(s.box[k])
    a.coulomb = int(nblib.CoulombType.Pme)
    a.rcoulomb, a.rlist, a.ewald_rtol, a.epsilon_rf, a.use_ewald_shift = 0.9, 1.0, 1e-5, 1.0, 0

    L = _lib.load()
    stream = torch.cuda.current_stream(dev)
    for call in range(2):
        f = torch.full((s.n * 3,), float("nan"), dtype=torch.float32, device=dev)
        e = torch.zeros(2, dtype=torch.float64, device=dev)
        vir = torch.zeros(9, dtype=torch.float64, device=dev)
        code = L.nbx_compute_noalloc(C.byref(a), C.c_void_p(f.data_ptr()), C.c_void_p(e.data_ptr()),
                                     C.c_void_p(vir.data_ptr()), C.c_void_p(stream.cuda_stream))
        assert code == 0, _lib.STATUS_NAMES.get(code, code)
        torch.cuda.synchronize()
        fn = f.cpu().numpy().reshape(-1, 3)
        assert np.isfinite(fn).all()
        assert rel_rms(fn, f_ref) <= FORCE_RTOL, call
        en = e.cpu().numpy()
        assert np.all(np.abs(en - e_ref) <= ENERGY_RTOL * np.abs(e_ref)), (call, en, e_ref)
        vn = vir.cpu().numpy().reshape(3, 3)
        xin = g["xq"][g["cells"], :3].astype(np.float64)
        scale = np.sqrt(np.sum((xin**2).sum(1) * (f_ref.astype(np.float64) ** 2).sum(1)))
        assert np.abs(vn - v_ref).max() <= FORCE_RTOL * scale, call


def test_noalloc_rejects_too_many_slots():
    from gmxapi_gb300 import _lib as lib

    a = lib.nbx_noalloc_args()
    a.num_atoms, a.num_slots, a.num_sci, a.num_types = 10, 65536 + 64, 1, 1
    a.xq = a.types = a.nbfp = a.cells = a.sci = a.cj4 = a.excl = 8  # never dereferenced
    a.rcoulomb, a.rlist = 0.9, 1.0
    code = lib.load().nbx_compute_noalloc(C.byref(a), C.c_void_p(8), None, None, None)
    assert code == 3  # NBX_ERR_LIST_OVERFLOW, before any device work
