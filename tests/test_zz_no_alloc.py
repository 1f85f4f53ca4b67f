"""nbx_compute_noalloc: the force evaluation for callers that may not allocate.

Some callers cannot call cudaMalloc -- an engine that owns every device
allocation through its own memory pool, or code running where allocation is
not allowed.  nbx_compute_noalloc evaluates forces, energies and the virial on
a pair list the caller already holds and keeps its scratch in a fixed device
array inside the library instead of allocating.  This file is named so that
pytest collects it last; it checks that entry point, through the C ABI, against
the allocating device path (nbx_compute) on two calls in a row, with the same
tolerances as the other parity tests, for Ewald (with and without the potential
shift), reaction field and plain cut-off Coulomb, and for forces only, forces +
energies and forces + energies + virial; at the largest type count the kernels
accept; and with a bounded device-side wait that gives up (the outputs become
NaN and nbx_noalloc_status reports the timeout).
"""
import ctypes as C

import numpy as np
import pytest

from gmxapi_gb300 import _lib, nblib, systems
from tests.helpers import rel_rms

pytestmark = pytest.mark.gpu

FORCE_RTOL = 1e-5
ENERGY_RTOL = {nblib.CoulombType.Pme: 1e-6, nblib.CoulombType.ReactionField: 5e-6, nblib.CoulombType.Cutoff: 5e-6}


def _device_inputs(calc, s, dev, opts):
    """The handle's atom data and list in the exported nbnxm layouts, as device tensors, and the
    nbx_noalloc_args that point at them."""
    import torch

    g = calc.grid()
    pl = calc.pairlist()
    ai = g["atom_indices"]
    types = np.where(ai >= 0, s.type[np.maximum(ai, 0)], s.ntypes).astype(np.int32)
    nt1 = s.ntypes + 1
    nbfp = np.zeros((nt1, nt1, 2), np.float32)
    nbfp[: s.ntypes, : s.ntypes] = s.nbfp.reshape(s.ntypes, s.ntypes, 2)

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
    a.coulomb = int(opts.coulomb_type)
    a.rcoulomb = float(opts.rcoulomb)
    a.rlist = float(opts.pairlist_cutoff)
    a.ewald_rtol, a.epsilon_rf, a.use_ewald_shift = float(opts.ewald_rtol), float(opts.epsilon_rf), int(
        opts.use_ewald_shift)
    return a, t, g


def _run_noalloc(a, n, dev, energies, virial):
    import torch

    f = torch.full((n * 3,), float("nan"), dtype=torch.float32, device=dev)
    e = torch.zeros(2, dtype=torch.float64, device=dev) if energies else None
    vir = torch.zeros(9, dtype=torch.float64, device=dev) if virial else None
    stream = torch.cuda.current_stream(dev)
    code = _lib.load().nbx_compute_noalloc(C.byref(a), C.c_void_p(f.data_ptr()),
                                           C.c_void_p(e.data_ptr()) if e is not None else None,
                                           C.c_void_p(vir.data_ptr()) if vir is not None else None,
                                           C.c_void_p(stream.cuda_stream))
    assert code == 0, _lib.STATUS_NAMES.get(code, code)
    status = _lib.load().nbx_noalloc_status(C.c_void_p(stream.cuda_stream))
    return (status, f.cpu().numpy().reshape(-1, 3), None if e is None else e.cpu().numpy(),
            None if vir is None else vir.cpu().numpy().reshape(3, 3))


def _check_against_allocating_path(s, opts, outputs):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    calc = nblib.ForceCalculator(s, opts)
    f_ref = calc.compute(s.x).copy()
    e_ref = calc.energies.copy()
    v_ref = calc.virial.copy()
    a, keep, g = _device_inputs(calc, s, dev, opts)
    calc.close()
    want_e = outputs in ("energies", "energies+virial")
    want_v = outputs == "energies+virial"
    xin = g["xq"][g["cells"], :3].astype(np.float64)
    vscale = np.sqrt(np.sum((xin**2).sum(1) * (f_ref.astype(np.float64) ** 2).sum(1)))
    for call in range(2):
        status, fn, en, vn = _run_noalloc(a, s.n, dev, want_e, want_v)
        assert status == 0, _lib.STATUS_NAMES.get(status, status)
        assert np.isfinite(fn).all()
        assert rel_rms(fn, f_ref) <= FORCE_RTOL, call
        if want_e:
            tol = ENERGY_RTOL[opts.coulomb_type]
            assert np.all(np.abs(en - e_ref) <= tol * np.abs(e_ref)), (call, en, e_ref)
        if want_v:
            assert np.abs(vn - v_ref).max() <= FORCE_RTOL * vscale, call


_OUTPUTS = ["forces", "energies", "energies+virial"]
_CASES = ([(nblib.CoulombType.Pme, False, 1.0, o) for o in _OUTPUTS]
          + [(nblib.CoulombType.Pme, True, 1.0, o) for o in _OUTPUTS]
          + [(nblib.CoulombType.ReactionField, False, 1.0, o) for o in _OUTPUTS]
          + [(nblib.CoulombType.Cutoff, False, 1.0, o) for o in _OUTPUTS]
          # reaction field with eps_rf = 78: forces only.  The Coulomb energy of this box is then a
          # residual of ~2e-5 of the summed pair magnitudes, and float pair energies (the
          # reference's are single precision too) leave ~4e-5 relative noise on it in either kernel
          + [(nblib.CoulombType.ReactionField, False, 78.0, "forces")])


@pytest.mark.parametrize("coulomb,shift,eps_rf,outputs", _CASES)
def test_noalloc_matches_allocating_path_twice(coulomb, shift, eps_rf, outputs):
    s = systems.spc_water(1000, 3.104, seed=21)
    opts = nblib.NBKernelOptions(coulomb_type=coulomb, pairlist_cutoff=1.0, rcoulomb=0.9,
                                 compute_virial_and_energy=True, use_ewald_shift=shift, epsilon_rf=eps_rf)
    _check_against_allocating_path(s, opts, outputs)


def test_noalloc_at_the_largest_type_count():
    """47 real types + the filler type: the type table and the per-warp stages need more than the
    default 48 KB of shared memory, which the kernels opt in to."""
    s = systems.lj_liquid(n=3000, ntypes=47, seed=9)
    opts = nblib.NBKernelOptions(coulomb_type=nblib.CoulombType.Pme, pairlist_cutoff=1.0, rcoulomb=0.9,
                                 compute_virial_and_energy=True)
    _check_against_allocating_path(s, opts, "energies+virial")


def test_noalloc_reports_a_timed_out_wait():
    """The stage barriers wait for bytes that never arrive (test hook): the bounded waits give up,
    the outputs are NaN and the status read-out says NBX_ERR_TIMEOUT; the next call is clean."""
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    s = systems.spc_water(300, 2.08, seed=3)
    opts = nblib.NBKernelOptions(coulomb_type=nblib.CoulombType.Pme, pairlist_cutoff=1.0, rcoulomb=0.9,
                                 compute_virial_and_energy=True)
    calc = nblib.ForceCalculator(s, opts)
    f_ref = calc.compute(s.x).copy()
    a, keep, _ = _device_inputs(calc, s, dev, opts)
    calc.close()
    L = _lib.load()
    L.nbx_noalloc_set_wait_test(1)
    try:
        status, fn, en, vn = _run_noalloc(a, s.n, dev, True, True)
    finally:
        L.nbx_noalloc_set_wait_test(0)
    assert status == 5, _lib.STATUS_NAMES.get(status, status)  # NBX_ERR_TIMEOUT
    assert np.isnan(fn).all() and np.isnan(en).all() and np.isnan(vn).all()
    status, fn, en, vn = _run_noalloc(a, s.n, dev, True, True)
    assert status == 0
    assert rel_rms(fn, f_ref) <= FORCE_RTOL


def test_noalloc_rejects_too_many_slots():
    from gmxapi_gb300 import _lib as lib

    a = lib.nbx_noalloc_args()
    a.num_atoms, a.num_slots, a.num_sci, a.num_types = 10, 65536 + 64, 1, 1
    a.xq = a.types = a.nbfp = a.cells = a.sci = a.cj4 = a.excl = 8  # never dereferenced
    a.rcoulomb, a.rlist = 0.9, 1.0
    code = lib.load().nbx_compute_noalloc(C.byref(a), C.c_void_p(8), None, None, None)
    assert code == 3  # NBX_ERR_LIST_OVERFLOW, before any device work


@pytest.mark.parametrize("num_atoms,num_slots", [(200, 128), (100, 130)])
def test_noalloc_rejects_inconsistent_sizes(num_atoms, num_slots):
    from gmxapi_gb300 import _lib as lib

    a = lib.nbx_noalloc_args()
    a.num_atoms, a.num_slots, a.num_sci, a.num_types = num_atoms, num_slots, 1, 1
    a.xq = a.types = a.nbfp = a.cells = a.sci = a.cj4 = a.excl = 8  # never dereferenced
    a.rcoulomb, a.rlist = 0.9, 1.0
    code = lib.load().nbx_compute_noalloc(C.byref(a), C.c_void_p(8), None, None, None)
    assert code == 1  # NBX_ERR_INVALID_INPUT, before any device work
