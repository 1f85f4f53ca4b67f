"""nblib-style façade over the GB300 engine (Python side).

Mirrors the reference's user interface for this path
(api/nblib/forcecalculator.h:75-109, kerneloptions.h:56-112):
``ForceCalculator(system, options).compute(x, forces)`` and
``updatePairList(x)``, with the same argument meaning (forces are
overwritten; coordinates are wrapped into the box once at construction like
SimulationState) and the same error behaviour (invalid input raises).  The
options add the pair-list parameters nblib keeps internal (separate rlist,
inner radius and dynamic-pruning interval).
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import enum

import numpy as np

from . import _lib


class CoulombType(enum.IntEnum):
    Pme = 0
    Cutoff = 1
    ReactionField = 2


class VdwModifier(enum.IntEnum):
    PotShift = 0
    ForceSwitch = 1
    PotSwitch = 2
    NoModifier = 3
    #: LJ-PME real space (vdwtype PME, geometric grid) with the potential shift
    LjPme = 4


class InputException(ValueError):
    """Raised for invalid systems or options (nblib::InputException)."""


def check(code: int, handle=None):
    """NBX_ERR_INVALID_INPUT as InputException (like nblib), other failures as NbxError."""
    if code == _lib.NBX_ERR_INVALID_INPUT:
        msg = _lib.load().nbx_last_error(handle)
        raise InputException(msg.decode() if msg else "invalid input")
    _lib.check(code, handle)


@dataclasses.dataclass
class NBKernelOptions:
    coulomb_type: CoulombType = CoulombType.Pme
    #: nblib's single cut-off: rc = rvdw = rlist (api/nblib/gmxsetup.cpp:230,242)
    pairlist_cutoff: float = 1.0
    compute_virial_and_energy: bool = False
    #: Coulomb/LJ cut-off when different from the list radius
    rcoulomb: float | None = None
    #: inner list radius for dynamic pruning (None: no separate inner list)
    rlist_inner: float | None = None
    nstlist: int = 10
    nstlist_prune: int = 0
    ewald_rtol: float = 1e-5
    epsilon_rf: float = 1.0
    use_ewald_shift: bool = False
    #: LJ modifier (mdp vdw-modifier): potential shift (nblib), force switch, potential switch, none
    vdw_modifier: "VdwModifier" = None
    #: switching distance for the switch modifiers (nm)
    rvdw_switch: float = 0.0
    #: LJ-PME (vdw_modifier LJPME): erfc-like tolerance of the LJ Ewald coefficient at rc
    ewald_rtol_lj: float = 1e-3

    def to_c(self) -> _lib.nbx_options:
        o = _lib.nbx_options()
        _lib.load().nbx_default_options(C.byref(o))
        o.coulomb = int(self.coulomb_type)
        o.rlist = float(self.pairlist_cutoff)
        o.rcoulomb = float(self.rcoulomb if self.rcoulomb is not None else self.pairlist_cutoff)
        o.rlist_inner = float(self.rlist_inner) if self.rlist_inner is not None else 0.0
        o.ewald_rtol = float(self.ewald_rtol)
        o.epsilon_rf = float(self.epsilon_rf)
        o.use_ewald_shift = int(bool(self.use_ewald_shift))
        o.nstlist = int(self.nstlist)
        o.nstlist_prune = int(self.nstlist_prune)
        o.compute_energy = int(bool(self.compute_virial_and_energy))
        o.vdw_modifier = int(self.vdw_modifier if self.vdw_modifier is not None else VdwModifier.PotShift)
        o.rvdw_switch = float(self.rvdw_switch)
        o.ewald_rtol_lj = float(self.ewald_rtol_lj)
        return o


def _fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _iptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


class ForceCalculator:
    """nblib::ForceCalculator on one GB300 GPU."""

    def __init__(self, system, options: NBKernelOptions | None = None, device: int = 0):
        self.options = options or NBKernelOptions()
        self.system = system
        self.n = system.n
        L = _lib.load()
        self._x = np.ascontiguousarray(system.x, np.float32).reshape(-1)
        self._q = np.ascontiguousarray(system.q, np.float32)
        self._t = np.ascontiguousarray(system.type, np.int32)
        self._nbfp = np.ascontiguousarray(system.nbfp, np.float32)
        self._ei = np.ascontiguousarray(system.excl_index, np.int32)
        el = system.excl_list if len(system.excl_list) else np.zeros(1, np.int32)
        self._el = np.ascontiguousarray(el, np.int32)
        desc = _lib.nbx_system_desc()
        desc.num_atoms = self.n
        desc.x = _fptr(self._x)
        desc.q = _fptr(self._q)
        desc.type = _iptr(self._t)
        desc.num_types = int(system.ntypes)
        desc.nbfp = _fptr(self._nbfp)
        desc.excl_index = _iptr(self._ei)
        desc.excl_list = _iptr(self._el)
        for d in range(3):
            desc.box[d] = float(system.box[d])
        self._opts = self.options.to_c()
        h = C.c_void_p()
        code = L.nbx_create(C.byref(desc), C.byref(self._opts), device, C.byref(h))
        if code != _lib.NBX_OK:
            msg = L.nbx_last_error(None).decode()
            if code == 1:
                raise InputException(msg)
            raise _lib.NbxError(code, msg)
        self.h = h
        self.energies = np.zeros(2)
        self.virial = np.zeros((3, 3))

    def close(self):
        if getattr(self, "h", None):
            _lib.load().nbx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- nblib interface ----
    def compute(self, x, forces=None, energies: bool | None = None):
        """Forces (N, 3) for coordinates x (N, 3); energies/virial when requested."""
        x = np.ascontiguousarray(x, np.float32).reshape(-1)
        if x.size != 3 * self.n:
            raise InputException("coordinate array has the wrong size")
        out = forces if forces is not None else np.empty((self.n, 3), np.float32)
        if out.dtype != np.float32 or not out.flags.c_contiguous or out.size != 3 * self.n:
            raise InputException("forces must be a contiguous float32 (N, 3) array")
        want = self.options.compute_virial_and_energy if energies is None else energies
        e = np.zeros(2)
        vir = np.zeros(9)
        code = _lib.load().nbx_compute(
            self.h, _fptr(x), _fptr(out),
            e.ctypes.data_as(C.POINTER(C.c_double)) if want else None,
            vir.ctypes.data_as(C.POINTER(C.c_double)) if want else None,
        )
        check(code, self.h)
        if want:
            self.energies = e
            self.virial = vir.reshape(3, 3)
        return out

    def update_pairlist(self, x):
        x = np.ascontiguousarray(x, np.float32).reshape(-1)
        check(_lib.load().nbx_update_pairlist(self.h, _fptr(x)), self.h)

    updatePairList = update_pairlist

    # ---- device-resident interface (raw device pointers) ----
    def search_device(self, x_ptr: int):
        check(_lib.load().nbx_search_device(self.h, C.c_void_p(x_ptr)), self.h)

    def prune_device(self, part: int):
        check(_lib.load().nbx_prune_device(self.h, part), self.h)

    def compute_device(self, x_ptr: int, f_ptr: int, e_ptr: int | None = None, vir_ptr: int | None = None):
        check(_lib.load().nbx_compute_device(self.h, C.c_void_p(x_ptr), C.c_void_p(f_ptr),
                                             C.c_void_p(e_ptr) if e_ptr else None,
                                             C.c_void_p(vir_ptr) if vir_ptr else None), self.h)

    def md_step_device(self, step: int, x_ptr: int, f_ptr: int, e_ptr: int | None = None,
                       vir_ptr: int | None = None):
        check(_lib.load().nbx_md_step_device(self.h, int(step), C.c_void_p(x_ptr), C.c_void_p(f_ptr),
                                             C.c_void_p(e_ptr) if e_ptr else None,
                                             C.c_void_p(vir_ptr) if vir_ptr else None), self.h)

    def md_step(self, step: int, x, forces=None, energies: bool = False):
        """One scheduled step (search / rolling prune / compute) with host arrays."""
        x = np.ascontiguousarray(x, np.float32).reshape(-1)
        out = forces if forces is not None else np.empty((self.n, 3), np.float32)
        e = np.zeros(2)
        vir = np.zeros(9)
        check(_lib.load().nbx_md_step(self.h, int(step), _fptr(x), _fptr(out),
                                      e.ctypes.data_as(C.POINTER(C.c_double)) if energies else None,
                                      vir.ctypes.data_as(C.POINTER(C.c_double)) if energies else None),
              self.h)
        if energies:
            self.energies = e
            self.virial = vir.reshape(3, 3)
        return out

    def set_parameters_device(self, q_ptr: int | None, nbfp_ptr: int | None):
        """New charges ([N] float32) and/or nbfp ([ntypes^2 * 2] float32) from device memory."""
        check(_lib.load().nbx_set_parameters_device(self.h, C.c_void_p(q_ptr) if q_ptr else None,
                                                    C.c_void_p(nbfp_ptr) if nbfp_ptr else None), self.h)

    def backward_device(self, x_ptr: int, gf_ptr: int, ge_ptr: int | None, gx_ptr: int | None,
                        gq_ptr: int | None, gnbfp_ptr: int | None):
        """Adjoint pass over the current list (all arguments are device pointers)."""
        vp = C.c_void_p
        check(_lib.load().nbx_backward_device(self.h, vp(x_ptr), vp(gf_ptr), vp(ge_ptr) if ge_ptr else None,
                                              vp(gx_ptr) if gx_ptr else None, vp(gq_ptr) if gq_ptr else None,
                                              vp(gnbfp_ptr) if gnbfp_ptr else None), self.h)

    def set_timing(self, enable: bool):
        check(_lib.load().nbx_set_timing(self.h, int(bool(enable))), self.h)

    def timings(self, reset: bool = False):
        """(summed force-kernel ms, force-kernel launches, all kernel launches)."""
        ms = C.c_double()
        cnt = (C.c_longlong * 2)()
        check(_lib.load().nbx_get_timings(self.h, C.byref(ms), cnt, int(reset)), self.h)
        return float(ms.value), int(cnt[0]), int(cnt[1])

    def set_force_accumulate(self, enable: bool):
        """Device calls add the nonbonded forces to the force buffer instead of overwriting it."""
        check(_lib.load().nbx_set_force_accumulate(self.h, int(bool(enable))), self.h)

    def set_force_kernel(self, tile: int = 1, stage_depth: int = 2, blocks_per_sm: int = 2):
        """Force-kernel shape: tile 1 = two atom pairs per lane (packed FP32x2), 0 = one pair per
        lane; stage_depth = j-cluster stage buffers per warp (2 or 3); blocks_per_sm = resident
        256-thread blocks per SM (2 or 3)."""
        check(_lib.load().nbx_set_force_kernel(self.h, int(tile), int(stage_depth), int(blocks_per_sm)), self.h)

    def force_kernel(self) -> tuple[int, int, int]:
        t, d, b = C.c_int(), C.c_int(), C.c_int()
        check(_lib.load().nbx_get_force_kernel(self.h, C.byref(t), C.byref(d), C.byref(b)), self.h)
        return t.value, d.value, b.value

    def set_list_balance(self, entries_per_sm: int):
        """Entries per SM below which long list entries are split (0: never); next search."""
        check(_lib.load().nbx_set_list_balance(self.h, int(entries_per_sm)), self.h)

    # ---- free-energy perturbation (nb_free_energy.cpp, dispatched from kerneldispatch.cpp:458-567) ----
    def set_free_energy(self, perturbed, qB, typeB, lambda_coul: float = 0.0, lambda_vdw: float = 0.0,
                        alpha_vdw: float = 0.5, alpha_coul: float = 0.5, sc_power: int = 1,
                        sc_sigma: float = 0.3, sc_sigma_min: float | None = None, x=None):
        """Perturb `perturbed` atoms between their topology state (A) and charges qB / types typeB
        (B); the list is rebuilt at x (default: the coordinates the calculator was built with)."""
        self._fep_p = np.ascontiguousarray(perturbed, np.int32)
        self._fep_q = np.ascontiguousarray(qB, np.float32)
        self._fep_t = np.ascontiguousarray(typeB, np.int32)
        if not (self._fep_p.shape == self._fep_q.shape == self._fep_t.shape):
            raise InputException("perturbed, qB and typeB differ in length")
        d = _lib.nbx_fep_desc()
        d.num_perturbed = int(self._fep_p.shape[0])
        d.perturbed = _iptr(self._fep_p)
        d.qB = _fptr(self._fep_q)
        d.typeB = _iptr(self._fep_t)
        d.lambda_coul = float(lambda_coul)
        d.lambda_vdw = float(lambda_vdw)
        d.alpha_vdw = float(alpha_vdw)
        d.alpha_coul = float(alpha_coul)
        d.lambda_power = int(sc_power)
        d.sigma6_def = float(sc_sigma) ** 6
        d.sigma6_min = float(sc_sigma if sc_sigma_min is None else sc_sigma_min) ** 6
        check(_lib.load().nbx_fep_enable(self.h, C.byref(d)), self.h)
        self.update_pairlist(self._x if x is None else x)

    def set_lambda(self, lambda_coul: float, lambda_vdw: float | None = None):
        lv = lambda_coul if lambda_vdw is None else lambda_vdw
        check(_lib.load().nbx_fep_set_lambda(self.h, float(lambda_coul), float(lv)), self.h)

    def free_energy_terms(self) -> dict:
        """{V_coul, V_lj, dvdl_coul, dvdl_lj} of the perturbed pairs from the last evaluation with energies."""
        out = np.zeros(4)
        check(_lib.load().nbx_fep_get_energies(self.h, out.ctypes.data_as(C.POINTER(C.c_double))), self.h)
        return {"V_coul": out[0], "V_lj": out[1], "dvdl_coul": out[2], "dvdl_lj": out[3]}

    def clear_free_energy(self, x=None):
        check(_lib.load().nbx_fep_disable(self.h), self.h)
        self.update_pairlist(self._x if x is None else x)

    def list_balance(self) -> dict:
        o = np.zeros(4, np.int32)
        check(_lib.load().nbx_get_list_balance(self.h, _iptr(o)), self.h)
        return {"min_ci_balanced": int(o[0]), "nsp_max": int(o[1]), "entries_unsplit": int(o[2]),
                "entries": int(o[3])}

    PHASES = ("force", "grid", "search_count", "search_write", "prune")

    def phase_timings(self, reset: bool = False) -> dict:
        """{phase: (summed ms, event pairs)} for force, grid, search passes and prune."""
        ms = (C.c_double * 5)()
        cnt = (C.c_longlong * 5)()
        check(_lib.load().nbx_get_phase_timings(self.h, ms, cnt, int(reset)), self.h)
        return {p: (float(ms[k]), int(cnt[k])) for k, p in enumerate(self.PHASES)}

    def set_stream(self, stream_ptr: int):
        check(_lib.load().nbx_set_stream(self.h, C.c_void_p(stream_ptr)), self.h)

    def synchronize(self):
        check(_lib.load().nbx_synchronize(self.h), self.h)

    # ---- layout export ----
    def sizes(self) -> dict:
        s = np.zeros(8, np.int32)
        check(_lib.load().nbx_get_sizes(self.h, _iptr(s)), self.h)
        keys = ["num_atoms", "ncx", "ncy", "num_cells", "num_sci", "num_cj4", "num_excl", "npad"]
        return dict(zip(keys, (int(v) for v in s)))

    def grid(self) -> dict:
        s = self.sizes()
        nc, npad = s["num_cells"], s["npad"]
        ncol = s["ncx"] * s["ncy"]
        ai = np.zeros(npad, np.int32)
        cells = np.zeros(self.n, np.int32)
        cxy = np.zeros(ncol + 1, np.int32)
        ncl = np.zeros(nc, np.int32)
        bb = np.zeros(nc * 8 * 6, np.float32)
        bbcz = np.zeros(nc * 2, np.float32)
        xq = np.zeros(npad * 4, np.float32)
        check(_lib.load().nbx_get_grid(self.h, _iptr(ai), _iptr(cells), _iptr(cxy), _iptr(ncl), _fptr(bb),
                                       _fptr(bbcz), _fptr(xq)), self.h)
        return {"atom_indices": ai, "cells": cells, "cxy_ind": cxy, "num_clusters": ncl,
                "bb": bb.reshape(-1, 6), "bbcz": bbcz.reshape(-1, 2), "xq": xq.reshape(-1, 4),
                "ncx": s["ncx"], "ncy": s["ncy"], "ncells": nc, "npad": npad}

    def pairlist(self) -> dict:
        s = self.sizes()
        sci = np.zeros(4 * s["num_sci"], np.int32)
        cj4 = np.zeros(8 * s["num_cj4"], np.int32)
        excl = np.zeros(32 * max(s["num_excl"], 1), np.uint32)
        outer = np.zeros(2 * s["num_cj4"], np.uint32)
        check(_lib.load().nbx_get_pairlist(self.h, _iptr(sci), _iptr(cj4),
                                           excl.ctypes.data_as(C.POINTER(C.c_uint32)),
                                           outer.ctypes.data_as(C.POINTER(C.c_uint32))), self.h)
        return {"sci": sci.reshape(-1, 4), "cj4": cj4.reshape(-1, 8), "excl": excl.reshape(-1, 32),
                "imask_outer": outer.reshape(-1, 2)}

    def pair_count(self) -> int:
        p = (C.c_longlong * 2)()
        check(_lib.load().nbx_get_pair_counts(self.h, p), self.h)
        return int(p[0])


def measure_fp32_peak(device: int = 0) -> float:
    t = C.c_double()
    check(_lib.load().nbx_measure_fp32_peak(device, C.byref(t)))
    return float(t.value)
