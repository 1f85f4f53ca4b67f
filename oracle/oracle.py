"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Used by tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` as the checker of the CUDA path; the product never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libnbnxm_oracle.so")
_lib = None

COULOMB_EWALD = 0
COULOMB_CUTOFF = 1
COULOMB_RF = 2


def build() -> str:
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        srcs = [os.path.join(_HERE, n) for n in ("nbnxm_oracle.c", "nbnxm_cpu_oracle.c", "nbnxm_oracle.h")]
        if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < max(os.path.getmtime(p) for p in srcs):
            build()
        L = C.CDLL(_LIB_PATH)
        vp = C.c_void_p
        fp = C.POINTER(C.c_float)
        ip = C.POINTER(C.c_int)
        dp = C.POINTER(C.c_double)
        L.orc_create.restype = vp
        L.orc_create.argtypes = [C.c_int, fp, fp, fp, ip, C.c_int, fp, ip, ip, C.c_int,
                                 C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int]
        for name in ("orc_destroy", "orc_grid", "orc_search"):
            getattr(L, name).argtypes = [vp]
            getattr(L, name).restype = None
        L.orc_set_coordinates.argtypes = [vp, fp]
        L.orc_set_x.argtypes = [vp, fp]
        L.orc_prune.argtypes = [vp, C.c_int, C.c_int, C.c_int]
        L.orc_set_vdw_modifier.argtypes = [vp, C.c_int, C.c_float]
        L.orc_balance.argtypes = [vp, C.c_int]
        L.orc_balance.restype = C.c_int
        L.orc_force.argtypes = [vp, C.c_int]
        L.orc_force_entries.argtypes = [vp, C.c_int, C.c_int, C.c_int]
        L.orc_force_entries_mt.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int]
        L.orc_force_entries_mt.restype = C.c_int
        L.orc_forces_original_order.argtypes = [vp, fp]
        L.orc_virial.argtypes = [vp, fp, fp, dp]
        L.orc_energies.argtypes = [vp, dp]
        L.orc_fshift.argtypes = [vp, fp]
        for name in ("orc_beta", "orc_table_scale", "orc_epsfac", "orc_rbb2"):
            getattr(L, name).argtypes = [vp]
            getattr(L, name).restype = C.c_float
        L.orc_table_size.argtypes = [vp]
        L.orc_table_size.restype = C.c_int
        L.orc_table.argtypes = [vp, fp, fp]
        L.orc_grid_dims.argtypes = [vp, ip, fp]
        L.orc_list_sizes.argtypes = [vp, ip]
        for name in ("orc_cxy_ind", "orc_num_clusters", "orc_atom_indices", "orc_cells",
                     "orc_types_grid", "orc_sci", "orc_cj4"):
            getattr(L, name).argtypes = [vp]
            getattr(L, name).restype = ip
        for name in ("orc_xq", "orc_bb", "orc_bbcz", "orc_fnb"):
            getattr(L, name).argtypes = [vp]
            getattr(L, name).restype = fp
        for name in ("orc_excl", "orc_imask_outer"):
            getattr(L, name).argtypes = [vp]
            getattr(L, name).restype = C.POINTER(C.c_uint32)
        L.orc_fp64_allpairs.argtypes = [C.c_int, fp, fp, fp, ip, C.c_int, fp, ip, ip, C.c_int,
                                        C.c_double, C.c_double, C.c_double, C.c_double,
                                        C.c_double, C.c_int, ip, C.c_int, dp, dp, C.c_int, C.c_double,
                                        C.c_double]
        L.orc_one_4pi_eps0.restype = C.c_double
        L.orc_cpu_create.restype = vp
        L.orc_cpu_create.argtypes = [C.c_int, fp, fp, fp, ip, C.c_int, fp, ip, ip, C.c_float, C.c_float,
                                     C.c_float, C.c_float]
        for name in ("orc_cpu_destroy", "orc_cpu_grid", "orc_cpu_search"):
            getattr(L, name).argtypes = [vp]
            getattr(L, name).restype = None
        L.orc_cpu_set_x.argtypes = [vp, fp]
        L.orc_cpu_force.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int]
        L.orc_cpu_force.restype = C.c_int
        L.orc_cpu_sizes.argtypes = [vp, ip]
        L.orc_cpu_list.argtypes = [vp, ip, ip]
        L.orc_cpu_grid_arrays.argtypes = [vp, ip, fp]
        L.orc_cpu_forces.argtypes = [vp, fp]
        L.orc_cpu_energies.argtypes = [vp, dp]
        _lib = L
    return _lib


def _f(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a, a.ctypes.data_as(C.POINTER(C.c_float))


def _i(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(C.POINTER(C.c_int))


def _copy(ptr, n, dtype):
    if n == 0:
        return np.zeros(0, dtype=dtype)
    return np.ctypeslib.as_array(ptr, shape=(n,)).copy().astype(dtype, copy=False)


class Oracle:
    """One system in the oracle: grid, GPU-layout list, prune, force kernel."""

    def __init__(self, system, coulomb=COULOMB_EWALD, rc=0.9, rlist=1.0, rlist_inner=None,
                 ewald_rtol=1e-5, epsilon_rf=1.0, use_ewald_shift=False, vdw_modifier=0, rvdw_switch=0.0):
        L = lib()
        self.system = system
        self._keep = []
        x, xp = _f(system.x)
        box, bp = _f(system.box)
        q, qp = _f(system.q)
        t, tp = _i(system.type)
        nb, nbp = _f(system.nbfp)
        ei, eip = _i(system.excl_index)
        el, elp = _i(system.excl_list if len(system.excl_list) else np.zeros(1, np.int32))
        self._keep += [x, box, q, t, nb, ei, el]
        self.coulomb = coulomb
        self.rc = rc
        self.rlist = rlist
        self.rlist_inner = rlist if rlist_inner is None else rlist_inner
        self.use_ewald_shift = use_ewald_shift
        self.c = L.orc_create(system.n, xp, bp, qp, tp, system.ntypes, nbp, eip, elp, coulomb,
                              rc, rlist, self.rlist_inner, ewald_rtol, epsilon_rf,
                              int(use_ewald_shift))
        if vdw_modifier:
            L.orc_set_vdw_modifier(self.c, int(vdw_modifier), float(rvdw_switch))

    def __del__(self):
        if getattr(self, "c", None):
            lib().orc_destroy(self.c)
            self.c = None

    # -- pipeline --
    def grid(self):
        lib().orc_grid(self.c)

    def search(self):
        lib().orc_search(self.c)

    def balance(self, min_ci_balanced):
        """Split long entries and sort entries by size, as the GPU list does."""
        return int(lib().orc_balance(self.c, int(min_ci_balanced)))

    def set_coordinates(self, x):
        a, p = _f(x)
        lib().orc_set_coordinates(self.c, p)

    def set_x(self, x):
        a, p = _f(x)
        lib().orc_set_x(self.c, p)

    def prune(self, fresh, part=0, nparts=1):
        lib().orc_prune(self.c, int(fresh), part, nparts)

    def force(self, energy=True):
        lib().orc_force(self.c, int(energy))

    def force_entries(self, e0, e1, energy=True):
        lib().orc_force_entries(self.c, int(e0), int(e1), int(energy))

    def force_entries_mt(self, e0, e1, energy=True, threads=1):
        """force_entries over `threads` POSIX threads (multi-core timing baseline)."""
        if lib().orc_force_entries_mt(self.c, int(e0), int(e1), int(energy), int(threads)) != 0:
            raise RuntimeError("threaded oracle kernel failed")

    def forces(self):
        f = np.empty((self.system.n, 3), dtype=np.float32)
        lib().orc_forces_original_order(self.c, f.ctypes.data_as(C.POINTER(C.c_float)))
        return f

    def energies(self):
        e = np.zeros(2, dtype=np.float64)
        lib().orc_energies(self.c, e.ctypes.data_as(C.POINTER(C.c_double)))
        return e  # (Vlj, Vcoul)

    def virial(self, x_inbox, f):
        xa, xp = _f(x_inbox)
        fa, fp_ = _f(f)
        v = np.zeros(9, dtype=np.float64)
        lib().orc_virial(self.c, xp, fp_, v.ctypes.data_as(C.POINTER(C.c_double)))
        return v.reshape(3, 3)

    def fshift(self):
        f = np.zeros(135, dtype=np.float32)
        lib().orc_fshift(self.c, f.ctypes.data_as(C.POINTER(C.c_float)))
        return f.reshape(45, 3)

    # -- setup values --
    @property
    def beta(self):
        return lib().orc_beta(self.c)

    @property
    def epsfac(self):
        return lib().orc_epsfac(self.c)

    @property
    def rbb2(self):
        return lib().orc_rbb2(self.c)

    def table(self):
        n = lib().orc_table_size(self.c)
        F = np.zeros(max(n, 1), np.float32)
        V = np.zeros(max(n, 1), np.float32)
        lib().orc_table(self.c, F.ctypes.data_as(C.POINTER(C.c_float)),
                        V.ctypes.data_as(C.POINTER(C.c_float)))
        return lib().orc_table_scale(self.c), F[:n], V[:n]

    # -- grid / list --
    def grid_arrays(self):
        L = lib()
        dims = np.zeros(6, np.int32)
        cs = np.zeros(4, np.float32)
        L.orc_grid_dims(self.c, dims.ctypes.data_as(C.POINTER(C.c_int)),
                        cs.ctypes.data_as(C.POINTER(C.c_float)))
        ncx, ncy, ncol, ncells, ncl, npad = (int(v) for v in dims)
        return {
            "ncx": ncx, "ncy": ncy, "ncol": ncol, "ncells": ncells, "nclusters_total": ncl,
            "npad": npad, "cell_size": cs[:2].copy(), "inv_cell_size": cs[2:].copy(),
            "cxy_ind": _copy(L.orc_cxy_ind(self.c), ncol + 1, np.int32),
            "num_clusters": _copy(L.orc_num_clusters(self.c), ncells, np.int32),
            "atom_indices": _copy(L.orc_atom_indices(self.c), npad, np.int32),
            "cells": _copy(L.orc_cells(self.c), self.system.n, np.int32),
            "xq": _copy(L.orc_xq(self.c), npad * 4, np.float32).reshape(-1, 4),
            "types": _copy(L.orc_types_grid(self.c), npad, np.int32),
            "bb": _copy(L.orc_bb(self.c), ncells * 8 * 6, np.float32).reshape(-1, 6),
            "bbcz": _copy(L.orc_bbcz(self.c), ncells * 2, np.float32).reshape(-1, 2),
        }

    def pairlist(self):
        L = lib()
        s = np.zeros(3, np.int32)
        L.orc_list_sizes(self.c, s.ctypes.data_as(C.POINTER(C.c_int)))
        nsci, ncj4, nexcl = (int(v) for v in s)
        return {
            "sci": _copy(L.orc_sci(self.c), nsci * 4, np.int32).reshape(-1, 4),
            "cj4": _copy(L.orc_cj4(self.c), ncj4 * 8, np.int32).reshape(-1, 8),
            "excl": _copy(L.orc_excl(self.c), nexcl * 32, np.uint32).reshape(-1, 32),
            "imask_outer": _copy(L.orc_imask_outer(self.c), ncj4 * 2, np.uint32).reshape(-1, 2),
        }

    def fnb(self):
        npad = self.grid_arrays()["npad"]
        return _copy(lib().orc_fnb(self.c), npad * 3, np.float32).reshape(-1, 3)


def fp64_allpairs(system, coulomb=COULOMB_EWALD, rc=0.9, beta=None, subset=None,
                  use_ewald_shift=False, epsilon_rf=1.0, vdw_modifier=0, rvdw_switch=0.0, beta_lj=0.0):
    """FP64 explicit-image forces (on ``subset``) and, for the full set, energies.
    vdw_modifier 4 is LJ-PME real space (geometric grid) with the LJ Ewald coefficient beta_lj."""
    L = lib()
    n = system.n
    epsfac = L.orc_one_4pi_eps0()
    if coulomb == COULOMB_CUTOFF:
        epsilon_rf = 1.0
    # the interaction constants are single-precision values in the reference
    # (gmxsetup.cpp:226-284, rf_util.cpp:54-66): use exactly those
    f32 = np.float32
    rcf = f32(rc)
    eps = f32(epsilon_rf)
    if eps == 0:
        k_rf = f32(1) / (f32(2) * rcf * rcf * rcf)
    else:
        k_rf = (eps - f32(1)) / (f32(2) * eps + f32(1)) / (rcf * rcf * rcf)
    c_rf = f32(1) / rcf + k_rf * rcf * rcf
    rc, k_rf, c_rf = float(rcf), float(k_rf), float(c_rf)
    full = subset is None
    sub = np.arange(n, dtype=np.int32) if full else np.ascontiguousarray(subset, dtype=np.int32)
    x, xp = _f(system.x)
    box, bp = _f(system.box)
    q, qp = _f(system.q)
    t, tp = _i(system.type)
    nb, nbp = _f(system.nbfp)
    ei, eip = _i(system.excl_index)
    el, elp = _i(system.excl_list if len(system.excl_list) else np.zeros(1, np.int32))
    s, sp = _i(sub)
    f = np.zeros((len(sub), 3), np.float64)
    e = np.zeros(2, np.float64)
    L.orc_fp64_allpairs(n, xp, bp, qp, tp, system.ntypes, nbp, eip, elp, coulomb, rc,
                        0.0 if beta is None else float(beta), epsfac, k_rf, c_rf,
                        int(use_ewald_shift), sp, len(sub), f.ctypes.data_as(C.POINTER(C.c_double)),
                        e.ctypes.data_as(C.POINTER(C.c_double)) if full else None, int(vdw_modifier),
                        float(np.float32(rvdw_switch)), float(beta_lj))
    return (f, e) if full else (f, None)


class CpuOracle:
    """The reference's CPU layout for one system (4-atom clusters, the simple 4x4 cluster pair list
    of makeClusterListSimple) and a 4-wide cluster-pair kernel (Ewald, potential-shift LJ): the
    list checker and the timed CPU baseline.  Coordinates are wrapped into the box."""

    def __init__(self, system, rc=0.9, rlist=1.0, beta=None, ewald_rtol=1e-5):
        L = lib()
        self.system = system
        box = np.asarray(system.box, np.float64)
        x = np.ascontiguousarray(np.asarray(system.x, np.float64) % box, dtype=np.float32)
        # values that round up to the box edge wrap to 0, as put_atoms_in_box does
        x = np.where(x >= box.astype(np.float32), np.float32(0), x).astype(np.float32)
        self._x, xp = _f(x)
        self._box, bp = _f(system.box)
        self._q, qp = _f(system.q)
        self._t, tp = _i(system.type)
        self._nb, nbp = _f(system.nbfp)
        self._ei, eip = _i(system.excl_index)
        self._el, elp = _i(system.excl_list if len(system.excl_list) else np.zeros(1, np.int32))
        if beta is None:
            beta = Oracle(system, rc=rc, rlist=rlist, ewald_rtol=ewald_rtol).beta
        self.beta = float(beta)
        epsfac = np.float32(L.orc_one_4pi_eps0())
        self.c = L.orc_cpu_create(system.n, xp, bp, qp, tp, system.ntypes, nbp, eip, elp, rc, rlist,
                                  self.beta, float(epsfac))

    def __del__(self):
        if getattr(self, "c", None):
            lib().orc_cpu_destroy(self.c)
            self.c = None

    def grid(self):
        lib().orc_cpu_grid(self.c)

    def search(self):
        lib().orc_cpu_search(self.c)

    def sizes(self):
        s = np.zeros(4, np.int32)
        lib().orc_cpu_sizes(self.c, s.ctypes.data_as(C.POINTER(C.c_int)))
        return {"clusters": int(s[0]), "entries": int(s[1]), "j_entries": int(s[2]), "geometric": bool(s[3])}

    def force(self, energy=True, threads=1, e0=0, e1=None):
        n = self.sizes()["entries"] if e1 is None else e1
        if lib().orc_cpu_force(self.c, int(e0), int(n), int(energy), int(threads)) != 0:
            raise RuntimeError("CPU kernel failed")

    def forces(self):
        f = np.empty((self.system.n, 3), np.float32)
        lib().orc_cpu_forces(self.c, f.ctypes.data_as(C.POINTER(C.c_float)))
        return f

    def energies(self):
        e = np.zeros(2, np.float64)
        lib().orc_cpu_energies(self.c, e.ctypes.data_as(C.POINTER(C.c_double)))
        return e

    def pairlist(self):
        sz = self.sizes()
        ci = np.zeros(max(1, sz["entries"]) * 4, np.int32)
        cj = np.zeros(max(1, sz["j_entries"]) * 2, np.int32)
        lib().orc_cpu_list(self.c, ci.ctypes.data_as(C.POINTER(C.c_int)), cj.ctypes.data_as(C.POINTER(C.c_int)))
        ai = np.zeros(sz["clusters"] * 4, np.int32)
        xs = np.zeros(sz["clusters"] * 16, np.float32)
        lib().orc_cpu_grid_arrays(self.c, ai.ctypes.data_as(C.POINTER(C.c_int)),
                                  xs.ctypes.data_as(C.POINTER(C.c_float)))
        return {"ci": ci[: 4 * sz["entries"]].reshape(-1, 4), "cj": cj[: 2 * sz["j_entries"]].reshape(-1, 2),
                "atom_indices": ai, "xs": xs.reshape(-1, 4, 4)}
