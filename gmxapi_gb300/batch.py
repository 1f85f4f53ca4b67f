"""Batched ensembles: many independent systems of uneven size on one GPU.

``BatchForceCalculator`` wraps the nbx_batch_* C ABI: per-system grids and
pair lists, one persistent force launch over all systems' list entries,
per-system FP64 energies and virials, and a CUDA graph for the step.
``autotune`` picks the force-kernel tile (one or two atom pairs per lane), the
j-stage depth, the launch shape and the rolling-prune interval by timing
candidate settings on the caller's own coordinate frames.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from .nblib import NBKernelOptions, _fptr, _iptr


class BatchForceCalculator:
    """Forces, energies and virials for a list of systems sharing types, nbfp and options."""

    def __init__(self, systems, options: NBKernelOptions | None = None, device: int = 0):
        self.options = options or NBKernelOptions()
        self.systems = list(systems)
        n = len(self.systems)
        descs = (_lib.nbx_system_desc * n)()
        self._keep = []
        for d, s in zip(descs, self.systems):
            x = np.ascontiguousarray(s.x, np.float32).reshape(-1)
            q = np.ascontiguousarray(s.q, np.float32)
            t = np.ascontiguousarray(s.type, np.int32)
            nb = np.ascontiguousarray(s.nbfp, np.float32)
            ei = np.ascontiguousarray(s.excl_index, np.int32)
            el = np.ascontiguousarray(s.excl_list if len(s.excl_list) else np.zeros(1, np.int32), np.int32)
            self._keep += [x, q, t, nb, ei, el]
            d.num_atoms, d.x, d.q, d.type = s.n, _fptr(x), _fptr(q), _iptr(t)
            d.num_types, d.nbfp, d.excl_index, d.excl_list = int(s.ntypes), _fptr(nb), _iptr(ei), _iptr(el)
            for k in range(3):
                d.box[k] = float(s.box[k])
        self._opts = self.options.to_c()
        h = C.c_void_p()
        L = _lib.load()
        code = L.nbx_batch_create(n, descs, C.byref(self._opts), device, C.byref(h))
        if code != 0:
            raise _lib.NbxError(code, L.nbx_batch_last_error(None).decode())
        self.h = h
        off = (C.c_int * (n + 1))()
        tot = C.c_longlong()
        self._check(L.nbx_batch_atoms(h, C.byref(tot), off))
        self.offsets = np.array(off[:], np.int64)
        self.total_atoms = int(tot.value)

    def _check(self, code):
        if code != 0:
            raise _lib.NbxError(code, _lib.load().nbx_batch_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            _lib.load().nbx_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- device-resident interface (raw device pointers) ----
    def set_stream(self, stream_ptr: int):
        self._check(_lib.load().nbx_batch_set_stream(self.h, C.c_void_p(stream_ptr)))

    def search_device(self, x_ptr: int):
        self._check(_lib.load().nbx_batch_search_device(self.h, C.c_void_p(x_ptr)))

    def compute_device(self, x_ptr, f_ptr, e_ptr=None, vir_ptr=None):
        self._check(_lib.load().nbx_batch_compute_device(self.h, C.c_void_p(x_ptr), C.c_void_p(f_ptr),
                                                         C.c_void_p(e_ptr) if e_ptr else None,
                                                         C.c_void_p(vir_ptr) if vir_ptr else None))

    def md_step_device(self, step, x_ptr, f_ptr, e_ptr=None, vir_ptr=None):
        self._check(_lib.load().nbx_batch_md_step_device(self.h, int(step), C.c_void_p(x_ptr), C.c_void_p(f_ptr),
                                                         C.c_void_p(e_ptr) if e_ptr else None,
                                                         C.c_void_p(vir_ptr) if vir_ptr else None))

    def sequential_md_step_device(self, step, x_ptr, f_ptr, e_ptr=None, vir_ptr=None):
        self._check(_lib.load().nbx_batch_sequential_md_step_device(
            self.h, int(step), C.c_void_p(x_ptr), C.c_void_p(f_ptr), C.c_void_p(e_ptr) if e_ptr else None,
            C.c_void_p(vir_ptr) if vir_ptr else None))

    # ---- adjoint / force matching (raw device pointers) ----
    def set_parameters_device(self, q_ptr: int | None, nbfp_ptr: int | None):
        self._check(_lib.load().nbx_batch_set_parameters_device(
            self.h, C.c_void_p(q_ptr) if q_ptr else None, C.c_void_p(nbfp_ptr) if nbfp_ptr else None))

    def backward_device(self, x_ptr, gf_ptr, ge_ptr=None, gx_ptr=None, gq_ptr=None, gnbfp_ptr=None):
        vp = C.c_void_p
        self._check(_lib.load().nbx_batch_backward_device(
            self.h, vp(x_ptr), vp(gf_ptr), vp(ge_ptr) if ge_ptr else None, vp(gx_ptr) if gx_ptr else None,
            vp(gq_ptr) if gq_ptr else None, vp(gnbfp_ptr) if gnbfp_ptr else None))

    def force_match_device(self, x_ptr, q_ptr, nbfp_ptr, ftarget_ptr, loss_ptr, gq_ptr, gnbfp_ptr, e_ptr=None,
                           vir_ptr=None):
        vp = C.c_void_p
        self._check(_lib.load().nbx_batch_force_match_device(
            self.h, vp(x_ptr), vp(q_ptr), vp(nbfp_ptr), vp(ftarget_ptr), vp(loss_ptr), vp(gq_ptr), vp(gnbfp_ptr),
            vp(e_ptr) if e_ptr else None, vp(vir_ptr) if vir_ptr else None))

    def set_graph(self, enable: bool):
        self._check(_lib.load().nbx_batch_set_graph(self.h, int(bool(enable))))

    def set_kernel_variant(self, variant: int):
        self._check(_lib.load().nbx_batch_set_kernel_variant(self.h, int(variant)))

    def set_force_kernel(self, tile: int = 1, stage_depth: int = 2):
        """Force-kernel tile (1: two atom pairs per lane, packed FP32x2; 0: one pair per lane) and
        j-stage buffers per warp (2 or 3)."""
        self._check(_lib.load().nbx_batch_set_force_kernel(self.h, int(tile), int(stage_depth)))

    def set_prune(self, nstlist_prune: int, rlist_inner: float):
        self._check(_lib.load().nbx_batch_set_prune(self.h, int(nstlist_prune), float(rlist_inner)))

    # ---- autotuner ----
    def autotune(self, frames, variants=(0, 1, 2, 3), prune_intervals=(4, 10, 20), steps=None,
                 buffer_at_10=0.05, tiles=((0, 2), (1, 2), (1, 3))):
        """Time every (tile, stage depth, launch shape, prune interval) on ``frames``; keep the fastest.

        frames: torch tensor (nframes, 3 * total_atoms) on the device, a trajectory segment of the
        workload.  tiles: (tile, stage depth) pairs of the force kernel (tile 1 = two atom pairs per
        lane in packed FP32x2 arithmetic, tile 0 = one pair per lane; depth = j-stage buffers per
        warp).  variants: launch shapes (0: 256x2, 1: 128x4, 2: 512x1, 3: 64x8 threads x blocks per
        SM).  For a prune interval n the inner radius is rc + buffer_at_10 * sqrt(n / 10) (a
        diffusive drift over n steps).  Each candidate runs the full schedule (search, rolling
        prune, compute with energies) over the frames; returns (best settings, timings in ms/step
        keyed by (tile, depth, variant, interval)).
        """
        import torch

        rc = self.options.rcoulomb if self.options.rcoulomb is not None else self.options.pairlist_cutoff
        nsys = len(self.systems)
        dev = frames.device
        f = torch.empty(frames.shape[1], dtype=torch.float32, device=dev)
        e = torch.empty(2 * nsys, dtype=torch.float64, device=dev)
        v = torch.empty(9 * nsys, dtype=torch.float64, device=dev)
        nfr = frames.shape[0] if steps is None else min(steps, frames.shape[0])
        results = {}
        for n in prune_intervals:
            rin = min(self.options.pairlist_cutoff, rc + buffer_at_10 * math.sqrt(n / 10.0))
            self.set_prune(n, rin)
            for tile, depth in tiles:
                self.set_force_kernel(tile, depth)
                for var in variants:
                    self.set_kernel_variant(var)
                    # warm-up pass (search + graph capture), then the timed pass
                    for t in range(min(3, nfr)):
                        self.md_step_device(t, frames[t].data_ptr(), f.data_ptr(), e.data_ptr(), v.data_ptr())
                    torch.cuda.synchronize()
                    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    a.record()
                    for t in range(nfr):
                        self.md_step_device(t, frames[t].data_ptr(), f.data_ptr(), e.data_ptr(), v.data_ptr())
                    b.record()
                    torch.cuda.synchronize()
                    results[(tile, depth, var, n)] = a.elapsed_time(b) / nfr
        best = min(results, key=results.get)
        tile, depth, var, n = best
        rin = min(self.options.pairlist_cutoff, rc + buffer_at_10 * math.sqrt(n / 10.0))
        self.set_prune(n, rin)
        self.set_force_kernel(tile, depth)
        self.set_kernel_variant(var)
        return {"tile": tile, "stage_depth": depth, "kernel_variant": var, "nstlist_prune": n,
                "rlist_inner": rin}, results
