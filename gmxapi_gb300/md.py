"""GPU-resident MD: nblib's LeapFrog and a device-side step loop (Python side).

``LeapFrog(inverse_masses, box).integrate(dt, x, v, f)`` mirrors nblib::LeapFrog
(api/nblib/integrator.h:71-90): host arrays updated in place, atoms put back in the box.
``MdRunner`` keeps coordinates, velocities and forces on the GPU and runs mdrun-style steps
(do_force + update, src/gromacs/mdlib/sim_util.cpp): the cluster-pair kernel with its search
and rolling-prune schedule, optional PME reciprocal space, leap-frog, energies every
``nstcalcenergy`` steps, all on one CUDA stream through ``nbx_md_run_device``.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .nblib import ForceCalculator, InputException, NBKernelOptions


def _check(code: int, handle=None):
    if code == _lib.NBX_OK:
        return
    msg = _lib.load().nbx_leapfrog_last_error(handle)
    text = msg.decode() if msg else ""
    if code == _lib.NBX_ERR_INVALID_INPUT:
        raise InputException(text or "invalid input")
    raise _lib.NbxError(code, text)


def _fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class LeapFrog:
    """nblib::LeapFrog on one GPU: v += f dt / m, x += v dt, atoms put in the box."""

    def __init__(self, inverse_masses, box, device: int = 0):
        self._im = np.ascontiguousarray(inverse_masses, np.float32)
        self.n = int(self._im.shape[0])
        b = (C.c_float * 3)(*[float(v) for v in box])
        h = C.c_void_p()
        _check(_lib.load().nbx_leapfrog_create(self.n, _fptr(self._im), b, device, C.byref(h)))
        self.h = h

    @classmethod
    def from_masses(cls, masses, box, device: int = 0):
        m = np.asarray(masses, np.float64)
        return cls((1.0 / m).astype(np.float32), box, device)

    def close(self):
        if getattr(self, "h", None):
            _lib.load().nbx_leapfrog_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def integrate(self, dt: float, x: np.ndarray, v: np.ndarray, f: np.ndarray):
        """Host arrays (N, 3) float32, x and v updated in place (LeapFrog::integrate)."""
        for a in (x, v):
            if a.dtype != np.float32 or not a.flags.c_contiguous or a.size != 3 * self.n:
                raise InputException("x and v must be contiguous float32 (N, 3) arrays")
        fc = np.ascontiguousarray(f, np.float32)
        _check(_lib.load().nbx_leapfrog_integrate(self.h, float(dt), _fptr(x), _fptr(v), _fptr(fc)), self.h)

    def integrate_device(self, dt: float, x_ptr: int, v_ptr: int, f_ptr: int, ekin_ptr: int | None = None):
        _check(_lib.load().nbx_leapfrog_integrate_device(self.h, float(dt), x_ptr, v_ptr, f_ptr, ekin_ptr), self.h)

    def set_stream(self, stream_ptr: int):
        _check(_lib.load().nbx_leapfrog_set_stream(self.h, stream_ptr), self.h)


class MdRunner:
    """GPU-resident MD of one system: nonbonded (+ PME) forces and leap-frog on the device.

    ``energies`` rows are {E_LJ, E_Coulomb real space, E_Coulomb reciprocal, E_kin} (kJ/mol, FP64);
    E_kin = 0.5 (KE(t - dt/2) + KE(t + dt/2)), so the row sum is the total energy at step t."""

    def __init__(self, system, masses, options: NBKernelOptions | None = None, dt: float = 0.002,
                 velocities=None, pme: bool = True, fourier_spacing: float = 0.12, device: int = 0):
        import torch

        from . import pme as pme_mod

        self.system = system
        self.options = options or NBKernelOptions()
        self.dt = float(dt)
        self.device = device
        self.calc = ForceCalculator(system, self.options, device=device)
        dev = torch.device("cuda", device)
        self.stream = torch.cuda.current_stream(dev)
        self.calc.set_stream(self.stream.cuda_stream)
        box = [float(b) for b in system.box]
        self.lf = LeapFrog.from_masses(masses, box, device)
        self.pme = None
        rc = self.options.rcoulomb if self.options.rcoulomb is not None else self.options.pairlist_cutoff
        if pme and int(self.options.coulomb_type) == 0:
            self.pme = pme_mod.Pme(box, pme_mod.grid_size(box, fourier_spacing),
                                   pme_mod.ewald_coefficient(rc, self.options.ewald_rtol),
                                   device=device)
        n = system.n
        self.x = torch.from_numpy(np.ascontiguousarray(system.x, np.float32).reshape(-1)).to(dev)
        v0 = np.zeros((n, 3), np.float32) if velocities is None else np.asarray(velocities, np.float32)
        self.v = torch.from_numpy(np.ascontiguousarray(v0).reshape(-1)).to(dev)
        self.f = torch.zeros(3 * n, dtype=torch.float32, device=dev)
        self.q = torch.from_numpy(np.ascontiguousarray(system.q, np.float32)).to(dev)
        self.step = 0
        torch.cuda.synchronize(dev)

    def close(self):
        for k in ("pme", "lf", "calc"):
            obj = getattr(self, k, None)
            if obj is not None:
                obj.close()
                setattr(self, k, None)

    def run(self, num_steps: int, nstcalcenergy: int = 0):
        """Runs num_steps steps; returns the energy rows (every nstcalcenergy steps, none for 0)."""
        import torch

        rows = (num_steps + nstcalcenergy - 1) // nstcalcenergy if nstcalcenergy > 0 else 0
        e = torch.zeros((max(rows, 1), 4), dtype=torch.float64, device=self.x.device)
        code = _lib.load().nbx_md_run_device(
            self.calc.h, self.pme.h if self.pme is not None else None, self.lf.h, self.step, int(num_steps),
            self.dt, self.x.data_ptr(), self.v.data_ptr(), self.f.data_ptr(), self.q.data_ptr(),
            max(1, nstcalcenergy), e.data_ptr() if rows else None)
        if code != _lib.NBX_OK:
            msg = _lib.load().nbx_leapfrog_last_error(self.lf.h).decode()
            nb_msg = _lib.load().nbx_last_error(self.calc.h)
            raise _lib.NbxError(code, msg or (nb_msg.decode() if nb_msg else ""))
        self.step += int(num_steps)
        self.calc.synchronize()
        return e[:rows].cpu().numpy() if rows else np.zeros((0, 4))

    def positions(self) -> np.ndarray:
        return self.x.cpu().numpy().reshape(-1, 3)

    def velocities(self) -> np.ndarray:
        return self.v.cpu().numpy().reshape(-1, 3)
