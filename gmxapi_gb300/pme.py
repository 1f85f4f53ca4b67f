"""Smooth-PME reciprocal space on one GB300 (Python side of the nbx_pme_* C ABI).

Mirrors the reference's PME interface for the Coulomb grid: ``Pme(box, grid,
ewald_coeff)`` is gmx_pme_init (src/gromacs/ewald/pme.h:140), ``compute`` /
``compute_device`` are gmx_pme_do (pme.h:181) adding the reciprocal-space forces
and returning the energy and the virial, ``grid_size`` is calcFftGrid
(src/gromacs/fft/calcgrid.h:46) and ``ewald_coefficient`` calc_ewaldcoeff_q
(src/gromacs/ewald/ewald_utils.h:68).  The stage methods (``splines_device``,
``spread_device``, ``solve_device``, ``gather_device``) are the entry points the
reference's PME unit tests drive (src/gromacs/ewald/tests/pmetestcommon.h).
Invalid input raises nblib's InputException; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .nblib import InputException


def _check(code: int, handle=None):
    if code == _lib.NBX_OK:
        return
    msg = _lib.load().nbx_pme_last_error(handle)
    text = msg.decode() if msg else ""
    if code == _lib.NBX_ERR_INVALID_INPUT:
        raise InputException(text or "invalid input")
    raise _lib.NbxError(code, text)


def ewald_coefficient(rcoulomb: float, ewald_rtol: float = 1e-5) -> float:
    """beta with erfc(beta rc) = ewald_rtol (single precision, like the reference)."""
    return float(_lib.load().nbx_ewald_coefficient(float(rcoulomb), float(ewald_rtol)))


def ewald_coefficient_lj(rvdw: float, ewald_rtol_lj: float = 1e-3) -> float:
    """beta_lj with exp(-x^2)(1 + x^2 + x^4/2) = ewald_rtol_lj, x = beta_lj rvdw (calc_ewaldcoeff_lj)."""
    return float(_lib.load().nbx_ewald_coefficient_lj(float(rvdw), float(ewald_rtol_lj)))


def grid_size(box, spacing: float = 0.12) -> tuple[int, int, int]:
    """PME grid sizes for the box edges and the largest grid spacing (calcFftGrid)."""
    b = (C.c_float * 3)(*[float(v) for v in box])
    n = (C.c_int * 3)()
    _check(_lib.load().nbx_pme_grid_size(b, float(spacing), n))
    return int(n[0]), int(n[1]), int(n[2])


class Fft3d:
    """The 3D real <-> half-complex transform of a grid [nx][ny][nz] on one GPU (hand-written,
    unnormalised; gmx_parallel_3dfft_init / _execute of src/gromacs/fft/parallel_3dfft.h on one
    rank).  ``execute_device(+1, real, cgrid)``: real -> half-complex [nx][ny][nz/2+1] float2;
    ``execute_device(-1, real, cgrid)``: back (cgrid overwritten)."""

    def __init__(self, grid, device: int = 0):
        self.grid = tuple(int(v) for v in grid)
        n = (C.c_int * 3)(*self.grid)
        h = C.c_void_p()
        _check(_lib.load().nbx_fft3d_create(n, int(device), C.byref(h)))
        self.h = h

    def execute_device(self, direction: int, real_ptr: int, cgrid_ptr: int, stream_ptr: int = 0):
        _check(_lib.load().nbx_fft3d_execute_device(self.h, int(direction), real_ptr, cgrid_ptr, stream_ptr))

    def close(self):
        if getattr(self, "h", None):
            _lib.load().nbx_fft3d_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Pme:
    """One PME grid of a rectangular box (pme_order 4) on one GPU: Coulomb (charges), or with
    ``lj=True`` the LJ-PME dispersion grid (geometric rule; coefficients sqrt(C6_ii), the
    reference's sqrt_c6A)."""

    def __init__(self, box, grid=None, ewald_coeff: float | None = None, *, rcoulomb: float = 1.0,
                 ewald_rtol: float = 1e-5, fourier_spacing: float = 0.12, epsilon_r: float = 1.0,
                 device: int = 0, lj: bool = False, ewald_rtol_lj: float = 1e-3):
        self.box = tuple(float(v) for v in box)
        if len(self.box) != 3:
            raise InputException("rectangular boxes only: three edge lengths")
        self.grid = tuple(int(v) for v in grid) if grid is not None else grid_size(self.box, fourier_spacing)
        self.lj = bool(lj)
        if ewald_coeff is not None:
            self.beta = float(ewald_coeff)
        else:
            self.beta = (ewald_coefficient_lj(rcoulomb, ewald_rtol_lj) if self.lj
                         else ewald_coefficient(rcoulomb, ewald_rtol))
        self.epsilon_r = float(epsilon_r)
        self.device = device
        b = (C.c_float * 3)(*self.box)
        n = (C.c_int * 3)(*self.grid)
        h = C.c_void_p()
        if self.lj:
            _check(_lib.load().nbx_pme_create_lj(b, n, self.beta, device, C.byref(h)))
        else:
            _check(_lib.load().nbx_pme_create(b, n, self.beta, self.epsilon_r, device, C.byref(h)))
        self.h = h
        self.energy = 0.0
        self.virial = np.zeros((3, 3))

    def close(self):
        if getattr(self, "h", None):
            _lib.load().nbx_pme_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- device-resident interface (raw device pointers, asynchronous on the handle's stream) ----
    def compute_device(self, natoms: int, x_ptr: int, q_ptr: int, f_ptr: int, e_ptr: int | None = None,
                       vir_ptr: int | None = None):
        """Adds the reciprocal-space forces to f; energy (double[1]) / virial (double[9]) when given."""
        _check(_lib.load().nbx_pme_compute_device(self.h, natoms, x_ptr, q_ptr, f_ptr, e_ptr, vir_ptr), self.h)

    def splines_device(self, natoms: int, x_ptr: int, idx_ptr: int, theta_ptr: int, dtheta_ptr: int):
        _check(_lib.load().nbx_pme_splines_device(self.h, natoms, x_ptr, idx_ptr, theta_ptr, dtheta_ptr), self.h)

    def spread_device(self, natoms: int, x_ptr: int, q_ptr: int, grid_ptr: int):
        _check(_lib.load().nbx_pme_spread_device(self.h, natoms, x_ptr, q_ptr, grid_ptr), self.h)

    def solve_device(self, cgrid_ptr: int, e_ptr: int | None = None, vir_ptr: int | None = None):
        _check(_lib.load().nbx_pme_solve_device(self.h, cgrid_ptr, e_ptr, vir_ptr), self.h)

    def gather_device(self, natoms: int, x_ptr: int, q_ptr: int, grid_ptr: int, f_ptr: int):
        _check(_lib.load().nbx_pme_gather_device(self.h, natoms, x_ptr, q_ptr, grid_ptr, f_ptr), self.h)

    def fft_device(self, direction: int, real_ptr: int, cgrid_ptr: int):
        """The grid's 3D transform: +1 real -> half-complex, -1 back (unnormalised; the complex
        grid is overwritten by the backward transform)."""
        _check(_lib.load().nbx_pme_fft_device(self.h, int(direction), real_ptr, cgrid_ptr), self.h)

    def set_stream(self, stream_ptr: int):
        _check(_lib.load().nbx_pme_set_stream(self.h, stream_ptr), self.h)

    def synchronize(self):
        _check(_lib.load().nbx_pme_synchronize(self.h), self.h)

    # ---- host-array interface ----
    def compute(self, x, q, forces=None, energies: bool = True):
        """Reciprocal-space forces (N, 3) for host coordinates x and charges q, added to
        `forces` when given (like gmx_pme_do) and returned; sets .energy and .virial."""
        import torch

        x = np.ascontiguousarray(x, np.float32).reshape(-1, 3)
        q = np.ascontiguousarray(q, np.float32).reshape(-1)
        if q.shape[0] != x.shape[0]:
            raise InputException("coordinates and charges differ in length")
        dev = torch.device("cuda", self.device)
        dx = torch.from_numpy(x).to(dev)
        dq = torch.from_numpy(q).to(dev)
        f0 = np.zeros_like(x) if forces is None else np.ascontiguousarray(forces, np.float32).reshape(-1, 3)
        df = torch.from_numpy(f0).to(dev)
        de = torch.zeros(1, dtype=torch.float64, device=dev)
        dv = torch.zeros(9, dtype=torch.float64, device=dev)
        torch.cuda.synchronize(dev)
        self.compute_device(x.shape[0], dx.data_ptr(), dq.data_ptr(), df.data_ptr(),
                            de.data_ptr() if energies else None, dv.data_ptr() if energies else None)
        self.synchronize()
        if energies:
            self.energy = float(de.item())
            self.virial = dv.cpu().numpy().reshape(3, 3)
        out = df.cpu().numpy()
        if forces is not None and isinstance(forces, np.ndarray) and forces.dtype == np.float32 \
                and forces.flags.c_contiguous:
            forces.reshape(-1, 3)[:] = out
            return forces
        return out
