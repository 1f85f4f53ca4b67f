"""CPU restatement of nblib's leap-frog and of a GPU-resident MD step (TEST INFRASTRUCTURE ONLY).

Used by tests/ and ``bench.py``'s CPU-baseline leg as the checker of the CUDA update kernel and
step loop; the product never imports it.

- ``put_in_box``: put_atoms_in_box, rectangular branch (src/gromacs/pbcutil/pbc.cpp:1430-1446):
  ``while (x < 0) x += L; while (x >= L) x -= L`` per coordinate, in float32.  Like the kernel it
  applies at most 4 single shifts and then a floor-based one (the reference's loops are unbounded).
- ``leapfrog``: nblib::LeapFrog::integrate (api/nblib/integrator.cpp:67-77), float32, in the
  reference's operation order ``v += f * dt * invmass; x += v * dt``; the kinetic energy is the mean
  of the half-step values before and after the update (FP64).
- ``md_run``: the step loop of ``nbx_md_run_device``: nonbonded forces from the C oracle (a fresh
  grid and list every step: forces do not depend on the list while it covers rc), PME forces from
  ``pme_oracle``, leap-frog; atoms put in the box only on the update before a search step.
"""
from __future__ import annotations

import numpy as np

from oracle import oracle as O
from oracle import pme_oracle

_WRAP_STEPS = 4


def put_in_box(x: np.ndarray, box) -> np.ndarray:
    x = np.array(x, dtype=np.float32, copy=True).reshape(-1, 3)
    for d in range(3):
        L = np.float32(box[d])
        col = x[:, d]
        for _ in range(_WRAP_STEPS):
            m = col < 0
            col[m] = col[m] + L
        for _ in range(_WRAP_STEPS):
            m = col >= L
            col[m] = col[m] - L
        far = (col < 0) | (col >= L)
        if far.any():
            y = (col[far] - L * np.floor(col[far] / L)).astype(np.float32)
            y[y < 0] += L
            y[y >= L] = 0.0
            col[far] = y
        x[:, d] = col
    return x


def leapfrog(x, v, f, inv_mass, dt, box, wrap=True):
    """One update; returns (x, v, ekin) with ekin = 0.5 (KE(t - dt/2) + KE(t + dt/2))."""
    x = np.asarray(x, dtype=np.float32).reshape(-1, 3)
    v = np.asarray(v, dtype=np.float32).reshape(-1, 3)
    f = np.asarray(f, dtype=np.float32).reshape(-1, 3)
    im = np.asarray(inv_mass, dtype=np.float32)[:, None]
    dt = np.float32(dt)
    vn = (v + (f * dt).astype(np.float32) * im).astype(np.float32)
    xn = (x + (vn * dt).astype(np.float32)).astype(np.float32)
    if wrap:
        xn = put_in_box(xn, box)
    with np.errstate(divide="ignore"):
        m = np.where(im[:, 0] > 0, 1.0 / im[:, 0].astype(np.float64), 0.0)
    ke = 0.25 * float((m[:, None] * (v.astype(np.float64) ** 2 + vn.astype(np.float64) ** 2)).sum())
    return xn, vn, ke


def md_run(system, inv_mass, x, v, num_steps, dt, *, rc=0.9, rlist=1.0, nstlist=10, pme_grid=None, beta=None,
           first_step=0, nstcalcenergy=1):
    """Returns (x, v, energy rows {E_LJ, E_Coulomb real, E_Coulomb reciprocal, E_kin})."""
    x = np.asarray(x, dtype=np.float32).reshape(-1, 3).copy()
    v = np.asarray(v, dtype=np.float32).reshape(-1, 3).copy()
    box = [float(b) for b in system.box]
    o = O.Oracle(system, rc=rc, rlist=rlist)
    rows = []
    for k in range(num_steps):
        step = first_step + k
        o.set_coordinates(x)
        o.grid()
        o.search()
        o.force(True)
        f = o.forces().astype(np.float32)
        e_lj, e_c = o.energies()
        e_rec = 0.0
        if pme_grid is not None:
            fr, e_rec, _ = pme_oracle.compute(x, system.q, box, pme_grid, beta, single=True)
            f = (f + fr.astype(np.float32)).astype(np.float32)
        wrap = (step + 1) % nstlist == 0
        x, v, ke = leapfrog(x, v, f, inv_mass, dt, box, wrap=wrap)
        if k % nstcalcenergy == 0:
            rows.append([e_lj, e_c, e_rec, ke])
    return x, v, np.array(rows)
