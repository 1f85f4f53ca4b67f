"""CPU restatement of the reference's smooth-PME reciprocal path (TEST INFRASTRUCTURE ONLY).

Used by tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``
as the checker of the CUDA PME kernels; the product never imports it.  FP64 numpy,
pme_order 4, rectangular boxes, one rank (no PME decomposition).  Each function
cites the reference code it restates (paths inside the GROMACS source tree):

- ``fft_grid_size``: calcFftGrid, src/gromacs/fft/calcgrid.cpp:63-160, with
  minGridPointsPerDim = minimalPmeGridSize = 2 (pme_order - 1), ewald/pme.cpp:488-500.
- ``bspline_moduli``: make_bspline_moduli + make_dft_mod,
  src/gromacs/ewald/calculate_spline_moduli.cpp:52-122.
- ``splines``: calc_interpolation_idx (pme_spread.cpp:65-140; t = n (x / L + 2),
  index = (int)t mod n via make_gridindex_to_localindex, pme_grid.cpp:779-830) and
  CALC_SPLINE (pme_spread.cpp:220-266).
- ``spread``: spread_coefficients_bsplines_thread + wrap_periodic_pmegrid: atom a adds
  q theta_x theta_y theta_z to points (index + 0..3) mod n.
- ``solve``: solve_pme_yzx, src/gromacs/ewald/pme_solve.cpp:332-587.
- ``solve_lj``: solve_pme_lj_yzx with the geometric combination rule (one grid),
  src/gromacs/ewald/pme_solve.cpp:588-915.
- ``gather``: gather_f_bsplines / do_fspline, src/gromacs/ewald/pme_gather.cpp:78-360.
- ``compute``: gmx_pme_do's Coulomb path (spread -> r2c FFT -> solve -> c2r FFT ->
  gather), src/gromacs/ewald/pme.cpp:1002-1300, with unnormalised transforms.

Pinned against the reference's own PME unit-test reference data (spline values,
gridline indices and spread grids; spline moduli; solved grids, energies and virials;
gathered forces: src/gromacs/ewald/tests/refdata, extracted into
tests/golden/pme_golden.json), and against ``ewald_reciprocal_exact``, a direct FP64
k-space Ewald sum (the textbook reciprocal-space energy, its forces, and its virial
1/2 dE/d(strain), which is GROMACS' -1/2 sum r (x) F convention).
"""
from __future__ import annotations

import math

import numpy as np

ORDER = 4
ONE_4PI_EPS0 = None  # set below from the same CODATA constants as the reference's units.h


def _one_4pi_eps0() -> float:
    # src/gromacs/math/units.h:69-79
    eps0 = (8.8541878128e-12 * 1e-9 * 1e3) / (1.602176634e-19 ** 2 * 6.02214076e23)
    return 1.0 / (4.0 * math.pi * eps0)


ONE_4PI_EPS0 = _one_4pi_eps0()

_GRID_INIT = (6, 8, 10, 12, 14, 16, 20, 24, 25, 28, 32, 36, 40, 42, 44)
_GRID_BASE = (45, 48, 50, 52, 54, 56, 60, 64, 70, 72, 75, 80, 81, 84)


def fft_grid_size(length: float, spacing: float, min_points: int = 2 * (ORDER - 1)) -> int:
    """calcFftGrid for one box edge (calcgrid.cpp:117-152)."""
    nmin = max(int(float(np.float32(np.float32(length) / np.float32(spacing))) + 0.999), min_points)
    if _GRID_INIT[-1] >= nmin:
        i = len(_GRID_INIT) - 1
        while i > 0 and _GRID_INIT[i - 1] >= nmin:
            i -= 1
        return _GRID_INIT[i]
    fac2 = 1
    while fac2 * _GRID_BASE[-1] < nmin:
        fac2 *= 2
    n = 0
    for i in range(len(_GRID_BASE) - 1, 0, -1):  # the reference's do-while stops before index 0
        attempt = fac2 * _GRID_BASE[i]
        if ((attempt % 4 == 0 and attempt != 140) or attempt == 90) and attempt >= nmin:
            n = attempt
    return n


def bspline_moduli(n: int, order: int = ORDER) -> np.ndarray:
    """|DFT of the cardinal B-spline of order `order - 1` at the integers|^2, with the
    zero at n/2 replaced by the neighbours' mean for even spline order and even n."""
    spline_order = order - 1
    data = np.zeros(spline_order)
    data[0] = 1.0
    for k in range(2, spline_order + 1):
        div = 1.0 / k
        for m in range(k - 1, 0, -1):
            data[m] = div * ((k - m) * data[m - 1] + (m + 1) * data[m])
        data[0] = div * data[0]
    i = np.arange(n)[:, None]
    j = np.arange(spline_order)[None, :]
    arg = 2.0 * np.pi * i * (j + 1) / n
    sc = (data[None, :] * np.cos(arg)).sum(1)
    ss = (data[None, :] * np.sin(arg)).sum(1)
    mod = sc * sc + ss * ss
    if spline_order % 2 == 0 and n % 2 == 0:
        mod[n // 2] = 0.5 * (mod[n // 2 - 1] + mod[n // 2 + 1])
    return mod


def splines(x: np.ndarray, box, n, single: bool = True):
    """Gridline indices idx[N,3] and B-spline weights / derivatives theta, dtheta [3,N,4].

    single=True forms the fractional coordinate t = n (x / L + 2) in float32 like the
    reference's ``real`` in a mixed-precision build (x * rxx, + shift, * n, each rounded);
    single=False forms it in FP64 like a double-precision build (the reference's PME
    unit-test data were generated that way).  The weights are FP64 from that fraction."""
    x32 = np.asarray(x, dtype=np.float32).reshape(-1, 3)
    N = x32.shape[0]
    idx = np.zeros((N, 3), dtype=np.int64)
    theta = np.zeros((3, N, ORDER))
    dtheta = np.zeros((3, N, ORDER))
    for d in range(3):
        if single:
            rec = np.float32(1.0) / np.float32(box[d])
            t = np.float32(n[d]) * ((x32[:, d] * rec).astype(np.float32) + np.float32(2.0))
            t = t.astype(np.float32)
            ti = np.floor(t).astype(np.int64)
            dr = (t - ti.astype(np.float32)).astype(np.float64)
        else:
            rec = 1.0 / float(np.float32(box[d]))
            t = n[d] * (x32[:, d].astype(np.float64) * rec + 2.0)
            ti = np.floor(t).astype(np.int64)
            dr = t - ti
        idx[:, d] = np.mod(ti, n[d])
        # CALC_SPLINE(4)
        data = np.zeros((N, ORDER))
        data[:, 1] = dr
        data[:, 0] = 1.0 - dr
        for k in range(3, ORDER):
            div = 1.0 / (k - 1.0)
            data[:, k - 1] = div * dr * data[:, k - 2]
            for l in range(1, k - 1):
                data[:, k - l - 1] = div * ((dr + l) * data[:, k - l - 2] + (k - l - dr) * data[:, k - l - 1])
            data[:, 0] = div * (1.0 - dr) * data[:, 0]
        dtheta[d, :, 0] = -data[:, 0]
        for k in range(1, ORDER):
            dtheta[d, :, k] = data[:, k - 1] - data[:, k]
        div = 1.0 / (ORDER - 1)
        data[:, ORDER - 1] = div * dr * data[:, ORDER - 2]
        for l in range(1, ORDER - 1):
            data[:, ORDER - l - 1] = div * ((dr + l) * data[:, ORDER - l - 2]
                                            + (ORDER - l - dr) * data[:, ORDER - l - 1])
        data[:, 0] = div * (1.0 - dr) * data[:, 0]
        theta[d] = data
    return idx, theta, dtheta


def _points(idx, n, d):
    return np.mod(idx[:, d][:, None] + np.arange(ORDER)[None, :], n[d])  # [N, 4]


def spread(idx, theta, q, n) -> np.ndarray:
    """Real grid [nx, ny, nz] of the spread charges."""
    q = np.asarray(q, dtype=np.float64)
    gx, gy, gz = (_points(idx, n, d) for d in range(3))
    w = (q[:, None, None, None] * theta[0][:, :, None, None] * theta[1][:, None, :, None]
         * theta[2][:, None, None, :])
    flat = (gx[:, :, None, None] * n[1] + gy[:, None, :, None]) * n[2] + gz[:, None, None, :]
    grid = np.zeros(n[0] * n[1] * n[2])
    np.add.at(grid, flat.ravel(), w.ravel())
    return grid.reshape(n)


def _solve_terms(n, box, beta, epsilon_r, bsp):
    """Per half-complex point: eterm, m2, mh (3 arrays), corner factor; (0,0,0) masked out."""
    nx, ny, nz = n
    nzc = nz // 2 + 1
    kx = np.arange(nx)
    ky = np.arange(ny)
    kz = np.arange(nzc)
    mx = np.where(kx < (nx + 1) // 2, kx, kx - nx).astype(np.float64)
    my = np.where(ky < (ny + 1) // 2, ky, ky - ny).astype(np.float64)
    mz = kz.astype(np.float64)
    rec = [1.0 / float(np.float32(b)) for b in box]
    mhx = (mx * rec[0])[:, None, None] * np.ones((1, ny, nzc))
    mhy = (my * rec[1])[None, :, None] * np.ones((nx, 1, nzc))
    mhz = (mz * rec[2])[None, None, :] * np.ones((nx, ny, 1))
    m2 = mhx * mhx + mhy * mhy + mhz * mhz
    vol = float(np.float32(box[0])) * float(np.float32(box[1])) * float(np.float32(box[2]))
    denom = (m2 * bsp[2][:nzc][None, None, :] * (np.pi * vol * bsp[1])[None, :, None]
             * bsp[0][:, None, None])
    factor = np.pi * np.pi / (beta * beta)
    elfac = ONE_4PI_EPS0 / epsilon_r
    with np.errstate(divide="ignore", invalid="ignore"):
        eterm = elfac * np.exp(-factor * m2) / denom
    eterm[0, 0, 0] = 1.0  # the reference skips (0,0,0): the element stays unchanged
    corner = np.where((kz == 0) | (kz == (nz + 1) // 2), 0.5, 1.0)[None, None, :] * np.ones((nx, ny, 1))
    return eterm, m2, (mhx, mhy, mhz), corner, factor


def solve(cgrid: np.ndarray, n, box, beta: float, epsilon_r: float = 1.0, bsp=None):
    """Scaled half-complex grid [nx, ny, nz/2+1], energy and virial (3x3)."""
    if bsp is None:
        bsp = [bspline_moduli(n[d]) for d in range(3)]
    eterm, m2, (mhx, mhy, mhz), corner, factor = _solve_terms(n, box, beta, epsilon_r, bsp)
    c = np.asarray(cgrid, dtype=np.complex128)
    struct2 = 2.0 * (c.real ** 2 + c.imag ** 2)
    ets2 = corner * eterm * struct2
    ets2[0, 0, 0] = 0.0
    with np.errstate(divide="ignore", invalid="ignore"):
        vf = (factor * m2 + 1.0) * 2.0 / m2
    vf[0, 0, 0] = 0.0
    energy = 0.5 * ets2.sum()
    mh = (mhx, mhy, mhz)
    vir = np.zeros((3, 3))
    for a in range(3):
        for b in range(a + 1):
            vir[a, b] = vir[b, a] = 0.25 * (ets2 * vf * mh[b] * mh[a] - (ets2 if a == b else 0.0)).sum()
    return c * eterm, energy, vir


def solve_lj(cgrid: np.ndarray, n, box, beta_lj: float, bsp=None):
    """solve_pme_lj_yzx, geometric combination (one grid; pme_solve.cpp:588-915): the
    dispersion influence function, energy (0.5 sum) and virial (0.25 sum).  Unlike the
    Coulomb solve, the k = 0 element is scaled too."""
    if bsp is None:
        bsp = [bspline_moduli(n[d]) for d in range(3)]
    nx, ny, nz = n
    nzc = nz // 2 + 1
    kx = np.arange(nx)
    ky = np.arange(ny)
    kz = np.arange(nzc)
    mx = np.where(kx < (nx + 1) // 2, kx, kx - nx).astype(np.float64)
    my = np.where(ky < (ny + 1) // 2, ky, ky - ny).astype(np.float64)
    rec = [1.0 / float(np.float32(b)) for b in box]
    mhx = (mx * rec[0])[:, None, None] * np.ones((1, ny, nzc))
    mhy = (my * rec[1])[None, :, None] * np.ones((nx, 1, nzc))
    mhz = (kz * rec[2])[None, None, :] * np.ones((nx, ny, 1))
    m2 = mhx * mhx + mhy * mhy + mhz * mhz
    vol = float(np.float32(box[0])) * float(np.float32(box[1])) * float(np.float32(box[2]))
    factor = np.pi * np.pi / (beta_lj * beta_lj)
    by = 3.0 * vol * bsp[1] / (np.pi * math.sqrt(np.pi) * beta_lj ** 3)
    denom = bsp[2][:nzc][None, None, :] * by[None, :, None] * bsp[0][:, None, None]
    t1 = np.exp(-factor * m2)
    mk = np.sqrt(factor * m2)
    from scipy.special import erfc as _erfc

    t2 = math.sqrt(math.pi) * mk * _erfc(mk)
    m2k = factor * m2
    eterm = -((1.0 - 2.0 * m2k) * t1 + 2.0 * m2k * t2) / denom
    vterm = 3.0 * (-t1 + t2) / denom
    c = np.asarray(cgrid, dtype=np.complex128)
    struct2 = 2.0 * (c.real ** 2 + c.imag ** 2)
    corner = np.where((kz == 0) | (kz == (nz + 1) // 2), 0.5, 1.0)[None, None, :]
    ets2 = corner * eterm * struct2
    ets2vf = corner * 2.0 * factor * vterm * struct2
    energy = 0.5 * ets2.sum()
    mh = (mhx, mhy, mhz)
    vir = np.zeros((3, 3))
    for a in range(3):
        for b in range(a + 1):
            vir[a, b] = vir[b, a] = 0.25 * (ets2vf * mh[b] * mh[a] - (ets2 if a == b else 0.0)).sum()
    return c * eterm, energy, vir


def gather(grid, idx, theta, dtheta, q, n, box) -> np.ndarray:
    """Reciprocal-space forces [N, 3] (not added to anything)."""
    q = np.asarray(q, dtype=np.float64)
    gx, gy, gz = (_points(idx, n, d) for d in range(3))
    g = grid[gx[:, :, None, None], gy[:, None, :, None], gz[:, None, None, :]]  # [N,4,4,4]
    fx = np.einsum("ni,nj,nk,nijk->n", dtheta[0], theta[1], theta[2], g)
    fy = np.einsum("ni,nj,nk,nijk->n", theta[0], dtheta[1], theta[2], g)
    fz = np.einsum("ni,nj,nk,nijk->n", theta[0], theta[1], dtheta[2], g)
    rec = [1.0 / float(np.float32(b)) for b in box]
    f = np.stack([fx * n[0] * rec[0], fy * n[1] * rec[1], fz * n[2] * rec[2]], axis=1)
    return -q[:, None] * f


def compute(x, q, box, n, beta: float, epsilon_r: float = 1.0, single: bool = True, lj: bool = False):
    """Forces [N,3], energy and virial of the PME reciprocal part (gmx_pme_do): the Coulomb grid,
    or with lj=True the LJ-PME dispersion grid (q = sqrt(C6_ii), beta = beta_lj, geometric)."""
    n = tuple(int(v) for v in n)
    idx, theta, dtheta = splines(x, box, n, single)
    grid = spread(idx, theta, q, n)
    cgrid = np.fft.rfftn(grid)
    if lj:
        cgrid, energy, vir = solve_lj(cgrid, n, box, beta)
    else:
        cgrid, energy, vir = solve(cgrid, n, box, beta, epsilon_r)
    pot = np.fft.irfftn(cgrid, s=n, axes=(0, 1, 2)) * (n[0] * n[1] * n[2])  # unnormalised inverse
    f = gather(pot, idx, theta, dtheta, q, n, box)
    return f, energy, vir


def ewald_reciprocal_exact(x, q, box, beta: float, kmax, epsilon_r: float = 1.0):
    """Direct FP64 k-space Ewald sum: energy, forces [N,3], virial (3x3).

    E = f/(2 pi V) sum_{m != 0} exp(-pi^2 m^2 / beta^2) / m^2 |S(m)|^2 with
    S(m) = sum_j q_j exp(2 pi i m.x_j), m = (kx/Lx, ky/Ly, kz/Lz), |k| <= kmax per axis,
    f = ONE_4PI_EPS0 / epsilon_r; virial = 1/2 d E / d strain (GROMACS' sign)."""
    x = np.asarray(x, dtype=np.float64).reshape(-1, 3)
    q = np.asarray(q, dtype=np.float64)
    L = np.asarray(box, dtype=np.float64)
    vol = L.prod()
    fac = ONE_4PI_EPS0 / epsilon_r
    ks = [np.arange(-k, k + 1) for k in kmax]
    K = np.stack(np.meshgrid(*ks, indexing="ij"), -1).reshape(-1, 3)
    K = K[np.any(K != 0, axis=1)]
    m = K / L[None, :]
    m2 = (m * m).sum(1)
    w = np.exp(-np.pi ** 2 * m2 / beta ** 2) / m2
    phase = 2.0 * np.pi * x @ m.T  # [N, M]
    c, s = np.cos(phase), np.sin(phase)
    Sre = q @ c
    Sim = q @ s
    S2 = Sre ** 2 + Sim ** 2
    pref = fac / (2.0 * np.pi * vol)
    energy = pref * (w * S2).sum()
    # dE/dx_j = pref * sum_m w * 2 * q_j * (-Sre sin + Sim cos) * 2 pi m
    g = q[:, None] * (-s * Sre[None, :] + c * Sim[None, :])  # [N, M]
    grad = pref * 2.0 * 2.0 * np.pi * (g * w[None, :]) @ m
    forces = -grad
    vf = 2.0 * (1.0 + np.pi ** 2 * m2 / beta ** 2) / m2
    vir = np.zeros((3, 3))
    for a in range(3):
        for b in range(3):
            term = pref * w * S2 * (vf * m[:, a] * m[:, b] - (1.0 if a == b else 0.0))
            vir[a, b] = 0.5 * term.sum()
    return energy, forces, vir
