"""Seeded synthetic systems for the short-range nonbonded path.

These stand in for the reference's own benchmark input (the 3000-atom SPC/E
box of ``src/gromacs/nbnxm/benchmark/bench_coords.h`` used by
``gmx nonbonded-benchmark``): SPC water at the same number density
(~100 atoms/nm^3), built from a jittered lattice with random orientations,
plus a random multi-type LJ + Coulomb liquid for force matching.

Everything uses ``numpy.random.default_rng`` (PCG64), which gives the same
stream on x86-64 and aarch64.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

#: SPC water (rigid): LJ on oxygen only, q_O = -0.82, q_H = +0.41.
SPC_SIGMA = 0.3166
SPC_EPSILON = 0.650
SPC_Q_O = -0.82
SPC_Q_H = 0.41
OH_LENGTH = 0.1
HOH_ANGLE_DEG = 109.47


@dataclasses.dataclass
class System:
    """One periodic rectangular system in nblib terms.

    ``nbfp`` holds ``ntypes*ntypes`` pairs ``{6*C6, 12*C12}`` like
    nblib's non-bonded parameter array (api/nblib/gmxsetup.cpp:143-166);
    exclusions are a CSR list per atom that includes the atom itself
    (gmx::ListOfLists as built by nblib's Topology).
    """

    x: np.ndarray  # (N, 3) float32
    box: np.ndarray  # (3,) float32
    q: np.ndarray  # (N,) float32
    type: np.ndarray  # (N,) int32
    ntypes: int
    nbfp: np.ndarray  # (ntypes*ntypes*2,) float32
    excl_index: np.ndarray  # (N+1,) int32
    excl_list: np.ndarray  # (nnz,) int32
    name: str = ""
    # per-type LJ parameters when the system was built from sigma/epsilon
    sigma: np.ndarray | None = None
    epsilon: np.ndarray | None = None

    @property
    def n(self) -> int:
        return int(self.x.shape[0])


def lj_c6_c12(sigma: float, epsilon: float) -> tuple[float, float]:
    s6 = sigma**6
    return 4.0 * epsilon * s6, 4.0 * epsilon * s6 * s6


def nbfp_from_c6c12(c6: np.ndarray, c12: np.ndarray) -> np.ndarray:
    """(nt, nt) C6/C12 matrices -> nblib's flat {6*C6, 12*C12} array."""
    nt = c6.shape[0]
    out = np.empty((nt, nt, 2), dtype=np.float64)
    out[..., 0] = 6.0 * c6
    out[..., 1] = 12.0 * c12
    return out.reshape(-1).astype(np.float32)


def _random_rotations(rng: np.random.Generator, n: int) -> np.ndarray:
    """Uniform random rotation matrices (Shoemake's unit-quaternion method)."""
    u1, u2, u3 = rng.random((3, n))
    a = np.sqrt(1.0 - u1)
    b = np.sqrt(u1)
    qx = a * np.sin(2 * np.pi * u2)
    qy = a * np.cos(2 * np.pi * u2)
    qz = b * np.sin(2 * np.pi * u3)
    qw = b * np.cos(2 * np.pi * u3)
    r = np.empty((n, 3, 3))
    r[:, 0, 0] = 1 - 2 * (qy * qy + qz * qz)
    r[:, 0, 1] = 2 * (qx * qy - qz * qw)
    r[:, 0, 2] = 2 * (qx * qz + qy * qw)
    r[:, 1, 0] = 2 * (qx * qy + qz * qw)
    r[:, 1, 1] = 1 - 2 * (qx * qx + qz * qz)
    r[:, 1, 2] = 2 * (qy * qz - qx * qw)
    r[:, 2, 0] = 2 * (qx * qz - qy * qw)
    r[:, 2, 1] = 2 * (qy * qz + qx * qw)
    r[:, 2, 2] = 1 - 2 * (qx * qx + qy * qy)
    return r


def spc_water(n_molecules: int, box_edge: float, seed: int, jitter: float = 0.03) -> System:
    """SPC water box: oxygens on a jittered cubic lattice, random orientations.

    The lattice has m^3 >= n_molecules sites of spacing box_edge/m; when
    m^3 > n_molecules a seeded subset of sites is used.  Each oxygen gets a
    uniform jitter in [-jitter, jitter] per coordinate.
    """
    rng = np.random.default_rng(seed)
    m = int(math.ceil(n_molecules ** (1.0 / 3.0) - 1e-9))
    while m**3 < n_molecules:
        m += 1
    spacing = box_edge / m
    g = np.arange(m, dtype=np.float64)
    sites = np.stack(np.meshgrid(g, g, g, indexing="ij"), axis=-1).reshape(-1, 3)
    if sites.shape[0] > n_molecules:
        pick = np.sort(rng.choice(sites.shape[0], size=n_molecules, replace=False))
        sites = sites[pick]
    o = (sites + 0.5) * spacing + rng.uniform(-jitter, jitter, size=(n_molecules, 3))
    half = math.radians(HOH_ANGLE_DEG) / 2.0
    body = np.array(
        [
            [OH_LENGTH * math.sin(half), 0.0, OH_LENGTH * math.cos(half)],
            [-OH_LENGTH * math.sin(half), 0.0, OH_LENGTH * math.cos(half)],
        ]
    )
    rot = _random_rotations(rng, n_molecules)
    h = o[:, None, :] + np.einsum("nij,kj->nki", rot, body)
    x = np.empty((n_molecules, 3, 3))
    x[:, 0] = o
    x[:, 1:] = h
    x = x.reshape(-1, 3)
    n = 3 * n_molecules
    q = np.tile(np.array([SPC_Q_O, SPC_Q_H, SPC_Q_H], dtype=np.float32), n_molecules)
    types = np.tile(np.array([0, 1, 1], dtype=np.int32), n_molecules)
    c6o, c12o = lj_c6_c12(SPC_SIGMA, SPC_EPSILON)
    c6 = np.array([[c6o, 0.0], [0.0, 0.0]])
    c12 = np.array([[c12o, 0.0], [0.0, 0.0]])
    # every atom excludes its own molecule (itself included)
    excl_index = np.arange(0, 3 * n + 1, 3, dtype=np.int32)
    mol = np.arange(n) // 3
    excl_list = (3 * mol[:, None] + np.arange(3)[None, :]).reshape(-1).astype(np.int32)
    return System(
        x=x.astype(np.float32),
        box=np.full(3, box_edge, dtype=np.float32),
        q=q,
        type=types,
        ntypes=2,
        nbfp=nbfp_from_c6c12(c6, c12),
        excl_index=excl_index,
        excl_list=excl_list,
        name=f"spc{n_molecules}",
    )


def water_small(seed: int = 1) -> System:
    """1,000 SPC waters (3,000 atoms) in a 3.104 nm cubic box."""
    return spc_water(1000, 3.104, seed)


def water_large(seed: int = 2) -> System:
    """96,000 SPC waters (288,000 atoms) in a 14.21 nm cubic box."""
    return spc_water(96000, 14.21, seed)


ARGON_SIGMA, ARGON_EPSILON, ARGON_MASS = 0.3405, 0.996, 39.948


def lj_fcc(cells: int = 6, lattice: float = 0.5256, charge: float = 0.0, seed: int = 0) -> System:
    """Argon-like Lennard-Jones atoms on an fcc lattice (4 per cubic cell of edge `lattice`),
    one type; with `charge` > 0 half of the atoms (seeded choice) carry +charge and half -charge.
    A relaxed starting structure for MD (no overlaps), unlike the random liquids."""
    rng = np.random.default_rng(seed)
    g = np.arange(cells, dtype=np.float64)
    corners = np.stack(np.meshgrid(g, g, g, indexing="ij"), axis=-1).reshape(-1, 1, 3)
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])[None] + 0.25
    x = ((corners + basis).reshape(-1, 3) * lattice).astype(np.float32)
    n = x.shape[0]
    q = np.zeros(n, np.float32)
    if charge > 0:
        sign = np.ones(n)
        sign[rng.permutation(n)[: n // 2]] = -1.0
        q = (sign * charge).astype(np.float32)
    c6, c12 = lj_c6_c12(ARGON_SIGMA, ARGON_EPSILON)
    return System(
        x=x,
        box=np.full(3, cells * lattice, dtype=np.float32),
        q=q,
        type=np.zeros(n, np.int32),
        ntypes=1,
        nbfp=nbfp_from_c6c12(np.array([[c6]]), np.array([[c12]])),
        excl_index=np.arange(n + 1, dtype=np.int32),
        excl_list=np.arange(n, dtype=np.int32),
        name=f"ljfcc{n}",
    )


#: Madelung constant of the rock-salt lattice, referred to the nearest-neighbour distance
MADELUNG_ROCK_SALT = 1.747564594633182


def rock_salt(cells: int = 4, nn_distance: float = 0.282) -> System:
    """A perfect rock-salt crystal of unit charges: `cells`^3 conventional cubic cells
    (8 ions each, lattice constant 2 * nn_distance), no Lennard-Jones, no exclusions
    but self.  Its electrostatic energy is -N/2 * MADELUNG_ROCK_SALT / nn_distance
    (times 1/(4 pi eps0)) and the force on every ion is zero."""
    g = np.arange(2 * cells, dtype=np.float64)
    idx = np.stack(np.meshgrid(g, g, g, indexing="ij"), axis=-1).reshape(-1, 3)
    x = (idx + 0.25) * nn_distance
    q = np.where(idx.sum(1) % 2 == 0, 1.0, -1.0).astype(np.float32)
    n = x.shape[0]
    return System(
        x=x.astype(np.float32),
        box=np.full(3, 2 * cells * nn_distance, dtype=np.float32),
        q=q,
        type=np.zeros(n, np.int32),
        ntypes=1,
        nbfp=np.zeros(2, np.float32),
        excl_index=np.arange(n + 1, dtype=np.int32),
        excl_list=np.arange(n, dtype=np.int32),
        name=f"rocksalt{n}",
    )


def uneven_ensemble(
    num_systems: int = 256, seed: int = 3, n_min: int = 500, n_max: int = 20000
) -> list[System]:
    """Independent SPC water boxes with atom counts log-uniform in [n_min, n_max].

    N_i = 3*round(exp(U(ln n_min, ln n_max))/3); edge = (N_i/3 * 0.0299)^(1/3).
    """
    rng = np.random.default_rng(seed)
    out = []
    for s in range(num_systems):
        n = 3 * int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max))) / 3.0))
        nmol = n // 3
        edge = (nmol * 0.0299) ** (1.0 / 3.0)
        sysx = spc_water(nmol, edge, seed * 100003 + s)
        sysx.name = f"ens{s}_n{n}"
        out.append(sysx)
    return out


def perturb(x: np.ndarray, rng: np.random.Generator, sigma: float = 0.002) -> np.ndarray:
    """Gaussian displacement of every coordinate (the per-step drift of the MD-like run)."""
    return (x + rng.normal(0.0, sigma, size=x.shape)).astype(np.float32)


def _clashes(x, types, dmin, edge, pairs):
    """The pairs (from a k-d tree query) closer than their type pair's minimum distance."""
    if len(pairs) == 0:
        return np.zeros((0, 2), np.int64)
    d = x[pairs[:, 0]] - x[pairs[:, 1]]
    d -= edge * np.round(d / edge)
    close = np.einsum("ij,ij->i", d, d) < dmin[types[pairs[:, 0]], types[pairs[:, 1]]] ** 2
    return pairs[close]


def force_matching_specs(num_systems: int = 64, n_min: int = 2000, n_max: int = 50000, ntypes: int = 8,
                         seed: int = 5) -> list[dict]:
    """Arguments of ``lj_liquid`` for an ensemble of log-uniform sizes sharing one set of
    per-type sigma / epsilon (drawn as in ``lj_liquid``)."""
    rng = np.random.default_rng(seed)
    sig_t = rng.uniform(0.25, 0.40, size=ntypes)
    eps_t = rng.uniform(0.1, 1.0, size=ntypes)
    sizes = np.exp(rng.uniform(np.log(n_min), np.log(n_max), size=num_systems)).astype(int)
    return [dict(n=int(n), ntypes=ntypes, seed=int(seed * 1000 + k), type_sigma=sig_t, type_epsilon=eps_t)
            for k, n in enumerate(sizes)]


def _lj_liquid_kwargs(kw: dict) -> System:
    return lj_liquid(**kw)


def force_matching_ensemble(num_systems: int = 64, n_min: int = 2000, n_max: int = 50000, ntypes: int = 8,
                            seed: int = 5, processes: int = 1) -> list[System]:
    """Random LJ + Coulomb liquids of log-uniform size sharing per-type sigma / epsilon;
    positions, types and charges per system.  ``processes`` > 1 builds them in a
    spawn-started process pool (safe after CUDA is initialised)."""
    specs = force_matching_specs(num_systems, n_min, n_max, ntypes, seed)
    if processes <= 1:
        return [lj_liquid(**kw) for kw in specs]
    import multiprocessing as mp

    with mp.get_context("spawn").Pool(processes) as pool:
        return pool.map(_lj_liquid_kwargs, specs)


def lj_liquid(
    n: int = 24000,
    ntypes: int = 8,
    density: float = 100.0,
    seed: int = 4,
    min_dist_fraction: float = 0.5,
    q_sigma: float = 0.4,
    sigma_range: tuple[float, float] = (0.25, 0.40),
    epsilon_range: tuple[float, float] = (0.1, 1.0),
    type_sigma: np.ndarray | None = None,
    type_epsilon: np.ndarray | None = None,
) -> System:
    """Random multi-type LJ + Coulomb liquid with Lorentz-Berthelot mixing.

    Types are drawn uniformly per atom; sigma_t ~ U(sigma_range),
    epsilon_t ~ U(epsilon_range); charges ~ N(0, q_sigma) shifted to a zero
    total.  Positions are uniform in a cubic box at ``density``; every pair
    closer than ``min_dist_fraction * sigma_ij`` is rejected and the
    higher-numbered atom redrawn, from uniform candidates tested against the
    atoms already accepted (more candidates per round as the free volume
    shrinks), until no such pair is left (periodic k-d trees).  At 100 atoms/nm^3 a fraction of 0.8 packs beyond random close
    packing, so it cannot finish; 0.5 is the default (packing fraction ~0.22).
    """
    from scipy.spatial import cKDTree

    rng = np.random.default_rng(seed)
    edge = (n / density) ** (1.0 / 3.0)
    sig_t = rng.uniform(*sigma_range, size=ntypes)
    eps_t = rng.uniform(*epsilon_range, size=ntypes)
    # parameters shared by an ensemble replace the drawn ones (the draws keep the stream)
    if type_sigma is not None:
        sig_t = np.asarray(type_sigma, np.float64)
    if type_epsilon is not None:
        eps_t = np.asarray(type_epsilon, np.float64)
    types = rng.integers(0, ntypes, size=n).astype(np.int32)
    q = rng.normal(0.0, q_sigma, size=n)
    q = (q - q.mean()).astype(np.float32)
    sig_ij = 0.5 * (sig_t[:, None] + sig_t[None, :])
    eps_ij = np.sqrt(eps_t[:, None] * eps_t[None, :])
    dmin = min_dist_fraction * sig_ij
    rmax = float(dmin.max())
    x = rng.uniform(0.0, edge, size=(n, 3))
    # first pass: of every clashing pair the higher-numbered atom is redrawn
    tree = cKDTree(x, boxsize=edge)
    redo = np.unique(_clashes(x, types, dmin, edge, tree.query_pairs(rmax, output_type="ndarray")).max(axis=1))
    kcand, kngb = 8, 16  # candidates per atom and round: doubled while fewer than half the atoms place
    for _round in range(10000):
        if len(redo) == 0:
            break
        fixed = np.setdiff1d(np.arange(n), redo)
        tree = cKDTree(x[fixed], boxsize=edge)
        cand = rng.uniform(0.0, edge, size=(len(redo), kcand, 3))
        dist, idx = tree.query(cand.reshape(-1, 3), k=kngb, distance_upper_bound=rmax)
        near = np.isfinite(dist)
        tj = types[fixed[np.where(near, idx, 0)]]
        ti = np.repeat(types[redo], kcand)[:, None]
        bad = near & (dist < dmin[ti, tj])
        ok = ~bad.any(axis=1) & ~near[:, -1]  # a full neighbour list is rejected outright
        ok = ok.reshape(len(redo), kcand)
        has = ok.any(axis=1)
        if has.mean() < 0.5:
            kcand = min(2 * kcand, 256)
        first = ok.argmax(axis=1)
        placed = redo[has]
        x[placed] = cand[has, first[has]]
        # candidates placed in the same round may clash with each other
        still = set(redo[~has].tolist())
        if len(placed) > 1:
            t2 = cKDTree(x[placed], boxsize=edge)
            pp = _clashes(x[placed], types[placed], dmin, edge, t2.query_pairs(rmax, output_type="ndarray"))
            still.update(placed[pp.max(axis=1)].tolist() if len(pp) else [])
        redo = np.array(sorted(still), dtype=np.int64)
    else:
        raise RuntimeError("rejection sampling did not converge")
    c6 = 4.0 * eps_ij * sig_ij**6
    c12 = 4.0 * eps_ij * sig_ij**12
    return System(
        x=x.astype(np.float32),
        box=np.full(3, edge, dtype=np.float32),
        q=q,
        type=types,
        ntypes=ntypes,
        nbfp=nbfp_from_c6c12(c6, c12),
        excl_index=np.arange(n + 1, dtype=np.int32),
        excl_list=np.arange(n, dtype=np.int32),
        name=f"lj{n}",
        sigma=sig_t.astype(np.float64),
        epsilon=eps_t.astype(np.float64),
    )
