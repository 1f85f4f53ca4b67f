"""The reference's CPU cluster pair list (4-atom clusters, makeClusterListSimple) and the 4-wide
cluster-pair kernel of the CPU baseline (oracle/nbnxm_cpu_oracle.c), checked on the CPU.

The CPU list is checked the way the GPU list is: as the set of atom-pair images it covers.  Every
image of an atom pair within rlist that is not a topology exclusion must be in the list exactly
once (half shell: one orientation per pair), excluded pairs must have their interaction bits
cleared, and forces and energies computed on it must match the GPU-layout oracle.
"""
import numpy as np
import pytest

from gmxapi_gb300 import systems
from oracle import oracle as O
from tests.helpers import rel_rms

SYSTEMS = {
    "water900": lambda: systems.spc_water(300, 2.08, seed=5),
    "water_small_box": lambda: systems.spc_water(170, 1.72, seed=6),  # edge < 2 rlist: several images
    "lj_liquid": lambda: systems.lj_liquid(n=1500, ntypes=8, seed=8),
}


def _shift_vector(s):
    tz, r = divmod(s, 15)
    ty, tx = divmod(r, 5)
    return np.array([tx - 2, ty - 1, tz - 1])


def _canonical(i, j, n):
    """One key per image pair: (i, j, n) and (j, i, -n) are the same interaction."""
    if i > j or (i == j and tuple(-n) > tuple(n)):
        return (j, i, tuple(-n))
    return (i, j, tuple(n))


def _listed_pairs(s, c):
    pl = c.pairlist()
    ai = pl["atom_indices"]
    keys, excluded_bits = [], []
    for ci, shift, a, b in pl["ci"]:
        n = _shift_vector(shift)
        for cj, excl in pl["cj"][a:b]:
            for ii in range(4):
                i = ai[ci * 4 + ii]
                for jj in range(4):
                    j = ai[cj * 4 + jj]
                    if i < 0 or j < 0:
                        continue
                    bit = (int(excl) >> (ii * 4 + jj)) & 1
                    # the image of j seen from the shifted i: x_i + n L - x_j
                    key = _canonical(int(i), int(j), n)
                    (keys if bit else excluded_bits).append(key)
    return keys, excluded_bits


def _required_pairs(s, rlist):
    box = np.asarray(s.box, np.float64)
    x = np.asarray(s.x, np.float64) % box
    excl = set()
    for i in range(s.n):
        for j in s.excl_list[s.excl_index[i]:s.excl_index[i + 1]]:
            excl.add((min(i, int(j)), max(i, int(j))))
    req = set()
    rng = [-2, -1, 0, 1, 2]
    for tx in rng:
        for ty in rng[1:4]:
            for tz in rng[1:4]:
                n = np.array([tx, ty, tz])
                d = x[:, None, :] + n * box - x[None, :, :]
                r2 = (d ** 2).sum(-1)
                ii, jj = np.nonzero(r2 < rlist * rlist)
                for i, j in zip(ii, jj):
                    if i == j and tx == 0 and ty == 0 and tz == 0:
                        continue
                    if (min(i, j), max(i, j)) in excl:
                        continue
                    req.add(_canonical(int(i), int(j), n))
    return req


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_cpu_list_covers_every_pair_within_rlist_once(name):
    s = SYSTEMS[name]()
    c = O.CpuOracle(s, rc=0.9, rlist=1.0)
    c.grid()
    c.search()
    keys, _ = _listed_pairs(s, c)
    assert len(keys) == len(set(keys)), "an atom-pair image is listed twice"
    missing = _required_pairs(s, 1.0) - set(keys)
    assert not missing, sorted(missing)[:5]


def test_cpu_list_clears_the_exclusion_bits():
    s = SYSTEMS["water900"]()
    c = O.CpuOracle(s, rc=0.9, rlist=1.0)
    c.grid()
    c.search()
    keys, cleared = _listed_pairs(s, c)
    excl = {(i, int(j)) for i in range(s.n) for j in s.excl_list[s.excl_index[i]:s.excl_index[i + 1]] if i < j}
    in_list_excluded = {(k[0], k[1]) for k in keys if k[2] == (0, 0, 0)} & excl
    assert not in_list_excluded
    # every intramolecular pair appears with its bits cleared (the molecules are whole in the box)
    assert excl <= {(k[0], k[1]) for k in cleared}


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_cpu_kernel_matches_the_gpu_layout_oracle(name):
    s = SYSTEMS[name]()
    o = O.Oracle(s, rc=0.9, rlist=1.0)
    o.grid()
    o.search()
    o.force(True)
    c = O.CpuOracle(s, rc=0.9, rlist=1.0, beta=o.beta)
    c.grid()
    c.search()
    for threads in (1, 3):
        c.force(True, threads=threads)
        assert rel_rms(c.forces(), o.forces()) <= 1e-5
        e, eo = c.energies(), o.energies()
        # LJ to 1e-6; the Coulomb sum of the 4-wide kernel is in float per vector lane
        assert abs(e[0] - eo[0]) <= 1e-6 * abs(eo[0])
        assert abs(e[1] - eo[1]) <= 2e-5 * abs(eo[1])
