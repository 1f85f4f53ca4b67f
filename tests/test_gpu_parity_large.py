"""Parity at the benchmark sizes: CUDA path vs the CPU oracle through the C ABI (GB300).

The 288,000-atom SPC water box (96,000 molecules, 14.21 nm, rc 0.9, rlist 1.0, rlist_inner 0.95)
the benchmark runs: grid arrays bit-exact, the pair list bit-exact as sorted sets of cluster pairs
with their atom-pair masks, the fresh prune's inner and outer masks, two parts of the rolling
prune after the coordinates moved, and forces / energies / virial within the force (1e-5 relative
RMS) and energy (1e-6) bars.  And a 32-system ensemble drawn from the benchmark's law (500 to
20,000 atoms, log-uniform; seven systems below 800 atoms, whose boxes are shorter than 2 rlist),
every system of the batched launch against the oracle.
"""
import numpy as np
import pytest

from gmxapi_gb300 import nblib, systems
from oracle import oracle as O
from tests.helpers import canonical_pairs, rel_rms

pytestmark = pytest.mark.gpu

FORCE_RTOL = 1e-5
ENERGY_RTOL = 1e-6
RLIST_INNER = 0.95


@pytest.fixture(scope="module")
def large():
    s = systems.water_large()
    opts = nblib.NBKernelOptions(coulomb_type=nblib.CoulombType.Pme, pairlist_cutoff=1.0, rcoulomb=0.9,
                                 rlist_inner=RLIST_INNER, nstlist=100, nstlist_prune=10,
                                 compute_virial_and_energy=True)
    calc = nblib.ForceCalculator(s, opts)  # grids, searches, balances and prunes the fresh list
    o = O.Oracle(s, rc=0.9, rlist=1.0, rlist_inner=RLIST_INNER)
    o.grid()
    o.search()
    o.balance(calc.list_balance()["min_ci_balanced"])
    o.prune(fresh=True)
    yield s, calc, o
    calc.close()


def _outer_sets(p):
    rows = []
    for sc, sh, c0, c1 in p["sci"]:
        for j4 in range(c0, c1):
            rows.append((sc, sh, tuple(p["cj4"][j4][:4]), tuple(p["imask_outer"][j4])))
    return sorted(rows)


def test_large_grid_bit_exact(large):
    s, calc, o = large
    g, r = calc.grid(), o.grid_arrays()
    assert (g["ncx"], g["ncy"], g["ncells"]) == (r["ncx"], r["ncy"], r["ncells"])
    for k in ("cxy_ind", "num_clusters", "atom_indices", "cells", "bbcz", "xq"):
        np.testing.assert_array_equal(g[k], r[k], err_msg=k)
    used = np.concatenate([np.arange(c * 8, c * 8 + k) for c, k in enumerate(r["num_clusters"])])
    np.testing.assert_array_equal(g["bb"][used], r["bb"][used])


def test_large_pairlist_and_fresh_prune_bit_exact(large):
    """Entries in the same order after balancing; the pair sets with the fresh prune's inner masks
    (rlist_inner) and the outer masks (rlist) kept for the rolling prune."""
    s, calc, o = large
    pg, po = calc.pairlist(), o.pairlist()
    np.testing.assert_array_equal(pg["sci"], po["sci"])
    a = canonical_pairs(pg["sci"], pg["cj4"], pg["excl"])
    b = canonical_pairs(po["sci"], po["cj4"], po["excl"])
    assert len(a) == len(b) > 1_000_000
    assert np.array_equal(a, b)
    assert _outer_sets(pg) == _outer_sets(po)


def test_large_forces_energies_virial_vs_oracle(large):
    s, calc, o = large
    f = calc.compute(s.x).copy()
    e, vir = calc.energies.copy(), calc.virial.copy()
    o.force(True)
    fo, eo = o.forces(), o.energies()
    err = rel_rms(f, fo)
    assert err <= FORCE_RTOL
    assert np.all(np.abs(e - eo) <= ENERGY_RTOL * np.abs(eo)), (e, eo)
    g = calc.grid()
    xin = g["xq"][g["cells"], :3]
    vo = o.virial(xin, fo)
    scale = np.sqrt(np.sum((xin.astype(np.float64) ** 2).sum(1) * (fo.astype(np.float64) ** 2).sum(1)))
    assert np.abs(vir - vo).max() <= FORCE_RTOL * scale
    print(f"288k: forces rel RMS vs oracle {err:.2e}, energies {np.abs(e - eo) / np.abs(eo)}")


def test_large_rolling_prune_two_parts_bit_exact(large):
    """Two of the five rolling-prune parts after two perturbed steps (sigma 0.002 nm, as the
    benchmark moves the atoms), then the forces on the pruned list."""
    s, calc, o = large
    rng = np.random.default_rng(31)
    x = s.x.copy()
    for part in range(2):
        x = systems.perturb(x, rng, 0.002)
        calc.compute(x)  # converts x into the grid layout with the last search's shifts
        calc.prune_device(part)
        calc.synchronize()
        o.set_x(x)
        o.prune(fresh=False, part=part, nparts=5)
    pg, po = calc.pairlist(), o.pairlist()
    assert np.array_equal(canonical_pairs(pg["sci"], pg["cj4"], pg["excl"]),
                          canonical_pairs(po["sci"], po["cj4"], po["excl"]))
    f = calc.compute(x)
    o.force(True)
    assert rel_rms(f, o.forces()) <= FORCE_RTOL


def test_ensemble_32_systems_each_vs_oracle():
    """32 systems of the uneven ensemble in one batched launch; every system's forces, energies
    and virial against its own oracle (the batch is not compared with itself)."""
    torch = pytest.importorskip("torch")
    from gmxapi_gb300.batch import BatchForceCalculator

    ens = systems.uneven_ensemble(32, seed=5, n_min=500, n_max=20000)
    assert sum(s.n < 800 for s in ens) >= 5 and max(s.n for s in ens) > 19000
    opts = nblib.NBKernelOptions(coulomb_type=nblib.CoulombType.Pme, pairlist_cutoff=1.0, rcoulomb=0.9,
                                 nstlist=10, compute_virial_and_energy=True)
    b = BatchForceCalculator(ens, opts)
    dev = torch.device("cuda:0")
    x = torch.from_numpy(np.concatenate([s.x.reshape(-1) for s in ens])).to(dev)
    f = torch.empty_like(x)
    e = torch.zeros(2 * len(ens), dtype=torch.float64, device=dev)
    v = torch.zeros(9 * len(ens), dtype=torch.float64, device=dev)
    b.compute_device(x.data_ptr(), f.data_ptr(), e.data_ptr(), v.data_ptr())
    torch.cuda.synchronize()
    fb = f.cpu().numpy()
    eb = e.cpu().numpy().reshape(-1, 2)
    vb = v.cpu().numpy().reshape(-1, 3, 3)
    b.close()
    worst = 0.0
    for i, s in enumerate(ens):
        o = O.Oracle(s, rc=0.9, rlist=1.0)
        o.grid()
        o.search()
        o.force(True)
        fo, eo = o.forces(), o.energies()
        off = b.offsets[i]
        fi = fb[3 * off:3 * (off + s.n)].reshape(-1, 3)
        err = rel_rms(fi, fo)
        worst = max(worst, err)
        assert err <= FORCE_RTOL, (i, s.n, err)
        assert np.all(np.abs(eb[i] - eo) <= ENERGY_RTOL * np.abs(eo)), (i, s.n, eb[i], eo)
        xin = o.grid_arrays()["xq"][o.grid_arrays()["cells"], :3]
        vo = o.virial(xin, fo)
        scale = np.sqrt(np.sum((xin.astype(np.float64) ** 2).sum(1) * (fo.astype(np.float64) ** 2).sum(1)))
        assert np.abs(vb[i] - vo).max() <= FORCE_RTOL * scale, (i, s.n)
    print(f"32-system ensemble ({sum(s.n for s in ens)} atoms): worst force rel RMS vs oracle {worst:.2e}")
