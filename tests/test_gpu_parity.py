"""CUDA path vs the CPU oracle, through the C ABI (needs a GB300).

Bars (from the path's specification):
  grid and pair list: bit-exact (lists compared as sorted sets of cluster
  pairs with their 64-bit atom-pair masks);
  forces: relative RMS <= 1e-5 against the oracle; energies relative <= 1e-6;
  every case also reports its error against the FP64 all-pairs sum.
"""
import numpy as np
import pytest

from gmxapi_gb300 import nblib, systems
from oracle import oracle as O
from tests.helpers import canonical_pairs, nblib_golden_system, rel_rms

pytestmark = pytest.mark.gpu

FORCE_RTOL = 1e-5
ENERGY_RTOL = 1e-6
# Reaction field sums q_i q_j (1/r - c_rf) over every pair out to rc with
# float 1/r, whose rounding alone puts a ~2e-6 noise floor on the total; the
# Ewald path (all benchmark configurations) keeps the 1e-6 bar.
ENERGY_RTOL_RF = 5e-6


def _pair(s, coulomb=nblib.CoulombType.Pme, rc=0.9, rlist=1.0, rlist_inner=None, prune=0):
    opts = nblib.NBKernelOptions(coulomb_type=coulomb, pairlist_cutoff=rlist, rcoulomb=rc,
                                 rlist_inner=rlist_inner, nstlist_prune=prune,
                                 compute_virial_and_energy=True)
    calc = nblib.ForceCalculator(s, opts)
    o = O.Oracle(s, coulomb=int(coulomb), rc=rc, rlist=rlist, rlist_inner=rlist_inner)
    o.grid()
    o.search()
    # the same split + size sort the engine applies to its list
    o.balance(calc.list_balance()["min_ci_balanced"])
    return calc, o


SYSTEMS = {
    "water3000": lambda: systems.water_small(),
    "water900": lambda: systems.spc_water(300, 2.08, seed=5),
    "water_small_box": lambda: systems.spc_water(170, 1.72, seed=6),  # edge < 2 rlist: multiple images
    "water_tiny": lambda: systems.spc_water(20, 0.84, seed=7),        # <= 64 atoms: one cell, shp_x = 2
    "lj_liquid": lambda: systems.lj_liquid(n=1500, ntypes=8, seed=8),
    # 47 types + the filler type, the most the kernels accept: the type table no longer fits the
    # default 48 KB of shared memory
    "lj_47_types": lambda: systems.lj_liquid(n=3000, ntypes=47, seed=9),
}


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_grid_bit_exact(name):
    s = SYSTEMS[name]()
    calc, o = _pair(s)
    g = calc.grid()
    r = o.grid_arrays()
    assert g["ncx"] == r["ncx"] and g["ncy"] == r["ncy"] and g["ncells"] == r["ncells"]
    np.testing.assert_array_equal(g["cxy_ind"], r["cxy_ind"])
    np.testing.assert_array_equal(g["num_clusters"], r["num_clusters"])
    np.testing.assert_array_equal(g["atom_indices"], r["atom_indices"])
    np.testing.assert_array_equal(g["cells"], r["cells"])
    np.testing.assert_array_equal(g["bbcz"], r["bbcz"])
    np.testing.assert_array_equal(g["xq"], r["xq"])
    # bounding boxes of the clusters in use
    used = np.concatenate([np.arange(c * 8, c * 8 + k) for c, k in enumerate(r["num_clusters"])])
    np.testing.assert_array_equal(g["bb"][used], r["bb"][used])


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_pairlist_bit_exact_as_sorted_sets(name):
    s = SYSTEMS[name]()
    calc, o = _pair(s)
    pg = calc.pairlist()
    po = o.pairlist()
    a = canonical_pairs(pg["sci"], pg["cj4"], pg["excl"])
    b = canonical_pairs(po["sci"], po["cj4"], po["excl"])
    assert len(a) == len(b)
    assert np.array_equal(a, b)
    # same entries (sci, shift) and cj4 count
    assert sorted(map(tuple, pg["sci"][:, :2])) == sorted(map(tuple, po["sci"][:, :2]))
    assert len(pg["cj4"]) == len(po["cj4"])


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_balanced_list_entries_match_oracle_in_order(name):
    """Split + large-first sort (split_sci_entry / sort_sci): the same entries in the same order."""
    s = SYSTEMS[name]()
    calc, o = _pair(s)
    bal = calc.list_balance()
    pg, po = calc.pairlist(), o.pairlist()
    np.testing.assert_array_equal(pg["sci"], po["sci"])
    sizes = pg["sci"][:, 3] - pg["sci"][:, 2]
    assert bal["entries"] == len(pg["sci"]) >= bal["entries_unsplit"]
    if bal["nsp_max"] > 0 and len(pg["cj4"]) > 0:
        # pieces are close to the target: no piece above twice its pair budget
        m0 = np.array([bin(int(v)).count("1") for v in pg["cj4"][:, 4].astype(np.uint32)])
        pairs = np.array([m0[a:b].sum() for a, b in pg["sci"][:, 2:4]])
        assert (pairs[sizes > 1] <= 2 * bal["nsp_max"] + 32).all()
    # large first, up to the size-class cap of twice the average
    cap = min(255, (2 * len(pg["cj4"])) // max(1, len(sizes)))
    cls = np.minimum(sizes, cap)
    assert (np.diff(cls) <= 0).all()


def _long_list_water(n_molecules=3000, seed=11):
    # water at rlist 2.0 nm: its cells find up to ~780 j-clusters (9,000 atoms), more than the 512
    # search records a cell starts with
    return systems.spc_water(n_molecules, (n_molecules * 0.0299) ** (1 / 3), seed=seed)


def test_search_records_grow_for_long_lists():
    """A cell that finds more j-clusters than its search records hold makes the search grow them and
    count again: the list and the forces still match the oracle."""
    s = _long_list_water()
    calc, o = _pair(s, rlist=2.0)
    pg, po = calc.pairlist(), o.pairlist()
    a = canonical_pairs(pg["sci"], pg["cj4"], pg["excl"])
    b = canonical_pairs(po["sci"], po["cj4"], po["excl"])
    assert len(a) == len(b) and np.array_equal(a, b)
    f = calc.compute(s.x)
    o.force(True)
    assert rel_rms(f, o.forces()) <= FORCE_RTOL
    calc.close()


def test_balancing_leaves_forces_unchanged():
    s = systems.water_small()
    calc, _o = _pair(s)
    f1 = calc.compute(s.x).copy()
    e1 = calc.energies.copy()
    calc.set_list_balance(0)
    calc.update_pairlist(s.x)
    assert calc.list_balance()["nsp_max"] == 0
    f2 = calc.compute(s.x)
    assert rel_rms(f2, f1) < 1e-6
    np.testing.assert_allclose(calc.energies, e1, rtol=1e-7)


@pytest.mark.parametrize("name", ["water3000", "water_small_box"])
def test_fresh_prune_masks_bit_exact(name):
    s = SYSTEMS[name]()
    calc, o = _pair(s, rlist_inner=0.95, prune=10)  # the engine prunes the fresh list at creation
    o.prune(fresh=True)
    pg = calc.pairlist()
    po = o.pairlist()
    assert np.array_equal(canonical_pairs(pg["sci"], pg["cj4"], pg["excl"]),
                          canonical_pairs(po["sci"], po["cj4"], po["excl"]))
    # outer masks, keyed by the canonical list position of each cj4
    def outer_sets(p):
        rows = []
        for sc, sh, c0, c1 in p["sci"]:
            for j4 in range(c0, c1):
                rows.append((sc, sh, tuple(p["cj4"][j4][:4]), tuple(p["imask_outer"][j4])))
        return sorted(rows)
    assert outer_sets(pg) == outer_sets(po)


@pytest.mark.parametrize("name", list(SYSTEMS))
@pytest.mark.parametrize("coulomb", [nblib.CoulombType.Pme, nblib.CoulombType.ReactionField])
def test_forces_energies_virial_vs_oracle(name, coulomb):
    s = SYSTEMS[name]()
    calc, o = _pair(s, coulomb=coulomb)
    f = calc.compute(s.x)
    e = calc.energies
    vir = calc.virial
    o.force(True)
    fo = o.forces()
    eo = o.energies()
    assert rel_rms(f, fo) <= FORCE_RTOL
    etol = ENERGY_RTOL if coulomb == nblib.CoulombType.Pme else ENERGY_RTOL_RF
    for k in range(2):
        if abs(eo[k]) > 0:
            assert abs(e[k] - eo[k]) <= etol * abs(eo[k]) + 1e-9, (k, e[k], eo[k])
    g = calc.grid()
    xin = g["xq"][g["cells"], :3]
    vo = o.virial(xin, fo)
    # the virial sums x_i (x) f_i: force errors within the force bar allow at most
    # ~FORCE_RTOL * sqrt(sum |x_i|^2 |f_i|^2) in each component
    scale = np.sqrt(np.sum((xin.astype(np.float64) ** 2).sum(1) * (fo.astype(np.float64) ** 2).sum(1)))
    assert np.abs(vir - vo).max() <= FORCE_RTOL * scale + 1e-9 * np.abs(vo).max()
    # error against the FP64 explicit-image sum is reported and bounded
    f64, e64 = O.fp64_allpairs(s, coulomb=int(coulomb), rc=0.9, beta=o.beta if coulomb == 0 else None)
    err64 = rel_rms(f, f64)
    print(f"{name} coulomb={int(coulomb)}: rel RMS vs oracle {rel_rms(f, fo):.2e}, vs FP64 {err64:.2e}")
    assert err64 <= 1e-5


@pytest.mark.parametrize("shape", [(0, 2, 2), (1, 3, 2), (1, 2, 3), (1, 3, 3)])
@pytest.mark.parametrize("name", ["water3000", "water_small_box", "water_tiny", "lj_liquid"])
@pytest.mark.parametrize("coulomb", [nblib.CoulombType.Pme, nblib.CoulombType.ReactionField])
def test_force_kernel_shapes_vs_oracle(name, coulomb, shape):
    """The other force-kernel shapes (one pair per lane; two pairs per lane with three stage buffers
    and/or three blocks per SM) against the oracle, F only and F + E; the default shape (two pairs
    per lane, two buffers, two blocks) is covered above."""
    s = SYSTEMS[name]()
    calc, o = _pair(s, coulomb=coulomb)
    calc.set_force_kernel(*shape)
    assert calc.force_kernel() == shape
    o.force(True)
    fo, eo = o.forces(), o.energies()
    f = calc.compute(s.x).copy()
    assert rel_rms(f, fo) <= FORCE_RTOL
    etol = ENERGY_RTOL if coulomb == nblib.CoulombType.Pme else ENERGY_RTOL_RF
    for k in range(2):
        if abs(eo[k]) > 0:
            assert abs(calc.energies[k] - eo[k]) <= etol * abs(eo[k]) + 1e-9, (k, calc.energies[k], eo[k])
    f_only = calc.compute(s.x, energies=False)
    assert rel_rms(f_only, fo) <= FORCE_RTOL


@pytest.mark.parametrize("key", ["argon", "spc_methanol"])
def test_nblib_golden_forces(key):
    """The reference's own nblib golden vectors (Cutoff Coulomb, rc = rlist = 1.0)."""
    s, ref = nblib_golden_system(key)
    opts = nblib.NBKernelOptions(coulomb_type=nblib.CoulombType.Cutoff, pairlist_cutoff=1.0)
    calc = nblib.ForceCalculator(s, opts)
    f = calc.compute(s.x)
    assert rel_rms(f, ref) <= FORCE_RTOL
    assert np.abs(f - ref).max() <= 5e-5 * np.abs(ref).max()


def test_rolling_prune_matches_oracle():
    s = systems.water_small()
    calc, o = _pair(s, rlist_inner=0.93, prune=10)
    o.prune(fresh=True)
    rng = np.random.default_rng(3)
    x = s.x.copy()
    for part in range(5):
        x = systems.perturb(x, rng, 0.01)
        calc.compute(x)  # converts x into the grid layout
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


def test_update_pairlist_after_motion():
    s = systems.spc_water(300, 2.08, seed=12)
    calc, o = _pair(s)
    x = systems.perturb(s.x, np.random.default_rng(1), 0.05)
    calc.update_pairlist(x)
    o.set_coordinates(x)
    o.grid()
    o.search()
    o.balance(calc.list_balance()["min_ci_balanced"])
    pg, po = calc.pairlist(), o.pairlist()
    np.testing.assert_array_equal(pg["sci"], po["sci"])
    assert np.array_equal(canonical_pairs(pg["sci"], pg["cj4"], pg["excl"]),
                          canonical_pairs(po["sci"], po["cj4"], po["excl"]))
    f = calc.compute(x)
    o.set_x(x)
    o.force(False)
    assert rel_rms(f, o.forces()) <= FORCE_RTOL


def test_invalid_input_raises():
    s = systems.spc_water(30, 1.0, seed=1)
    bad = systems.spc_water(30, 1.0, seed=1)
    bad.x[3, 1] = np.nan
    with pytest.raises(nblib.InputException):
        nblib.ForceCalculator(bad)
    calc = nblib.ForceCalculator(s)
    with pytest.raises(nblib.InputException):
        calc.compute(np.zeros((5, 3), np.float32))


def test_repeat_compute_stable_and_changes_after_update():
    """UpdateChangesForces (api/nblib/tests/nbkernelsystem.cpp:137-185).

    The GPU sums forces with atomics, so repeats agree to rounding, not bitwise."""
    s, _ = nblib_golden_system("spc_methanol")
    calc = nblib.ForceCalculator(s, nblib.NBKernelOptions(coulomb_type=nblib.CoulombType.Cutoff))
    f1 = calc.compute(s.x).copy()
    f2 = calc.compute(s.x)
    assert rel_rms(f2, f1) < 1e-6
    x2 = systems.perturb(s.x, np.random.default_rng(0), 0.001)
    f3 = calc.compute(x2)
    assert np.all(f3 != f1)


def test_large_box_force_error_vs_fp64_on_subset():
    """The 288,000-atom SPC box (96,000 molecules, 14.21 nm): GPU forces on a random
    3,000-atom subset against the FP64 explicit-image sum."""
    s = systems.water_large()
    opts = nblib.NBKernelOptions(coulomb_type=nblib.CoulombType.Pme, pairlist_cutoff=1.0, rcoulomb=0.9,
                                 compute_virial_and_energy=True)
    calc = nblib.ForceCalculator(s, opts)
    f = calc.compute(s.x)
    sub = np.sort(np.random.default_rng(17).choice(s.n, 3000, replace=False)).astype(np.int32)
    beta = O.Oracle(systems.water_small(), rc=0.9, rlist=1.0).beta  # beta depends on rc and rtol only
    f64, _ = O.fp64_allpairs(s, coulomb=0, rc=0.9, beta=beta, subset=sub)
    err = rel_rms(f[sub], f64)
    print(f"288k box, 3000-atom subset: rel RMS vs FP64 {err:.2e}")
    assert err <= 1e-5


@pytest.mark.parametrize("mod", [nblib.VdwModifier.ForceSwitch, nblib.VdwModifier.PotSwitch,
                                 nblib.VdwModifier.NoModifier])
@pytest.mark.parametrize("name", ["water3000", "lj_liquid"])
def test_lj_modifiers_vs_oracle(name, mod):
    """vdw-modifier force switch / potential switch (rvdw_switch 0.7 nm) and plain cut-off:
    forces, energies and virial against the oracle (kernel_ref_inner.h switch terms) and
    forces against the FP64 sum."""
    s = SYSTEMS[name]()
    opts = nblib.NBKernelOptions(coulomb_type=nblib.CoulombType.Pme, pairlist_cutoff=1.0, rcoulomb=0.9,
                                 compute_virial_and_energy=True, vdw_modifier=mod, rvdw_switch=0.7)
    calc = nblib.ForceCalculator(s, opts)
    o = O.Oracle(s, rc=0.9, rlist=1.0, vdw_modifier=int(mod), rvdw_switch=0.7)
    o.grid()
    o.search()
    o.balance(calc.list_balance()["min_ci_balanced"])
    f = calc.compute(s.x)
    o.force(True)
    assert rel_rms(f, o.forces()) <= FORCE_RTOL
    eo = o.energies()
    for k in range(2):
        assert abs(calc.energies[k] - eo[k]) <= ENERGY_RTOL * abs(eo[k]) + 1e-9, (k, calc.energies[k], eo[k])
    f64, _ = O.fp64_allpairs(s, rc=0.9, beta=o.beta, vdw_modifier=int(mod), rvdw_switch=0.7)
    assert rel_rms(f, f64) <= FORCE_RTOL


def test_switch_modifiers_rejected_where_unsupported():
    s = systems.lj_liquid(n=600, ntypes=4, seed=3)
    with pytest.raises(nblib.InputException):
        nblib.ForceCalculator(s, nblib.NBKernelOptions(vdw_modifier=nblib.VdwModifier.ForceSwitch,
                                                       rvdw_switch=1.2))


def _water_like(x, q, types, box, excl=None):
    n = len(x)
    ei = np.arange(n + 1, dtype=np.int32) if excl is None else excl[0]
    el = np.arange(n, dtype=np.int32) if excl is None else excl[1]
    w = systems.water_small()
    return systems.System(x=np.asarray(x, np.float32).reshape(-1, 3), box=np.asarray(box, np.float32),
                          q=np.asarray(q, np.float32), type=np.asarray(types, np.int32), ntypes=w.ntypes,
                          nbfp=w.nbfp, excl_index=ei, excl_list=el, name="edge")


@pytest.mark.parametrize("coulomb", [nblib.CoulombType.Pme, nblib.CoulombType.ReactionField])
def test_single_atom_only_self_energy(coulomb):
    """One charged atom: no pairs, zero force, the energy is the self term alone."""
    s = _water_like([[0.5, 0.6, 0.7]], [0.5], [0], [3.0, 3.0, 3.0])
    calc, o = _pair(s, coulomb=coulomb)
    f = calc.compute(s.x)
    o.force(True)
    assert np.all(f == 0.0)
    np.testing.assert_allclose(calc.energies, o.energies(), rtol=1e-6, atol=1e-9)
    assert calc.energies[1] < 0 and calc.energies[0] == 0.0


def test_coincident_charges_stay_finite():
    """Two non-excluded charges (no LJ) at the same position: the minimum-distance clamp
    (c_nbnxnMinDistanceSquared, pairlist.h:146) keeps the Coulomb terms finite, as in the
    reference.  (With LJ, 12 C12 r^-14 at the clamp overflows float in the reference too.)"""
    s = _water_like([[1.0, 1.0, 1.0], [1.0, 1.0, 1.0], [1.5, 1.1, 1.0]], [0.4, -0.3, 0.1], [1, 1, 1],
                    [3.0, 3.0, 3.0])
    calc, o = _pair(s)
    f = calc.compute(s.x)
    o.force(True)
    assert np.all(np.isfinite(f)) and np.all(np.isfinite(calc.energies))
    assert rel_rms(f, o.forces()) <= FORCE_RTOL
    np.testing.assert_allclose(calc.energies, o.energies(), rtol=1e-5)


def test_list_grows_when_atoms_spread_out():
    """Atoms first crowded into one corner octant, then spread over the whole box: the
    search count pass finds a longer list and the capacity grows before the write pass."""
    s = systems.spc_water(300, 2.08, seed=5)
    x = s.x.copy()
    s.x = (x * np.float32(0.5)).astype(np.float32)
    calc, o = _pair(s)
    n0 = calc.sizes()["num_cj4"]
    calc.update_pairlist(x)
    o.set_coordinates(x)
    o.grid()
    o.search()
    o.balance(calc.list_balance()["min_ci_balanced"])
    assert calc.sizes()["num_cj4"] > n0
    pg, po = calc.pairlist(), o.pairlist()
    assert np.array_equal(canonical_pairs(pg["sci"], pg["cj4"], pg["excl"]),
                          canonical_pairs(po["sci"], po["cj4"], po["excl"]))
    f = calc.compute(x)
    o.set_x(x)
    o.force(False)
    assert rel_rms(f, o.forces()) <= FORCE_RTOL


def test_far_outside_box_is_an_input_error():
    """put_atoms_in_box bound: a coordinate more than 127 box lengths out is rejected."""
    s = systems.spc_water(30, 1.0, seed=1)
    calc = nblib.ForceCalculator(s)
    x = s.x.copy()
    x[0, 0] += 200.0
    with pytest.raises(nblib.InputException):
        calc.update_pairlist(x)
