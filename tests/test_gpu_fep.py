"""The perturbed-pair (free-energy) kernel through the C ABI vs the free-energy oracle (needs a GB300).

Bars: total forces (cluster path + perturbed pairs) rel-RMS <= 1e-5 and energies <= 1e-5 against
the FP64 oracle sum (all-pairs over the masked system + the free-energy oracle); the perturbed-pair
energies and dV/dlambda within 1e-5 of the system's energy (+1e-4 relative) of the oracle's; with
state B equal to A and no soft-core, forces, energies and the virial equal the plain path's at
every lambda.
"""
import numpy as np
import pytest

from gmxapi_gb300 import nblib, systems
from oracle import fep_oracle as F
from oracle import oracle as O
from tests.helpers import rel_rms
from tests.test_fep_oracle import EPS_RF, RC, _ic, _masked

pytestmark = pytest.mark.gpu


def _system(name):
    if name == "water":
        return systems.spc_water(300, 2.08, seed=5)
    if name == "lj":
        return systems.lj_liquid(n=1500, ntypes=4, seed=8)
    # the LJ liquid with an extra all-zero type: atoms that vanish in state B
    s = systems.lj_liquid(n=1500, ntypes=4, seed=8)
    nt = s.ntypes
    nb = np.zeros((nt + 1, nt + 1, 2), np.float32)
    nb[:nt, :nt] = np.asarray(s.nbfp, np.float32).reshape(nt, nt, 2)
    return systems.System(x=s.x, box=s.box, q=s.q, type=s.type, ntypes=nt + 1, nbfp=nb.reshape(-1),
                          excl_index=s.excl_index, excl_list=s.excl_list)


def _perturbation(s, seed, vanish=False):
    rng = np.random.default_rng(seed)
    pert = np.sort(rng.choice(s.n, 40, replace=False)).astype(np.int32)
    qB = (s.q[pert] * -0.5 + rng.normal(0, 0.2, len(pert))).astype(np.float32)
    tB = rng.integers(0, s.ntypes - (1 if vanish else 0), len(pert)).astype(np.int32)
    if vanish:  # every fourth perturbed atom disappears in state B (soft-core on both terms)
        tB[::4] = s.ntypes - 1
        qB[::4] = 0.0
    return pert, qB, tB


def _calc(s, coulomb):
    ct = nblib.CoulombType.Pme if coulomb == "ewald" else nblib.CoulombType.ReactionField
    opts = nblib.NBKernelOptions(coulomb_type=ct, pairlist_cutoff=1.0, rcoulomb=RC, epsilon_rf=EPS_RF,
                                 compute_virial_and_energy=True)
    return nblib.ForceCalculator(s, opts)


@pytest.mark.parametrize("name", ["water", "lj", "lj_vanishing"])
@pytest.mark.parametrize("coulomb", ["ewald", "rf"])
@pytest.mark.parametrize("lam,soft,power", [(0.0, True, 1), (0.35, True, 1), (0.8, True, 2), (0.5, False, 1),
                                            (1.0, True, 1)])
def test_fep_matches_oracle(name, coulomb, lam, soft, power):
    s = _system(name)
    pert, qB, tB = _perturbation(s, 3, vanish=(name == "lj_vanishing"))
    calc = _calc(s, coulomb)
    alpha = 0.5 if soft else 0.0
    calc.set_free_energy(pert, qB, tB, lambda_coul=lam, lambda_vdw=lam, alpha_vdw=alpha, alpha_coul=alpha,
                         sc_power=power)
    f = calc.compute(s.x).astype(np.float64)
    e = calc.energies.copy()
    terms = calc.free_energy_terms()
    calc.close()
    ic, ctype = _ic(s, coulomb)
    qB_full = s.q.copy()
    qB_full[pert] = qB
    tB_full = s.type.copy()
    tB_full[pert] = tB
    sc = F.SoftCore(alpha_vdw=alpha, alpha_coul=alpha, lambda_power=power) if soft else None
    ff, vc, vv, dc, dv, _ = F.compute(s, pert, qB_full, tB_full, lam, lam, sc, ic)
    fm, em = O.fp64_allpairs(_masked(s, pert), coulomb=ctype, rc=RC,
                             beta=ic.beta if coulomb == "ewald" else None, epsilon_rf=EPS_RF)
    f_ref = fm + ff
    assert rel_rms(f, f_ref) <= 1e-5
    assert e[0] == pytest.approx(em[0] + vv, rel=1e-5)
    assert e[1] == pytest.approx(em[1] + vc, rel=1e-5)
    # the perturbed-pair sums are small differences of large float terms (self terms, exclusion
    # corrections): their error is bounded by the energy bar of the whole system
    tol_c = 1e-5 * abs(e[1])
    tol_v = 1e-5 * abs(e[0]) + 1e-3
    assert terms["V_coul"] == pytest.approx(vc, abs=tol_c + 1e-4 * abs(vc))
    assert terms["V_lj"] == pytest.approx(vv, abs=tol_v + 1e-4 * abs(vv))
    assert terms["dvdl_coul"] == pytest.approx(dc, abs=tol_c + 1e-4 * abs(dc))
    assert terms["dvdl_lj"] == pytest.approx(dv, abs=tol_v + 1e-4 * abs(dv))


@pytest.mark.parametrize("coulomb", ["ewald", "rf"])
def test_unchanged_state_equals_the_plain_path(coulomb):
    """B = A without soft-core: forces, energies and virial as without perturbation, any lambda."""
    s = _system("water")
    rng = np.random.default_rng(4)
    pert = np.sort(rng.choice(s.n, 60, replace=False)).astype(np.int32)
    calc = _calc(s, coulomb)
    f0 = calc.compute(s.x).astype(np.float64)
    e0, v0 = calc.energies.copy(), calc.virial.copy()
    for lam in (0.0, 0.4, 1.0):
        calc.set_free_energy(pert, s.q[pert], s.type[pert], lambda_coul=lam, lambda_vdw=lam, alpha_vdw=0.0,
                             alpha_coul=0.0)
        f = calc.compute(s.x).astype(np.float64)
        assert rel_rms(f, f0) <= 2e-6
        # reaction field sums q_i q_j (1/r - c_rf) with float 1/r out to rc: ~2e-6 noise on the
        # total, so the two summation routes agree to the RF energy bar of the parity tests
        np.testing.assert_allclose(calc.energies, e0, rtol=2e-6 if coulomb == "ewald" else 5e-6)
        np.testing.assert_allclose(calc.virial, v0, rtol=0, atol=2e-6 * np.abs(v0).max())
        t = calc.free_energy_terms()
        assert abs(t["dvdl_coul"]) <= 1e-5 * (abs(t["V_coul"]) + 1) and abs(t["dvdl_lj"]) <= 1e-5 * (abs(t["V_lj"]) + 1)
    calc.clear_free_energy()
    f = calc.compute(s.x).astype(np.float64)
    assert rel_rms(f, f0) <= 1e-6
    np.testing.assert_allclose(calc.energies, e0, rtol=1e-6)
    calc.close()


def test_dvdl_is_the_lambda_derivative_on_the_gpu():
    s = _system("lj")
    pert, qB, tB = _perturbation(s, 5)
    calc = _calc(s, "ewald")
    calc.set_free_energy(pert, qB, tB, lambda_coul=0.5, lambda_vdw=0.5)
    h = 2e-3

    def energy(lc, lv):
        calc.set_lambda(lc, lv)
        calc.compute(s.x)
        return calc.energies.sum(), calc.free_energy_terms()

    _, t = energy(0.5, 0.5)
    ep, _ = energy(0.5 + h, 0.5)
    em, _ = energy(0.5 - h, 0.5)
    assert t["dvdl_coul"] == pytest.approx((ep - em) / (2 * h), rel=2e-3, abs=1e-2)
    ep, _ = energy(0.5, 0.5 + h)
    em, _ = energy(0.5, 0.5 - h)
    assert t["dvdl_lj"] == pytest.approx((ep - em) / (2 * h), rel=2e-3, abs=1e-2)
    calc.close()


def test_md_with_perturbed_atoms_runs():
    """The MD step loop with perturbed atoms: the rows stay finite and conserve energy over 200 steps."""
    from gmxapi_gb300 import md

    s = systems.lj_fcc(cells=6, lattice=0.5256, charge=0.2, seed=3)
    rng = np.random.default_rng(6)
    pert = np.sort(rng.choice(s.n, 20, replace=False)).astype(np.int32)
    v0 = (rng.standard_normal((s.n, 3)) * np.sqrt(0.00831446 * 100.0 / systems.ARGON_MASS)).astype(np.float32)
    opts = nblib.NBKernelOptions(pairlist_cutoff=1.1, rcoulomb=0.9, nstlist=10, compute_virial_and_energy=True,
                                 use_ewald_shift=True)
    run = md.MdRunner(s, np.full(s.n, systems.ARGON_MASS, np.float32), opts, dt=0.002, velocities=v0, pme=False)
    run.calc.set_free_energy(pert, np.zeros(len(pert), np.float32), s.type[pert], lambda_coul=0.5, lambda_vdw=0.5)
    rows = run.run(200, nstcalcenergy=10)
    et = rows.sum(axis=1)
    assert np.all(np.isfinite(et))
    assert abs(et[-1] - et[0]) <= 5e-3 * rows[:, 3].mean()
    run.close()


@pytest.mark.parametrize("bad", ["index", "type", "power", "repeat", "lambda"])
def test_invalid_perturbation_raises(bad):
    s = _system("water")
    calc = _calc(s, "ewald")
    pert = np.array([1, 5, 9], np.int32)
    qB = np.zeros(3, np.float32)
    tB = np.zeros(3, np.int32)
    kw = {}
    if bad == "index":
        pert[1] = s.n
    elif bad == "type":
        tB[0] = s.ntypes
    elif bad == "power":
        kw["sc_power"] = 3
    elif bad == "repeat":
        pert[2] = 1
    with pytest.raises(nblib.InputException):
        if bad == "lambda":
            calc.set_free_energy(pert, qB, tB)
            calc.set_lambda(1.5)
        else:
            calc.set_free_energy(pert, qB, tB, **kw)
    calc.close()
