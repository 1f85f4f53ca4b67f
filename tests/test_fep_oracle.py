"""The free-energy oracle pinned by its end states against the pinned FP64 all-pairs oracle (CPU)."""
import numpy as np
import pytest

from gmxapi_gb300 import systems
from oracle import fep_oracle as F
from oracle import oracle as O

RC = 0.9
RC32 = float(np.float32(RC))  # the interaction constants are single precision in the reference
EPS_RF = 78.0


def _masked(s, perturbed):
    """The system with the perturbed atoms uncharged and of an all-zero LJ type."""
    nt = s.ntypes
    nb = np.asarray(s.nbfp, np.float32).reshape(nt, nt, 2)
    nb2 = np.zeros((nt + 1, nt + 1, 2), np.float32)
    nb2[:nt, :nt] = nb
    q = s.q.copy()
    t = s.type.copy()
    q[perturbed] = 0.0
    t[perturbed] = nt
    return systems.System(x=s.x, box=s.box, q=q, type=t, ntypes=nt + 1, nbfp=nb2.reshape(-1),
                          excl_index=s.excl_index, excl_list=s.excl_list)


def _ic(s, coulomb):
    if coulomb == "ewald":
        beta = float(O.Oracle(s, rc=RC, rlist=1.0).beta)
        return (F.Interaction(coulomb="ewald", rc=RC32, beta=beta, cpot6=-RC32 ** -6, cpot12=-RC32 ** -12),
                O.COULOMB_EWALD)
    # reaction field with eps_rf = 78 (k_rf, c_rf in single precision, rf_util.cpp:54-66)
    eps, rcf = np.float32(EPS_RF), np.float32(RC)
    k_rf = (eps - np.float32(1)) / (np.float32(2) * eps + np.float32(1)) / (rcf * rcf * rcf)
    c_rf = np.float32(1) / rcf + k_rf * rcf * rcf
    return (F.Interaction(coulomb="rf", rc=RC32, k_rf=float(k_rf), c_rf=float(c_rf), cpot6=-RC32 ** -6,
                          cpot12=-RC32 ** -12), O.COULOMB_RF)


SYSTEMS = {
    "water": lambda: systems.spc_water(300, 2.08, seed=5),
    "lj_liquid": lambda: systems.lj_liquid(n=800, ntypes=4, seed=8),
}


@pytest.mark.parametrize("name", list(SYSTEMS))
@pytest.mark.parametrize("coulomb", ["ewald", "rf"])
@pytest.mark.parametrize("lam,soft", [(0.0, True), (1.0, True), (0.37, False)])
def test_end_states_reduce_to_the_plain_kernel(name, coulomb, lam, soft):
    """B = A: the perturbed atoms' pairs give what the plain all-pairs sum gives for them
    (the difference between the full and the masked system), at every lambda without
    soft-core and at lambda 0 and 1 with it."""
    s = SYSTEMS[name]()
    rng = np.random.default_rng(1)
    pert = np.sort(rng.choice(s.n, 30, replace=False))
    ic, ctype = _ic(s, coulomb)
    sc = F.SoftCore(alpha_vdw=0.5, alpha_coul=0.5, lambda_power=1) if soft else None
    f, vc, vv, dc, dv, vir = F.compute(s, pert, s.q, s.type, lam, lam, sc, ic)
    beta = ic.beta if coulomb == "ewald" else None
    f_full, e_full = O.fp64_allpairs(s, coulomb=ctype, rc=RC, beta=beta, epsilon_rf=EPS_RF)
    f_mask, e_mask = O.fp64_allpairs(_masked(s, pert), coulomb=ctype, rc=RC, beta=beta, epsilon_rf=EPS_RF)
    assert vv == pytest.approx(e_full[0] - e_mask[0], rel=1e-9, abs=1e-9)
    assert vc == pytest.approx(e_full[1] - e_mask[1], rel=1e-9, abs=1e-9)
    np.testing.assert_allclose(f, f_full - f_mask, rtol=0, atol=1e-8 * np.abs(f_full).max())
    if not soft:  # with soft-core the two copies of the same state sit on different soft-core paths
        assert abs(dc) < 1e-9 * max(1.0, abs(vc)) and abs(dv) < 1e-9 * max(1.0, abs(vv))


@pytest.mark.parametrize("power", [1, 2])
@pytest.mark.parametrize("coulomb", ["ewald", "rf"])
def test_dvdl_is_the_lambda_derivative(power, coulomb):
    """Charges and LJ types change between the states (some atoms vanish: soft-core active);
    dV/dlambda equals the central difference of V(lambda) (lambda_coul = lambda_vdw)."""
    s = systems.lj_liquid(n=800, ntypes=4, seed=8)
    rng = np.random.default_rng(2)
    pert = np.sort(rng.choice(s.n, 40, replace=False))
    qB = s.q.copy()
    qB[pert] = rng.normal(0, 0.5, len(pert)).astype(np.float32)
    tB = s.type.copy()
    tB[pert] = rng.integers(0, s.ntypes, len(pert))
    # a quarter of the perturbed atoms vanish in state B (zero LJ type and charge)
    nt = s.ntypes
    nb = np.asarray(s.nbfp, np.float32).reshape(nt, nt, 2)
    nb2 = np.zeros((nt + 1, nt + 1, 2), np.float32)
    nb2[:nt, :nt] = nb
    s2 = systems.System(x=s.x, box=s.box, q=s.q, type=s.type, ntypes=nt + 1, nbfp=nb2.reshape(-1),
                        excl_index=s.excl_index, excl_list=s.excl_list)
    gone = pert[::4]
    tB[gone] = nt
    qB[gone] = 0.0
    ic, _ = _ic(s2, coulomb)
    sc = F.SoftCore(alpha_vdw=0.5, alpha_coul=0.5, lambda_power=power)
    h = 1e-5
    for lam in (0.2, 0.5, 0.9):
        _, vc, vv, dc, dv, _ = F.compute(s2, pert, qB, tB, lam, lam, sc, ic)
        _, vcp, vvp, _, _, _ = F.compute(s2, pert, qB, tB, lam + h, lam + h, sc, ic)
        _, vcm, vvm, _, _, _ = F.compute(s2, pert, qB, tB, lam - h, lam - h, sc, ic)
        assert dc == pytest.approx((vcp - vcm) / (2 * h), rel=1e-5, abs=1e-6)
        assert dv == pytest.approx((vvp - vvm) / (2 * h), rel=1e-5, abs=1e-6)


def test_forces_are_the_gradient():
    s = systems.lj_liquid(n=400, ntypes=3, seed=3)
    rng = np.random.default_rng(3)
    pert = np.sort(rng.choice(s.n, 12, replace=False))
    qB = s.q.copy()
    qB[pert] *= -1.0
    ic, _ = _ic(s, "ewald")
    sc = F.SoftCore()
    f, *_ = F.compute(s, pert, qB, s.type, 0.4, 0.6, sc, ic)
    hstep = 1e-6
    x0 = s.x.astype(np.float64)
    for a, d in ((pert[0], 0), (pert[5], 2), (int(np.setdiff1d(np.arange(s.n), pert)[7]), 1)):
        e = []
        for sign in (1, -1):
            x = x0.copy()
            x[a, d] += sign * hstep
            s2 = systems.System(x=x, box=s.box, q=s.q, type=s.type, ntypes=s.ntypes, nbfp=s.nbfp,
                                excl_index=s.excl_index, excl_list=s.excl_list)
            _, vc, vv, *_ = F.compute(s2, pert, qB, s.type, 0.4, 0.6, sc, ic)
            e.append(vc + vv)
        assert -(e[0] - e[1]) / (2 * hstep) == pytest.approx(f[a, d], rel=1e-5, abs=1e-4)
