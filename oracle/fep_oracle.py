"""CPU restatement of the reference's free-energy (perturbed) nonbonded kernel (TEST INFRASTRUCTURE ONLY).

Used by tests/ as the checker of the CUDA free-energy kernel; the product never imports it.
FP64 numpy, vectorised over pairs.  Restates nb_free_energy_kernel
(src/gromacs/gmxlib/nonbonded/nb_free_energy.cpp:200-850) for one perturbed-atom pair list:

- lambda factors LFC / LFV (1 - lambda for state A, lambda for B), DLF = (-1, +1), soft-core
  factors lfac / dlfac for sc-power 1 or 2 and sc-r-power 6 (:372-388);
- per pair and state: sigma^6 = C12/C6 (clamped below at sigma6_min; sigma6_def when C6 or C12 is
  zero), soft-core only when one end state has C12 = 0 (:480-509); r_C = (alpha_C lfac sigma^6 +
  r^6)^(1/6), r_V likewise (:520-548);
- Coulomb: Ewald qq (1/r_C - sh_ewald) within rc on r (:553-565), reaction field
  qq (1/r_C + k_rf r_C^2 - c_rf) within rc on r_C; Lennard-Jones with the potential-shift
  constants within rvdw on r_V (:573-590);
- assembly of forces, energies and dV/dlambda (:620-645);
- excluded pairs: reaction field k_rf r^2 - c_rf (:647-667), Ewald: the reciprocal-space part
  -qq erf(beta r)/r subtracted for pairs within rc and for excluded pairs (:669-723), halved for
  the self pair.  The reference interpolates erf(beta r)/r from its Ewald table; here it is
  analytic.  The reference keeps an excluded pair's correction while the pair is in its list
  (r < rlist); here while r < rc, as the cluster kernel does.

Parity unpinned: the reference holds no test data for this kernel and its compiled code is not
run here, so no reference output checks the soft-core branches at intermediate lambda.  What is
checked: at lambda = 0 (1) with state B (A) equal to A (B) it reduces to the pinned cluster-pair
oracle for the same pairs (``tests/test_fep_oracle.py``), and dV/dlambda equals the central
difference of V(lambda).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from oracle import pme_oracle


@dataclass
class SoftCore:
    alpha_vdw: float = 0.5
    alpha_coul: float = 0.5
    lambda_power: int = 1     # sc-power (1 or 2)
    sigma6_def: float = 0.3 ** 6
    sigma6_min: float = 0.3 ** 6


@dataclass
class Interaction:
    coulomb: str = "ewald"    # "ewald" or "rf"
    rc: float = 0.9
    beta: float = 3.4705
    sh_ewald: float = 0.0
    k_rf: float = 0.0
    c_rf: float = 0.0
    cpot6: float = 0.0        # dispersion shift (potential-shift modifier: -1/rc^6)
    cpot12: float = 0.0       # repulsion shift (-1/rc^12)
    epsfac: float = pme_oracle.ONE_4PI_EPS0


def lambda_factors(lam_coul, lam_vdw, lam_power):
    LFC = np.array([1.0 - lam_coul, lam_coul])
    LFV = np.array([1.0 - lam_vdw, lam_vdw])
    DLF = np.array([-1.0, 1.0])
    scp = 6.0
    lfac_c = (1 - LFC) ** 2 if lam_power == 2 else (1 - LFC)
    dlfac_c = DLF * lam_power / scp * ((1 - LFC) if lam_power == 2 else 1.0)
    lfac_v = (1 - LFV) ** 2 if lam_power == 2 else (1 - LFV)
    dlfac_v = DLF * lam_power / scp * ((1 - LFV) if lam_power == 2 else 1.0)
    return LFC, LFV, DLF, lfac_c, dlfac_c, lfac_v, dlfac_v


def pair_list(x, box, perturbed, excl_index, excl_list, rc):
    """Pairs with at least one perturbed atom, each once (minimum image; box >= 2 rc):
    returns i, j, dx (x_i - x_j, minimum image), excluded flag.  Self pairs are separate."""
    x = np.asarray(x, np.float64).reshape(-1, 3)
    L = np.asarray(box, np.float64)
    pert = np.zeros(x.shape[0], bool)
    pert[np.asarray(perturbed, int)] = True
    rows = []
    for i in np.flatnonzero(pert):
        ex = set(int(a) for a in excl_list[excl_index[i]:excl_index[i + 1]])
        d = x[i][None, :] - x
        d -= L * np.round(d / L)
        r2 = (d * d).sum(1)
        for j in np.flatnonzero(r2 < rc * rc):
            if j == i or (pert[j] and j < i):
                continue
            rows.append((i, j, d[j], j in ex))
    if not rows:
        return np.zeros(0, int), np.zeros(0, int), np.zeros((0, 3)), np.zeros(0, bool)
    i = np.array([r[0] for r in rows])
    j = np.array([r[1] for r in rows])
    dx = np.array([r[2] for r in rows])
    ex = np.array([r[3] for r in rows])
    return i, j, dx, ex


def kernel(i, j, dx, excluded, qA, qB, tA, tB, nbfp, ntypes1, lam_coul, lam_vdw, sc: SoftCore | None,
           ic: Interaction, self_atoms=()):
    """Forces on the pair atoms [(N,3) dict-free: returns fi per pair], and the sums.

    Returns (f_pair [P,3] force on i (minus on j), Vc, Vv, dvdl_c, dvdl_v, self energy terms
    included in Vc / dvdl_c)."""
    soft = sc is not None and (sc.alpha_vdw != 0 or sc.alpha_coul != 0)
    lam_power = sc.lambda_power if sc is not None else 1
    LFC, LFV, DLF, lfac_c, dlfac_c, lfac_v, dlfac_v = lambda_factors(lam_coul, lam_vdw, lam_power)
    qA = np.asarray(qA, np.float64)
    qB = np.asarray(qB, np.float64)
    nb = np.asarray(nbfp, np.float64).reshape(-1, 2)
    rsq = (dx * dx).sum(1)
    r = np.sqrt(rsq)
    with np.errstate(divide="ignore"):
        rinv = np.where(rsq > 0, 1.0 / r, 0.0)
    inc = ~excluded
    rc = ic.rc
    Fscal = np.zeros_like(r)
    Vc = Vv = dVc = dVv = 0.0
    qq = [ic.epsfac * qA[i] * qA[j], ic.epsfac * qB[i] * qB[j]]
    tt = [np.asarray(tA)[i] * ntypes1 + np.asarray(tA)[j], np.asarray(tB)[i] * ntypes1 + np.asarray(tB)[j]]
    c6 = [nb[tt[0], 0], nb[tt[1], 0]]
    c12 = [nb[tt[0], 1], nb[tt[1], 1]]
    if soft:
        rpm2 = rsq * rsq
        rp = rpm2 * rsq
        both = (c12[0] > 0) & (c12[1] > 0)
        a_v = np.where(both, 0.0, sc.alpha_vdw)
        a_c = np.where(both, 0.0, sc.alpha_coul)
    else:
        rpm2 = rinv * rinv
        rp = np.ones_like(r)
    for s in range(2):
        m = inc & ((qq[s] != 0) | (c6[s] != 0) | (c12[s] != 0))
        if soft:
            with np.errstate(divide="ignore", invalid="ignore"):
                sig6 = np.where((c6[s] > 0) & (c12[s] > 0), 0.5 * c12[s] / np.where(c6[s] > 0, c6[s], 1.0),
                                sc.sigma6_def)
            sig6 = np.where((c6[s] > 0) & (c12[s] > 0) & (sig6 < sc.sigma6_min), sc.sigma6_min, sig6)
            rpinvC = 1.0 / (a_c * lfac_c[s] * sig6 + rp)
            rpinvV = 1.0 / (a_v * lfac_v[s] * sig6 + rp)
            rinvC, rC = rpinvC ** (1.0 / 6.0), rpinvC ** (-1.0 / 6.0)
            rinvV, rV = rpinvV ** (1.0 / 6.0), rpinvV ** (-1.0 / 6.0)
        else:
            sig6 = np.zeros_like(r)
            rpinvC = rpinvV = np.ones_like(r)
            rinvC, rC, rinvV, rV = rinv, r, rinv, r
        if ic.coulomb == "ewald":
            ce = m & (qq[s] != 0) & (r < rc)
            Vcs = np.where(ce, qq[s] * (rinvC - ic.sh_ewald), 0.0)
            FCs = np.where(ce, qq[s] * rinvC, 0.0)
        else:
            ce = m & (qq[s] != 0) & (rC < rc)
            Vcs = np.where(ce, qq[s] * (rinvC + ic.k_rf * rC * rC - ic.c_rf), 0.0)
            FCs = np.where(ce, qq[s] * (rinvC - 2.0 * ic.k_rf * rC * rC), 0.0)
        ve = m & ((c6[s] != 0) | (c12[s] != 0)) & (rV < rc)
        rinv6 = rpinvV if soft else rinvV ** 6
        v6 = c6[s] * rinv6
        v12 = c12[s] * rinv6 * rinv6
        Vvs = np.where(ve, (v12 + c12[s] * ic.cpot12) / 12.0 - (v6 + c6[s] * ic.cpot6) / 6.0, 0.0)
        FVs = np.where(ve, v12 - v6, 0.0)
        FCs = FCs * rpinvC
        FVs = FVs * rpinvV
        Vc += float((LFC[s] * Vcs).sum())
        Vv += float((LFV[s] * Vvs).sum())
        Fscal += LFC[s] * FCs * rpm2 + LFV[s] * FVs * rpm2
        if soft:
            dVc += float((Vcs * DLF[s] + LFC[s] * a_c * dlfac_c[s] * FCs * sig6).sum())
            dVv += float((Vvs * DLF[s] + LFV[s] * a_v * dlfac_v[s] * FVs * sig6).sum())
        else:
            dVc += float((Vcs * DLF[s]).sum())
            dVv += float((Vvs * DLF[s]).sum())
    # excluded pairs (reaction field) and the reciprocal-space part (Ewald)
    if ic.coulomb == "ewald":
        b = ic.beta
        corr = r < rc
        with np.errstate(divide="ignore", invalid="ignore"):
            v_lr = np.where(corr & (r > 0), np.array([math.erf(b * t) for t in r]) * rinv, 0.0)
            dv = np.where(corr & (r > 0),
                          (2.0 * b / math.sqrt(math.pi) * np.exp(-b * b * rsq)) * rinv - v_lr * rinv, 0.0)
        f_lr = -dv * rinv
        for s in range(2):
            Vc -= float((LFC[s] * qq[s] * v_lr).sum())
            Fscal -= LFC[s] * qq[s] * f_lr
            dVc -= float((DLF[s] * qq[s] * v_lr).sum())
    else:
        ex = excluded & (r < rc)
        VV = np.where(ex, ic.k_rf * rsq - ic.c_rf, 0.0)
        FF = np.where(ex, -2.0 * ic.k_rf, 0.0)
        for s in range(2):
            Vc += float((LFC[s] * qq[s] * VV).sum())
            Fscal += LFC[s] * qq[s] * FF
            dVc += float((DLF[s] * qq[s] * VV).sum())
    # self pairs of the perturbed atoms: half of the r = 0 excluded term
    for a in self_atoms:
        qqs = [ic.epsfac * qA[a] * qA[a], ic.epsfac * qB[a] * qB[a]]
        vself = 2.0 * ic.beta / math.sqrt(math.pi) if ic.coulomb == "ewald" else ic.c_rf
        for s in range(2):
            Vc -= 0.5 * LFC[s] * qqs[s] * vself
            dVc -= 0.5 * DLF[s] * qqs[s] * vself
    fpair = Fscal[:, None] * dx
    return fpair, Vc, Vv, dVc, dVv


def compute(system, perturbed, qB, tB, lam_coul, lam_vdw, sc: SoftCore | None, ic: Interaction):
    """The free-energy kernel's contribution for a System: forces (N,3), Vc, Vv, dvdl_c, dvdl_v, virial."""
    n = system.n
    i, j, dx, ex = pair_list(system.x, system.box, perturbed, system.excl_index, system.excl_list, ic.rc)
    fp, Vc, Vv, dVc, dVv = kernel(i, j, dx, ex, system.q, qB, system.type, tB, system.nbfp, system.ntypes, lam_coul,
                                  lam_vdw, sc, ic, self_atoms=perturbed)
    f = np.zeros((n, 3))
    np.add.at(f, i, fp)
    np.add.at(f, j, -fp)
    vir = -0.5 * np.einsum("pa,pb->ab", dx, fp)
    return f, Vc, Vv, dVc, dVv, vir
