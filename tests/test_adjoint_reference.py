"""The FP64 autograd all-pairs functional used to check the adjoint kernel.

Pinned two ways on the CPU: its forces (-dE/dx by autograd) against the C
oracle's FP64 explicit-image forces and energies, and its second derivatives
(gradients of a loss of the forces) against FP64 central differences with
step 1e-6.
"""
import numpy as np
import pytest
import torch

from gmxapi_gb300 import systems
from oracle import oracle as orc
from oracle.fp64_autograd import COULOMB_EWALD, COULOMB_RF, AllPairsFP64

RC = 0.8
FD_STEP = 1e-6


def _lb(sigma, epsilon):
    sig = 0.5 * (sigma[:, None] + sigma[None, :])
    eps = torch.sqrt(epsilon[:, None] * epsilon[None, :])
    s6 = sig**6
    c6 = 4.0 * eps * s6
    return torch.stack((6.0 * c6, 12.0 * c6 * s6), dim=-1)


def _constants(s, coulomb):
    o = orc.Oracle(s, coulomb=coulomb, rc=RC, rlist=RC + 0.1)
    return o.beta, orc.lib().orc_one_4pi_eps0()


@pytest.fixture(scope="module")
def liquid():
    return systems.lj_liquid(n=500, ntypes=4, seed=11)


@pytest.fixture(scope="module")
def water():
    return systems.spc_water(170, 1.72, seed=6)


@pytest.mark.parametrize("coulomb", [COULOMB_EWALD, COULOMB_RF])
@pytest.mark.parametrize("which", ["liquid", "water"])
def test_forces_match_c_oracle(which, coulomb, request):
    s = request.getfixturevalue(which)
    beta, epsfac = _constants(s, coulomb)
    ref = AllPairsFP64(s, RC, beta, epsfac, coulomb=coulomb)
    x = torch.tensor(s.x, dtype=torch.float64)
    q = torch.tensor(s.q, dtype=torch.float64)
    nbfp = torch.tensor(s.nbfp, dtype=torch.float64).reshape(s.ntypes, s.ntypes, 2)
    f, e = ref.forces_energies(x, q, nbfp)
    fo, eo = orc.fp64_allpairs(s, coulomb=coulomb, rc=RC, beta=beta)
    f = f.detach().numpy()
    assert np.sqrt(np.mean((f - fo) ** 2) / np.mean(fo**2)) < 1e-10
    np.testing.assert_allclose(e.detach().numpy(), eo, rtol=1e-10, atol=1e-8)


def _loss(ref, x, q, sigma, epsilon, g_f, g_e):
    f, e = ref.forces_energies(x, q, _lb(sigma, epsilon))
    return (g_f * f).sum() + (g_e * e).sum()


@pytest.mark.parametrize("coulomb", [COULOMB_EWALD, COULOMB_RF])
def test_second_derivatives_match_central_differences(liquid, coulomb):
    s = liquid
    beta, epsfac = _constants(s, coulomb)
    ref = AllPairsFP64(s, RC, beta, epsfac, coulomb=coulomb)
    rng = np.random.default_rng(3)
    g_f = torch.tensor(rng.normal(size=(s.n, 3)))
    g_e = torch.tensor([0.7, -0.3], dtype=torch.float64)
    x = torch.tensor(s.x, dtype=torch.float64, requires_grad=True)
    q = torch.tensor(s.q, dtype=torch.float64, requires_grad=True)
    sig = torch.tensor(s.sigma, dtype=torch.float64, requires_grad=True)
    eps = torch.tensor(s.epsilon, dtype=torch.float64, requires_grad=True)
    loss = _loss(ref, x, q, sig, eps, g_f, g_e)
    gx, gq, gs, ge = torch.autograd.grad(loss, (x, q, sig, eps))

    def at(dx=0.0, dq=0.0, ds=0.0, de=0.0):
        xx = (x.detach() + dx).requires_grad_(True)
        return float(_loss(ref, xx, q.detach() + dq, sig.detach() + ds, eps.detach() + de, g_f, g_e).detach())

    # directional derivative along a random displacement, and single parameters
    v = torch.tensor(rng.normal(size=(s.n, 3)))
    fd = (at(dx=FD_STEP * v) - at(dx=-FD_STEP * v)) / (2 * FD_STEP)
    an = float((gx * v).sum())
    assert abs(fd - an) <= 1e-6 * max(1.0, abs(an)), (fd, an)
    for k in (0, 7, 123):
        e_k = torch.zeros(s.n, dtype=torch.float64)
        e_k[k] = 1.0
        fd = (at(dq=FD_STEP * e_k) - at(dq=-FD_STEP * e_k)) / (2 * FD_STEP)
        assert abs(fd - float(gq[k])) <= 1e-6 * max(1.0, abs(fd)), (k, fd, float(gq[k]))
    for t in range(s.ntypes):
        e_t = torch.zeros(s.ntypes, dtype=torch.float64)
        e_t[t] = 1.0
        fd = (at(ds=FD_STEP * e_t) - at(ds=-FD_STEP * e_t)) / (2 * FD_STEP)
        assert abs(fd - float(gs[t])) <= 1e-5 * max(1.0, abs(fd)), (t, fd, float(gs[t]))
        fd = (at(de=FD_STEP * e_t) - at(de=-FD_STEP * e_t)) / (2 * FD_STEP)
        assert abs(fd - float(ge[t])) <= 1e-6 * max(1.0, abs(fd)), (t, fd, float(ge[t]))
