"""Adjoint (backward) kernel against the FP64 autograd all-pairs functional.

For a loss L = sum G.F + gE.E of the GPU forces and energies, the gradients
with respect to coordinates (a Hessian-vector product), charges and per-type
sigma/epsilon (through the Lorentz-Berthelot table) are compared with the same
loss differentiated by autograd in FP64 over all pairs, on a 2,000-atom random
LJ + Coulomb liquid with 8 types and on SPC water (exclusions), for Ewald and
reaction-field electrostatics.  The FP64 functional itself is pinned against
central differences and the C oracle by the CPU tests.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from gmxapi_gb300 import systems  # noqa: E402
from gmxapi_gb300.adjoint import DifferentiableNonbonded, lorentz_berthelot_nbfp  # noqa: E402
from gmxapi_gb300.nblib import CoulombType, NBKernelOptions  # noqa: E402
from oracle import oracle as orc  # noqa: E402
from oracle.fp64_autograd import COULOMB_EWALD, COULOMB_RF, AllPairsFP64  # noqa: E402

pytestmark = pytest.mark.gpu

RC = 0.9
RLIST = 1.0
# FP32 pair arithmetic against FP64: relative RMS over all atoms / parameters
GX_RTOL = 2e-5
GQ_RTOL = 2e-5
GPARAM_RTOL = 2e-5

DEV = "cuda:0"


def rel_rms(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.sqrt(np.sum((a - b) ** 2) / np.sum(b**2)))


def _water_params(s):
    """Per-type sigma/epsilon of SPC water (H has none: epsilon 0)."""
    sig = np.array([systems.SPC_SIGMA, systems.SPC_SIGMA])
    eps = np.array([systems.SPC_EPSILON, 0.0])
    return sig, eps


CASES = {
    "liquid2000": lambda: systems.lj_liquid(n=2000, ntypes=8, seed=21),
    "water900": lambda: systems.spc_water(300, 2.08, seed=8),
}


def _params(s):
    if s.sigma is not None:
        return np.asarray(s.sigma, np.float64), np.asarray(s.epsilon, np.float64)
    return _water_params(s)


def _gpu(s, coulomb, g_f, g_e, loss_kind="linear", f_target=None):
    opts = NBKernelOptions(coulomb_type=CoulombType.Pme if coulomb == COULOMB_EWALD else CoulombType.ReactionField,
                           pairlist_cutoff=RLIST, rcoulomb=RC, epsilon_rf=1.0 if coulomb == COULOMB_EWALD else 0.0)
    eng = DifferentiableNonbonded(s, opts)
    sig0, eps0 = _params(s)
    x = torch.tensor(s.x, dtype=torch.float32, device=DEV, requires_grad=True)
    q = torch.tensor(s.q, dtype=torch.float32, device=DEV, requires_grad=True)
    sig = torch.tensor(sig0, dtype=torch.float64, device=DEV, requires_grad=True)
    eps = torch.tensor(eps0, dtype=torch.float64, device=DEV, requires_grad=True)
    f, e = eng(x, q, lorentz_berthelot_nbfp(sig, eps))
    if loss_kind == "linear":
        loss = (torch.tensor(g_f, dtype=torch.float32, device=DEV) * f).sum() + (
            torch.tensor(g_e, device=DEV) * e).sum()
    else:
        ft = torch.tensor(f_target, dtype=torch.float32, device=DEV)
        loss = ((f - ft) ** 2).sum()
    loss.backward()
    out = dict(f=f.detach().cpu().numpy(), e=e.detach().cpu().numpy(), gx=x.grad.cpu().numpy(),
               gq=q.grad.cpu().numpy(), gsig=sig.grad.cpu().numpy(), geps=eps.grad.cpu().numpy())
    eng.close()
    return out


def _fp64(s, coulomb, g_f, g_e, loss_kind="linear", f_target=None):
    o = orc.Oracle(s, coulomb=coulomb, rc=RC, rlist=RLIST, epsilon_rf=1.0 if coulomb == COULOMB_EWALD else 0.0)
    ref = AllPairsFP64(s, RC, o.beta, orc.lib().orc_one_4pi_eps0(), coulomb=coulomb,
                       epsilon_rf=1.0 if coulomb == COULOMB_EWALD else 0.0)
    sig0, eps0 = _params(s)
    x = torch.tensor(s.x, dtype=torch.float64, requires_grad=True)
    q = torch.tensor(s.q, dtype=torch.float64, requires_grad=True)
    sig = torch.tensor(sig0, dtype=torch.float64, requires_grad=True)
    eps = torch.tensor(eps0, dtype=torch.float64, requires_grad=True)
    f, e = ref.forces_energies(x, q, lorentz_berthelot_nbfp(sig, eps))
    if loss_kind == "linear":
        loss = (torch.tensor(g_f) * f).sum() + (torch.tensor(g_e) * e).sum()
    else:
        loss = ((f - torch.tensor(f_target, dtype=torch.float64)) ** 2).sum()
    gx, gq, gs, ge = torch.autograd.grad(loss, (x, q, sig, eps))
    return dict(f=f.detach().numpy(), e=e.detach().numpy(), gx=gx.numpy(), gq=gq.numpy(), gsig=gs.numpy(),
                geps=ge.numpy())


def _compare(g, r, params=True):
    errs = {k: rel_rms(g[k], r[k]) for k in ("f", "gx", "gq", "gsig", "geps")}
    assert errs["f"] < 1e-5, errs
    assert errs["gx"] < GX_RTOL, errs
    assert errs["gq"] < GQ_RTOL, errs
    if params:
        assert errs["gsig"] < GPARAM_RTOL, errs
        assert errs["geps"] < GPARAM_RTOL, errs
    return errs


@pytest.mark.parametrize("coulomb", [COULOMB_EWALD, COULOMB_RF])
@pytest.mark.parametrize("name", list(CASES))
def test_adjoint_linear_loss_matches_fp64_autograd(name, coulomb):
    s = CASES[name]()
    rng = np.random.default_rng(5)
    g_f = rng.normal(size=(s.n, 3))
    g_e = np.array([0.3, -0.2])
    g = _gpu(s, coulomb, g_f, g_e)
    r = _fp64(s, coulomb, g_f, g_e)
    errs = _compare(g, r, params=s.sigma is not None)
    print(name, coulomb, errs)


def test_adjoint_force_matching_loss_matches_fp64_autograd():
    """Loss sum |F - F_target|^2 with F_target at parameters perturbed by up to 5 %."""
    s = CASES["liquid2000"]()
    rng = np.random.default_rng(9)
    t = systems.System(**{**s.__dict__})
    t.sigma = s.sigma * rng.uniform(0.95, 1.05, s.ntypes)
    t.epsilon = s.epsilon * rng.uniform(0.95, 1.05, s.ntypes)
    t.q = (s.q * rng.uniform(0.95, 1.05, s.n)).astype(np.float32)
    nb = lorentz_berthelot_nbfp(torch.tensor(t.sigma), torch.tensor(t.epsilon)).numpy()
    t.nbfp = nb.reshape(-1).astype(np.float32)
    f_target, _ = orc.fp64_allpairs(t, rc=RC, beta=orc.Oracle(s, rc=RC, rlist=RLIST).beta)
    g = _gpu(s, COULOMB_EWALD, None, None, loss_kind="match", f_target=f_target)
    r = _fp64(s, COULOMB_EWALD, None, None, loss_kind="match", f_target=f_target)
    errs = _compare(g, r)
    print(errs)


def test_energy_gradient_is_minus_force():
    """With G = 0 and dL/dE = 1 the coordinate gradient is dE/dx = -F."""
    s = CASES["water900"]()
    g = _gpu(s, COULOMB_EWALD, np.zeros((s.n, 3)), np.array([1.0, 1.0]))
    assert rel_rms(g["gx"], -g["f"]) < 1e-5


def test_adjoint_is_repeatable():
    s = CASES["liquid2000"]()
    rng = np.random.default_rng(1)
    g_f = rng.normal(size=(s.n, 3))
    a = _gpu(s, COULOMB_EWALD, g_f, np.array([0.1, 0.1]))
    b = _gpu(s, COULOMB_EWALD, g_f, np.array([0.1, 0.1]))
    for k in ("gx", "gq", "gsig", "geps"):
        assert rel_rms(a[k], b[k]) < 1e-5


def test_adjoint_rejects_too_many_types():
    s = systems.lj_liquid(n=600, ntypes=16, seed=2)
    eng = DifferentiableNonbonded(s)
    x = torch.tensor(s.x, device=DEV, requires_grad=True)
    q = torch.tensor(s.q, device=DEV)
    nbfp = torch.tensor(s.nbfp, device=DEV).reshape(16, 16, 2)
    f, e = eng(x, q, nbfp)
    with pytest.raises(Exception, match="15"):
        f.sum().backward()
    eng.close()


def test_gradient_step_captured_in_a_cuda_graph_matches_eager():
    """The whole force-matching step (Lorentz-Berthelot table, forward, loss, backward) captured in
    one CUDA graph and replayed gives the eager gradients (the engine's stream switch must not
    synchronise while the graph is being captured)."""
    s = CASES["liquid2000"]()
    eng = DifferentiableNonbonded(s)
    x = torch.tensor(s.x, device=DEV, requires_grad=True)
    q = torch.tensor(s.q, device=DEV, requires_grad=True)
    sig = torch.tensor(s.sigma, dtype=torch.float64, device=DEV, requires_grad=True)
    eps = torch.tensor(s.epsilon, dtype=torch.float64, device=DEV, requires_grad=True)
    with torch.no_grad():
        f_t, _ = eng(x, q * 1.02, lorentz_berthelot_nbfp(sig * 0.98, eps * 1.03))
    eng.search(x)

    def step():
        f, _e = eng(x, q, lorentz_berthelot_nbfp(sig, eps), search=False)
        ((f - f_t) ** 2).sum().backward()

    step()
    eager = [t.grad.clone() for t in (x, q, sig, eps)]
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        for _ in range(2):
            for t in (x, q, sig, eps):
                t.grad = None
            step()
    torch.cuda.current_stream().wait_stream(side)
    for t in (x, q, sig, eps):
        t.grad = None
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        step()
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    for a, t in zip(eager, (x, q, sig, eps)):
        assert rel_rms(t.grad.cpu(), a.cpu()) < 1e-5  # atomics sum in another order
    eng.close()


@pytest.mark.parametrize("nt", [1, 8, 15])
def test_lorentz_berthelot_kernels_match_torch(nt):
    """The one-kernel combination rule and its adjoint against the torch formula (FP64)."""
    rng = np.random.default_rng(nt)
    sig = torch.tensor(rng.uniform(0.25, 0.45, nt), dtype=torch.float64, device=DEV, requires_grad=True)
    eps = torch.tensor(rng.uniform(0.05, 1.2, nt), dtype=torch.float64, device=DEV, requires_grad=True)
    g = torch.tensor(rng.normal(size=(nt, nt, 2)), dtype=torch.float64, device=DEV)
    t = lorentz_berthelot_nbfp(sig, eps)
    (t * g).sum().backward()
    s_c, e_c = sig.detach().cpu().requires_grad_(), eps.detach().cpu().requires_grad_()
    t_c = lorentz_berthelot_nbfp(s_c, e_c)
    (t_c * g.cpu()).sum().backward()
    np.testing.assert_allclose(t.detach().cpu().numpy(), t_c.detach().numpy(), rtol=1e-13)
    np.testing.assert_allclose(sig.grad.cpu().numpy(), s_c.grad.numpy(), rtol=1e-11, atol=1e-12)
    np.testing.assert_allclose(eps.grad.cpu().numpy(), e_c.grad.numpy(), rtol=1e-11, atol=1e-12)


def test_fused_force_matching_loss_matches_the_torch_expression():
    """force_matching_loss (one kernel each way) against ((f - f_t) ** 2).sum(): the loss in FP64,
    the gradients of a full force-matching step, and the step captured in a CUDA graph."""
    from gmxapi_gb300.adjoint import force_matching_loss

    s = CASES["liquid2000"]()
    eng = DifferentiableNonbonded(s)
    x = torch.tensor(s.x, device=DEV, requires_grad=True)
    q = torch.tensor(s.q, device=DEV, requires_grad=True)
    sig = torch.tensor(s.sigma, dtype=torch.float64, device=DEV, requires_grad=True)
    eps = torch.tensor(s.epsilon, dtype=torch.float64, device=DEV, requires_grad=True)
    with torch.no_grad():
        f_t, _ = eng(x, q * 1.02, lorentz_berthelot_nbfp(sig * 0.98, eps * 1.03))
    eng.search(x)
    params = (x, q, sig, eps)

    def step(fused):
        for t in params:
            t.grad = None
        f, _e = eng(x, q, lorentz_berthelot_nbfp(sig, eps), search=False)
        loss = force_matching_loss(f, f_t) if fused else ((f.double() - f_t.double()) ** 2).sum()
        loss.backward()
        return loss.detach().clone(), [t.grad.clone() for t in params]

    l_ref, g_ref = step(False)
    l_fused, g_fused = step(True)
    # the two steps' forces differ by the order of their atomic sums; the losses of one force array:
    with torch.no_grad():
        f, _e = eng(x, q, lorentz_berthelot_nbfp(sig, eps), search=False)
        a = float(force_matching_loss(f, f_t))
        b = float(((f.double() - f_t.double()) ** 2).sum())
    assert abs(a - b) <= 1e-12 * abs(b)
    assert abs(float(l_fused) - float(l_ref)) <= 1e-6 * abs(float(l_ref))
    for a, b in zip(g_fused, g_ref):
        assert rel_rms(a.cpu(), b.cpu()) < 1e-5
    # inside a CUDA graph: the same gradients after replays
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        for _ in range(2):
            step(True)
    torch.cuda.current_stream().wait_stream(side)
    for t in params:
        t.grad = None
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        f, _e = eng(x, q, lorentz_berthelot_nbfp(sig, eps), search=False)
        force_matching_loss(f, f_t).backward()
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    for a, t in zip(g_ref, params):
        assert rel_rms(t.grad.cpu(), a.cpu()) < 1e-5
    with pytest.raises(TypeError):
        force_matching_loss(f_t.double(), f_t.double())
    eng.close()
