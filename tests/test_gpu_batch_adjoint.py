"""Batched adjoint and batched force matching.

The batch's backward pass must equal the single-system adjoint of every member
(gradients with respect to coordinates and charges per system, the type-table
gradient summed over systems), and one force-matching step (one CUDA-graph
launch: parameters -> forces -> loss -> adjoint) must match the FP64 autograd
all-pairs functional of the same loss on a small ensemble with shared sigma,
epsilon and per-type charge scales.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from gmxapi_gb300 import systems  # noqa: E402
from gmxapi_gb300.adjoint import (  # noqa: E402
    BatchForceMatcher,
    DifferentiableNonbonded,
    TypeScaledCharges,
    lorentz_berthelot_nbfp,
)
from gmxapi_gb300.batch import BatchForceCalculator  # noqa: E402
from gmxapi_gb300.nblib import CoulombType, NBKernelOptions  # noqa: E402
from oracle import oracle as orc  # noqa: E402
from oracle.fp64_autograd import COULOMB_EWALD, AllPairsFP64  # noqa: E402

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def rel_rms(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.sqrt(np.sum((a - b) ** 2) / np.sum(b**2)))


def _opts():
    return NBKernelOptions(coulomb_type=CoulombType.Pme, pairlist_cutoff=1.0, rcoulomb=0.9, nstlist_prune=0,
                           compute_virial_and_energy=True)


def _ensemble(sizes=(2000, 2600, 3100), seed=7):
    rng = np.random.default_rng(seed)
    sig = rng.uniform(0.25, 0.40, 8)
    eps = rng.uniform(0.1, 1.0, 8)
    return [systems.lj_liquid(n=n, ntypes=8, seed=seed * 10 + k, type_sigma=sig, type_epsilon=eps)
            for k, n in enumerate(sizes)], sig, eps


@pytest.mark.parametrize("graph", [False, True])
def test_batch_backward_matches_single_systems(graph):
    ens, sig, eps = _ensemble()
    b = BatchForceCalculator(ens, _opts())
    b.set_graph(graph)
    stream = torch.cuda.current_stream().cuda_stream
    b.set_stream(stream)
    x = torch.cat([torch.tensor(s.x).reshape(-1) for s in ens]).to(DEV)
    n = x.numel() // 3
    b.search_device(x.data_ptr())
    rng = np.random.default_rng(3)
    gf = torch.tensor(rng.normal(size=3 * n), dtype=torch.float32, device=DEV)
    ge = torch.tensor(rng.normal(size=2 * len(ens)), dtype=torch.float64, device=DEV)
    gx = torch.empty(3 * n, device=DEV)
    gq = torch.empty(n, device=DEV)
    gp = torch.empty(8, 8, 2, dtype=torch.float64, device=DEV)
    b.backward_device(x.data_ptr(), gf.data_ptr(), ge.data_ptr(), gx.data_ptr(), gq.data_ptr(), gp.data_ptr())
    torch.cuda.synchronize()
    gp_sum = np.zeros((8, 8, 2))
    for k, s in enumerate(ens):
        o0, o1 = int(b.offsets[k]), int(b.offsets[k + 1])
        eng = DifferentiableNonbonded(s, _opts())
        eng.calc.set_stream(stream)
        xs = torch.tensor(s.x, device=DEV)
        eng.search(xs)
        gxs = torch.empty(s.n, 3, device=DEV)
        gqs = torch.empty(s.n, device=DEV)
        gps = torch.empty(8, 8, 2, dtype=torch.float64, device=DEV)
        eng.calc.backward_device(xs.data_ptr(), gf[3 * o0:3 * o1].contiguous().data_ptr(),
                                 ge[2 * k:2 * k + 2].contiguous().data_ptr(), gxs.data_ptr(), gqs.data_ptr(),
                                 gps.data_ptr())
        torch.cuda.synchronize()
        assert rel_rms(gx[3 * o0:3 * o1].cpu(), gxs.reshape(-1).cpu()) < 1e-5
        assert rel_rms(gq[o0:o1].cpu(), gqs.cpu()) < 1e-5
        gp_sum += gps.cpu().numpy()
        eng.close()
    assert rel_rms(gp.cpu().numpy(), gp_sum) < 1e-6
    b.close()


def _fp64_loss_grads(ens, sig, eps, qscale, q0, f_target):
    """FP64 autograd over all pairs of every system: loss and d loss / d(sigma, epsilon, qscale)."""
    s64 = torch.tensor(sig, dtype=torch.float64, requires_grad=True)
    e64 = torch.tensor(eps, dtype=torch.float64, requires_grad=True)
    k64 = torch.tensor(qscale, dtype=torch.float64, requires_grad=True)
    nbfp = lorentz_berthelot_nbfp(s64, e64)
    beta = orc.Oracle(ens[0], rc=0.9, rlist=1.0).beta
    epsfac = orc.lib().orc_one_4pi_eps0()
    total = 0.0
    off = 0
    for s in ens:
        ref = AllPairsFP64(s, 0.9, beta, epsfac, coulomb=COULOMB_EWALD)
        x = torch.tensor(s.x, dtype=torch.float64, requires_grad=True)
        q = torch.tensor(q0[off:off + s.n], dtype=torch.float64) * k64[torch.tensor(s.type, dtype=torch.long)]
        f, _ = ref.forces_energies(x, q, nbfp)
        ft = torch.tensor(f_target[3 * off:3 * (off + s.n)], dtype=torch.float64).reshape(-1, 3)
        total = total + ((f - ft) ** 2).sum()
        off += s.n
    gs, ge, gk = torch.autograd.grad(total, (s64, e64, k64))
    return float(total.detach()), gs.numpy(), ge.numpy(), gk.numpy()


def test_force_matching_step_matches_fp64_autograd():
    ens, sig, eps = _ensemble(sizes=(2000, 2400), seed=9)
    q0 = np.concatenate([s.q for s in ens]).astype(np.float64)
    types = np.concatenate([s.type for s in ens]).astype(np.int64)
    rng = np.random.default_rng(2)
    # targets: the engine's own forces at parameters perturbed by up to 5 %
    sig_t, eps_t = sig * rng.uniform(0.95, 1.05, 8), eps * rng.uniform(0.95, 1.05, 8)
    qs_t = rng.uniform(0.95, 1.05, 8)
    b = BatchForceCalculator(ens, _opts())
    b.set_stream(torch.cuda.current_stream().cuda_stream)
    x = torch.cat([torch.tensor(s.x).reshape(-1) for s in ens]).to(DEV)
    b.search_device(x.data_ptr())
    q_t = torch.tensor(q0 * qs_t[types], dtype=torch.float32, device=DEV)
    nb_t = lorentz_berthelot_nbfp(torch.tensor(sig_t), torch.tensor(eps_t)).float().contiguous().to(DEV)
    b.set_parameters_device(q_t.data_ptr(), nb_t.data_ptr())
    f_target = torch.empty_like(x)
    b.compute_device(x.data_ptr(), f_target.data_ptr())
    torch.cuda.synchronize()
    b.close()

    m = BatchForceMatcher(ens, f_target)
    s_p = torch.tensor(sig, dtype=torch.float64, device=DEV, requires_grad=True)
    e_p = torch.tensor(eps, dtype=torch.float64, device=DEV, requires_grad=True)
    k_p = torch.ones(8, dtype=torch.float64, device=DEV, requires_grad=True)
    charges = TypeScaledCharges(torch.tensor(q0, device=DEV), torch.tensor(types, device=DEV), 8)
    for rep in range(2):  # second call replays the captured graph
        for p in (s_p, e_p, k_p):
            p.grad = None
        loss = m(charges(k_p), lorentz_berthelot_nbfp(s_p, e_p))
        loss.backward()
    l64, gs, ge, gk = _fp64_loss_grads(ens, sig, eps, np.ones(8), q0, f_target.cpu().numpy())
    print("loss", float(loss), l64, "grads", rel_rms(s_p.grad.cpu(), gs), rel_rms(e_p.grad.cpu(), ge),
          rel_rms(k_p.grad.cpu(), gk))
    assert abs(float(loss) - l64) <= 2e-5 * l64
    assert rel_rms(s_p.grad.cpu(), gs) < 2e-5
    assert rel_rms(e_p.grad.cpu(), ge) < 2e-5
    assert rel_rms(k_p.grad.cpu(), gk) < 2e-5
    m.close()


def test_benchmarked_force_matching_batch_subset_vs_fp64():
    """The force-matching benchmark's own batch (64 liquids, 2,000-50,000 atoms, seed 5), on the
    subset its FP64 all-pairs reference can afford: the two smallest systems (2,007 and 2,095 atoms)
    with the benchmark's target construction (forces at parameters perturbed by up to 5 %, seed 21)
    and its list (static, at rc).  Loss and gradients against FP64 autograd."""
    from gmxapi_gb300.adjoint import static_list_options

    specs = sorted(systems.force_matching_specs(64), key=lambda k: k["n"])[:2]
    ens = [systems.lj_liquid(**kw) for kw in specs]
    assert [s.n for s in ens] == [2007, 2095]
    sig, eps = ens[0].sigma, ens[0].epsilon
    q0 = np.concatenate([s.q for s in ens]).astype(np.float64)
    types = np.concatenate([s.type for s in ens]).astype(np.int64)
    rng = np.random.default_rng(21)
    pert = [rng.uniform(0.95, 1.05, 8) for _ in range(3)]
    opts = static_list_options(0.9)
    opts.compute_virial_and_energy = True
    b = BatchForceCalculator(ens, opts)
    b.set_stream(torch.cuda.current_stream().cuda_stream)
    x = torch.cat([torch.tensor(s.x).reshape(-1) for s in ens]).to(DEV)
    b.search_device(x.data_ptr())
    q_t = torch.tensor(q0 * pert[2][types], dtype=torch.float32, device=DEV)
    nb_t = lorentz_berthelot_nbfp(torch.tensor(sig * pert[0]), torch.tensor(eps * pert[1])).float().contiguous().to(DEV)
    b.set_parameters_device(q_t.data_ptr(), nb_t.data_ptr())
    f_target = torch.empty_like(x)
    b.compute_device(x.data_ptr(), f_target.data_ptr())
    torch.cuda.synchronize()
    b.close()
    m = BatchForceMatcher(ens, f_target, opts)
    s_p = torch.tensor(sig, dtype=torch.float64, device=DEV, requires_grad=True)
    e_p = torch.tensor(eps, dtype=torch.float64, device=DEV, requires_grad=True)
    k_p = torch.ones(8, dtype=torch.float64, device=DEV, requires_grad=True)
    charges = TypeScaledCharges(torch.tensor(q0, device=DEV), torch.tensor(types, device=DEV), 8)
    loss = m(charges(k_p), lorentz_berthelot_nbfp(s_p, e_p))
    loss.backward()
    l64, gs, ge, gk = _fp64_loss_grads(ens, sig, eps, np.ones(8), q0, f_target.cpu().numpy())
    errs = (abs(float(loss) - l64) / l64, rel_rms(s_p.grad.cpu(), gs), rel_rms(e_p.grad.cpu(), ge),
            rel_rms(k_p.grad.cpu(), gk))
    print("benchmarked batch, 2 smallest systems: loss rel err %.2e, grad rel RMS sigma %.2e epsilon %.2e "
          "charge scale %.2e" % errs)
    assert errs[0] <= 2e-5 and max(errs[1:]) < 2e-5
    m.close()
