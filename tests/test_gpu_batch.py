"""Batched ensemble (nbx_batch_*) against the single-system path, through the C ABI (GB300)."""
import numpy as np
import pytest

from gmxapi_gb300 import nblib, systems
from gmxapi_gb300.batch import BatchForceCalculator
from tests.helpers import rel_rms

pytestmark = pytest.mark.gpu

FORCE_RTOL = 1e-5
ENERGY_RTOL = 1e-6


def _ensemble(nsys=12, seed=9, n_min=300, n_max=3000):
    return systems.uneven_ensemble(nsys, seed=seed, n_min=n_min, n_max=n_max)


def _opts(prune=0, rlist_inner=None):
    return nblib.NBKernelOptions(coulomb_type=nblib.CoulombType.Pme, pairlist_cutoff=1.0, rcoulomb=0.9,
                                 rlist_inner=rlist_inner, nstlist=10, nstlist_prune=prune,
                                 compute_virial_and_energy=True)


@pytest.mark.parametrize("graph", [True, False])
@pytest.mark.parametrize("variant", [0, 1, 2, 3])
@pytest.mark.parametrize("tile,depth", [(0, 2), (1, 2), (1, 3)])
def test_batch_matches_single_systems(graph, variant, tile, depth):
    torch = pytest.importorskip("torch")
    ens = _ensemble()
    b = BatchForceCalculator(ens, _opts())
    if variant == 2:
        b.set_stream(0)  # the legacy default stream (graphs are captured on a private stream)
    b.set_graph(graph)
    b.set_kernel_variant(variant)
    b.set_force_kernel(tile, depth)
    dev = torch.device("cuda:0")
    x = torch.from_numpy(np.concatenate([s.x.reshape(-1) for s in ens])).to(dev)
    f = torch.empty_like(x)
    e = torch.zeros(2 * len(ens), dtype=torch.float64, device=dev)
    v = torch.zeros(9 * len(ens), dtype=torch.float64, device=dev)
    for rep in range(2):  # second call replays the graph
        b.compute_device(x.data_ptr(), f.data_ptr(), e.data_ptr(), v.data_ptr())
        torch.cuda.synchronize()
        fb = f.cpu().numpy()
        eb = e.cpu().numpy().reshape(-1, 2)
        vb = v.cpu().numpy().reshape(-1, 3, 3)
        for i, s in enumerate(ens):
            calc = nblib.ForceCalculator(s, _opts())
            fs = calc.compute(s.x)
            o = b.offsets[i]
            assert rel_rms(fb[3 * o:3 * (o + s.n)].reshape(-1, 3), fs) <= FORCE_RTOL, (i, s.n)
            assert np.all(np.abs(eb[i] - calc.energies) <= ENERGY_RTOL * np.abs(calc.energies)), (i, eb[i])
            assert np.abs(vb[i] - calc.virial).max() <= 1e-5 * np.abs(calc.virial).max() + 1e-3, i
            calc.close()
    b.close()


def test_batched_search_grows_records():
    """Long-list systems (water at rlist 2.0 nm, cells beyond their initial 512 search records)
    through the batched search, whose systems search concurrently on several streams and grow
    their records between the two rounds: forces and energies equal the single-system path."""
    torch = pytest.importorskip("torch")
    ens = [systems.spc_water(m, (m * 0.0299) ** (1 / 3), seed=11 + k) for k, m in enumerate((3000, 2500, 400))]
    opts = nblib.NBKernelOptions(coulomb_type=nblib.CoulombType.Pme, pairlist_cutoff=2.0, rcoulomb=0.9,
                                 nstlist=10, compute_virial_and_energy=True)
    b = BatchForceCalculator(ens, opts)
    dev = torch.device("cuda:0")
    x = torch.from_numpy(np.concatenate([s.x.reshape(-1) for s in ens])).to(dev)
    f = torch.empty_like(x)
    e = torch.zeros(2 * len(ens), dtype=torch.float64, device=dev)
    b.search_device(x.data_ptr())  # the batched search (creation searched each system on its own)
    b.compute_device(x.data_ptr(), f.data_ptr(), e.data_ptr(), None)
    torch.cuda.synchronize()
    fb = f.cpu().numpy()
    eb = e.cpu().numpy().reshape(-1, 2)
    for i, s in enumerate(ens):
        calc = nblib.ForceCalculator(s, opts)
        fs = calc.compute(s.x)
        o = b.offsets[i]
        assert rel_rms(fb[3 * o:3 * (o + s.n)].reshape(-1, 3), fs) <= FORCE_RTOL, (i, s.n)
        assert np.all(np.abs(eb[i] - calc.energies) <= ENERGY_RTOL * np.abs(calc.energies)), (i, eb[i])
        calc.close()
    b.close()


def test_batched_schedule_matches_sequential():
    """The scheduled batch step (search, batched rolling prune, compute) equals the per-system steps."""
    torch = pytest.importorskip("torch")
    ens = _ensemble(nsys=8, seed=10)
    opts = _opts(prune=4, rlist_inner=0.94)
    a = BatchForceCalculator(ens, opts)
    s = BatchForceCalculator(ens, opts)
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(4)
    x = np.concatenate([e.x.reshape(-1) for e in ens]).astype(np.float32)
    fa = torch.empty(x.size, dtype=torch.float32, device=dev)
    fs = torch.empty_like(fa)
    ea = torch.zeros(2 * len(ens), dtype=torch.float64, device=dev)
    es = torch.zeros_like(ea)
    for step in range(12):
        x = (x + rng.normal(0, 0.003, size=x.shape)).astype(np.float32)
        xd = torch.from_numpy(x).to(dev)
        a.md_step_device(step, xd.data_ptr(), fa.data_ptr(), ea.data_ptr())
        s.sequential_md_step_device(step, xd.data_ptr(), fs.data_ptr(), es.data_ptr())
        torch.cuda.synchronize()
        assert rel_rms(fa.cpu().numpy(), fs.cpu().numpy()) <= FORCE_RTOL, step
        assert np.all(np.abs(ea.cpu().numpy() - es.cpu().numpy()) <= ENERGY_RTOL * np.abs(es.cpu().numpy())), step


def test_autotune_picks_a_setting():
    torch = pytest.importorskip("torch")
    ens = _ensemble(nsys=6, seed=11)
    b = BatchForceCalculator(ens, _opts(prune=10, rlist_inner=0.95))
    dev = torch.device("cuda:0")
    x0 = torch.from_numpy(np.concatenate([s.x.reshape(-1) for s in ens])).to(dev)
    frames = x0[None, :] + 0.002 * torch.randn((12, x0.numel()), device=dev).cumsum(0)
    best, timings = b.autotune(frames, variants=(0, 1), prune_intervals=(4, 10), tiles=((0, 2), (1, 2), (1, 3)))
    assert best["kernel_variant"] in (0, 1) and best["nstlist_prune"] in (4, 10)
    assert (best["tile"], best["stage_depth"]) in ((0, 2), (1, 2), (1, 3))
    assert len(timings) == 12 and all(t > 0 for t in timings.values())
