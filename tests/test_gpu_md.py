"""GPU-resident MD: leap-frog kernel, force accumulation, the step loop vs the MD oracle (needs a GB300).

Bars: the leap-frog update is bit-exact against the float32 oracle (same operations in the same
order, no contraction); kinetic energies within 1e-8 (per-atom |v|^2 in float, sums in FP64); the nblib integrator test's analytic bound;
MD trajectories of 20 steps (nonbonded + PME + leap-frog) within 2e-5 nm of the oracle's and energy
rows within 1e-5; total-energy drift of an NVE liquid bounded.
"""
import numpy as np
import pytest

from oracle import md_oracle as M
from oracle import pme_oracle as P
from tests.helpers import rel_rms

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def md():
    from gmxapi_gb300 import md as md_mod

    return md_mod


def test_leapfrog_host_call_is_bit_exact(md):
    rng = np.random.default_rng(1)
    box = (2.3, 1.7, 3.1)
    n = 5000
    x = ((rng.random((n, 3)) * 1.4 - 0.2) * np.array(box)).astype(np.float32)  # some outside the box
    v = rng.standard_normal((n, 3)).astype(np.float32)
    f = (rng.standard_normal((n, 3)) * 300).astype(np.float32)
    im = (1.0 / rng.uniform(1.0, 40.0, n)).astype(np.float32)
    lf = md.LeapFrog(im, box)
    xg, vg = x.copy(), v.copy()
    lf.integrate(0.002, xg, vg, f)
    xo, vo, _ = M.leapfrog(x, v, f, im, 0.002, box)
    np.testing.assert_array_equal(vg, vo)
    np.testing.assert_array_equal(xg, xo)
    lf.close()


def test_leapfrog_reproduces_nblib_integrator_test(md):
    """api/nblib/tests/integrator.cpp IntegratorWorks on the GPU."""
    dt, steps = 0.001, 100
    lf = md.LeapFrog(np.ones(1, np.float32), (100.0, 100.0, 100.0))
    x = np.zeros((1, 3), np.float32)
    v = np.zeros((1, 3), np.float32)
    f = np.array([[1.0, 2.0, 0.0]], np.float32)
    for step in range(steps):
        t = step * dt
        np.testing.assert_allclose(x[0], 0.5 * f[0] * t * t, rtol=0, atol=steps * 5e-6)
        np.testing.assert_allclose(v[0], f[0] * t, rtol=0, atol=steps * 5e-6)
        lf.integrate(dt, x, v, f)
    lf.close()


def test_leapfrog_device_kinetic_energy(md):
    rng = np.random.default_rng(2)
    box = (3.0, 3.0, 3.0)
    n = 100000  # several blocks per SM: the completion counter and partial sums
    x = (rng.random((n, 3)) * 3.0).astype(np.float32)
    v = rng.standard_normal((n, 3)).astype(np.float32)
    f = (rng.standard_normal((n, 3)) * 100).astype(np.float32)
    im = (1.0 / rng.uniform(1.0, 16.0, n)).astype(np.float32)
    lf = md.LeapFrog(im, box)
    dx, dv, df = (torch.from_numpy(a.reshape(-1).copy()).cuda() for a in (x, v, f))
    e = torch.zeros(1, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    for k in range(3):  # repeated calls reuse the counter
        lf.integrate_device(0.002, dx.data_ptr(), dv.data_ptr(), df.data_ptr(), e.data_ptr())
        torch.cuda.synchronize()
        x, v, ke = M.leapfrog(x, v, f, im, 0.002, box)
        # per-atom |v|^2 in float (FMA), the sum over atoms in FP64
        assert e.item() == pytest.approx(ke, rel=1e-8)
    np.testing.assert_array_equal(dx.cpu().numpy().reshape(-1, 3), x)
    lf.close()


def test_force_accumulate(md):
    from gmxapi_gb300 import nblib, systems

    s = systems.spc_water(300, 2.08, seed=5)
    opts = nblib.NBKernelOptions(pairlist_cutoff=1.0, rcoulomb=0.9)
    calc = nblib.ForceCalculator(s, opts)
    dx = torch.from_numpy(s.x.reshape(-1).copy()).cuda()
    f_alone = torch.zeros(3 * s.n, device="cuda")
    torch.cuda.synchronize()
    calc.compute_device(dx.data_ptr(), f_alone.data_ptr())
    calc.synchronize()
    calc.set_force_accumulate(True)
    base = torch.full((3 * s.n,), 2.5, device="cuda")
    f = base.clone()
    torch.cuda.synchronize()
    calc.compute_device(dx.data_ptr(), f.data_ptr())
    calc.synchronize()
    np.testing.assert_allclose((f - base).cpu().numpy(), f_alone.cpu().numpy(), rtol=0,
                               atol=2e-6 * float(f_alone.abs().max()))
    # the host-array call still overwrites
    fh = calc.compute(s.x)
    assert rel_rms(fh.reshape(-1), f_alone.cpu().numpy()) <= 1e-6
    calc.close()


def _liquid():
    """864 argon-like atoms from an fcc lattice, charges +-0.3 e (so PME matters)."""
    from gmxapi_gb300 import systems

    s = systems.lj_fcc(cells=6, lattice=0.5256, charge=0.3, seed=21)
    masses = np.full(s.n, systems.ARGON_MASS, np.float32)
    return s, masses


@pytest.mark.parametrize("with_pme,prune", [(True, False), (False, False), (True, True)])
def test_md_run_matches_oracle(md, with_pme, prune):
    """prune: dynamic pruning to rlist_inner 0.92 every 4 steps (2 rolling parts), against the
    oracle's unpruned list: pruning drops only pairs that stay beyond rc, so the trajectory is the
    same."""
    from gmxapi_gb300 import nblib
    from gmxapi_gb300 import pme as pm

    s, masses = _liquid()
    rng = np.random.default_rng(4)
    v0 = (rng.standard_normal((s.n, 3)) * np.sqrt(0.00831446 * 120.0 / 39.948)).astype(np.float32)
    extra = {"rlist_inner": 0.92, "nstlist_prune": 4} if prune else {}
    opts = nblib.NBKernelOptions(pairlist_cutoff=1.0, rcoulomb=0.9, nstlist=10, compute_virial_and_energy=True,
                                 **extra)
    run = md.MdRunner(s, masses, opts, dt=0.002, velocities=v0, pme=with_pme)
    rows = run.run(20, nstcalcenergy=1)
    box = [float(b) for b in s.box]
    grid = pm.grid_size(box, 0.12) if with_pme else None
    beta = pm.ewald_coefficient(0.9, 1e-5)
    xo, vo, ro = M.md_run(s, 1.0 / masses.astype(np.float64), s.x, v0, 20, 0.002, rc=0.9, rlist=1.0, nstlist=10,
                          pme_grid=grid, beta=beta)
    xg, vg = run.positions(), run.velocities()
    # compare positions as periodic images
    d = xg - xo
    d -= np.round(d / np.array(box)) * np.array(box)
    assert np.abs(d).max() <= 2e-5
    assert rel_rms(vg, vo) <= 2e-5
    assert rows.shape == (20, 4)
    for c in range(4):
        if np.abs(ro[:, c]).max() > 0:
            np.testing.assert_allclose(rows[:, c], ro[:, c], rtol=1e-5, atol=1e-5 * np.abs(ro[:, c]).max())
    run.close()


def test_md_nve_energy_drift(md):
    """2,000 steps (4 ps) of NVE argon-like atoms with charges (LJ + Ewald + PME), started from
    the lattice at 120 K: total-energy drift bounded."""
    from gmxapi_gb300 import nblib

    s, masses = _liquid()
    rng = np.random.default_rng(7)
    v0 = (rng.standard_normal((s.n, 3)) * np.sqrt(0.00831446 * 120.0 / 39.948)).astype(np.float32)
    opts = nblib.NBKernelOptions(pairlist_cutoff=1.1, rcoulomb=0.9, nstlist=10, compute_virial_and_energy=True,
                                 use_ewald_shift=True)
    run = md.MdRunner(s, masses, opts, dt=0.002, velocities=v0, pme=True, fourier_spacing=0.1)
    rows = run.run(2000, nstcalcenergy=20)
    etot = rows.sum(axis=1)
    ekin = rows[:, 3]
    drift = abs(etot[-1] - etot[0])
    print(f"NVE: E_tot {etot[0]:.3f} -> {etot[-1]:.3f}, mean E_kin {ekin.mean():.3f}, "
          f"fluctuation {etot.std():.4f}")
    assert np.all(np.isfinite(etot))
    assert drift <= 2e-3 * ekin.mean()  # measured ~3e-5
    run.close()


def test_leapfrog_kernel_reproduces_the_reference_leapfrog_test(md):
    """The reference's own LeapFrogTest.SimpleIntegration data (10 cases without coupling) through
    the GPU update; the kernel puts atoms in the box, so positions are compared modulo the box
    (edges 25, 10, 10 nm), within the reference test's tolerance (absolute, steps x 5e-6) plus the
    rounding of the wrap."""
    import json
    import os

    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "leapfrog_golden.json")) as fh:
        cases = json.load(fh)["cases"]
    box = np.array([25.0, 10.0, 10.0])
    for case in cases:
        n = case["num_atoms"]
        i = np.arange(n)
        x = np.stack([(i % 21) * 1.0, 6.5 - (i % 13) * 1.0, np.zeros(n)], -1).astype(np.float32)
        v = np.tile(np.array(case["v0"], np.float32), (n, 1))
        f = np.tile(np.array(case["f0"], np.float32), (n, 1))
        im = (1.0 / (1.0 + (i % 100))).astype(np.float32)
        lf = md.LeapFrog(im, tuple(box))
        for _ in range(case["num_steps"]):
            lf.integrate(case["dt"], x, v, f)
        lf.close()
        want = np.array(case["final_x"])
        want = want - np.floor(want / box) * box
        d = np.abs(x - want)
        d = np.minimum(d, box - d)  # a coordinate on the box edge may wrap to either side
        tol = case["tolerance"] + 2e-6
        assert d.max() <= tol, (case["index"], d.max())
        np.testing.assert_allclose(v, case["final_v"], rtol=0, atol=case["tolerance"])
