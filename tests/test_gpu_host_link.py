"""Host arrays in mapped pinned memory: the kernels read the coordinates and write the forces in
place over the host link instead of staging them with copies (needs a GB300).

Bar: the same forces as the copy-staged path (pageable numpy arrays) to 1e-6 relative RMS (only the
order of the j-force atomics differs between runs), the same energies to 1e-9 and virial to 1e-5 of
its largest element, over a schedule with search steps, rolling-prune steps and plain steps.
"""
import numpy as np
import pytest

from gmxapi_gb300 import nblib, systems
from tests.helpers import rel_rms

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _opts():
    return nblib.NBKernelOptions(pairlist_cutoff=1.0, rcoulomb=0.9, rlist_inner=0.95, nstlist=10,
                                 nstlist_prune=4, compute_virial_and_energy=True)


def _pinned(a):
    t = torch.from_numpy(np.ascontiguousarray(a, np.float32)).pin_memory()
    return t, t.numpy()


def test_md_steps_with_mapped_host_arrays_match_staged_copies():
    s = systems.spc_water(1000, 3.104, seed=11)
    rng = np.random.default_rng(4)
    staged = nblib.ForceCalculator(s, _opts())
    mapped = nblib.ForceCalculator(s, _opts())
    x = s.x.astype(np.float32).copy()
    xt, xp = _pinned(x)
    ft, fp = _pinned(np.zeros_like(x))
    for step in range(25):
        x += rng.normal(0.0, 0.002, x.shape).astype(np.float32)
        xp[:] = x
        fa = staged.md_step(step, x, energies=True)
        mapped.md_step(step, xp, forces=fp, energies=True)
        assert rel_rms(fp.astype(np.float64), fa.astype(np.float64)) <= 1e-6, step
        assert np.allclose(mapped.energies, staged.energies, rtol=1e-9, atol=0.0), step
        # the virial sums x (x) f over float forces whose j-parts are added by atomics in any order
        assert np.allclose(mapped.virial, staged.virial, rtol=1e-4, atol=1e-5 * np.abs(staged.virial).max())
    staged.close()
    mapped.close()


def test_compute_with_mapped_host_arrays_matches_staged_copies():
    s = systems.spc_water(1000, 3.104, seed=12)
    a = nblib.ForceCalculator(s, _opts())
    b = nblib.ForceCalculator(s, _opts())
    x = s.x.astype(np.float32)
    xt, xp = _pinned(x)
    ft, fp = _pinned(np.full_like(x, 7.0))  # overwritten, not accumulated
    fa = a.compute(x)
    b.compute(xp, forces=fp)
    assert rel_rms(fp.astype(np.float64), fa.astype(np.float64)) <= 1e-6
    assert np.allclose(b.energies, a.energies, rtol=1e-9, atol=0.0)
    a.close()
    b.close()


@pytest.mark.parametrize("pinned", ["x", "f"])
def test_one_mapped_array_and_one_pageable(pinned):
    """Each host array takes its own route: in place when mapped, copied otherwise."""
    s = systems.spc_water(1000, 3.104, seed=13)
    a = nblib.ForceCalculator(s, _opts())
    b = nblib.ForceCalculator(s, _opts())
    x = s.x.astype(np.float32)
    xt, xp = _pinned(x)
    ft, fp = _pinned(np.zeros_like(x))
    for step in range(12):
        fa = a.md_step(step, x, energies=True)
        if pinned == "x":
            fb = b.md_step(step, xp, energies=True)
        else:
            fb = b.md_step(step, x, forces=fp, energies=True)
        assert rel_rms(fb.astype(np.float64), fa.astype(np.float64)) <= 1e-6, step
        assert np.allclose(b.energies, a.energies, rtol=1e-9, atol=0.0), step
    a.close()
    b.close()
