"""CUDA PME kernels vs the reference's PME test data and the PME oracle (needs a GB300).

The kernels compute in float32 (fractions, weights, grids, eterm) with FP64 energy and
virial sums, like the reference's mixed-precision build; the oracle and the reference
data are FP64.  Bars: gridline indices exact; spline weights within 1e-6 of the
float32-fraction oracle; solved grids, energies and virials within 1e-5 relative of
the reference data; forces of the whole pipeline within 1e-5 relative RMS of the
oracle; energies within 1e-5 relative.
"""
import json
import os

import numpy as np
import pytest

from oracle import pme_oracle as P
from tests.helpers import rel_rms

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "pme_golden.json")
FORCE_RTOL = 1e-5
ENERGY_RTOL = 1e-5


@pytest.fixture(scope="module")
def golden():
    with open(GOLDEN) as fh:
        return json.load(fh)


@pytest.fixture(scope="module")
def pm():
    from gmxapi_gb300 import pme

    return pme


def dev(a, dtype=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


def f32(a):
    return np.asarray(a, dtype=np.float32).astype(np.float64)


def run_splines(p, x):
    N = x.shape[0]
    dx = dev(x)
    idx = torch.zeros((N, 3), dtype=torch.int32, device="cuda")
    th = torch.zeros((3, N, 4), device="cuda")
    dth = torch.zeros((3, N, 4), device="cuda")
    torch.cuda.synchronize()
    p.splines_device(N, dx.data_ptr(), idx.data_ptr(), th.data_ptr(), dth.data_ptr())
    p.synchronize()
    return idx.cpu().numpy(), th.cpu().numpy().astype(np.float64), dth.cpu().numpy().astype(np.float64)


def run_spread(p, x, q):
    dx, dq = dev(x), dev(q)
    grid = torch.full(p.grid, 7.0, device="cuda")  # spread must overwrite
    torch.cuda.synchronize()
    p.spread_device(x.shape[0], dx.data_ptr(), dq.data_ptr(), grid.data_ptr())
    p.synchronize()
    return grid.cpu().numpy().astype(np.float64)


def test_splines_match_reference_data(golden, pm):
    for case in golden["spline_spread"]:
        p = pm.Pme(case["box"], case["grid"], 3.0)
        x = np.array(case["x"], np.float32)
        idx, th, dth = run_splines(p, x)
        assert idx.tolist() == case["idx"]
        o_idx, o_th, o_dth = P.splines(x, case["box"], case["grid"], single=True)
        np.testing.assert_array_equal(idx, o_idx)
        np.testing.assert_allclose(th, o_th, rtol=0, atol=1e-6)
        np.testing.assert_allclose(dth, o_dth, rtol=0, atol=2e-6)
        for d in range(3):
            np.testing.assert_allclose(th[d].ravel(), case["theta"][d], rtol=0, atol=1e-5)
            np.testing.assert_allclose(dth[d].ravel(), case["dtheta"][d], rtol=0, atol=2e-5)
        p.close()


def test_spread_matches_reference_data(golden, pm):
    for case in golden["spline_spread"]:
        p = pm.Pme(case["box"], case["grid"], 3.0)
        x = np.array(case["x"], np.float32)
        grid = run_spread(p, x, np.array(case["q"], np.float32))
        got = {f"Cell {i} {j} {k}": grid[i, j, k] for i, j, k in zip(*np.nonzero(grid))}
        assert set(got) == set(case["grid_values"])
        ref = np.array([case["grid_values"][k] for k in sorted(got)])
        val = np.array([got[k] for k in sorted(got)])
        # relative to the largest point: the tiny corner weights carry the float32 fraction's error
        assert np.max(np.abs(val - ref)) <= 1e-5 * np.max(np.abs(ref))
        o_idx, o_th, _ = P.splines(x, case["box"], case["grid"], single=True)
        o_grid = P.spread(o_idx, o_th, f32(case["q"]), tuple(case["grid"]))
        assert np.max(np.abs(grid - o_grid)) <= 1e-6 * np.max(np.abs(o_grid))
        p.close()


@pytest.mark.parametrize("layout", ["uniform", "crowded", "odd_z"])
def test_spread_paths_match_oracle(pm, layout):
    """nz % 4 == 0 spreads with 16-byte vector reductions, other nz with scalar atomics; the
    crowded case piles every atom onto a few grid points (maximal atomic contention)."""
    rng = np.random.default_rng(5)
    box = (3.0, 3.2, 2.8)
    grid = (32, 36, 28) if layout != "odd_z" else (32, 36, 25)
    N = 6000
    if layout == "crowded":
        x = (rng.random((N, 3)) * 0.3 + 1.0).astype(np.float32)  # all in one 0.3 nm cube
    else:
        x = (rng.random((N, 3)) * np.array(box) * 1.5 - 0.25 * np.array(box)).astype(np.float32)
    q = rng.standard_normal(N).astype(np.float32)
    q[::7] = 0.0
    p = pm.Pme(box, grid, 3.0)
    g = run_spread(p, x, q)
    idx, th, _ = P.splines(x, box, grid, single=True)
    ref = P.spread(idx, th, q, grid)
    assert np.max(np.abs(g - ref)) <= 1e-5 * np.max(np.abs(ref))
    f = p.compute(x, q)
    ref_f, ref_e, _ = P.compute(x, q, box, grid, 3.0, single=True)
    assert rel_rms(f, ref_f) <= FORCE_RTOL
    assert p.energy == pytest.approx(ref_e, rel=ENERGY_RTOL)
    p.close()


def _complex_input(case):
    n = case["grid"]
    c = np.zeros((n[0], n[1], n[2] // 2 + 1, 2), np.float32)
    for (i, j, k), (re, im) in case["input"]:
        c[i, j, k] = (re, im)
    return c


@pytest.mark.parametrize("energy", [True, False])
def test_solve_matches_reference_data(golden, pm, energy):
    for case in golden["solve"]:
        p = pm.Pme(case["box"], case["grid"], case["beta"], epsilon_r=case["epsilon_r"])
        c = dev(_complex_input(case))
        e = torch.zeros(1, dtype=torch.float64, device="cuda")
        v = torch.zeros(9, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        p.solve_device(c.data_ptr(), e.data_ptr() if energy else None, v.data_ptr() if energy else None)
        p.synchronize()
        out = c.cpu().numpy().astype(np.float64)
        for key, val in case["output"].items():
            parts = key.split()
            got = out[int(parts[1]), int(parts[2]), int(parts[3]), 0 if parts[4] == "re" else 1]
            assert got == pytest.approx(val, rel=1e-5, abs=1e-30)
        if energy:
            assert e.item() == pytest.approx(case["energy"], rel=ENERGY_RTOL, abs=1e-30)
            vir = v.cpu().numpy().reshape(3, 3)
            for key, val in case["virial"].items():
                _, a, b = key.split()
                assert vir[int(a), int(b)] == pytest.approx(val, rel=1e-5, abs=1e-30)
            np.testing.assert_array_equal(vir, vir.T)
        p.close()


def test_gather_matches_oracle(pm):
    rng = np.random.default_rng(11)
    box = (2.3, 1.9, 2.7)
    n = (20, 16, 24)
    N = 500
    x = (rng.random((N, 3)) * np.array(box) * 3 - np.array(box)).astype(np.float32)  # images -1..2 boxes
    q = rng.standard_normal(N).astype(np.float32)
    grid = rng.standard_normal(n).astype(np.float32)
    p = pm.Pme(box, n, 3.0)
    dx, dq, dg = dev(x), dev(q), dev(grid)
    f0 = rng.standard_normal((N, 3)).astype(np.float32)
    df = dev(f0)
    torch.cuda.synchronize()
    p.gather_device(N, dx.data_ptr(), dq.data_ptr(), dg.data_ptr(), df.data_ptr())
    p.synchronize()
    f = df.cpu().numpy().astype(np.float64) - f0  # gather adds
    idx, th, dth = P.splines(x, box, n, single=True)
    ref = P.gather(grid.astype(np.float64), idx, th, dth, q, n, box)
    assert rel_rms(f, ref) <= 1e-6
    p.close()


def _systems():
    from gmxapi_gb300 import systems

    return {
        "water900": lambda: systems.spc_water(300, 2.08, seed=5),
        "water3000": lambda: systems.water_small(),
        "lj_liquid_charged": lambda: systems.lj_liquid(n=1500, ntypes=8, seed=8),
        "water_tiny": lambda: systems.spc_water(20, 0.84, seed=7),
    }


@pytest.mark.parametrize("name", ["water900", "water3000", "lj_liquid_charged", "water_tiny"])
@pytest.mark.parametrize("spacing", [0.12, 0.1])
def test_compute_matches_oracle(pm, name, spacing):
    s = _systems()[name]()
    box = [float(b) for b in s.box]
    n = P.fft_grid_size(box[0], spacing), P.fft_grid_size(box[1], spacing), P.fft_grid_size(box[2], spacing)
    beta = pm.ewald_coefficient(0.9, 1e-5)
    p = pm.Pme(box, n, beta)
    f = p.compute(s.x, s.q)
    ref_f, ref_e, ref_v = P.compute(s.x, s.q, box, n, beta, single=True)
    assert rel_rms(f, ref_f) <= FORCE_RTOL
    assert p.energy == pytest.approx(ref_e, rel=ENERGY_RTOL)
    assert np.max(np.abs(p.virial - ref_v)) <= ENERGY_RTOL * np.max(np.abs(ref_v))
    p.close()


def test_compute_adds_to_forces_and_images_agree(pm):
    from gmxapi_gb300 import systems

    s = systems.spc_water(300, 2.08, seed=5)
    box = [float(b) for b in s.box]
    p = pm.Pme(box, (20, 20, 20), 3.12)
    base = np.full((s.n, 3), 1.5, np.float32)
    f = p.compute(s.x, s.q, forces=base.copy())
    e = p.energy
    f_alone = p.compute(s.x, s.q)
    np.testing.assert_allclose(f - 1.5, f_alone, rtol=0, atol=2e-5 * np.abs(f_alone).max())
    # the same atoms one box length away (and two, and minus one) in each dimension
    shifts = np.array([[1, -1, 2], [-1, 2, 1]], np.float32) * np.array(box, np.float32)
    for sh in shifts:
        x_img = s.x + sh  # rounded to float32 again: up to 8x coarser than the in-box coordinates
        f_img = p.compute(x_img, s.q)
        ref_f, ref_e, _ = P.compute(x_img, s.q, box, (20, 20, 20), 3.12, single=True)
        assert rel_rms(f_img, ref_f) <= FORCE_RTOL
        assert p.energy == pytest.approx(ref_e, rel=ENERGY_RTOL)
        assert rel_rms(f_img, f_alone) <= 5e-5
        assert p.energy == pytest.approx(e, rel=1e-5)
    p.close()


def test_repeated_calls_keep_their_state(pm):
    """One handle through many calls of different sizes (the solve's completion counter and
    partial sums are reused): every energy equals the oracle's."""
    from gmxapi_gb300 import systems

    s = systems.rock_salt(cells=4, nn_distance=0.282)
    box = [float(b) for b in s.box]
    n = (20, 20, 20)
    p = pm.Pme(box, n, 3.12)
    _, ref_e, _ = P.compute(s.x, s.q, box, n, 3.12, single=True)
    rng = np.random.default_rng(9)
    for k in range(4):
        p.compute(s.x, s.q, energies=(k % 2 == 1))
        if k % 2 == 1:
            assert p.energy == pytest.approx(ref_e, rel=ENERGY_RTOL)
        # a larger system on the same handle
        x = (rng.random((3000 * (k + 1), 3)) * np.array(box)).astype(np.float32)
        q = rng.standard_normal(x.shape[0]).astype(np.float32)
        p.compute(x, q)
        assert p.energy == pytest.approx(P.compute(x, q, box, n, 3.12, single=True)[1], rel=ENERGY_RTOL)
    p.compute(s.x, s.q)
    assert p.energy == pytest.approx(ref_e, rel=ENERGY_RTOL)
    p.close()


def test_empty_and_uncharged(pm):
    p = pm.Pme((2.0, 2.0, 2.0), (16, 16, 16), 3.12)
    f = p.compute(np.zeros((0, 3), np.float32), np.zeros(0, np.float32))
    assert f.shape == (0, 3) and p.energy == 0.0 and not p.virial.any()
    x = np.random.default_rng(3).random((50, 3)).astype(np.float32) * 2
    f = p.compute(x, np.zeros(50, np.float32))
    assert not f.any() and p.energy == 0.0
    p.close()


def test_full_ewald_reproduces_the_madelung_constant(pm):
    """Real space (cluster-pair kernel, self term included) + reciprocal space (PME) on a
    perfect rock-salt crystal: E = -N/2 M f / a and zero force on every ion."""
    from gmxapi_gb300 import nblib, systems

    s = systems.rock_salt(cells=4, nn_distance=0.282)
    rc = 1.0
    opts = nblib.NBKernelOptions(coulomb_type=nblib.CoulombType.Pme, pairlist_cutoff=rc, rcoulomb=rc,
                                 compute_virial_and_energy=True)
    calc = nblib.ForceCalculator(s, opts)
    f_real = calc.compute(s.x).astype(np.float64)
    e_real = calc.energies[1]
    box = [float(b) for b in s.box]
    p = pm.Pme(box, pm.grid_size(box, 0.1), pm.ewald_coefficient(rc, 1e-5))
    f_rec = p.compute(s.x, s.q).astype(np.float64)
    e_madelung = -s.n / 2 * systems.MADELUNG_ROCK_SALT * P.ONE_4PI_EPS0 / 0.282
    assert e_real + p.energy == pytest.approx(e_madelung, rel=2e-5)
    f = f_real + f_rec
    assert np.abs(f).max() <= 1e-3 * P.ONE_4PI_EPS0 / 0.282 ** 2
    p.close()
    calc.close()


def test_water_288k_matches_oracle(pm):
    """The benchmark box: 288,000 atoms, 120^3 grid."""
    from gmxapi_gb300 import systems

    s = systems.water_large()
    box = [float(b) for b in s.box]
    n = pm.grid_size(box, 0.12)
    assert n == (120, 120, 120)
    beta = pm.ewald_coefficient(0.9, 1e-5)
    p = pm.Pme(box, n, beta)
    f = p.compute(s.x, s.q)
    ref_f, ref_e, ref_v = P.compute(s.x, s.q, box, n, beta, single=True)
    assert rel_rms(f, ref_f) <= FORCE_RTOL
    assert p.energy == pytest.approx(ref_e, rel=ENERGY_RTOL)
    assert np.max(np.abs(p.virial - ref_v)) <= ENERGY_RTOL * np.max(np.abs(ref_v))
    # PME does not conserve momentum (energies, not forces, are interpolated): the net force
    # is the oracle's, to float32 accumulation
    net = f.astype(np.float64).sum(0)
    assert np.abs(net - ref_f.sum(0)).max() <= 1e-5 * np.abs(ref_f).max() * np.sqrt(s.n)
    p.close()
