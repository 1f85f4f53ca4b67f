"""The PME oracle against the reference's own PME unit-test data and an exact Ewald sum (CPU)."""
import json
import os

import numpy as np
import pytest

from oracle import pme_oracle as P

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "pme_golden.json")


@pytest.fixture(scope="module")
def golden():
    with open(GOLDEN) as fh:
        return json.load(fh)


def f32(a):
    """The reference's test inputs are float literals (0.12F), widened to double."""
    return np.asarray(a, dtype=np.float32).astype(np.float64)


def test_spline_moduli_match_reference_data(golden):
    for case in golden["moduli"]:
        for d, key in enumerate("xyz"):
            ref = np.array(case[key])
            got = P.bspline_moduli(case["grid"][d])
            np.testing.assert_allclose(got, ref, rtol=1e-13, atol=0)


def test_splines_and_spread_match_reference_data(golden):
    assert len(golden["spline_spread"]) == 6
    for case in golden["spline_spread"]:
        n = tuple(case["grid"])
        idx, theta, dtheta = P.splines(np.array(case["x"]), case["box"], n, single=False)
        assert idx.tolist() == case["idx"]  # includes coordinates beyond 2 box lengths and negative ones
        for d in range(3):
            np.testing.assert_allclose(theta[d].ravel(), case["theta"][d], rtol=0, atol=1e-14)
            np.testing.assert_allclose(dtheta[d].ravel(), case["dtheta"][d], rtol=0, atol=1e-14)
        grid = P.spread(idx, theta, f32(case["q"]), n)
        got = {f"Cell {i} {j} {k}": grid[i, j, k] for i, j, k in zip(*np.nonzero(grid))}
        assert set(got) == set(case["grid_values"])
        for key, val in case["grid_values"].items():
            assert got[key] == pytest.approx(val, rel=1e-12)


def test_single_precision_fraction_stays_close(golden):
    """The float32 fraction (what the CUDA kernels compute) changes the weights by ~1e-6 at most."""
    for case in golden["spline_spread"]:
        idx, theta, _ = P.splines(np.array(case["x"]), case["box"], tuple(case["grid"]), single=True)
        assert idx.tolist() == case["idx"]
        for d in range(3):
            np.testing.assert_allclose(theta[d].ravel(), case["theta"][d], rtol=0, atol=1e-5)


def _complex_grid(case):
    n = case["grid"]
    c = np.zeros((n[0], n[1], n[2] // 2 + 1), dtype=np.complex128)
    for (i, j, k), (re, im) in case["input"]:
        c[i, j, k] = f32(re) + 1j * f32(im)
    return c


def test_solve_matches_reference_data(golden):
    assert len(golden["solve"]) == 12
    for case in golden["solve"]:
        out, energy, vir = P.solve(_complex_grid(case), tuple(case["grid"]), case["box"], case["beta"],
                                   case["epsilon_r"])
        for key, val in case["output"].items():
            parts = key.split()
            v = out[int(parts[1]), int(parts[2]), int(parts[3])]
            got = v.real if parts[4] == "re" else v.imag
            assert got == pytest.approx(val, rel=1e-12, abs=1e-300)
        assert energy == pytest.approx(case["energy"], rel=1e-12, abs=1e-300)
        for key, val in case["virial"].items():
            _, a, b = key.split()
            assert vir[int(a), int(b)] == pytest.approx(val, rel=1e-12, abs=1e-300)
            assert vir[int(b), int(a)] == vir[int(a), int(b)]


def test_gather_matches_reference_data(golden):
    assert len(golden["gather"]) == 12
    for case in golden["gather"]:
        n = tuple(case["grid"])
        grid = np.zeros(n)
        for (i, j, k), val in case["grid_values"]:
            grid[i, j, k] = f32(val)
        N = len(case["q"])
        theta = f32(case["theta"]).reshape(3, N, 4)
        dtheta = f32(case["dtheta"]).reshape(3, N, 4)
        f = P.gather(grid, np.array(case["idx"]), theta, dtheta, f32(case["q"]), n, case["box"])
        np.testing.assert_allclose(f, np.array(case["forces"]), rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize("length,spacing,expected", [
    (2.0, 0.12, 20),     # nmin 17 -> first listed size >= 17
    (0.5, 0.12, 6),      # minimalPmeGridSize
    (5.2, 0.12, 44),     # nmin 44: last of the initial list
    (5.5, 0.12, 48),     # nmin 46 -> 48 (45 is not a multiple of 4)
    (10.8, 0.12, 96),    # nmin 90: 2 * 45 = 90 is never tried, the search stops before the first base size
    (10.6, 0.12, 96),    # nmin 89
    (14.21, 0.12, 120),  # the 288k-atom water box
    (16.5, 0.12, 144),   # nmin 138: 140 is excluded
])
def test_fft_grid_size(length, spacing, expected):
    assert P.fft_grid_size(length, spacing) == expected


def _random_neutral(seed, n, box):
    rng = np.random.default_rng(seed)
    x = rng.random((n, 3)) * np.asarray(box)
    q = rng.standard_normal(n)
    return x, q - q.mean()


def test_pme_converges_to_exact_ewald_sum():
    """Spread / solve / gather against a direct FP64 k-space sum: error falls like h^4."""
    box = [2.1, 2.3, 1.9]
    x, q = _random_neutral(1, 60, box)
    beta = 3.12
    e_ex, f_ex, v_ex = P.ewald_reciprocal_exact(x, q, box, beta, [30, 30, 30])
    errs = []
    for spacing in (0.08, 0.04):
        n = [P.fft_grid_size(b, spacing) for b in box]
        f, e, v = P.compute(x, q, box, n, beta, single=False)
        rr = np.sqrt(((f - f_ex) ** 2).sum() / (f_ex ** 2).sum())
        errs.append(rr)
        assert abs(e - e_ex) / abs(e_ex) < 2e-4
        assert np.max(np.abs(v - v_ex)) / np.max(np.abs(v_ex)) < 2e-3
    assert errs[0] < 1e-3 and errs[1] < errs[0] / 5


def test_exact_virial_is_half_the_strain_derivative():
    box = [2.1, 2.3, 1.9]
    x, q = _random_neutral(2, 40, box)
    beta = 3.12
    _, _, vir = P.ewald_reciprocal_exact(x, q, box, beta, [24, 24, 24])
    eps = 1e-6
    for a in range(3):
        bp, bm = list(box), list(box)
        bp[a] *= 1 + eps
        bm[a] *= 1 - eps
        xp, xm = x.copy(), x.copy()
        xp[:, a] *= 1 + eps
        xm[:, a] *= 1 - eps
        ep = P.ewald_reciprocal_exact(xp, q, bp, beta, [24, 24, 24])[0]
        em = P.ewald_reciprocal_exact(xm, q, bm, beta, [24, 24, 24])[0]
        assert 0.5 * (ep - em) / (2 * eps) == pytest.approx(vir[a, a], rel=1e-6)


def test_exact_forces_are_the_energy_gradient():
    box = [2.1, 2.3, 1.9]
    x, q = _random_neutral(3, 12, box)
    _, f, _ = P.ewald_reciprocal_exact(x, q, box, 3.12, [20, 20, 20])
    h = 1e-6
    for i, d in ((0, 0), (5, 1), (11, 2)):
        xp, xm = x.copy(), x.copy()
        xp[i, d] += h
        xm[i, d] -= h
        ep = P.ewald_reciprocal_exact(xp, q, box, 3.12, [20, 20, 20])[0]
        em = P.ewald_reciprocal_exact(xm, q, box, 3.12, [20, 20, 20])[0]
        assert -(ep - em) / (2 * h) == pytest.approx(f[i, d], rel=1e-5, abs=1e-3)


def test_lj_solve_matches_reference_data(golden):
    assert len(golden["solve_lj"]) == 12
    for case in golden["solve_lj"]:
        out, energy, vir = P.solve_lj(_complex_grid(case), tuple(case["grid"]), case["box"], case["beta_lj"])
        for key, val in case["output"].items():
            parts = key.split()
            v = out[int(parts[1]), int(parts[2]), int(parts[3])]
            got = v.real if parts[4] == "re" else v.imag
            assert got == pytest.approx(val, rel=1e-10, abs=1e-300)
        assert energy == pytest.approx(case["energy"], rel=1e-10)
        for key, val in case["virial"].items():
            _, a, b = key.split()
            assert vir[int(a), int(b)] == pytest.approx(val, rel=1e-9, abs=1e-12 * abs(case["energy"]))


def test_lj_pme_reproduces_the_fcc_lattice_energy():
    """LJ-PME real space (FP64 all-pairs, geometric grid) + the dispersion grid on an argon fcc
    crystal: the untruncated lattice sums 0.5 N (C12 A12 / a^12 - C6 A6 / a^6), A6 = 14.45392,
    A12 = 12.13188, less the repulsion's potential shift inside rc."""
    from gmxapi_gb300 import build, systems

    build.build()
    from gmxapi_gb300 import pme as pm
    from oracle import oracle as O

    s = systems.lj_fcc(cells=6, lattice=0.5256, charge=0.0, seed=0)
    rc = 0.9
    bl = pm.ewald_coefficient_lj(rc, 1e-3)
    f_real, e_real = O.fp64_allpairs(s, rc=rc, beta=3.47, vdw_modifier=4, beta_lj=bl)
    nb = np.asarray(s.nbfp).reshape(-1, 2)
    c6, c12 = float(nb[0, 0]) / 6.0, float(nb[0, 1]) / 12.0
    box = [float(b) for b in s.box]
    f_rec, e_rec, _ = P.compute(s.x, np.full(s.n, np.sqrt(c6)), box, (40, 40, 40), bl, single=False, lj=True)
    a = 0.5256 / np.sqrt(2.0)
    d = s.x[0] - s.x
    d -= np.round(d / s.box) * s.box
    r = np.sqrt((d * d).sum(1))
    n_rc = int(np.sum((r > 0) & (r < rc)))
    expect = 0.5 * s.n * (c12 * 12.13188 / a ** 12 - c6 * 14.45392 / a ** 6) - 0.5 * s.n * n_rc * c12 / rc ** 12
    assert e_real[0] + e_rec == pytest.approx(expect, rel=2e-5)
    assert np.abs(f_real + f_rec).max() < 1e-2  # lattice sites are force-free


def test_fft_golden_vector_is_numpy_rfftn():
    """The reference's 3D FFT test vector (tests/golden/fft_golden.json, from FFFTest3D.Real5_6_9)
    is numpy's unnormalised rfftn forward and N * irfftn backward in the engine's layout."""
    import json
    import os

    import numpy as np

    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "fft_golden.json")) as fh:
        g = json.load(fh)
    grid = g["grid"]
    nzc = grid[2] // 2 + 1
    x = np.array(g["forward_input"]).reshape(grid)
    want = np.array(g["forward_output"]).reshape(grid[0], grid[1], nzc, 2)
    np.testing.assert_allclose(np.fft.rfftn(x), want[..., 0] + 1j * want[..., 1], rtol=1e-12, atol=1e-10)
    c = np.array(g["backward_input"]).reshape(grid[0], grid[1], nzc, 2)
    back = np.fft.irfftn(c[..., 0] + 1j * c[..., 1], s=grid, axes=(0, 1, 2)) * np.prod(grid)
    np.testing.assert_allclose(back, np.array(g["backward_output"]).reshape(grid), rtol=1e-12, atol=1e-10)
    assert g["reference_complex_axis_order"] == ["y", "kz", "x"]
