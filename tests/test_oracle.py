"""The CPU oracle itself: pinned to the reference's golden vectors and to FP64.

Mirrors api/nblib/tests/nbkernelsystem.cpp (ArgonForcesAreCorrect,
SpcMethanolForcesAreCorrect, UpdateChangesForces) at the reference's own
tolerance (api/nblib/tests/testhelpers.h:72-77: 200 single-precision ULP).
"""
import numpy as np
import pytest

from gmxapi_gb300 import systems
from oracle import oracle as O
from tests.helpers import canonical_pairs, nblib_golden_system, rel_rms, ulp_distance


@pytest.mark.parametrize("key", ["argon", "spc_methanol"])
def test_oracle_matches_nblib_golden(key):
    s, ref = nblib_golden_system(key)
    o = O.Oracle(s, coulomb=O.COULOMB_CUTOFF, rc=1.0, rlist=1.0)
    o.grid()
    o.search()
    o.force(energy=False)
    f = o.forces()
    assert ulp_distance(f, ref).max() <= 200


def test_oracle_repeatable_and_changes_with_update():
    s, _ = nblib_golden_system("spc_methanol")
    o = O.Oracle(s, coulomb=O.COULOMB_CUTOFF, rc=1.0, rlist=1.0)
    o.grid()
    o.search()
    o.force(False)
    f1 = o.forces()
    o.force(False)
    assert np.array_equal(f1, o.forces())
    o.set_x(s.x + np.float32(0.001))
    o.force(False)
    assert not np.array_equal(f1, o.forces())


def test_ewald_coefficient_and_table():
    s = systems.water_small()
    o = O.Oracle(s, rc=0.9, rlist=1.0)
    # beta from erfc(beta*rc) = 1e-5 (ewald/ewald_utils.cpp:46-71)
    assert abs(o.beta - 3.4705) < 1e-3
    scale, F, V = o.table()
    assert len(F) == int(0.9 * scale) + 2
    # the F table approximates -d/dr erf(beta r)/r
    from math import erf, exp, pi, sqrt
    b = o.beta
    for r in (0.1, 0.3, 0.6, 0.85):
        exact = -(2 * b / sqrt(pi) * exp(-(b * r) ** 2) / r - erf(b * r) / r**2)
        k = int(r * scale)
        eps = r * scale - k
        approx = (1 - eps) * F[k] + eps * F[k + 1]
        assert abs(approx - exact) < 1e-5 * max(1.0, abs(exact))


def test_oracle_vs_fp64_allpairs_water():
    s = systems.water_small()
    o = O.Oracle(s, rc=0.9, rlist=1.0)
    o.grid()
    o.search()
    o.force(True)
    f = o.forces()
    f64, e64 = O.fp64_allpairs(s, rc=0.9, beta=o.beta)
    assert rel_rms(f, f64) < 1e-5
    e = o.energies()
    assert abs(e[0] - e64[0]) / abs(e64[0]) < 1e-5
    assert abs(e[1] - e64[1]) / abs(e64[1]) < 1e-5


def test_pairlist_covers_every_pair_within_rlist():
    """Every atom pair closer than rlist is in exactly one list entry."""
    s = systems.spc_water(300, 2.08, seed=7)
    o = O.Oracle(s, rc=0.9, rlist=1.0)
    o.grid()
    o.search()
    g = o.grid_arrays()
    pl = o.pairlist()
    rows = canonical_pairs(pl["sci"], pl["cj4"], pl["excl"])
    xq = g["xq"]
    ai = g["atom_indices"]
    box = s.box.astype(np.float64)
    shifts = np.array([[(k - 2) * box[0], (l - 1) * box[1], (m - 1) * box[2]]
                       for m in range(3) for l in range(3) for k in range(5)])
    count = {}
    for r in rows:
        ci, cj, sh, mask = int(r["ci"]), int(r["cj"]), int(r["shift"]), int(r["mask"])
        for ic in range(8):
            a = ai[ci * 8 + ic]
            for jc in range(8):
                b = ai[cj * 8 + jc]
                if a < 0 or b < 0:
                    continue
                d = xq[ci * 8 + ic, :3] + shifts[sh] - xq[cj * 8 + jc, :3]
                if d @ d < 1.0:
                    key = (min(a, b), max(a, b))
                    if (mask >> (ic * 8 + jc)) & 1:
                        count[key] = count.get(key, 0) + 1
    # brute force: pairs within rlist (minimum image suffices: box > 2 rlist)
    x = s.x.astype(np.float64) % box
    n = s.n
    mol = np.arange(n) // 3
    for a in range(n):
        d = x[a + 1:] - x[a]
        d -= box * np.round(d / box)
        r2 = (d * d).sum(1)
        for k in np.nonzero(r2 < 0.99)[0]:
            b = a + 1 + k
            if mol[a] == mol[b]:
                assert (a, b) not in count  # excluded pairs are masked out
            else:
                assert count.get((a, b), 0) == 1, (a, b)


def test_balancing_splits_and_sorts_without_changing_pairs():
    """split_sci_entry + sort_sci in the oracle: a partition of each entry's cj4
    groups into pieces, entries ordered large-first, the same cluster pairs."""
    s = systems.water_small()
    o = O.Oracle(s, rc=0.9, rlist=1.0)
    o.grid()
    o.search()
    p0 = o.pairlist()
    before = canonical_pairs(p0["sci"], p0["cj4"], p0["excl"])
    nsp_max = o.balance(44 * 152)
    p1 = o.pairlist()
    assert nsp_max >= 36
    assert len(p1["sci"]) > len(p0["sci"])
    assert np.array_equal(canonical_pairs(p1["sci"], p1["cj4"], p1["excl"]), before)
    # every cj4 group in exactly one entry
    covered = np.zeros(len(p1["cj4"]), int)
    for _sc, _sh, a, b in p1["sci"]:
        covered[a:b] += 1
    assert (covered == 1).all()
    sizes = p1["sci"][:, 3] - p1["sci"][:, 2]
    cap = min(255, 2 * len(p1["cj4"]) // len(sizes))
    assert (np.diff(np.minimum(sizes, cap)) <= 0).all()
    # a large grid (>= min_ci_balanced cells) is only sorted
    o2 = O.Oracle(s, rc=0.9, rlist=1.0)
    o2.grid()
    o2.search()
    assert o2.balance(1) == 0
    assert len(o2.pairlist()["sci"]) == len(p0["sci"])


def test_erfc_expansion_coefficients_match_their_fit():
    """The force kernels' erfc(x) = t P(t) exp(-x^2) coefficients (nbx_internal.cuh erfc_poly)
    recomputed: Chebyshev interpolation of erfc(x) exp(x^2) / t at 8 nodes of t in
    [1 / (1 + 0.47 * 4), 1], converted to monomials in t; and the expansion's accuracy."""
    import math
    import os
    import re

    from scipy.special import erfc

    n, p, xmax = 8, 0.47, 4.0
    tmin = 1 / (1 + p * xmax)
    mid, half = 0.5 * (1 + tmin), 0.5 * (1 - tmin)
    cheb = np.zeros(n)
    for k in range(n):
        th = math.pi * (k + 0.5) / n
        t = mid + half * math.cos(th)
        x = (1 / t - 1) / p
        g = math.erfc(x) * math.exp(x * x) / t
        cheb += 2.0 / n * g * np.cos(np.arange(n) * th)
    cheb[0] *= 0.5
    mono_u = np.polynomial.chebyshev.cheb2poly(cheb)
    mono_t = np.zeros(n)
    for k in range(n):
        term = np.polynomial.polynomial.polypow([-mid / half, 1 / half], k)
        mono_t[: len(term)] += mono_u[k] * term
    src = open(os.path.join(os.path.dirname(__file__), "..", "gmxapi_gb300", "csrc", "nbx_internal.cuh")).read()
    body = src[src.index("float erfc_poly(float t)"):]
    body = body[: body.index("}")]
    lits = [float(v) for v in re.findall(r"([-+]?\d\.\d+e[-+]\d+)f", body)]
    coef = np.array(lits[::-1])  # Horner order: highest first
    assert len(coef) == n
    np.testing.assert_allclose(coef, mono_t.astype(np.float32), rtol=1e-6, atol=1e-8)
    x = np.linspace(0.0, xmax, 100001)
    t = 1 / (1 + np.float32(p) * x)
    approx = t * np.polyval(coef[::-1], t) * np.exp(-x * x)
    assert (np.abs(approx - erfc(x)) / erfc(x)).max() < 2e-7


@pytest.mark.parametrize("mod", [1, 2, 3])
def test_oracle_lj_modifiers_vs_fp64(mod):
    """Force switch, potential switch and plain cut-off (rvdw_switch 0.7 nm) in the oracle's
    float kernel against the FP64 explicit-image sum, on the random LJ + Coulomb liquid."""
    s = systems.lj_liquid(n=1500, ntypes=4, seed=12)
    o = O.Oracle(s, rc=0.9, rlist=1.0, vdw_modifier=mod, rvdw_switch=0.7)
    o.grid()
    o.search()
    o.force(energy=True)
    f64, e64 = O.fp64_allpairs(s, rc=0.9, beta=o.beta, vdw_modifier=mod, rvdw_switch=0.7)
    assert rel_rms(o.forces(), f64) < 1e-5
    np.testing.assert_allclose(o.energies(), e64, rtol=1e-5)
    # the modifier changes the result relative to the potential shift
    o0 = O.Oracle(s, rc=0.9, rlist=1.0)
    o0.grid()
    o0.search()
    o0.force(energy=True)
    assert abs(o0.energies()[0] - o.energies()[0]) > 1e-6 * abs(o0.energies()[0])


def test_erf_series_coefficients_and_accuracy():
    """The excluded-pair energies' sqrt(pi)/2 erf(x)/x = 1 - w/3 + w^2 R(w) (nbx_internal.cuh
    erf_over_x_series, w = x^2 <= 1): the float coefficients of R are 1/(n! (2n+1)) for n = 2..13
    rounded to float32, and the hybrid evaluation (1 - w/3 in FP64, the tail in float32 with
    fused multiply-adds) stays within 1.5e-8 relative of the exact function."""
    import math
    import os
    import re

    from scipy.special import erf

    src = open(os.path.join(os.path.dirname(__file__), "..", "gmxapi_gb300", "csrc", "nbx_internal.cuh")).read()
    body = src[src.index("double erf_over_x_series(double wd)"):]
    body = body[: body.index("return")]
    lits = [float(v.rstrip("f")) for v in re.findall(r"[-+]?\d+\.\d+e[-+]\d+f", body)]
    want = [1.0 / (math.factorial(n) * (2 * n + 1)) for n in range(13, 1, -1)]
    assert len(lits) == len(want)
    for got, w in zip(lits, want):
        assert np.float32(got) == np.float32(w)
    c = [np.float32(v) for v in lits]

    def fma32(a, b, d):  # a float32 fused multiply-add, rounded once
        return np.float32(np.float64(a) * np.float64(b) + np.float64(d))

    worst = 0.0
    for wd in np.linspace(1e-6, 1.0, 4001):
        w = np.float32(wd)
        r = c[0]
        for k in c[1:]:
            r = fma32(r, -w, k)
        s = (1.0 - wd / 3.0) + float(np.float32(np.float32(w * w) * r))  # FP64 part: fma on the GPU
        x = math.sqrt(wd)
        exact = erf(x) / x * math.sqrt(math.pi) / 2
        worst = max(worst, abs(s - exact) / exact)
    assert worst <= 1.5e-8, worst


def test_shift_numbering_is_the_references():
    """The shift index the pair-list entries carry (xyz2is: 5 (3 (z + 1) + y + 1) + x + 2, central
    22, as in the oracle and the search kernels) against the reference's calc_shifts output for its
    test box (PbcTest.CalcShiftsWorks, tests/golden/shift_golden.json), whose 45 vectors are all
    distinct: vector n = x a + y b + z c for the decomposition of n."""
    import json
    import os

    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "shift_golden.json")) as fh:
        g = json.load(fh)
    a, b, c = (np.array(r) for r in g["box"])
    got = []
    for n in range(45):
        x, y, z = n % 5 - 2, (n // 5) % 3 - 1, n // 15 - 1
        assert 5 * (3 * (z + 1) + y + 1) + x + 2 == n
        got.append(x * a + y * b + z * c)
    np.testing.assert_allclose(np.array(got), np.array(g["shift_vectors"]), rtol=0, atol=1e-9)
    assert 5 * (3 * 1 + 1) + 2 == 22  # the central shift (no image), CENTRAL / kCentral
