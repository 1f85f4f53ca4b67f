"""LJ-PME: the real-space grid part in the cluster kernel and the dispersion grid (needs a GB300).

Bars: real-space forces rel-RMS <= 1e-5 and energies <= 1e-5 against the FP64 all-pairs oracle with
the LJ-PME grid part; the dispersion grid's forces and energy within 1e-5 of the PME oracle and its
solve within 1e-5 of the reference's LJ solver test data; real + reciprocal space reproduce the
untruncated fcc lattice energy.
"""
import json
import os

import numpy as np
import pytest

from gmxapi_gb300 import nblib, systems
from oracle import oracle as O
from oracle import pme_oracle as P
from tests.helpers import rel_rms

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "pme_golden.json")


def _opts(rc=0.9, rlist=1.0):
    return nblib.NBKernelOptions(pairlist_cutoff=rlist, rcoulomb=rc, vdw_modifier=nblib.VdwModifier.LjPme,
                                 compute_virial_and_energy=True)


@pytest.mark.parametrize("name", ["water", "lj_liquid", "fcc"])
def test_real_space_matches_fp64(name):
    from gmxapi_gb300 import pme as pm

    s = {"water": lambda: systems.spc_water(300, 2.08, seed=5),
         "lj_liquid": lambda: systems.lj_liquid(n=1500, ntypes=4, seed=8),
         "fcc": lambda: systems.lj_fcc(cells=6, lattice=0.5256, charge=0.2, seed=2)}[name]()
    calc = nblib.ForceCalculator(s, _opts())
    f = calc.compute(s.x).astype(np.float64)
    e = calc.energies.copy()
    calc.close()
    beta = pm.ewald_coefficient(0.9, 1e-5)
    bl = pm.ewald_coefficient_lj(0.9, 1e-3)
    f_ref, e_ref = O.fp64_allpairs(s, rc=0.9, beta=beta, vdw_modifier=4, beta_lj=bl)
    assert rel_rms(f, f_ref) <= 1e-5
    assert e[0] == pytest.approx(e_ref[0], rel=1e-5, abs=1e-5 * abs(e_ref[1]))
    assert e[1] == pytest.approx(e_ref[1], rel=1e-5)


def test_dispersion_grid_matches_oracle():
    from gmxapi_gb300 import pme as pm

    s = systems.lj_liquid(n=1500, ntypes=4, seed=8)
    box = [float(b) for b in s.box]
    nb = np.asarray(s.nbfp, np.float64).reshape(s.ntypes, s.ntypes, 2)
    coef = np.sqrt(nb[s.type, s.type, 0] / 6.0).astype(np.float32)  # sqrt(C6_ii)
    grid = pm.grid_size(box, 0.12)
    bl = pm.ewald_coefficient_lj(0.9, 1e-3)
    p = pm.Pme(box, grid, bl, lj=True)
    f = p.compute(s.x, coef)
    rf, re, rv = P.compute(s.x, coef, box, grid, bl, single=True, lj=True)
    assert rel_rms(f, rf) <= 1e-5
    assert p.energy == pytest.approx(re, rel=1e-5)
    assert np.max(np.abs(p.virial - rv)) <= 1e-5 * np.max(np.abs(rv))
    p.close()


def test_lj_solve_matches_reference_data():
    from gmxapi_gb300 import pme as pm

    golden = json.load(open(GOLDEN))
    for case in golden["solve_lj"]:
        p = pm.Pme(case["box"], case["grid"], case["beta_lj"], lj=True)
        n = case["grid"]
        c = np.zeros((n[0], n[1], n[2] // 2 + 1, 2), np.float32)
        for (i, j, k), (re_, im_) in case["input"]:
            c[i, j, k] = (re_, im_)
        dc = torch.from_numpy(c).cuda()
        e = torch.zeros(1, dtype=torch.float64, device="cuda")
        v = torch.zeros(9, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        p.solve_device(dc.data_ptr(), e.data_ptr(), v.data_ptr())
        p.synchronize()
        out = dc.cpu().numpy().astype(np.float64)
        # the influence function cancels to O(1/b) e^-b at large b, so far-tail values carry float
        # error; like the reference's solver test, tolerances scale with max(1, largest value) for
        # the grid, 10 for the energy and 1000 for the virial (pmesolvetest.cpp)
        scale = max([1.0] + [abs(v_) for v_ in case["output"].values()])
        for key, val in case["output"].items():
            parts = key.split()
            got = out[int(parts[1]), int(parts[2]), int(parts[3]), 0 if parts[4] == "re" else 1]
            assert got == pytest.approx(val, rel=1e-5, abs=1e-6 * scale)
        assert e.item() == pytest.approx(case["energy"], rel=1e-5, abs=1e-6 * 10.0)
        vir = v.cpu().numpy().reshape(3, 3)
        for key, val in case["virial"].items():
            _, a, b = key.split()
            assert vir[int(a), int(b)] == pytest.approx(val, rel=1e-5, abs=1e-6 * 1000.0)
        p.close()


def test_lj_pme_reproduces_the_fcc_lattice_energy():
    from gmxapi_gb300 import pme as pm

    s = systems.lj_fcc(cells=6, lattice=0.5256, charge=0.0, seed=0)
    calc = nblib.ForceCalculator(s, _opts())
    f_real = calc.compute(s.x).astype(np.float64)
    e_real = calc.energies[0]
    calc.close()
    nb = np.asarray(s.nbfp).reshape(-1, 2)
    c6, c12 = float(nb[0, 0]) / 6.0, float(nb[0, 1]) / 12.0
    box = [float(b) for b in s.box]
    p = pm.Pme(box, (40, 40, 40), pm.ewald_coefficient_lj(0.9, 1e-3), lj=True)
    f_rec = p.compute(s.x, np.full(s.n, np.sqrt(c6), np.float32)).astype(np.float64)
    a = 0.5256 / np.sqrt(2.0)
    d = s.x[0] - s.x
    d -= np.round(d / s.box) * s.box
    r = np.sqrt((d * d).sum(1))
    n_rc = int(np.sum((r > 0) & (r < 0.9)))
    expect = 0.5 * s.n * (c12 * 12.13188 / a ** 12 - c6 * 14.45392 / a ** 6) - 0.5 * s.n * n_rc * c12 / 0.9 ** 12
    assert e_real + p.energy == pytest.approx(expect, rel=3e-5)
    assert np.abs(f_real + f_rec).max() < 2e-2
    p.close()


def test_ljpme_rejected_where_unsupported():
    s = systems.spc_water(300, 2.08, seed=5)
    calc = nblib.ForceCalculator(s, _opts())
    with pytest.raises(nblib.InputException):
        calc.set_free_energy(np.array([1], np.int32), np.zeros(1, np.float32), np.zeros(1, np.int32))
    calc.close()
