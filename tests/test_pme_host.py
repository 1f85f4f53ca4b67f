"""Host-side PME entry points of the C ABI: grid sizes, the Ewald coefficient, input checks (no GPU)."""
import math

import numpy as np
import pytest

from oracle import pme_oracle as P


@pytest.fixture(scope="module")
def pme_mod():
    from gmxapi_gb300 import build

    build.build()
    from gmxapi_gb300 import pme

    return pme


def test_grid_size_matches_oracle(pme_mod):
    rng = np.random.default_rng(7)
    lengths = list(rng.uniform(0.6, 40.0, 300)) + [2.0, 5.2, 5.5, 10.6, 10.8, 14.21, 16.5]
    for spacing in (0.16, 0.12, 0.1):
        for a, b, c in np.reshape(lengths[: 3 * (len(lengths) // 3)], (-1, 3)):
            got = pme_mod.grid_size((a, b, c), spacing)
            assert got == tuple(P.fft_grid_size(v, spacing) for v in (a, b, c))


def test_ewald_coefficient_solves_the_tolerance(pme_mod):
    for rc, rtol in ((0.9, 1e-5), (1.0, 1e-5), (1.2, 1e-6), (0.9, 1e-3)):
        beta = pme_mod.ewald_coefficient(rc, rtol)
        assert math.erfc(beta * rc) == pytest.approx(rtol, rel=1e-3)
    assert pme_mod.ewald_coefficient(0.9, 0.0) == pme_mod.ewald_coefficient(0.9, 1e-5)


@pytest.mark.parametrize("box,grid,beta", [
    ((2.0, 2.0, 2.0), (5, 16, 16), 3.0),      # below minimalPmeGridSize (6)
    ((2.0, 2.0, 2.0), (16, 16, 0), 3.0),
    ((2.0, -1.0, 2.0), (16, 16, 16), 3.0),    # non-positive box edge
    ((2.0, 2.0, 2.0), (16, 16, 16), 0.0),     # non-positive Ewald coefficient
    ((2.0, 2.0, 2.0), (16, 16, 5000), 3.0),   # above the supported grid size
])
def test_invalid_input_raises(pme_mod, box, grid, beta):
    from gmxapi_gb300.nblib import InputException

    with pytest.raises(InputException):
        pme_mod.Pme(box, grid, beta)


def test_grid_size_rejects_bad_spacing(pme_mod):
    from gmxapi_gb300.nblib import InputException

    with pytest.raises(InputException):
        pme_mod.grid_size((2.0, 2.0, 2.0), 0.0)
    with pytest.raises(InputException):
        pme_mod.grid_size((2.0, 0.0, 2.0), 0.12)


def test_create_without_gpu_reports_no_device(pme_mod):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from gmxapi_gb300 import _lib

    with pytest.raises(_lib.NbxError) as ei:
        pme_mod.Pme((2.0, 2.0, 2.0), (16, 16, 16), 3.0)
    assert ei.value.code == _lib.NBX_ERR_NO_DEVICE
