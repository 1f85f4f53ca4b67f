"""The hand-written 3D real <-> half-complex transform of the PME grids (needs a GB300).

Through nbx_fft3d_* (the transform alone) and nbx_pme_fft_device (a PME handle's grid).  Pinned by
the reference's own 3D FFT test (FFFTest3D.Real5_6_9: src/gromacs/fft/tests/fft.cpp
with refdata/FFFTest3D_Real5_6_9.xml, converted by tests/golden/make_fft_golden.py), forward and
backward, and checked against FP64 numpy transforms on grid sizes with every supported prime
factor (butterflies 2, 3, 4, 5; direct DFT stages 7, 11, 13, 17, 19, 23), odd and even z lengths, and the benchmark's 120^3 and 192^3 grids.
Bars (float32 arithmetic against FP64): relative RMS 2e-6, largest error 1e-5 of the output's RMS.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "fft_golden.json")


def _fft(grid):
    from gmxapi_gb300 import pme

    return pme.Fft3d(tuple(grid))


def _forward(p, grid, x):
    nzc = grid[2] // 2 + 1
    dr = torch.as_tensor(np.ascontiguousarray(x, np.float32), device="cuda")
    dc = torch.zeros((grid[0], grid[1], nzc, 2), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    p.execute_device(1, dr.data_ptr(), dc.data_ptr())
    torch.cuda.synchronize()
    c = dc.cpu().numpy().astype(np.float64)
    return c[..., 0] + 1j * c[..., 1]


def _backward(p, grid, c):
    dc = torch.as_tensor(np.ascontiguousarray(np.stack([c.real, c.imag], -1), np.float32), device="cuda")
    dr = torch.full(tuple(grid), 7.0, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    p.execute_device(-1, dr.data_ptr(), dc.data_ptr())
    torch.cuda.synchronize()
    return dr.cpu().numpy().astype(np.float64)


def _check(got, want):
    rms = np.sqrt(np.mean(np.abs(want) ** 2))
    err = np.abs(got - want)
    assert np.sqrt(np.mean(err**2)) <= 2e-6 * rms, np.sqrt(np.mean(err**2)) / rms
    assert err.max() <= 1e-5 * rms, err.max() / rms


def test_reference_3d_fft_test_vector():
    with open(GOLDEN) as fh:
        g = json.load(fh)
    grid = g["grid"]
    nzc = grid[2] // 2 + 1
    p = _fft(grid)
    x = np.array(g["forward_input"]).reshape(grid)
    want = np.array(g["forward_output"]).reshape(grid[0], grid[1], nzc, 2)
    _check(_forward(p, grid, x), want[..., 0] + 1j * want[..., 1])
    c = np.array(g["backward_input"]).reshape(grid[0], grid[1], nzc, 2)
    _check(_backward(p, grid, c[..., 0] + 1j * c[..., 1]), np.array(g["backward_output"]).reshape(grid))
    p.close()


# the last four cover every compile-time length (96, 120, 128, 144, 160, 192) on every axis
GRIDS = [(16, 16, 16), (20, 16, 24), (32, 36, 25), (7, 11, 13), (1, 8, 5), (44, 52, 70), (45, 9, 81), (19, 17, 23),
         (120, 120, 120), (192, 192, 192), (96, 144, 160), (160, 128, 96), (128, 96, 144), (144, 160, 128)]


@pytest.mark.parametrize("grid", GRIDS)
def test_forward_and_backward_match_fp64_numpy(grid):
    rng = np.random.default_rng(sum(grid))
    p = _fft(grid)
    x = rng.standard_normal(grid).astype(np.float32)
    _check(_forward(p, grid, x), np.fft.rfftn(x.astype(np.float64)))
    # backward of a Hermitian spectrum (the transform of real data) and of a random one
    c = np.fft.rfftn(rng.standard_normal(grid))
    _check(_backward(p, grid, c), np.fft.irfftn(c, s=grid, axes=(0, 1, 2)) * np.prod(grid))
    c = rng.standard_normal(c.shape) + 1j * rng.standard_normal(c.shape)
    _check(_backward(p, grid, c), np.fft.irfftn(c, s=grid, axes=(0, 1, 2)) * np.prod(grid))
    p.close()


def test_round_trip_is_n_times_identity():
    grid = (24, 30, 28)
    p = _fft(grid)
    x = np.random.default_rng(5).standard_normal(grid)
    _check(_backward(p, grid, _forward(p, grid, x)) / np.prod(grid), x)
    p.close()


def test_pme_handle_transform_matches():
    """The PME handle's own transform (nbx_pme_fft_device) is the same plan."""
    from gmxapi_gb300 import pme

    grid = (24, 20, 18)
    p = pme.Pme((2.0, 2.0, 2.0), grid, 3.0)
    x = np.random.default_rng(2).standard_normal(grid).astype(np.float32)
    dr = torch.as_tensor(x, device="cuda")
    dc = torch.zeros((grid[0], grid[1], grid[2] // 2 + 1, 2), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    p.fft_device(1, dr.data_ptr(), dc.data_ptr())
    p.synchronize()
    c = dc.cpu().numpy().astype(np.float64)
    _check(c[..., 0] + 1j * c[..., 1], np.fft.rfftn(x.astype(np.float64)))
    p.close()


def test_unsupported_grid_is_an_input_error():
    from gmxapi_gb300 import pme

    for grid in ((257, 16, 16), (16, 1031, 16), (0, 8, 8)):
        with pytest.raises(Exception, match="prime factors|null"):
            pme.Fft3d(grid)
