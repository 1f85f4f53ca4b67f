"""Leap-frog oracle against the reference's integrator test; leap-frog C ABI input checks (no GPU)."""
import numpy as np
import pytest

from oracle import md_oracle as M


def test_oracle_leapfrog_reproduces_nblib_integrator_test():
    """api/nblib/tests/integrator.cpp IntegratorWorks: one atom of mass 1 under a constant force
    (1, 2, 0), dt 0.001, 100 steps in a 100 nm box, within 100 * 5e-6 of the analytic motion."""
    dt, steps = 0.001, 100
    x = np.zeros((1, 3), np.float32)
    v = np.zeros((1, 3), np.float32)
    f = np.array([[1.0, 2.0, 0.0]], np.float32)
    im = np.ones(1, np.float32)
    tol = steps * 0.000005
    for step in range(steps):
        t = step * dt
        np.testing.assert_allclose(x[0], 0.5 * f[0] * t * t, rtol=0, atol=tol)
        np.testing.assert_allclose(v[0], f[0] * t, rtol=0, atol=tol)
        x, v, _ = M.leapfrog(x, v, f, im, dt, (100.0, 100.0, 100.0))


def _reference_put_in_box(x, box):
    """The reference's unbounded while loops (pbc.cpp:1430-1446), float32."""
    x = np.array(x, np.float32).reshape(-1, 3)
    for i in range(x.shape[0]):
        for d in range(3):
            L = np.float32(box[d])
            while x[i, d] < 0:
                x[i, d] = np.float32(x[i, d] + L)
            while x[i, d] >= L:
                x[i, d] = np.float32(x[i, d] - L)
    return x


def test_put_in_box_matches_the_reference_loops():
    rng = np.random.default_rng(3)
    box = (2.3, 1.7, 3.1)
    # up to four box lengths away: the same float additions as the reference
    x = (rng.random((4000, 3)) * 9.0 - 4.5) * np.array(box)
    x = x.astype(np.float32)
    np.testing.assert_array_equal(M.put_in_box(x, box), _reference_put_in_box(x, box))
    edge = np.array([[0.0, 1.7, -0.0], [2.3, -1e-9, 3.1 * 4], [-2.3, 1.7 * 2, 3.1 - 1e-7]], np.float32)
    np.testing.assert_array_equal(M.put_in_box(edge, box), _reference_put_in_box(edge, box))
    # far away: a floor-based shift (the reference would loop), still inside [0, L)
    far = np.array([[1e4, -3e3, 777.7]], np.float32)
    w = M.put_in_box(far, box)
    assert np.all(w >= 0) and np.all(w < np.array(box, np.float32))


@pytest.fixture(scope="module")
def md_mod():
    from gmxapi_gb300 import build

    build.build()
    from gmxapi_gb300 import md

    return md


@pytest.mark.parametrize("im,box", [
    (np.array([1.0, -1.0], np.float32), (2.0, 2.0, 2.0)),    # negative inverse mass
    (np.array([1.0, np.inf], np.float32), (2.0, 2.0, 2.0)),  # infinite inverse mass
    (np.array([1.0, 1.0], np.float32), (2.0, 0.0, 2.0)),     # non-positive box edge
])
def test_leapfrog_invalid_input_raises(md_mod, im, box):
    from gmxapi_gb300.nblib import InputException

    with pytest.raises(InputException):
        md_mod.LeapFrog(im, box)


def test_leapfrog_without_gpu_reports_no_device(md_mod):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from gmxapi_gb300 import _lib

    with pytest.raises(_lib.NbxError) as ei:
        md_mod.LeapFrog(np.ones(4, np.float32), (2.0, 2.0, 2.0))
    assert ei.value.code == _lib.NBX_ERR_NO_DEVICE


def _leapfrog_golden():
    import json
    import os

    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "leapfrog_golden.json")) as fh:
        return json.load(fh)["cases"]


def _leapfrog_start(case):
    import numpy as np

    n = case["num_atoms"]
    i = np.arange(n)
    x = np.stack([(i % 21) * 1.0, 6.5 - (i % 13) * 1.0, np.zeros(n)], -1).astype(np.float32)
    v = np.tile(np.array(case["v0"], np.float32), (n, 1))
    f = np.tile(np.array(case["f0"], np.float32), (n, 1))
    im = (1.0 / (1.0 + (i % 100))).astype(np.float32)
    return x, v, f, im


def test_leapfrog_oracle_reproduces_the_reference_leapfrog_test():
    """The reference's own LeapFrogTest.SimpleIntegration data (src/gromacs/mdlib/tests/leapfrog.cpp,
    the 10 cases without coupling; tests/golden/leapfrog_golden.json) within that test's tolerance
    (absolute, steps x 5e-6), with the positions left unwrapped as the reference test does."""
    import numpy as np

    from oracle import md_oracle as M

    for case in _leapfrog_golden():
        x, v, f, im = _leapfrog_start(case)
        for _ in range(case["num_steps"]):
            x, v, _ = M.leapfrog(x, v, f, im, case["dt"], (1e3, 1e3, 1e3), wrap=False)
        np.testing.assert_allclose(x, case["final_x"], rtol=0, atol=case["tolerance"])
        np.testing.assert_allclose(v, case["final_v"], rtol=0, atol=case["tolerance"])
