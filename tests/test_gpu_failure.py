"""Failure detection on the GPU without a fault: the force kernel's bounded waits.

The force kernel waits (on mbarriers) for the bulk copies that stage j-clusters in
shared memory.  Each wait gives up after one second, flags a timeout in the list
header and lets the warp leave, so a stalled copy becomes an error code instead of a
hung GPU.  The test hook arms the barriers for bytes that never arrive: the compute
must report NBX_ERR_TIMEOUT within seconds, and after the hook is off and the list is
rebuilt the same handle must compute correct forces again.
"""
import time

import pytest

from gmxapi_gb300 import _lib, nblib, systems
from oracle import oracle as O
from tests.helpers import rel_rms

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape", [(1, 2, 2), (1, 3, 3), (0, 2, 2)])
def test_stage_wait_times_out_and_the_handle_recovers(shape):
    s = systems.spc_water(300, 2.08, seed=5)
    calc = nblib.ForceCalculator(s, nblib.NBKernelOptions(pairlist_cutoff=1.0, rcoulomb=0.9))
    calc.set_force_kernel(*shape)
    L = _lib.load()
    assert L.nbx_set_wait_test(calc.h, 1) == _lib.NBX_OK
    t0 = time.time()
    with pytest.raises(_lib.NbxError) as err:
        calc.compute(s.x)
    assert err.value.code == _lib.NBX_ERR_TIMEOUT
    assert time.time() - t0 < 60
    assert L.nbx_set_wait_test(calc.h, 0) == _lib.NBX_OK
    calc.update_pairlist(s.x)  # a search clears the status
    f = calc.compute(s.x)
    o = O.Oracle(s, rc=0.9, rlist=1.0)
    o.grid()
    o.search()
    o.force(energy=False)
    assert rel_rms(f, o.forces()) <= 1e-5
