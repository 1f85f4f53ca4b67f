"""gmxapi_gb300: the GROMACS nbnxm short-range nonbonded path on GB300 (sm_103a).

``gmxapi_gb300.nblib`` is the nblib-style façade over the C ABI in
include/nbnxm_gb300.h; ``gmxapi_gb300.systems`` builds the seeded synthetic
systems; ``gmxapi_gb300.adjoint`` holds the torch.autograd binding.
"""
from . import systems  # noqa: F401

__all__ = ["systems", "nblib", "build"]
