"""ctypes binding of the C ABI in include/nbnxm_gb300.h.

The engine is the in-tree shared library gmxapi_gb300/lib/libnbnxm_gb300.so,
built by gmxapi_gb300/build.py (``python -c "import __graft_entry__ as g;
g.build()"``).  There is no fallback: if the library is missing, loading
raises.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libnbnxm_gb300.so")

NBX_OK = 0
NBX_ERR_INVALID_INPUT = 1
NBX_ERR_OUT_OF_MEMORY = 2
NBX_ERR_LIST_OVERFLOW = 3
NBX_ERR_CUDA = 4
NBX_ERR_TIMEOUT = 5
NBX_ERR_NO_DEVICE = 6
NBX_ERR_STATE = 7
STATUS_NAMES = {
    0: "NBX_OK",
    1: "NBX_ERR_INVALID_INPUT",
    2: "NBX_ERR_OUT_OF_MEMORY",
    3: "NBX_ERR_LIST_OVERFLOW",
    4: "NBX_ERR_CUDA",
    5: "NBX_ERR_TIMEOUT",
    6: "NBX_ERR_NO_DEVICE",
    7: "NBX_ERR_STATE",
}

#: every function include/nbnxm_gb300.h declares
EXPORTED = [
    "nbx_default_options", "nbx_create", "nbx_destroy", "nbx_last_error", "nbx_update_pairlist",
    "nbx_compute", "nbx_set_stream", "nbx_get_stream", "nbx_search_device", "nbx_prune_device",
    "nbx_compute_device", "nbx_md_step_device", "nbx_synchronize", "nbx_get_sizes", "nbx_get_grid",
    "nbx_get_pairlist", "nbx_get_pair_counts", "nbx_measure_fp32_peak", "nbx_md_step",
    "nbx_set_timing", "nbx_get_timings", "nbx_compute_noalloc", "nbx_noalloc_status", "nbx_noalloc_set_wait_test",
    "nbx_batch_create", "nbx_batch_destroy", "nbx_batch_last_error", "nbx_batch_atoms", "nbx_batch_set_stream",
    "nbx_batch_search_device", "nbx_batch_prune_device", "nbx_batch_compute_device", "nbx_batch_md_step_device",
    "nbx_batch_sequential_md_step_device", "nbx_batch_set_graph", "nbx_batch_set_kernel_variant",
    "nbx_batch_set_prune", "nbx_batch_set_force_kernel", "nbx_backward_device", "nbx_set_parameters_device",
    "nbx_get_phase_timings", "nbx_set_list_balance", "nbx_get_list_balance",
    "nbx_batch_set_parameters_device", "nbx_batch_backward_device", "nbx_batch_force_match_device",
    "nbx_set_wait_test", "nbx_set_force_kernel", "nbx_get_force_kernel",
    "nbx_ewald_coefficient", "nbx_pme_grid_size", "nbx_pme_create", "nbx_pme_destroy", "nbx_pme_last_error",
    "nbx_pme_set_stream", "nbx_pme_synchronize", "nbx_pme_get_info", "nbx_pme_compute_device",
    "nbx_pme_splines_device", "nbx_pme_spread_device", "nbx_pme_solve_device", "nbx_pme_gather_device",
    "nbx_pme_fft_device", "nbx_fft3d_create", "nbx_fft3d_destroy", "nbx_fft3d_execute_device",
    "nbx_get_options", "nbx_set_force_accumulate", "nbx_get_force_accumulate", "nbx_leapfrog_create", "nbx_leapfrog_destroy",
    "nbx_leapfrog_last_error", "nbx_leapfrog_set_stream", "nbx_leapfrog_integrate", "nbx_leapfrog_integrate_device",
    "nbx_md_run_device", "nbx_fep_enable", "nbx_fep_set_lambda", "nbx_fep_get_energies", "nbx_fep_energies_device",
    "nbx_fep_disable", "nbx_pme_create_lj", "nbx_ewald_coefficient_lj", "nbx_lb_table_device",
    "nbx_lb_table_backward_device", "nbx_match_loss_device",
]


class nbx_system_desc(C.Structure):
    _fields_ = [
        ("num_atoms", C.c_int),
        ("x", C.POINTER(C.c_float)),
        ("q", C.POINTER(C.c_float)),
        ("type", C.POINTER(C.c_int)),
        ("num_types", C.c_int),
        ("nbfp", C.POINTER(C.c_float)),
        ("excl_index", C.POINTER(C.c_int)),
        ("excl_list", C.POINTER(C.c_int)),
        ("box", C.c_float * 3),
    ]


class nbx_options(C.Structure):
    _fields_ = [
        ("coulomb", C.c_int),
        ("rcoulomb", C.c_float),
        ("rlist", C.c_float),
        ("rlist_inner", C.c_float),
        ("ewald_rtol", C.c_float),
        ("epsilon_rf", C.c_float),
        ("use_ewald_shift", C.c_int),
        ("nstlist", C.c_int),
        ("nstlist_prune", C.c_int),
        ("compute_energy", C.c_int),
        ("vdw_modifier", C.c_int),
        ("rvdw_switch", C.c_float),
        ("ewald_rtol_lj", C.c_float),
    ]


class nbx_noalloc_args(C.Structure):
    _fields_ = [
        ("num_atoms", C.c_int),
        ("num_slots", C.c_int),
        ("num_sci", C.c_int),
        ("xq", C.c_void_p),
        ("types", C.c_void_p),
        ("num_types", C.c_int),
        ("nbfp", C.c_void_p),
        ("cells", C.c_void_p),
        ("sci", C.c_void_p),
        ("cj4", C.c_void_p),
        ("excl", C.c_void_p),
        ("excl_index", C.c_void_p),
        ("excl_list", C.c_void_p),
        ("box", C.c_float * 3),
        ("coulomb", C.c_int),
        ("rcoulomb", C.c_float),
        ("rlist", C.c_float),
        ("ewald_rtol", C.c_float),
        ("epsilon_rf", C.c_float),
        ("use_ewald_shift", C.c_int),
    ]


class nbx_fep_desc(C.Structure):
    _fields_ = [
        ("num_perturbed", C.c_int),
        ("perturbed", C.POINTER(C.c_int)),
        ("qB", C.POINTER(C.c_float)),
        ("typeB", C.POINTER(C.c_int)),
        ("lambda_coul", C.c_float),
        ("lambda_vdw", C.c_float),
        ("alpha_vdw", C.c_float),
        ("alpha_coul", C.c_float),
        ("lambda_power", C.c_int),
        ("sigma6_def", C.c_float),
        ("sigma6_min", C.c_float),
    ]


class NbxError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


_lib = None


def load():
    """Load the engine library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"{LIB_PATH} is missing: build it with gmxapi_gb300.build.build() "
            "(nvcc, sm_103a); there is no CPU fallback"
        )
    L = C.CDLL(LIB_PATH)
    vp, ip, fp, dp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_float), C.POINTER(C.c_double)
    u32p, llp = C.POINTER(C.c_uint32), C.POINTER(C.c_longlong)
    L.nbx_default_options.argtypes = [C.POINTER(nbx_options)]
    L.nbx_default_options.restype = None
    L.nbx_create.argtypes = [C.POINTER(nbx_system_desc), C.POINTER(nbx_options), C.c_int, C.POINTER(vp)]
    L.nbx_destroy.argtypes = [vp]
    L.nbx_last_error.argtypes = [vp]
    L.nbx_last_error.restype = C.c_char_p
    L.nbx_update_pairlist.argtypes = [vp, fp]
    L.nbx_compute.argtypes = [vp, fp, fp, dp, dp]
    L.nbx_set_stream.argtypes = [vp, vp]
    L.nbx_get_stream.argtypes = [vp]
    L.nbx_get_stream.restype = vp
    L.nbx_search_device.argtypes = [vp, vp]
    L.nbx_prune_device.argtypes = [vp, C.c_int]
    L.nbx_compute_device.argtypes = [vp, vp, vp, vp, vp]
    L.nbx_md_step_device.argtypes = [vp, C.c_longlong, vp, vp, vp, vp]
    L.nbx_synchronize.argtypes = [vp]
    L.nbx_get_sizes.argtypes = [vp, ip]
    L.nbx_get_grid.argtypes = [vp, ip, ip, ip, ip, fp, fp, fp]
    L.nbx_get_pairlist.argtypes = [vp, ip, ip, u32p, u32p]
    L.nbx_get_pair_counts.argtypes = [vp, llp]
    L.nbx_measure_fp32_peak.argtypes = [C.c_int, dp]
    L.nbx_md_step.argtypes = [vp, C.c_longlong, fp, fp, dp, dp]
    L.nbx_set_timing.argtypes = [vp, C.c_int]
    L.nbx_get_timings.argtypes = [vp, dp, llp, C.c_int]
    L.nbx_get_phase_timings.argtypes = [vp, dp, llp, C.c_int]
    L.nbx_set_list_balance.argtypes = [vp, C.c_int]
    L.nbx_set_wait_test.argtypes = [vp, C.c_int]
    L.nbx_set_force_kernel.argtypes = [vp, C.c_int, C.c_int, C.c_int]
    L.nbx_get_force_kernel.argtypes = [vp, ip, ip, ip]
    L.nbx_batch_set_parameters_device.argtypes = [vp, vp, vp]
    L.nbx_batch_backward_device.argtypes = [vp] * 7
    L.nbx_batch_force_match_device.argtypes = [vp] * 10
    L.nbx_get_list_balance.argtypes = [vp, ip]
    L.nbx_compute_noalloc.argtypes = [C.POINTER(nbx_noalloc_args), vp, vp, vp, vp]
    L.nbx_noalloc_status.argtypes = [vp]
    L.nbx_noalloc_set_wait_test.argtypes = [C.c_int]
    L.nbx_batch_create.argtypes = [C.c_int, C.POINTER(nbx_system_desc), C.POINTER(nbx_options), C.c_int,
                                   C.POINTER(vp)]
    L.nbx_batch_destroy.argtypes = [vp]
    L.nbx_batch_last_error.argtypes = [vp]
    L.nbx_batch_last_error.restype = C.c_char_p
    L.nbx_batch_atoms.argtypes = [vp, llp, ip]
    L.nbx_batch_set_stream.argtypes = [vp, vp]
    L.nbx_batch_search_device.argtypes = [vp, vp]
    L.nbx_batch_prune_device.argtypes = [vp, C.c_int]
    L.nbx_batch_compute_device.argtypes = [vp, vp, vp, vp, vp]
    L.nbx_batch_md_step_device.argtypes = [vp, C.c_longlong, vp, vp, vp, vp]
    L.nbx_batch_sequential_md_step_device.argtypes = [vp, C.c_longlong, vp, vp, vp, vp]
    L.nbx_batch_set_graph.argtypes = [vp, C.c_int]
    L.nbx_batch_set_kernel_variant.argtypes = [vp, C.c_int]
    L.nbx_batch_set_prune.argtypes = [vp, C.c_int, C.c_float]
    L.nbx_batch_set_force_kernel.argtypes = [vp, C.c_int, C.c_int]
    L.nbx_backward_device.argtypes = [vp, vp, vp, vp, vp, vp, vp]
    L.nbx_set_parameters_device.argtypes = [vp, vp, vp]
    L.nbx_lb_table_device.argtypes = [vp, vp, C.c_int, vp, vp]
    L.nbx_lb_table_backward_device.argtypes = [vp, vp, C.c_int, vp, vp, vp, vp]
    L.nbx_match_loss_device.argtypes = [vp, vp, C.c_longlong, vp, vp, vp]
    L.nbx_ewald_coefficient.argtypes = [C.c_float, C.c_float]
    L.nbx_ewald_coefficient.restype = C.c_float
    L.nbx_pme_grid_size.argtypes = [fp, C.c_float, ip]
    L.nbx_pme_create.argtypes = [fp, ip, C.c_float, C.c_float, C.c_int, C.POINTER(vp)]
    L.nbx_pme_destroy.argtypes = [vp]
    L.nbx_pme_create_lj.argtypes = [fp, ip, C.c_float, C.c_int, C.POINTER(vp)]
    L.nbx_ewald_coefficient_lj.argtypes = [C.c_float, C.c_float]
    L.nbx_ewald_coefficient_lj.restype = C.c_float
    L.nbx_pme_last_error.argtypes = [vp]
    L.nbx_pme_last_error.restype = C.c_char_p
    L.nbx_pme_set_stream.argtypes = [vp, vp]
    L.nbx_pme_synchronize.argtypes = [vp]
    L.nbx_pme_get_info.argtypes = [vp, ip, fp]
    L.nbx_pme_compute_device.argtypes = [vp, C.c_int, vp, vp, vp, vp, vp]
    L.nbx_pme_splines_device.argtypes = [vp, C.c_int, vp, vp, vp, vp]
    L.nbx_pme_spread_device.argtypes = [vp, C.c_int, vp, vp, vp]
    L.nbx_pme_solve_device.argtypes = [vp, vp, vp, vp]
    L.nbx_pme_gather_device.argtypes = [vp, C.c_int, vp, vp, vp, vp]
    L.nbx_pme_fft_device.argtypes = [vp, C.c_int, vp, vp]
    L.nbx_fft3d_create.argtypes = [C.POINTER(C.c_int), C.c_int, C.POINTER(vp)]
    L.nbx_fft3d_destroy.argtypes = [vp]
    L.nbx_fft3d_execute_device.argtypes = [vp, C.c_int, vp, vp, vp]
    L.nbx_get_options.argtypes = [vp, C.POINTER(nbx_options)]
    L.nbx_set_force_accumulate.argtypes = [vp, C.c_int]
    L.nbx_get_force_accumulate.argtypes = [vp, C.POINTER(C.c_int)]
    L.nbx_leapfrog_create.argtypes = [C.c_int, fp, fp, C.c_int, C.POINTER(vp)]
    L.nbx_leapfrog_destroy.argtypes = [vp]
    L.nbx_leapfrog_last_error.argtypes = [vp]
    L.nbx_leapfrog_last_error.restype = C.c_char_p
    L.nbx_leapfrog_set_stream.argtypes = [vp, vp]
    L.nbx_leapfrog_integrate.argtypes = [vp, C.c_float, fp, fp, fp]
    L.nbx_leapfrog_integrate_device.argtypes = [vp, C.c_float, vp, vp, vp, vp]
    L.nbx_fep_enable.argtypes = [vp, C.POINTER(nbx_fep_desc)]
    L.nbx_fep_set_lambda.argtypes = [vp, C.c_float, C.c_float]
    L.nbx_fep_get_energies.argtypes = [vp, dp]
    L.nbx_fep_energies_device.argtypes = [vp]
    L.nbx_fep_energies_device.restype = vp
    L.nbx_fep_disable.argtypes = [vp]
    L.nbx_md_run_device.argtypes = [vp, vp, vp, C.c_longlong, C.c_int, C.c_float, vp, vp, vp, vp, C.c_int, vp]
    for name in EXPORTED:
        f = getattr(L, name)
        if f.restype is C.c_int or name not in ("nbx_default_options", "nbx_last_error", "nbx_get_stream",
                                                "nbx_batch_last_error", "nbx_pme_last_error",
                                                "nbx_ewald_coefficient", "nbx_leapfrog_last_error",
                                                "nbx_fep_energies_device", "nbx_ewald_coefficient_lj"):
            f.restype = C.c_int
    _lib = L
    return L


def check(code: int, handle=None):
    if code != NBX_OK:
        msg = load().nbx_last_error(handle)
        raise NbxError(code, msg.decode() if msg else "")
