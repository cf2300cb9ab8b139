"""ctypes loader for libmcigpu.so (include/mcig.h).

The library is the only compute path: if it is missing and cannot be built,
import fails loudly; there is no CPU fallback.
"""
import ctypes
import os

from . import build as _build

_LIB = None

c_int = ctypes.c_int
c_int64 = ctypes.c_int64
c_double = ctypes.c_double
c_void_p = ctypes.c_void_p
P_double = ctypes.POINTER(ctypes.c_double)
P_int64 = ctypes.POINTER(ctypes.c_int64)
P_int = ctypes.POINTER(ctypes.c_int)
P_uint8 = ctypes.POINTER(ctypes.c_uint8)
P_uint32 = ctypes.POINTER(ctypes.c_uint32)

# name -> (restype, argtypes)
SIGNATURES = {
    "mcig_last_error": (ctypes.c_char_p, []),
    "mcig_version": (ctypes.c_char_p, []),
    "mcig_create": (c_int, [c_int, c_int64, c_int, c_int, ctypes.POINTER(c_void_p)]),
    "mcig_destroy": (c_int, [c_void_p]),
    "mcig_get_ndim": (c_int, [c_void_p, P_int]),
    "mcig_get_nchains": (c_int64, [c_void_p]),
    "mcig_set_precision": (c_int, [c_void_p, c_int]),
    "mcig_get_stream": (c_void_p, [c_void_p]),
    "mcig_set_kernel": (c_int, [c_void_p, c_int]),
    "mcig_set_phase_fusion": (c_int, [c_void_p, c_int]),
    "mcig_set_calibration_split": (c_int, [c_void_p, c_int]),
    "mcig_set_lanes": (c_int, [c_void_p, c_int]),
    "mcig_set_sampling_chunks": (c_int, [c_void_p, c_int]),
    "mcig_set_fp64_decision": (c_int, [c_void_p, c_int]),
    "mcig_get_decision_stats": (c_int, [c_void_p, P_int64, P_int64, P_double]),
    "mcig_set_seed": (c_int, [c_void_p, ctypes.c_uint64]),
    "mcig_set_x": (c_int, [c_void_p, P_double, c_int64]),
    "mcig_get_x": (c_int, [c_void_p, P_double]),
    "mcig_center_x": (c_int, [c_void_p]),
    "mcig_set_mrt2step": (c_int, [c_void_p, c_double]),
    "mcig_set_mrt2step_i": (c_int, [c_void_p, c_int, c_double]),
    "mcig_get_mrt2step": (c_int, [c_void_p, c_int64, c_int, P_double]),
    "mcig_get_nstepsizes": (c_int, [c_void_p, P_int]),
    "mcig_get_mrt2steps": (c_int, [c_void_p, P_double]),
    "mcig_set_target_acceptance_rate": (c_int, [c_void_p, c_double]),
    "mcig_set_nfind_mrt2_iterations": (c_int, [c_void_p, c_int]),
    "mcig_set_ndecorrelation_steps": (c_int, [c_void_p, c_int64]),
    "mcig_set_trial_move": (c_int, [c_void_p, c_int, c_int, c_int, c_int, P_int]),
    "mcig_set_multistep_move": (c_int, [c_void_p, c_int, c_int, c_int, c_double]),
    "mcig_multistep_add_pdf": (c_int, [c_void_p, c_int, P_double, c_int]),
    "mcig_add_sampling_function": (c_int, [c_void_p, c_int, P_double, c_int]),
    "mcig_pop_sampling_function": (c_int, [c_void_p]),
    "mcig_clear_sampling_functions": (c_int, [c_void_p]),
    "mcig_get_npdf": (c_int, [c_void_p, P_int]),
    "mcig_add_observable": (c_int, [c_void_p, c_int, P_double, c_int, c_int, c_int, c_int, c_int]),
    "mcig_add_observable_default": (c_int, [c_void_p, c_int, P_double, c_int, c_int, c_int]),
    "mcig_pop_observable": (c_int, [c_void_p]),
    "mcig_clear_observables": (c_int, [c_void_p]),
    "mcig_get_nobs": (c_int, [c_void_p, P_int]),
    "mcig_get_nobsdim": (c_int, [c_void_p, P_int]),
    "mcig_set_full_storage": (c_int, [c_void_p, c_int]),
    "mcig_set_irange": (c_int, [c_void_p, P_double, P_double]),
    "mcig_reset_domain": (c_int, [c_void_p]),
    "mcig_integrate": (c_int, [c_void_p, c_int64, P_double, P_double, c_int, c_int]),
    "mcig_get_chain_results": (c_int, [c_void_p, P_double, P_double]),
    "mcig_store_observables_on_file": (c_int, [c_void_p, ctypes.c_char_p, c_int]),
    "mcig_clear_observable_file": (c_int, [c_void_p]),
    "mcig_store_walker_positions_on_file": (c_int, [c_void_p, ctypes.c_char_p, c_int]),
    "mcig_clear_walker_file": (c_int, [c_void_p]),
    "mcig_get_acceptance_rate": (c_int, [c_void_p, P_double]),
    "mcig_get_counts": (c_int, [c_void_p, P_int64, P_int64]),
    "mcig_get_obs_data": (c_int, [c_void_p, c_int, P_double, P_int64]),
    "mcig_get_obs_data_chains": (c_int, [c_void_p, c_int, c_int64, c_int64, P_double, P_int64]),
    "mcig_get_step_counters": (c_int, [c_void_p, ctypes.POINTER(ctypes.c_uint64)]),
    "mcig_set_replay": (c_int, [c_void_p, P_double, c_int64, P_int64]),
    "mcig_set_record_accepts": (c_int, [c_void_p, c_int]),
    "mcig_get_accept_bits": (c_int, [c_void_p, P_uint8, P_int64]),
    "mcig_estimate": (c_int, [c_int, c_int, c_int64, c_int, P_double, P_double, P_double]),
    "mcig_accumulate_walk": (c_int, [c_int, c_int, P_double, c_int, c_int, c_int, c_int, c_int64, P_double, P_uint8,
                                     P_double, P_int64]),
    "mcig_get_last_timings": (c_int, [c_void_p, P_double, P_int64]),
    "mcig_philox_block": (c_int, [c_int, P_uint32, P_uint32, P_uint32]),
    "mcig_batch_create": (c_int, [ctypes.POINTER(c_void_p), c_int, P_int64, c_int, c_int, ctypes.POINTER(c_void_p)]),
    "mcig_batch_run": (c_int, [c_void_p, P_double, P_double]),
    "mcig_batch_destroy": (c_int, [c_void_p]),
    "mcig_batch_last_ms": (c_int, [c_void_p, P_double]),
    "mcig_batch_get_tuning": (c_int, [c_void_p, P_int, P_int]),
    "mcig_batch_set_tuning": (c_int, [c_void_p, c_int, P_int]),
    "mcig_batch_autotune": (c_int, [c_void_p, ctypes.c_char_p]),
    "mcig_flow_nparams": (c_int64, [c_int, c_int]),
    "mcig_flow_create": (c_int, [c_int, c_int, c_int, ctypes.c_uint64, c_int, ctypes.POINTER(c_void_p)]),
    "mcig_flow_destroy": (c_int, [c_void_p]),
    "mcig_flow_get_params": (c_int, [c_void_p, ctypes.POINTER(ctypes.c_float), P_int64]),
    "mcig_flow_set_params": (c_int, [c_void_p, ctypes.POINTER(ctypes.c_float), c_int64]),
    "mcig_flow_tc_selftest": (c_int, [c_int, c_void_p, c_void_p, c_int, c_int, ctypes.POINTER(ctypes.c_float)]),
    "mcig_flow_set_tensor_path": (c_int, [c_void_p, c_int]),
    "mcig_flow_forward": (c_int, [c_void_p, P_double, c_int64, P_double, P_double]),
    "mcig_flow_inverse": (c_int, [c_void_p, P_double, c_int64, P_double, P_double]),
    "mcig_flow_loss_grad": (c_int, [c_void_p, P_double, c_int64, P_double, ctypes.POINTER(ctypes.c_float)]),
    "mcig_flow_train": (c_int, [c_void_p, P_double, c_int64, c_int, c_int, c_double, P_double]),
    "mcig_integrate_flow": (c_int, [c_void_p, c_void_p, c_int64, c_int, c_int64, c_int, c_int, c_double, P_double,
                                    P_double, c_int, c_int, P_double]),
    "mcig_mjblocker_estimate_noalloc": (c_int, [c_void_p, c_int64, c_int, c_void_p, c_void_p, c_void_p]),
    "mcig_plugin_load": (c_int, [ctypes.c_char_p, ctypes.POINTER(c_void_p)]),
    "mcig_plugin_unload": (c_int, [c_void_p]),
    "mcig_plugin_counts": (c_int, [c_void_p, P_int, P_int]),
    "mcig_set_plugin": (c_int, [c_void_p, c_void_p]),
    "mcig_plugin_nmoves": (c_int, [c_void_p, P_int]),
    "mcig_set_user_move": (c_int, [c_void_p, c_int, P_double, c_int]),
}


def lib_path():
    return _build.LIB


def load():
    """Load (building first if needed) libmcigpu.so and declare every signature."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    try:
        _build.build()
    except Exception as e:  # no nvcc here: use an existing build or fail
        if not os.path.exists(path):
            raise ImportError("libmcigpu.so is not built and cannot be built: %s" % e)
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = L
    return L
