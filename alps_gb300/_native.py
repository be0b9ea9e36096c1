"""Loads the native library (alps_gb300/lib/libalps_gb300.so) and declares
its C-ABI for ctypes.

There is no Python or CPU implementation of the library behind this module:
if the shared object is missing or unusable, every call raises.
"""
import ctypes as C
import os
import threading

from . import _abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libalps_gb300.so")
_lib = None
_lock = threading.Lock()


class NativeLibraryMissing(RuntimeError):
    pass


def lib():
    """Returns the loaded library, raising NativeLibraryMissing if it was not
    built (run ``python -m alps_gb300.build`` or __graft_entry__.build())."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise NativeLibraryMissing(
                "alps_gb300 native library not built: %s is missing (run python alps_gb300/build.py)" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        P = C.POINTER
        dp = P(C.c_double)
        cp = P(_abi.alps_complex)
        vp = C.c_void_p
        sig = {
            "alps_version": ([], C.c_char_p),
            "alps_error_string": ([C.c_int], C.c_char_p),
            "alps_system_defaults": ([P(_abi.alps_system)], None),
            "alps_species_defaults": ([P(_abi.alps_species)], None),
            "alps_create": ([P(_abi.alps_system), P(vp)], C.c_int),
            "alps_destroy": ([vp], None),
            "alps_set_species": ([vp, C.c_int, P(_abi.alps_species), dp, dp, dp], C.c_int),
            "alps_prepare": ([vp], C.c_int),
            "alps_get_fit": ([vp, C.c_int, dp], C.c_int),
            "alps_set_fit": ([vp, C.c_int, dp], C.c_int),
            "alps_get_f0_rel": ([vp, C.c_int, dp, dp, dp, dp, dp], C.c_int),
            "alps_calc_eigen": ([vp, C.c_int, C.POINTER(_abi.alps_complex), C.c_int, C.c_int,
                                 C.POINTER(_abi.alps_eigen)], C.c_int),
            "alps_server_create": ([C.c_size_t, C.c_int, P(vp)], C.c_int),
            "alps_server_destroy": ([vp], None),
            "alps_server_submit": ([vp, P(_abi.alps_request), P(C.c_int64)], C.c_int),
            "alps_server_poll": ([vp, C.c_int64, P(C.c_int)], C.c_int),
            "alps_server_wait": ([vp, C.c_int64], C.c_int),
            "alps_server_stats": ([vp, P(C.c_int64), P(C.c_int), P(C.c_size_t)], C.c_int),
            "alps_set_k": ([vp, C.c_double, C.c_double], C.c_int),
            "alps_get_nmax": ([vp, P(C.c_int)], C.c_int),
            "alps_set_precision": ([vp, C.c_int], C.c_int),
            "alps_disp": ([vp, _abi.alps_complex, cp, cp, cp, cp], C.c_int),
            "alps_disp_batch": ([vp, C.c_int, cp, cp], C.c_int),
            "alps_disp_batch_device": ([vp, C.c_int, vp, vp, vp], C.c_int),
            "alps_secant": ([vp, C.c_int, C.c_int, cp, P(C.c_int), cp], C.c_int),
            "alps_secant_ex": ([vp, C.c_int, C.c_int, cp, C.c_double, P(C.c_int), cp, P(C.c_int)], C.c_int),
            "alps_map": ([vp, P(_abi.alps_map_params), cp, cp, dp], C.c_int),
            "alps_find_minima": ([dp, C.c_int, C.c_int, C.c_int, P(C.c_int), P(C.c_int)], C.c_int),
            "alps_run_input": ([C.c_char_p, C.c_char_p], C.c_int),
            "alps_read_input": ([C.c_char_p, P(_abi.alps_input)], C.c_int),
            "alps_read_f0": ([C.c_char_p, C.c_int, C.c_int, dp, dp, dp], C.c_int),
            "alps_generate_f0": ([P(_abi.alps_dist_params), C.c_int, C.c_int, dp, dp, dp, dp], C.c_int),
            "alps_get_stats": ([vp, P(_abi.alps_stats)], C.c_int),
            "alps_set_profiling": ([vp, C.c_int], C.c_int),
            "alps_disp_batch_noalloc": ([vp, C.c_int, vp, vp, vp, P(C.c_size_t)], C.c_int),
            "alps_batch_status": ([vp, vp], C.c_int),
            "alps_prepare_many": ([P(vp), C.c_int, P(C.c_int)], C.c_int),
            "alps_set_k_many": ([P(vp), C.c_int, dp, dp, P(C.c_int)], C.c_int),
            "alps_solve_many": ([P(vp), C.c_int, C.c_int, cp, C.c_double, P(C.c_int), cp, P(C.c_int)], C.c_int),
            "alps_tc_product": ([vp, vp, vp, C.c_int, C.c_int, C.c_int, C.c_int, P(C.c_int)], C.c_int),
            "alps_autotune": ([vp, C.c_int, vp, P(_abi.alps_tune_result)], C.c_int),
            "alps_server_get_profile": ([vp, P(_abi.alps_server_profile)], C.c_int),
            "alps_tune_clear": ([], C.c_int),
            "alps_get_profile": ([vp, dp, P(C.c_int64)], C.c_int),
            "alps_interpolate": ([dp, dp, dp, C.c_int, P(_abi.alps_interp_params), dp, dp, dp], C.c_int),
            "alps_run_interpolation": ([C.c_char_p, C.c_char_p], C.c_int),
        }
        for name, (args, res) in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
        return _lib


def check(status, where):
    if status != 0:
        msg = lib().alps_error_string(status).decode()
        raise _abi.AlpsError(status, "%s: %s" % (where, msg))


def exported_symbols():
    """Names of every function include/alps_gb300.h declares."""
    return [
        "alps_version", "alps_error_string", "alps_system_defaults", "alps_species_defaults", "alps_create",
        "alps_destroy", "alps_set_species", "alps_prepare", "alps_get_fit", "alps_set_fit", "alps_set_k",
        "alps_get_nmax", "alps_set_precision", "alps_disp", "alps_disp_batch", "alps_disp_batch_device",
        "alps_secant", "alps_secant_ex", "alps_solve_many", "alps_prepare_many", "alps_set_k_many", "alps_map", "alps_find_minima", "alps_run_input", "alps_generate_f0", "alps_get_stats",
        "alps_set_profiling", "alps_get_profile", "alps_disp_batch_noalloc", "alps_batch_status", "alps_tc_product", "alps_read_input", "alps_read_f0",
        "alps_autotune", "alps_tune_clear", "alps_get_f0_rel", "alps_calc_eigen", "alps_server_create", "alps_server_destroy", "alps_server_submit",
        "alps_server_poll", "alps_server_wait", "alps_server_stats", "alps_server_get_profile", "alps_interpolate", "alps_run_interpolation",
    ]
