"""ctypes binding of libsfft.so (the C interface of include/sfft.h).

There is no fallback: if the library is missing this module raises, and a
plan cannot be made without a CUDA device.
"""
import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsfft.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "sfft.h")

SFFT_VERSION_1, SFFT_VERSION_2, SFFT_VERSION_3 = 0, 1, 2
SFFT_PREC_FP64, SFFT_PREC_FP32 = 0, 1
SFFT_IN_C128, SFFT_IN_C64 = 0, 1
FFTW_MEASURE = 0
FFTW_ESTIMATE = 1 << 6


class Options(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int), ("device", ctypes.c_int), ("max_batch", ctypes.c_int)]


class Params(ctypes.Structure):
    _fields_ = [("Bcst_loc", ctypes.c_double), ("Bcst_est", ctypes.c_double), ("Comb_cst", ctypes.c_double),
                ("loc_loops", ctypes.c_int), ("est_loops", ctypes.c_int), ("threshold_loops", ctypes.c_int),
                ("comb_loops", ctypes.c_int), ("tolerance_loc", ctypes.c_double),
                ("tolerance_est", ctypes.c_double)]


class ServerOptions(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("max_batch", ctypes.c_int), ("hbm_budget_bytes", ctypes.c_long),
                ("k_round", ctypes.c_int), ("tune_invalid", ctypes.c_int), ("v2_voted", ctypes.c_int)]


class Plan(ctypes.Structure):
    _fields_ = [("version", ctypes.c_int), ("n", ctypes.c_uint), ("k", ctypes.c_uint),
                ("data", ctypes.c_void_p)]


_lib = None


def header_functions():
    """Names of the functions include/sfft.h declares."""
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    block = src.split('extern "C" {', 1)[1].split("#ifdef __cplusplus\n}", 1)[0]
    return sorted(set(re.findall(r"\b(sfft_\w+)\s*\(", block)))


def load(build_if_missing=False):
    """The loaded library (ctypes.CDLL) with argument types set."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if build_if_missing:
            from . import build
            build.build()
        else:
            raise ImportError(f"{LIB_PATH} is not built (python -m sfft_gb300.build)")
    L = ctypes.CDLL(LIB_PATH)
    vp, cp, ci, cl = ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_long
    PP = ctypes.POINTER(Plan)
    L.sfft_malloc.restype = vp
    L.sfft_malloc.argtypes = [ctypes.c_size_t]
    L.sfft_free.argtypes = [vp]
    L.sfft_make_plan.restype = PP
    L.sfft_make_plan.argtypes = [ci, ci, ci, ci]
    L.sfft_make_plan_ex.restype = PP
    L.sfft_make_plan_ex.argtypes = [ci, ci, ci, ci, ctypes.POINTER(Options)]
    L.sfft_free_plan.argtypes = [PP]
    L.sfft_exec.argtypes = [PP, vp, vp]
    L.sfft_exec_many.argtypes = [PP, ci, vp, vp]
    L.sfft_last_error.restype = cp
    L.sfft_output_capacity.restype = cl
    L.sfft_output_capacity.argtypes = [PP]
    L.sfft_exec_sparse.restype = cl
    L.sfft_exec_sparse.argtypes = [PP, vp, vp, vp, cl]
    L.sfft_exec_batch.restype = ci
    L.sfft_exec_batch.argtypes = [PP, ci, vp, ci, vp, vp, vp, cl, vp]
    L.sfft_exec_many_sparse.restype = ci
    L.sfft_exec_many_sparse.argtypes = [PP, ci, vp, vp, vp, vp, cl]
    L.sfft_sync.restype = ci
    L.sfft_sync.argtypes = [PP]
    L.sfft_debug_fetch.restype = cl
    L.sfft_debug_fetch.argtypes = [PP, ci, vp, cl]
    L.sfft_debug_median_network.restype = ci
    L.sfft_debug_median_network.argtypes = [ci, vp, cl]
    L.sfft_describe_plan.restype = ci
    L.sfft_describe_plan.argtypes = [ci, ci, ci, ctypes.POINTER(cl), ci]
    L.sfft_describe_filter.restype = ci
    L.sfft_describe_filter.argtypes = [ci, ci, ci, ci, vp, cl, vp, cl]
    L.sfft_profile.restype = ci
    L.sfft_profile.argtypes = [PP, ci]
    L.sfft_profile_read.restype = cl
    L.sfft_profile_read.argtypes = [PP, ctypes.POINTER(ctypes.c_double), ci]
    L.sfft_make_plan_params.restype = PP
    L.sfft_make_plan_params.argtypes = [ci, ci, ci, ctypes.POINTER(Params), ctypes.POINTER(Options)]
    L.sfft_plan_footprint.restype = cl
    L.sfft_plan_footprint.argtypes = [PP]
    L.sfft_exec_batch_ex.restype = ci
    L.sfft_exec_batch_ex.argtypes = [PP, ci, vp, ci, vp, vp, vp, vp, cl, vp]
    L.sfft_plan_stream.restype = vp
    L.sfft_plan_stream.argtypes = [PP]
    L.sfft_server_create.restype = vp
    L.sfft_server_create.argtypes = [ctypes.POINTER(ServerOptions)]
    L.sfft_server_destroy.argtypes = [vp]
    L.sfft_server_submit.restype = cl
    L.sfft_server_submit.argtypes = [vp, ci, ci, ci, ci, vp, ci, ctypes.c_uint]
    L.sfft_server_wait.restype = cl
    L.sfft_server_wait.argtypes = [vp, cl, vp, vp, cl, ctypes.POINTER(ctypes.c_double)]
    L.sfft_server_count.restype = cl
    L.sfft_server_count.argtypes = [vp, cl, ctypes.c_double]
    L.sfft_server_wait_for.restype = cl
    L.sfft_server_wait_for.argtypes = L.sfft_server_wait.argtypes + [ctypes.c_double]
    L.sfft_describe_plan_params.restype = ci
    L.sfft_describe_plan_params.argtypes = [ci, ci, ci, ctypes.POINTER(Params), ctypes.POINTER(ctypes.c_long), ci]
    L.sfft_plan_v2_voted.restype = ci
    L.sfft_plan_v2_voted.argtypes = [PP, ci]
    L.sfft_tuned_params.restype = ci
    L.sfft_tuned_params.argtypes = [ci, ci, ci, ctypes.POINTER(Params)]
    L.sfft_tuned_k.restype = ci
    L.sfft_tuned_k.argtypes = [ci]
    L.sfft_mixed_create.restype = vp
    L.sfft_mixed_create.argtypes = [ci, vp, vp, vp, vp, ci, ci, ci]
    L.sfft_mixed_exec.restype = ci
    L.sfft_mixed_exec.argtypes = [vp, vp, vp]
    L.sfft_mixed_sync.restype = ci
    L.sfft_mixed_sync.argtypes = [vp]
    L.sfft_mixed_result.restype = ci
    L.sfft_mixed_result.argtypes = [vp, ci, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(ci),
                                    ctypes.POINTER(cl)]
    L.sfft_mixed_result_host.restype = cl
    L.sfft_mixed_result_host.argtypes = [vp, ci, vp, vp, cl]
    L.sfft_mixed_set_persistent.restype = ci
    L.sfft_mixed_set_persistent.argtypes = [vp, ci]
    L.sfft_mixed_groups.restype = ci
    L.sfft_mixed_groups.argtypes = [vp]
    L.sfft_mixed_destroy.argtypes = [vp]
    L.sfft_mixed_stream.restype = vp
    L.sfft_mixed_stream.argtypes = [vp]
    L.sfft_server_plan_bytes.restype = cl
    L.sfft_server_plan_bytes.argtypes = [ci, ci, ci, ci, ci]
    L.sfft_server_stats.restype = ci
    L.sfft_server_stats.argtypes = [vp, ctypes.POINTER(cl), ci]
    L.sfft_exec_noalloc.restype = cl
    L.sfft_exec_noalloc.argtypes = [PP, vp, ci, vp, vp, cl, vp, vp]
    L.sfft_kernel_launches.restype = cl
    L.sfft_kernel_launches.argtypes = []
    _lib = L
    return L


def last_error():
    return load().sfft_last_error().decode()
