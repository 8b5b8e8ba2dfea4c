"""Loader and ctypes declarations of libtileqr.so (include/tileqr.h).

The library is built in-tree (nextla.jl_gb300/tileqr_build.py).  There is no CPU
fallback: if the shared library is missing, every call raises.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libtileqr.so")

_I = ctypes.c_int
_C = ctypes.c_char
_P = ctypes.c_void_p

# name -> argument types (without the precision prefix); every entry point
# returns int and ends with a cudaStream_t.
SIGNATURES = {
    "geqr2": [_I, _I, _P, _I, _P, _P, _P],
    "larft": [_C, _C, _I, _I, _P, _I, _P, _P, _I, _P],
    "larfb": [_C, _C, _C, _C, _I, _I, _I, _P, _I, _P, _I, _P, _I, _P, _I, _P],
    "geqrt": [_I, _I, _I, _P, _I, _P, _I, _P, _P, _P],
    "unmqr": [_C, _C, _I, _I, _I, _I, _P, _I, _P, _I, _P, _I, _P, _I, _P],
    "tsqrt": [_I, _I, _I, _I, _P, _I, _P, _I, _P, _I, _P, _P, _P],
    "tsmqr": [_C, _C, _I, _I, _I, _I, _I, _I, _P, _I, _P, _I, _P, _I, _P, _I, _P, _I, _P],
    "parfb": [_C, _C, _C, _C, _I, _I, _I, _I, _I, _I, _P, _I, _P, _I, _P, _I, _P, _I, _P, _I, _P],
    "ttqrt": [_I, _I, _I, _P, _I, _P, _I, _P, _I, _P, _P, _P],
    "pamm": [_C, _C, _C, _C, _I, _I, _I, _I, _P, _I, _P, _I, _P, _I, _P, _I, _P],
    "ttmqr": [_C, _C, _I, _I, _I, _I, _I, _I, _P, _I, _P, _I, _P, _I, _P, _I, _P, _I, _P],
    "tile_geqrf": [_I, _I, _I, _I, _P, _I, _P, _I, _P, _I, _P],
    "tile_unmqr": [_C, _I, _I, _I, _I, _I, _P, _I, _P, _I, _P, _I, _P],
    "trsm_lun": [_I, _I, _P, _I, _P, _I, _P],
    "tile_gels": [_I, _I, _I, _I, _I, _P, _I, _P, _I, _P, _I, _P, _I, _P],
    "tile_geqrf_tree": [_I, _I, _I, _I, _P, _I, _P, _P, _I, _P, _P, _I, _I, _P, _I, _P],
    "tile_unmqr_tree": [_C, _I, _I, _I, _I, _I, _P, _I, _P, _P, _I, _P, _I, _P],
    "tile_geqrf_hqr": [_I, _I, _I, _I, _I, _P, _I, _P, _P, _I, _P, _P, _I, _I, _P, _I, _P],
    "tile_unmqr_hqr": [_C, _I, _I, _I, _I, _I, _I, _P, _I, _P, _P, _I, _P, _I, _P],
}

# routines that also exist for ComplexF64 (prefix z) and ComplexF32 (prefix c)
COMPLEX = ("geqr2", "larft", "larfb", "geqrt", "unmqr", "tsqrt", "tsmqr", "parfb", "ttqrt", "ttmqr",
           "tile_geqrf", "tile_unmqr", "trsm_lun", "tile_gels", "pamm", "tile_geqrf_tree", "tile_unmqr_tree",
           "tile_geqrf_hqr", "tile_unmqr_hqr")


def prefixes(name):
    return ("d", "s", "z", "c") if name in COMPLEX else ("d", "s")


# measurement hooks without a precision prefix: name -> (argtypes, restype)
DIAG = {
    "tqr_launch_count": ([], ctypes.c_ulonglong),
    "tqr_profile_enable": ([_I], None),
    "tqr_profile_read": ([ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_double),
                          ctypes.POINTER(ctypes.c_double)], _I),
    "tqr_fp64_peak_probe": ([_I, _I, _P, _P], _I),
    "tqr_fp64_mma_probe": ([_I, _I, _I, _P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), _P],
                           _I),
    "tqr_tile_dag_worksize": ([_I, _I, _I, _I, ctypes.POINTER(ctypes.c_size_t)], _I),
    "tqr_dtile_geqrf_dag": ([_I, _I, _I, _I, _P, _I, _P, _I, _P, _I, _P, ctypes.c_size_t, _P], _I),
    "tqr_stile_geqrf_dag": ([_I, _I, _I, _I, _P, _I, _P, _I, _P, _I, _P, ctypes.c_size_t, _P], _I),
    "tqr_ztile_geqrf_dag": ([_I, _I, _I, _I, _P, _I, _P, _I, _P, _I, _P, ctypes.c_size_t, _P], _I),
    "tqr_ctile_geqrf_dag": ([_I, _I, _I, _I, _P, _I, _P, _I, _P, _I, _P, ctypes.c_size_t, _P], _I),
    "tqr_tile_dag_status": ([_P, ctypes.POINTER(_I), ctypes.POINTER(_I), _P], _I),
    "tqr_tile_dag_wait_selftest": ([_I, _I, _I, _I, _P, _I, _P, _I, _P, _I, _P, ctypes.c_size_t, _I, _P], _I),
    "tqr_tile_dag_check": ([_I, _I, _I, _I, ctypes.POINTER(ctypes.c_longlong)], _I),
    "tqr_tile_autotune": ([_I, _I, _I, _I, ctypes.POINTER(_I), ctypes.POINTER(_I), _P], _I),
    "tqr_tile_tuning": ([_I, _I, _I, ctypes.POINTER(_I), ctypes.POINTER(_I)], _I),
    "tqr_tile_dag_stats": ([_P, ctypes.POINTER(ctypes.c_ulonglong), _P], _I),
    "tqr_dtile_geqrf_noalloc": ([_I, _I, _I, _I, _P, _I, _P, _I, _P, _I, _P], _I),
    "tqr_tile_noalloc_status": ([ctypes.POINTER(_I), ctypes.POINTER(_I), _P], _I),
    "tqr_tile_noalloc_check": ([_I, _I, _I, _I, ctypes.POINTER(ctypes.c_longlong)], _I),
    "tqr_tile_dag_simulate": ([_I, _I, _I, _I, _I, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                               ctypes.POINTER(ctypes.c_double)], _I),
    "tqr_tile_dag_check_rhs": ([_I, _I, _I, _I, _I, ctypes.POINTER(ctypes.c_longlong)], _I),
    "tqr_tile_gels_worksize": ([_I, _I, _I, _I, _I, ctypes.POINTER(ctypes.c_size_t)], _I),
    "tqr_dtile_gels_dag": ([_I, _I, _I, _I, _I, _P, _I, _P, _I, _P, _I, _P, _I, _P, ctypes.c_size_t, _P], _I),
    "tqr_stile_gels_dag": ([_I, _I, _I, _I, _I, _P, _I, _P, _I, _P, _I, _P, _I, _P, ctypes.c_size_t, _P], _I),
    "tqr_dsgels_worksize": ([_I, _I, _I, _I, _I, ctypes.POINTER(ctypes.c_size_t)], _I),
    "tqr_dsgels_phases": ([ctypes.POINTER(ctypes.c_double), ctypes.POINTER(_I)], _I),
    "tqr_dsgels_fp64_panels": ([_I], _I),
    "tqr_dsgels_hqr_group": ([_I], _I),
    "tqr_dsgels_trsv_pipelined": ([_I], _I),
    "tqr_dsgels_trsv_pipe_check": ([_I, ctypes.POINTER(ctypes.c_longlong)], _I),
    "tqr_stile_geqrf_hqr_dag_f64p": ([_I, _I, _I, _I, _I, _P, _I, _P, _P, _I, _P, _P, _I, _I, _P, _I, _P,
                                      ctypes.c_size_t, _P], _I),
    "tqr_tile_hqr_dag_check_tc": ([_I, _I, _I, _I, _I, _I, ctypes.POINTER(ctypes.c_longlong)], _I),
    "tqr_tile_hqr_dag_check_wy": ([_I, _I, _I, _I, _I, _I, ctypes.POINTER(ctypes.c_longlong),
                                   ctypes.POINTER(ctypes.c_longlong)], _I),
    "tqr_stile_geqrf_dag_f64p": ([_I, _I, _I, _I, _P, _I, _P, _I, _P, _I, _P, ctypes.c_size_t, _P], _I),
    "tqr_dsgels": ([_I, _I, _I, _I, _I, _P, _I, _P, _I, _P, _I, _I, ctypes.c_double, _P, ctypes.c_size_t,
                    ctypes.POINTER(_I), ctypes.POINTER(ctypes.c_double), _P], _I),
    "tqr_batched_problem_bytes": ([], _I),
    "tqr_batched_plan": ([_I, _I, _P, _P, _P, _P, _P, ctypes.POINTER(ctypes.c_longlong),
                          ctypes.POINTER(ctypes.c_longlong)], _I),
    "tqr_batched_worksize": ([_I, ctypes.POINTER(ctypes.c_size_t)], _I),
    "tqr_batched_autotune": ([_I, _I, _P], _I),
    "tqr_batched_tuning": ([_I, _I, ctypes.POINTER(_I), ctypes.POINTER(_I)], _I),
    "tqr_dbatched_gels": ([_I, _P, _P, _P, _P, _P, ctypes.c_size_t, _P], _I),
    "tqr_sbatched_gels": ([_I, _P, _P, _P, _P, _P, ctypes.c_size_t, _P], _I),
    "tqr_batched_status": ([_P, ctypes.POINTER(_I), ctypes.POINTER(_I), _P], _I),
    "tqr_zbatched_gels": ([_I, _P, _P, _P, _P, _P, ctypes.c_size_t, _P], _I),
    "tqr_cbatched_gels": ([_I, _P, _P, _P, _P, _P, ctypes.c_size_t, _P], _I),
    "tqr_dbatched_residual": ([_I, _P, _P, _P, _P, _P, _P], _I),
    "tqr_sbatched_residual": ([_I, _P, _P, _P, _P, _P, _P], _I),
    "tqr_batched_graph": ([_I, _I, _P, _P, _P, _P, _P, ctypes.c_size_t, ctypes.POINTER(_P)], _I),
    "tqr_batched_graph_launch": ([_P, _P], _I),
    "tqr_batched_graph_destroy": ([_P], _I),
    "tqr_tile_tree_dag_worksize": ([_I, _I, _I, _I, _I, ctypes.POINTER(ctypes.c_size_t)], _I),
    "tqr_tile_hqr_dag_worksize": ([_I, _I, _I, _I, _I, _I, ctypes.POINTER(ctypes.c_size_t)], _I),
    "tqr_tile_hqr_dag_check": ([_I, _I, _I, _I, _I, _I, ctypes.POINTER(ctypes.c_longlong)], _I),
    "tqr_dtile_geqrf_hqr_dag": ([_I, _I, _I, _I, _I, _P, _I, _P, _P, _I, _P, _P, _I, _I, _P, _I, _P, ctypes.c_size_t,
                                 _P], _I),
    "tqr_stile_geqrf_hqr_dag": ([_I, _I, _I, _I, _I, _P, _I, _P, _P, _I, _P, _P, _I, _I, _P, _I, _P, ctypes.c_size_t,
                                 _P], _I),
    "tqr_ztile_geqrf_hqr_dag": ([_I, _I, _I, _I, _I, _P, _I, _P, _P, _I, _P, _P, _I, _I, _P, _I, _P, ctypes.c_size_t,
                                 _P], _I),
    "tqr_ctile_geqrf_hqr_dag": ([_I, _I, _I, _I, _I, _P, _I, _P, _P, _I, _P, _P, _I, _I, _P, _I, _P, ctypes.c_size_t,
                                 _P], _I),
    "tqr_ztile_geqrf_tree_dag": ([_I, _I, _I, _I, _P, _I, _P, _P, _I, _P, _P, _I, _I, _P, _I, _P, ctypes.c_size_t,
                                  _P], _I),
    "tqr_ctile_geqrf_tree_dag": ([_I, _I, _I, _I, _P, _I, _P, _P, _I, _P, _P, _I, _I, _P, _I, _P, ctypes.c_size_t,
                                  _P], _I),
    "tqr_tile_hqr_dag_check_strips": ([_I, _I, _I, _I, _I, _I, _I, ctypes.POINTER(ctypes.c_longlong)], _I),
    "tqr_tile_tree_dag_check": ([_I, _I, _I, _I, _I, ctypes.POINTER(ctypes.c_longlong)], _I),
    "tqr_tile_tree_dag_status": ([_P, ctypes.POINTER(_I), ctypes.POINTER(_I), _P], _I),
    "tqr_dtile_geqrf_tree_dag": ([_I, _I, _I, _I, _P, _I, _P, _P, _I, _P, _P, _I, _I, _P, _I, _P, ctypes.c_size_t,
                                  _P], _I),
    "tqr_stile_geqrf_tree_dag": ([_I, _I, _I, _I, _P, _I, _P, _P, _I, _P, _P, _I, _I, _P, _I, _P, ctypes.c_size_t,
                                  _P], _I),
    "tqr_tile_dag_tensor_cores": ([_I], _I),
    "tqr_tile_dag_order_quantum": ([ctypes.c_double], ctypes.c_double),
    "tqr_tile_tc_tma": ([_I], _I),
    "tqr_tile_tc_wy": ([_I], _I),
    "tqr_tile_dag_occupancy": ([_I, _I, ctypes.POINTER(_I), ctypes.POINTER(_I)], _I),
    "tqr_tile_dag_check_tc": ([_I, _I, _I, _I, _I, ctypes.POINTER(ctypes.c_longlong)], _I),
    "tqr_stsmqr_tc": ([_I, _I, _I, _I, _P, _I, _P, _I, _P, _I, _P, _I, _P, _P], _I),
    "tqr_swy_slot_bytes": ([], ctypes.c_size_t),
    "tqr_swy_build": ([_I, _I, _P, _I, _P, _I, _I, _P, ctypes.c_size_t, _P, _P], _I),
    "tqr_swy_apply": ([_I, _I, _I, _I, _P, _I, _P, _I, _P, _P, _P], _I),
    "tqr_stsmqr_wy": ([_I, _I, _I, _I, _P, _I, _P, _I, _P, _I, _P, _I, _P, ctypes.c_size_t, _P, _P], _I),
    "tqr_qr_batched_worksize": ([_I, _I, _I, _I, ctypes.POINTER(ctypes.c_size_t)], _I),
    "tqr_zqr_batched_fwd": ([_I, _I, _I, _I, _P, _P, _P, _P, _P, ctypes.c_size_t, _P], _I),
    "tqr_cqr_batched_fwd": ([_I, _I, _I, _I, _P, _P, _P, _P, _P, ctypes.c_size_t, _P], _I),
    "tqr_zqr_batched_bwd": ([_I, _I, _I, _I, _P, _P, _P, _P, _P, _P, ctypes.c_size_t, _P], _I),
    "tqr_cqr_batched_bwd": ([_I, _I, _I, _I, _P, _P, _P, _P, _P, _P, ctypes.c_size_t, _P], _I),
    "tqr_dqr_batched_fwd": ([_I, _I, _I, _I, _P, _P, _P, _P, _P, ctypes.c_size_t, _P], _I),
    "tqr_sqr_batched_fwd": ([_I, _I, _I, _I, _P, _P, _P, _P, _P, ctypes.c_size_t, _P], _I),
    "tqr_dqr_batched_bwd": ([_I, _I, _I, _I, _P, _P, _P, _P, _P, _P, ctypes.c_size_t, _P], _I),
    "tqr_sqr_batched_bwd": ([_I, _I, _I, _I, _P, _P, _P, _P, _P, _P, ctypes.c_size_t, _P], _I),
}

_lib = None


class LibraryMissing(RuntimeError):
    pass


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise LibraryMissing(
                f"{LIB_PATH} is not built; run nextla.jl_gb300/tileqr_build.py (no CPU fallback exists)")
        L = ctypes.CDLL(LIB_PATH)
        for name, args in SIGNATURES.items():
            for p in prefixes(name):
                f = getattr(L, f"tqr_{p}{name}")
                f.argtypes = args
                f.restype = _I
        for name, (args, res) in DIAG.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def launch_count():
    return int(lib().tqr_launch_count())


def profile_enable(on):
    lib().tqr_profile_enable(1 if on else 0)


def profile_read():
    """(launches, device ms, algorithmic flops) of the timed trailing updates."""
    n = ctypes.c_longlong(0)
    ms = ctypes.c_double(0)
    fl = ctypes.c_double(0)
    rc = lib().tqr_profile_read(ctypes.byref(n), ctypes.byref(ms), ctypes.byref(fl))
    if rc != 0:
        raise RuntimeError(f"tqr_profile_read: CUDA error {rc}")
    return n.value, ms.value, fl.value


def fn(prefix, name):
    if prefix not in prefixes(name) and name in SIGNATURES:
        raise TypeError(f"{name} has no {'complex' if prefix in 'zc' else prefix} form")
    return getattr(lib(), f"tqr_{prefix}{name}")


def exported_symbols():
    """Every tqr_* symbol the header declares, as (name, present) pairs."""
    L = lib()
    out = []
    for name in SIGNATURES:
        for p in prefixes(name):
            out.append((f"tqr_{p}{name}", hasattr(L, f"tqr_{p}{name}")))
    return out
