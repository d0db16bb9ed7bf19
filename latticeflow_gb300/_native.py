"""ctypes binding of the C ABI declared in include/latticeflow_gpu.h.

The library is the in-tree ``_lib/liblatticeflow_gpu.so``; there is no
fallback: if it is missing, loading raises ``NativeLibraryMissing``.
"""
import ctypes
import os

from ._build import LIB

P = ctypes.c_void_p
I = ctypes.c_int
SZ = ctypes.c_size_t

# every symbol declared in include/latticeflow_gpu.h: name -> (restype, argtypes)
PROTOTYPES = {
    "lf_last_error": (ctypes.c_char_p, []),
    "lf_is_valid_solver": (I, [ctypes.c_char_p]),
    "lf_is_valid_kernel": (I, [ctypes.c_char_p]),
    "lf_kernel_dimension": (I, [ctypes.c_char_p]),
    "lf_valid_kernel_names": (SZ, [ctypes.c_char_p, SZ]),
    "lf_valid_solver_names": (SZ, [ctypes.c_char_p, SZ]),
    "lf_kernel_info": (I, [ctypes.c_char_p, P, P, P, P]),
    "lf_create": (I, [ctypes.c_char_p, ctypes.c_char_p, I, P, P]),
    "lf_destroy": (None, [P]),
    "lf_n_dimensions": (I, [P]),
    "lf_shape": (I, [P, P]),
    "lf_n_nodes": (SZ, [P]),
    "lf_n_filling_edges": (I, [P]),
    "lf_edge_deltas": (I, [P, P]),
    "lf_add_energy_potentials": (I, [P, P, P]),
    "lf_add_energy_potentials_device": (I, [P, P, P]),
    "lf_add_capacities": (I, [P, P, P, P]),
    "lf_run": (I, [P]),
    "lf_run_time": (ctypes.c_double, [P]),
    "lf_get_cut": (I, [P, P]),
    "lf_get_cut_max": (I, [P, P]),
    "lf_get_flow": (I, [P, P, P]),
    "lf_get_levels": (I, [P, P]),
    "lf_get_level_sets": (I, [P, P]),
    "lf_get_stats": (I, [P, P, P, P]),
    "lf_set_tuning": (I, [P, I, I, I]),
    "lf_set_param": (I, [P, ctypes.c_char_p, I]),
    "lf_clear": (I, [P]),
    "lf_set_profiling": (I, [P, I]),
    "lf_get_profile": (I, [P, P, P]),
    "lf_get_stream": (I, [P, P]),
    "lf_get_layout": (I, [P, P, P, P]),
    "lf_tv_2d": (I, [ctypes.c_char_p, SZ, SZ, P, ctypes.c_double, P, P]),
    "lf_tv_2d_level_sets": (I, [ctypes.c_char_p, SZ, SZ, P, ctypes.c_double, P, P, P]),
    "lf_tv_2d_path": (I, [ctypes.c_char_p, SZ, SZ, P, SZ, P, P]),
    "lf_tv_2d_path_stats": (I, [ctypes.c_char_p, SZ, SZ, P, SZ, P, P, P]),
    "lf_tv_2d_batch": (I, [ctypes.c_char_p, SZ, SZ, SZ, P, SZ, P, P, P, SZ]),
    "lf_batch_create": (I, [P]),
    "lf_batch_destroy": (None, [P]),
    "lf_batch_add": (I, [P, ctypes.c_char_p, I, P, P]),
    "lf_batch_size": (I, [P]),
    "lf_batch_add_energy_potentials": (I, [P, I, P, P]),
    "lf_batch_add_capacities": (I, [P, I, P, P, P]),
    "lf_batch_add_capacities_packed": (I, [P, P, P, P]),
    "lf_batch_get_cuts_packed": (I, [P, P, I]),
    "lf_batch_get_flows": (I, [P, P, P]),
    "lf_batch_clear": (I, [P]),
    "lf_batch_run": (I, [P]),
    "lf_batch_run_time": (ctypes.c_double, [P]),
    "lf_batch_get_cut": (I, [P, I, P]),
    "lf_batch_get_cut_max": (I, [P, I, P]),
    "lf_batch_get_flow": (I, [P, I, P, P]),
    "lf_batch_set_param": (I, [P, ctypes.c_char_p, I]),
    "lf_batch_get_stats": (I, [P, P, P, P]),
    "lf_cut_2d_noalloc": (I, [ctypes.c_char_p, SZ, SZ, P, P, P, P, P, P]),
    "lf_server_create": (I, [I, SZ, P]),
    "lf_server_destroy": (None, [P]),
    "lf_server_submit_tv": (I, [P, ctypes.c_char_p, SZ, SZ, P, ctypes.c_double, P]),
    "lf_server_submit_cut": (I, [P, ctypes.c_char_p, SZ, SZ, P, P, P, P]),
    "lf_server_wait": (I, [P, ctypes.c_int64, ctypes.c_double, P]),
    "lf_server_get_tv": (I, [P, ctypes.c_int64, P, P]),
    "lf_server_get_cut": (I, [P, ctypes.c_int64, P, P, P]),
    "lf_server_release": (I, [P, ctypes.c_int64]),
    "lf_server_cancel": (I, [P, ctypes.c_int64]),
    "lf_server_inject_alloc_failures": (I, [P, I]),
    "lf_server_stats": (I, [P, P, P, P, P, P]),
    "lf_server_set_max_group": (I, [P, I]),
    "lf_server_group_stats": (I, [P, P, P]),
}

LF_OK = 0
LF_ERR_BAD_NAME = 1
LF_ERR_SHAPE = 2
LF_ERR_RANGE = 3
LF_ERR_NO_CONVERGENCE = 4
LF_ERR_OOM = 5
LF_ERR_CUDA = 6
LF_ERR_INVALID = 7
LF_ERR_STATE = 8


class NativeLibraryMissing(ImportError):
    pass


class LatticeFlowError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("[%d] %s" % (code, msg))
        self.code = code


class BadSolverOrKernelName(ValueError):
    """Mirror of latticeQBP::BadSolverOrKernelName (solver/interface.hpp:152-168)."""


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise NativeLibraryMissing(
                "liblatticeflow_gpu.so is not built; run __graft_entry__.build() "
                "or python -m latticeflow_gb300._build")
        L = ctypes.CDLL(LIB)
        for name, (res, args) in PROTOTYPES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def last_error():
    return lib().lf_last_error().decode()


def check(rc):
    if rc == LF_OK:
        return
    msg = last_error()
    if rc == LF_ERR_BAD_NAME:
        raise BadSolverOrKernelName(msg)
    if rc in (LF_ERR_SHAPE, LF_ERR_INVALID):
        raise ValueError(msg)
    if rc == LF_ERR_RANGE:
        raise OverflowError(msg)
    raise LatticeFlowError(rc, msg)
