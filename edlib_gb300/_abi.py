"""ctypes binding of libedgpu.so (the C ABI declared in include/edgpu.h).

The library is built in-tree by ``edlib_gb300.build`` and loaded from ``edlib_gb300/_lib``.  There
is no fallback: if the library is missing, ``lib()`` raises.
"""
import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libedgpu.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "edgpu.h")

OK = 0
NOT_CONVERGED = 1
ERR_ARG, ERR_CUDA, ERR_CAPACITY, ERR_COLLISION, ERR_STATE = -1, -2, -3, -4, -5
STORAGES = {"CRS": 0, "SRS": 1, "SOCRS": 2}
# "mixed": the eigen-solve in FP32 (as "fp32"); Green's functions, susceptibilities and static observables
# from FP64 eigenvectors (the kept pairs continued in FP64) with FP64 recurrences
PRECISIONS = {"fp64": 0, "fp32": 1, "mixed": 2}
OPERATORS = {"Sz": 0, "N": 1}

_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)
_LL = ctypes.POINTER(ctypes.c_longlong)
_VP = ctypes.c_void_p


class DiagParams(ctypes.Structure):
    _fields_ = [("storage", ctypes.c_int), ("precision", ctypes.c_int), ("nev", ctypes.c_int), ("ncv", ctypes.c_int),
                ("eigenvalues_only", ctypes.c_int), ("tol", ctypes.c_double), ("maxitr", ctypes.c_int),
                ("sectors", _I), ("n_sectors", ctypes.c_int), ("multiplicity_check", ctypes.c_int),
                ("max_batch", ctypes.c_int)]


class GfParams(ctypes.Structure):
    _fields_ = [("beta", ctypes.c_double), ("nomega", ctypes.c_int), ("nlanc", ctypes.c_int),
                ("cutoff", ctypes.c_double), ("precision", ctypes.c_int), ("orbitals", _I),
                ("n_orbitals", ctypes.c_int), ("max_batch", ctypes.c_int), ("mesh", ctypes.c_int),
                ("emin", ctypes.c_double), ("emax", ctypes.c_double)]


_SIGS = {
    "edgpu_ctx_create": (ctypes.c_int, [ctypes.POINTER(_VP), ctypes.c_int, ctypes.c_size_t]),
    "edgpu_ctx_destroy": (ctypes.c_int, [_VP]),
    "edgpu_last_error": (ctypes.c_char_p, [_VP]),
    "edgpu_ctx_device_bytes": (ctypes.c_size_t, [_VP]),
    "edgpu_ctx_stream": (ctypes.c_void_p, [_VP]),
    "edgpu_model_hubbard": (ctypes.c_int, [_VP, ctypes.c_int, _D, _D, _D, _D, _D, ctypes.POINTER(_VP)]),
    "edgpu_model_siam": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_int, _D, _D, _D, ctypes.c_double, _D,
                                        ctypes.POINTER(_VP)]),
    "edgpu_model_destroy": (ctypes.c_int, [_VP]),
    "edgpu_model_transitions": (ctypes.c_int, [_VP, ctypes.c_int]),
    "edgpu_model_set_limits": (ctypes.c_int, [_VP, ctypes.c_size_t, ctypes.c_size_t]),
    "edgpu_binom": (ctypes.c_longlong, [_VP, ctypes.c_int, ctypes.c_int]),
    "edgpu_basis": (ctypes.c_int, [_VP, ctypes.c_int, _I]),
    "edgpu_ninv": (ctypes.c_int, [_VP, ctypes.c_int, _I]),
    "edgpu_sector_order": (ctypes.c_int, [_VP, _I, ctypes.c_int, _I, _I]),
    "edgpu_fill": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_int, ctypes.c_int, _LL]),
    "edgpu_av": (ctypes.c_int, [_VP, _D, _D, ctypes.c_longlong, ctypes.c_int, ctypes.c_int]),
    "edgpu_a_adag": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _D, _D,
                                    ctypes.c_int]),
    "edgpu_vv": (ctypes.c_int, [_VP, _D, _D, ctypes.c_longlong, _D]),
    "edgpu_spmv": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_int, ctypes.c_int, _VP, _VP, ctypes.c_int,
                                  ctypes.c_longlong, ctypes.c_int, ctypes.c_int, _VP]),
    "edgpu_diag": (ctypes.c_int, [_VP, ctypes.POINTER(DiagParams), _I]),
    "edgpu_diag_many": (ctypes.c_int, [ctypes.POINTER(_VP), ctypes.c_int, ctypes.POINTER(DiagParams), _I]),
    "edgpu_greens_function_many": (ctypes.c_int, [ctypes.POINTER(_VP), ctypes.c_int, ctypes.POINTER(GfParams),
                                                  ctypes.POINTER(_D), ctypes.POINTER(_D), _D]),
    "edgpu_chiloc_many": (ctypes.c_int, [ctypes.POINTER(_VP), ctypes.c_int, ctypes.POINTER(GfParams), ctypes.c_int, _D,
                                         ctypes.POINTER(_D), ctypes.POINTER(_D), _D]),
    "edgpu_diag_sector": (ctypes.c_int, [_VP, ctypes.POINTER(DiagParams), ctypes.c_int, ctypes.c_int, _D, _I, _D,
                                         ctypes.c_longlong]),
    "edgpu_eigenpairs": (ctypes.c_int, [_VP, _D, _I, _I, ctypes.c_int]),
    "edgpu_eigenvector": (ctypes.c_int, [_VP, ctypes.c_int, _D, ctypes.c_longlong]),
    "edgpu_greens_function": (ctypes.c_int, [_VP, ctypes.POINTER(GfParams), _D, _D, _D]),
    "edgpu_chiloc": (ctypes.c_int, [_VP, ctypes.POINTER(GfParams), ctypes.c_int, ctypes.c_double, _D, _D, _D]),
    "edgpu_refine_eigenpairs": (ctypes.c_int, [ctypes.POINTER(_VP), ctypes.c_int, ctypes.c_double, ctypes.c_double]),
    "edgpu_static_observables": (ctypes.c_int, [_VP, ctypes.c_double, ctypes.c_double, _D, _D, _D, _D, _D, _D, _D,
                                                _D]),
    "edgpu_lanczos": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_int, ctypes.c_int, _D, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_int, _D, _D, _I]),
    "edgpu_frac_points": (ctypes.c_int, [_VP, _D, _D, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                         _D, ctypes.c_int, _D]),
    "edgpu_stats": (ctypes.c_int, [_VP, _LL, _LL, _LL, _D]),
    "edgpu_bench_spmv": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int, _D, _D]),
    "edgpu_bench_spmv_batch": (ctypes.c_int, [ctypes.POINTER(_VP), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                              ctypes.c_int, _D, _D, _LL]),
    "edgpu_bench_cgs": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_int, _D, _D, _D, _D]),
    "edgpu_server_create": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_size_t, ctypes.POINTER(_VP)]),
    "edgpu_server_destroy": (ctypes.c_int, [_VP]),
    "edgpu_server_submit": (ctypes.c_int, [_VP, _VP, ctypes.POINTER(DiagParams), ctypes.POINTER(GfParams), _D, _D, _D,
                                           ctypes.POINTER(ctypes.c_longlong)]),
    "edgpu_server_step": (ctypes.c_int, [_VP, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    "edgpu_server_poll": (ctypes.c_int, [_VP, ctypes.c_longlong, ctypes.POINTER(ctypes.c_int),
                                         ctypes.POINTER(ctypes.c_int)]),
    "edgpu_greens_function_weighted": (ctypes.c_int, [_VP, ctypes.POINTER(GfParams), _D, ctypes.c_int, _D, _D]),
    "edgpu_self_energy": (ctypes.c_int, [_VP, ctypes.POINTER(GfParams), _D, _D, _D]),
    "edgpu_operator_tuning": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                             _D]),
    "edgpu_launch_count": (ctypes.c_longlong, []),
    "edgpu_selftest_bulk_wait": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                                ctypes.POINTER(ctypes.c_int)]),
    "edgpu_vv_noalloc": (ctypes.c_int, [_VP, _VP, ctypes.c_longlong, _VP, _VP]),
}

_lib = None


def header_symbols():
    """Names of every function declared in include/edgpu.h."""
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(edgpu_[a-z0-9_]+)\s*\(", txt)))


def lib():
    """Load libedgpu.so (raises if it has not been built: there is no CPU fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libedgpu.so is not built (%s); run edlib_gb300.build.build()" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


class EdgpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("edgpu error %d: %s" % (code, msg))
        self.code = code


def dptr(a):
    return a.ctypes.data_as(_D)


def iptr(a):
    return a.ctypes.data_as(_I)
