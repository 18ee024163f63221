"""ctypes binding of the in-tree CUDA library ``libshenfun_gb300.so``.

The library is the product's only compute path: there is no CPU fallback.
Importing the package does not need a GPU, but any call that would compute
raises ``SgpuError`` when the library or a CUDA device is missing.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libshenfun_gb300.so")

# status codes (include/shenfun_gb300.h)
OK, ERR_ARG, ERR_UNSUPPORTED, ERR_CUDA, ERR_NOMEM, ERR_NONFINITE, ERR_ZERO_PIVOT, ERR_TIMEOUT, \
    ERR_SCRATCH_LIMIT = range(9)
REAL, COMPLEX = 0, 1
BASIS_ORTHO, BASIS_SD, BASIS_SB, BASIS_SN = 0, 1, 2, 3
BASIS_BC = 0x10  # flag: non-homogeneous boundary values
XF_R2C, XF_C2R, XF_C2C_FWD, XF_C2C_BWD, XF_DCT2, XF_DCT3, XF_CHEB_SCALAR, XF_CHEB_FORWARD, \
    XF_CHEB_BACKWARD = range(1, 10)
PLAIN_F64, MIXED_DF, FP32_REFINED = 0, 1, 2
FORMS = {"plain": PLAIN_F64, "mixed": MIXED_DF, PLAIN_F64: PLAIN_F64, MIXED_DF: MIXED_DF}


class SgpuError(RuntimeError):
    def __init__(self, status, where=""):
        self.status = status
        msg = _status_string(status)
        super().__init__(f"{where}: {msg} (status {status})" if where else msg)


_lib = None

_i64 = ctypes.c_int64
_int = ctypes.c_int
_vp = ctypes.c_void_p
_dbl = ctypes.c_double

# name: (restype, argtypes)
SIGNATURES = {
    "sgpu_status_string": (ctypes.c_char_p, [_int]),
    "sgpu_version": (_int, []),
    "sgpu_device_ok": (_int, []),
    "sgpu_plan_create": (_int, [ctypes.POINTER(_vp), _int, _int, _int, _int]),
    "sgpu_plan_destroy": (_int, [_vp]),
    "sgpu_plan_execute": (_int, [_vp, _vp, _vp, _i64, _i64, _int, _dbl, _vp]),
    "sgpu_plan_workspace_size": (_int, [_vp, _i64, _i64, _int, ctypes.POINTER(ctypes.c_size_t)]),
    "sgpu_plan_execute_ws": (_int, [_vp, _vp, _vp, _i64, _i64, _int, _dbl, _vp, ctypes.c_size_t, _vp]),
    "sgpu_plan_set_variant": (_int, [_vp, _int]),
    "sgpu_plan_execute_blocks": (_int, [_vp, _vp, _vp, _i64, _i64, _int, _dbl, _vp, ctypes.c_size_t, _i64, _vp]),
    "sgpu_last_error": (_int, [_vp]),
    "sgpu_helmholtz_solve_refined": (_int, [_vp, _vp, _vp, _vp, _vp, _vp, _i64, _i64, _i64, _int, _dbl, _int, _int,
                                            _vp, _vp]),
    "sgpu_band_sep_factor32": (_int, [_int, _int, _int, _vp, _vp, _vp, _i64, _vp, _vp]),
    "sgpu_band_sep_solve_refined": (_int, [_vp, _vp, _vp, _vp, _int, _int, _int, _vp, _vp, _vp, _i64, _i64, _i64,
                                           _int, _dbl, _int, _vp, _vp]),
    "sgpu_set_wait_limit_ns": (_int, [ctypes.c_ulonglong]),
    "sgpu_plan_get_variant": (_int, [_vp, ctypes.POINTER(_int)]),
    "sgpu_fourier_pad": (_int, [_vp, _vp, _i64, _int, _int, _i64, _int, _vp]),
    "sgpu_fourier_truncate": (_int, [_vp, _vp, _i64, _int, _int, _i64, _int, _vp]),
    "sgpu_banded_LU": (_int, [_vp, _int, _vp, _i64, _vp]),
    "sgpu_banded_Solve": (_int, [_vp, _vp, _int, _vp, _i64, _i64, _i64, _int, _vp]),
    "sgpu_TDMA_LU": (_int, [_vp, _i64, _vp]),
    "sgpu_TDMA_Solve": (_int, [_vp, _vp, _i64, _i64, _i64, _int, _vp]),
    "sgpu_PDMA_LU": (_int, [_vp, _i64, _vp]),
    "sgpu_PDMA_Solve": (_int, [_vp, _vp, _i64, _i64, _i64, _int, _vp]),
    "sgpu_LU_Helmholtz": (_int, [_i64, _vp, _vp, _int, _vp, _vp, _vp, _vp, _i64, _i64, _vp]),
    "sgpu_Solve_Helmholtz": (_int, [_vp, _vp, _int, _vp, _vp, _vp, _vp, _i64, _i64, _i64, _int, _vp]),
    "sgpu_Helmholtz_matvec": (_int, [_vp, _vp, _vp, _vp, _i64, _i64, _i64, _int, _vp]),
    "sgpu_Helmholtz_Neumann_matvec": (_int, [_vp, _vp, _vp, _vp, _i64, _i64, _i64, _int, _vp]),
    "sgpu_bc_apply": (_int, [_vp, _vp, _vp, _vp, _vp, _vp, _i64, _i64, _i64, _int, _int, _vp]),
    "sgpu_Poisson_Solve_ADD": (_int, [_vp, _vp, _dbl, _i64, _i64, _i64, _int, _vp]),
    "sgpu_Poisson_Solve_ANN": (_int, [_vp, _vp, _dbl, _dbl, _i64, _i64, _i64, _int, _vp]),
    "sgpu_helmholtz_factor": (_int, [_i64, _vp, _vp, _int, _i64, _i64, _int, _vp, _vp]),
    "sgpu_helmholtz_solve_cached": (_int, [_vp, _vp, _vp, _int, _i64, _i64, _i64, _int, _int, _vp]),
    "sgpu_band_sep_factor": (_int, [_int, _int, _int, _vp, _vp, _vp, _i64, _vp, _vp]),
    "sgpu_band_sep_matvec": (_int, [_vp, _vp, _int, _int, _int, _vp, _vp, _vp, _i64, _i64, _i64, _int, _vp]),
    "sgpu_band_sep_solve": (_int, [_vp, _vp, _vp, _vp, _int, _i64, _i64, _i64, _int, _vp]),
    "sgpu_helmholtz_create": (_int, [ctypes.POINTER(_vp), _int, _vp, _int, _dbl, _int]),
    "sgpu_helmholtz_create_on": (_int, [ctypes.POINTER(_vp), _int, _vp, _int, _dbl, _int, _vp]),
    "sgpu_plan_cache_clear": (_int, []),
    "sgpu_helmholtz_destroy": (_int, [_vp]),
    "sgpu_helmholtz_shape": (_int, [_vp, _vp, _vp]),
    "sgpu_helmholtz_workspace_size": (_int, [_vp, ctypes.POINTER(ctypes.c_size_t)]),
    "sgpu_helmholtz_solve": (_int, [_vp, _vp, _vp, _vp, ctypes.c_size_t, _vp]),
    "sgpu_helmholtz_solve_noalloc": (_int, [_vp, _vp, _vp, _vp]),
    "sgpu_leggauss": (_int, [_int, _vp, _vp]),
    "sgpu_legendre_plan_create": (_int, [ctypes.POINTER(_vp), _int, _int, _int]),
    "sgpu_legendre_plan_destroy": (_int, [_vp]),
    "sgpu_legendre_nodes": (_int, [_vp, _vp, _vp]),
    "sgpu_legendre_execute": (_int, [_vp, _int, _vp, _vp, _i64, _i64, _int, _vp]),
    "sgpu_legendre_workspace_size": (_int, [_vp, _i64, _i64, _int, ctypes.POINTER(ctypes.c_size_t)]),
    "sgpu_legendre_execute_ws": (_int, [_vp, _int, _vp, _vp, _i64, _i64, _int, _vp, ctypes.c_size_t, _vp]),
    "sgpu_wait_timeouts": (_int, [ctypes.POINTER(ctypes.c_uint)]),
    "sgpu_LU_Biharmonic": (_int, [_dbl] + [_vp] * 18 + [_i64, _i64, _i64, _vp]),
    "sgpu_Biharmonic_factor_pr": (_int, [_vp] * 4 + [_i64, _i64, _i64, _vp]),
    "sgpu_Biharmonic_Solve": (_int, [_vp] * 9 + [_dbl, _i64, _i64, _i64, _i64, _int, _vp]),
    "sgpu_Biharmonic_matvec": (_int, [_vp, _vp, _dbl] + [_vp] * 13 + [_i64, _i64, _i64, _i64, _int, _vp]),
    "sgpu_SolverGeneric1ND_solve_data": (_int, [_vp, _vp, _int, _int, _i64, _i64, _i64, _i64, _i64, _int, _vp]),
    "sgpu_DMA_Solve": (_int, [_int, _vp, _vp, _i64, _i64, _i64, _i64, _i64, _int, _vp]),
    "sgpu_helmholtz_batch_workspace_size": (_int, [_vp, _int, ctypes.POINTER(ctypes.c_size_t)]),
    "sgpu_helmholtz_factor_ptr": (_int, [_vp, ctypes.POINTER(_vp)]),
    "sgpu_helmholtz_plan_handles": (_int, [_vp, _vp, _vp]),
    "sgpu_helmholtz_solve_batch": (_int, [_vp, _int, _vp, _vp, _vp, _vp, ctypes.c_size_t, _vp]),
    "sgpu_helmholtz_solve_cached_batch": (_int, [_vp, _vp, _vp, _int, _int, _i64, _i64, _i64, _int, _int, _vp]),
    "sgpu_band_sep_solve_batch": (_int, [_vp, _vp, _vp, _vp, _int, _int, _i64, _i64, _i64, _int, _vp]),
    "sgpu_line_gemm": (_int, [_vp, _vp, _vp, _i64, _i64, _i64, _i64, _int, _vp, _int, _vp]),
    "sgpu_scalar_product": (_int, [_vp] * 5 + [_int, _i64, _i64, _i64, _i64, _int, _vp, ctypes.c_size_t, _vp]),
    "sgpu_evaluate_expansion_all": (_int, [_vp] * 4 + [_int, _i64, _i64, _i64, _i64, _i64, _int, _vp,
                                                       ctypes.c_size_t, _vp]),
}


def _status_string(status):
    if _lib is not None:
        return _lib.sgpu_status_string(status).decode()
    return f"status {status}"


def load(path=LIB_PATH):
    """Load the library (once) and declare every exported signature."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise SgpuError(ERR_UNSUPPORTED,
                        f"CUDA library not built ({path}); run shenfun_gb300.build.build()")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def call(name, *args):
    """Call an entry point and raise on a non-zero status."""
    lib = load()
    st = getattr(lib, name)(*args)
    if st != OK:
        raise SgpuError(st, name)
    return st


def check_device(stream=None):
    """Synchronise `stream` (a torch stream or None for the current one) and
    raise SgpuError(ERR_TIMEOUT) when a tensor-core launch since the last
    check gave up a bounded wait (its outputs are invalid)."""
    from .device import stream_handle
    call("sgpu_last_error", stream_handle(stream))
