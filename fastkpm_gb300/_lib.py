"""ctypes binding of include/fastkpm_gb300.h (the C ABI of libfastkpm_gb300.so).

The shared library is built in-tree by fastkpm_gb300/build.py. Loading fails
loudly when it is missing: there is no CPU fallback.
"""
import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libfastkpm_gb300.so")

FK_OK, FK_ERR_ARG, FK_ERR_OOM, FK_ERR_PATTERN, FK_ERR_TIMEOUT = 0, 1, 2, 3, 4
FK_ERR_CUDA, FK_ERR_STATE, FK_ERR_NODEV, FK_ERR_UNSUPPORTED = 5, 6, 7, 8
FK_REAL, FK_COMPLEX = 0, 1
FK_PREC_FP64, FK_PREC_FP32, FK_PREC_DS = 0, 1, 2
FK_KERNEL_STEP, FK_KERNEL_ADJOINT, FK_KERNEL_OUTER, FK_KERNEL_HELPER = 0, 1, 2, 3
FK_OPT_FUSE_D, FK_OPT_NP, FK_OPT_CTAS_PER_SM, FK_OPT_STAGE_H, FK_OPT_GRAPHS = 0, 1, 2, 3, 4
FK_OPT_NP_STEP, FK_OPT_NP_ADJOINT, FK_OPT_NP_OUTER, FK_OPT_TMA = 5, 6, 7, 8
FK_OPT_UPLOAD = 9
FK_OPT_PRIORITY = 10
FK_OPT_ADJ_SPLIT = 11
FK_OPT_PIPE = 12
FK_OPT_ACC64 = 13
FK_OPT_CTA_WAVES = 14
FK_OPT_WARP_ROWS = 15
FK_OPT_ADJ_SWEEP = 16

PRECISIONS = {"fp64": FK_PREC_FP64, "fp32": FK_PREC_FP32, "ds": FK_PREC_DS}

_p = C.c_void_p
_i = C.c_int
_d = C.c_double
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)

# name -> (restype, argtypes)
SIGNATURES = {
    "fk_version": (C.c_char_p, []),
    "fk_status_string": (C.c_char_p, [_i]),
    "fk_device_count": (_i, [_ip]),
    "fk_device_memory": (_i, [_i, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
    "fk_device_fma_rate": (_i, [_i, _i, _dp]),
    "fk_engine_create": (_i, [_i, _i, _i, C.POINTER(_p)]),
    "fk_engine_destroy": (_i, [_p]),
    "fk_engine_last_error": (C.c_char_p, [_p]),
    "fk_engine_set_stream": (_i, [_p, _p]),
    "fk_engine_synchronize": (_i, [_p]),
    "fk_engine_set_option": (_i, [_p, _i, _i]),
    "fk_engine_get_option": (_i, [_p, _i, _ip]),
    "fk_engine_set_H": (_i, [_p, _i, _i, _i, _ip, _ip, _dp, _d, _d]),
    "fk_engine_set_R": (_i, [_p, _i, _i, _dp]),
    "fk_engine_get_R": (_i, [_p, _dp]),
    "fk_engine_set_R_sparse": (_i, [_p, _i, _i, _i, _ip, _dp]),
    "fk_engine_moments": (_i, [_p, _i, _dp]),
    "fk_engine_moments_async": (_i, [_p, _i]),
    "fk_engine_fetch_moments": (_i, [_p, _dp]),
    "fk_engine_stoch_matrix": (_i, [_p, _i, _dp, _i, _i, _ip, _ip, _dp]),
    "fk_engine_autodiff_matrix": (_i, [_p, _i, _dp, _i, _i, _ip, _ip, _dp]),
    "fk_engine_stoch_matrix_async": (_i, [_p, _i, _dp, _i, _i, _ip, _ip]),
    "fk_engine_autodiff_matrix_async": (_i, [_p, _i, _dp, _i, _i, _ip, _ip]),
    "fk_engine_fetch_D": (_i, [_p, _dp]),
    "fk_engine_energy_scale": (_i, [_p, _i, _i, _i, _ip, _ip, _dp, _d, _i, _dp, _dp, _dp]),
    "fk_engine_expansion_coefficients": (_i, [_p, _i, _i, _i, _d, _d, _d, _d, _dp]),
    "fk_engine_kpm_filling": (_i, [_p, _i, _d, _d, _d, _dp, _dp]),
    "fk_engine_moments2_v1": (_i, [_p, _i, _i, _ip, _ip, _dp, _i, _ip, _ip, _dp, _i, _i, _dp]),
    "fk_engine_moments2_v2": (_i, [_p, _i, _i, _ip, _ip, _dp, _i, _ip, _ip, _dp, _dp, _dp]),
    "fk_engine_solve_filling": (_i, [_p, _i, _i, _d, _d, _d, _i, _i, _ip, _ip, _dp, _dp, _dp]),
    "fk_engine_set_profiling": (_i, [_p, _i]),
    "fk_engine_profile_read": (_i, [_p, _i, C.POINTER(C.c_longlong), _dp]),
    "fk_engine_profile_reset": (_i, [_p]),
    "fk_engine_memory": (_i, [_p, C.POINTER(C.c_size_t)]),
    "fk_engine_timer_start": (_i, [_p]),
    "fk_host_register": (_i, [_p, C.c_size_t]),
    "fk_host_unregister": (_i, [_p]),
    "fk_engine_timer_stop": (_i, [_p, _dp]),
    "fk_batch_create": (_i, [_i, _i, _i, C.POINTER(_p)]),
    "fk_batch_destroy": (_i, [_p]),
    "fk_batch_last_error": (C.c_char_p, [_p]),
    "fk_batch_add": (_i, [_p, _i, _i, _i, _ip, _ip, _dp, _d, _d, _i, _dp, _ip]),
    "fk_batch_commit": (_i, [_p]),
    "fk_batch_moments": (_i, [_p, _i, _dp]),
    "fk_batch_autodiff_matrix": (_i, [_p, _i, _dp, _dp]),
    "fk_batch_set_option": (_i, [_p, _i, _i]),
    "fk_batch_get_option": (_i, [_p, _i, _ip]),
    "fk_batch_autotune": (_i, [_p, _i, _ip, _ip, _ip, _ip, _dp]),
    "fk_batch_profile_moments": (_i, [_p, _i, _dp, _ip]),
    "fk_batch_timer_start": (_i, [_p]),
    "fk_batch_timer_stop": (_i, [_p, _dp]),
    "fk_batch_info": (_i, [_p, _ip, C.POINTER(C.c_longlong), C.POINTER(C.c_size_t)]),
    "fk_moments_noalloc": (_i, [_i, _i, _i, _p, _p, _p, C.c_longlong, _i, _p, _p, _i, _dp, _p]),
    "fk_bsr_build": (_i, [_i, _i, _i, _i, _ip, _ip, _dp, _ip, _ip, _ip, _dp, _ip]),
    "fk_bsr_symmetrize": (_i, [_i, _i, _i, _i, _ip, _ip, _ip, _dp]),
    "fk_probe_identity": (_i, [_i, _i, _i, _i, _dp]),
    "fk_probe_uncorrelated": (_i, [_i, _i, _i, C.c_uint32, C.c_ulonglong, _i, _i, _dp]),
    "fk_probe_correlated": (_i, [_i, _i, _ip, C.c_uint32, C.c_ulonglong, _i, _i, _dp]),
    "fk_jackson_kernel": (_i, [_i, _dp]),
    "fk_expansion_coefficients": (_i, [_i, _i, _i, _d, _d, _d, _d, _dp]),
}

_lib = None


def load(path=None):
    """Load libfastkpm_gb300.so (once) and attach the C signatures."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or os.environ.get("FKPM_LIB_PATH") or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(
            "libfastkpm_gb300.so is not built (%s); run `python -c 'import __graft_entry__ as g; g.build()'`"
            % path)
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class FkError(RuntimeError):
    def __init__(self, status, where, detail=""):
        self.status = status
        lib = load()
        msg = "%s: %s" % (where, lib.fk_status_string(status).decode())
        if detail:
            msg += " (%s)" % detail
        super().__init__(msg)
