"""ctypes binding of libmsfem_gpu.so (C-ABI declared in include/msfem_gpu.h).

The structures below mirror include/msfem_gpu.h field by field.  The library
is loaded from this package's ``lib/`` folder (built by ``build.py``); a
missing library raises instead of falling back to anything else.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(_HERE, "lib")
LIB_PATH = os.path.join(LIB_DIR, "libmsfem_gpu.so")

# msfem_status_code
OK = 0
ERR_INVALID_ARG = -1
ERR_CUDA = -2
ERR_NO_DEVICE = -3
ERR_UNSUPPORTED = -4
ERR_OUT_OF_MEMORY = -5
ERR_NOT_CONVERGED = -6

# msfem_cell_status
CELL_CONVERGED = 0
CELL_MAXIT = 1
CELL_NAN = 2
CELL_BAD_INPUT = 3

# msfem_coef_kind
COEF_CONSTANT = 0
COEF_REFERENCE = 1
COEF_SINSIN = 2
COEF_FOURIER = 3
COEF_SPHERES = 4
COEF_TABULATED = 5

PREC_FP64 = 0
PREC_MIXED = 1
MEM_HOST = 0
MEM_DEVICE = 1
WARM_NONE = 0
WARM_USER = 1
WARM_SURROGATE = 2

# cudaStreamLegacy: the legacy default stream (a NULL stream selects the
# handle's own non-blocking stream in msfem_set_stream)
CUDA_STREAM_LEGACY = 1

MAX_N_2D = 32
MAX_N_3D = 24
NOALLOC_MAX_CELLS = 65536

_dp = ctypes.POINTER(ctypes.c_double)
_i32p = ctypes.POINTER(ctypes.c_int32)
_i64p = ctypes.POINTER(ctypes.c_int64)


class CoefDesc(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("ncomp", ctypes.c_int32),
        ("params", ctypes.c_double * 8),
        ("qp_values", ctypes.c_void_p),
        ("qp_offset", ctypes.c_void_p),
        ("modes", ctypes.c_void_p),
        ("n_modes", ctypes.c_int32),
        ("n_spheres", ctypes.c_int32),
        ("spheres", ctypes.c_void_p),
    ]


class BatchDesc(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int32),
        ("n_cells", ctypes.c_int32),
        ("n_fine", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("corners", ctypes.c_void_p),
        ("n_fine_per_cell", ctypes.c_void_p),
        ("coef", CoefDesc),
        ("f_value", ctypes.c_double),
        ("tol", ctypes.c_double),
        ("maxit", ctypes.c_int32),
        ("memory", ctypes.c_int32),
        ("warm_start", ctypes.c_int32),
        ("check_interval", ctypes.c_int32),
        ("warm_basis", ctypes.c_void_p),
        ("tol_absolute", ctypes.c_int32),
        ("reserved0", ctypes.c_int32),
        ("f_qp_values", ctypes.c_void_p),
        ("f_qp_offset", ctypes.c_void_p),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("solves", ctypes.c_int64),
        ("cells_converged", ctypes.c_int64),
        ("cells_failed", ctypes.c_int64),
        ("iterations_total", ctypes.c_int64),
        ("iterations_max", ctypes.c_int32),
        ("refinements_max", ctypes.c_int32),
        ("max_rel_residual", ctypes.c_double),
        ("kernel_ms", ctypes.c_double),
        ("total_ms", ctypes.c_double),
        ("kernel_launches", ctypes.c_int32),
        ("ctas_per_sm", ctypes.c_int32),
        ("h2d_bytes", ctypes.c_int64),
        ("d2h_bytes", ctypes.c_int64),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class Tuning(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int32),
        ("n_max", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("variant", ctypes.c_int32),
        ("threads", ctypes.c_int32),
        ("rows_per_thread", ctypes.c_int32),
        ("ctas_per_sm", ctypes.c_int32),
        ("check_interval", ctypes.c_int32),
        ("inner_tol", ctypes.c_float),
        ("n_variants", ctypes.c_int32),
        ("ms_per_solve", ctypes.c_double),
        ("cheb_ratio", ctypes.c_float),
        ("poly_degree", ctypes.c_int32),
        ("cluster_ctas", ctypes.c_int32),
        ("coarse_spacing", ctypes.c_int32),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


# Every entry point include/msfem_gpu.h declares: name -> (restype, argtypes)
EXPORTS = {
    "msfem_describe_tuning": (ctypes.c_int, [ctypes.POINTER(Tuning)]),
    "msfem_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int]),
    "msfem_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "msfem_set_stream": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "msfem_graph_info": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64),
                                        ctypes.POINTER(ctypes.c_int64)]),
    "msfem_run_batch": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BatchDesc),
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.POINTER(Stats)]),
    "msfem_energy_error": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BatchDesc),
                                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_void_p]),
    "msfem_reconstruct": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BatchDesc), ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_void_p]),
    "msfem_tabulate_coefficient": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BatchDesc),
                                                  ctypes.c_int32, ctypes.c_void_p]),
    "msfem_tabulated_size": (ctypes.c_int64, [ctypes.POINTER(BatchDesc), ctypes.c_int32]),
    "msfem_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BatchDesc), ctypes.c_int32,
                                      ctypes.POINTER(Tuning)]),
    "msfem_set_tuning": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Tuning)]),
    "msfem_run_batch_noalloc": (ctypes.c_int, [ctypes.POINTER(BatchDesc), ctypes.c_void_p,
                                               ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                               ctypes.c_void_p, ctypes.c_void_p]),
    "msfem_surrogate_param_count": (ctypes.c_int64, []),
    "msfem_surrogate_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64,
                                              ctypes.POINTER(ctypes.c_void_p)]),
    "msfem_surrogate_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "msfem_surrogate_set_params": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "msfem_surrogate_get_params": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "msfem_surrogate_features": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BatchDesc),
                                                ctypes.c_void_p]),
    "msfem_surrogate_targets": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                               ctypes.c_void_p]),
    "msfem_surrogate_predict": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                               ctypes.c_void_p]),
    "msfem_surrogate_gradients": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                 ctypes.c_int32, ctypes.c_void_p,
                                                 ctypes.POINTER(ctypes.c_double)]),
    "msfem_surrogate_train_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                  ctypes.c_int32, ctypes.c_float,
                                                  ctypes.POINTER(ctypes.c_double)]),
    "msfem_attach_surrogate": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "msfem_last_error": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t]),
    "msfem_version": (ctypes.c_char_p, []),
}

_lib = None


def load(path=None):
    """Load libmsfem_gpu.so and declare its signatures.  Raises OSError when
    the library has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise OSError(f"libmsfem_gpu.so not found at {p}: run build() first")
    lib = ctypes.CDLL(p)
    for name, (res, args) in EXPORTS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def last_error(lib=None):
    lib = lib or load()
    buf = ctypes.create_string_buffer(1024)
    lib.msfem_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


class MsfemError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"msfem error {code}: {msg}")
        self.code = code
