"""ctypes binding of libstonewall.so (the C ABI in include/stonewall.h).

There is no fallback: if the library is missing or cannot be loaded, every
call raises NativeUnavailable.  Run ``python -m stonewall.build`` (or
``__graft_entry__.build()``) first.
"""
import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libstonewall.so")

# status codes / dtypes / flags (include/stonewall.h)
SW_OK, SW_ERR_BAD_ARG, SW_ERR_OOM, SW_ERR_NONFINITE, SW_ERR_TIMEOUT, SW_ERR_CUDA, SW_ERR_UNSUPPORTED = range(7)
SW_ERR_TOO_LARGE = 7
SW_STATUS_NONFINITE, SW_STATUS_TIMEOUT = 1, 2
SW_F32, SW_F64, SW_F16_SHIFT, SW_BF16_SHIFT = range(4)
SW_NOISE_UNIFORM, SW_NOISE_GAUSSIAN = 0, 1
FORCE_SCALE = 2.0 ** 40

DTYPE_NAMES = {"f32": SW_F32, "fp32": SW_F32, "float32": SW_F32,
               "f64": SW_F64, "fp64": SW_F64, "float64": SW_F64,
               "f16": SW_F16_SHIFT, "fp16": SW_F16_SHIFT, "f16s": SW_F16_SHIFT,
               "bf16": SW_BF16_SHIFT, "bf16s": SW_BF16_SHIFT}
DTYPE_BYTES = {SW_F32: 4, SW_F64: 8, SW_F16_SHIFT: 2, SW_BF16_SHIFT: 2}


# Held while a CUDA graph is captured (the solver's chunks, the batch graphs) and by helper threads
# around their own GPU work (the solve server's mask packing), so that no other thread's
# allocations, copies or stream queries fall inside a capture and invalidate it.
CAPTURE_LOCK = threading.RLock()


class NativeUnavailable(RuntimeError):
    pass


class StonewallError(RuntimeError):
    def __init__(self, status, what, cuda_error=0):
        self.status, self.cuda_error = status, cuda_error
        msg = f"{what}: {_status_string(status)}"
        if status == SW_ERR_CUDA:
            msg += f" (cudaError {cuda_error})"
        super().__init__(msg)


class SwGeom(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32), ("pitch", ctypes.c_int32)]


_lib = None


def _status_string(status):
    try:
        return lib().sw_status_string(status).decode()
    except NativeUnavailable:
        return f"status {status}"


def lib():
    """The loaded library (loads it on first use)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise NativeUnavailable(f"{LIB_PATH} is not built; run `python -m stonewall.build` "
                                "(there is no CPU fallback)")
    _lib = load(LIB_PATH)
    return _lib


def load(path):
    """A CDLL of the library at path (the product library, or the bounds-checked build) with the
    argument and result types of every entry point set."""
    try:
        L = ctypes.CDLL(path)
    except OSError as e:
        raise NativeUnavailable(f"cannot load {path}: {e}") from e
    P, G = ctypes.c_void_p, ctypes.POINTER(SwGeom)
    i32, i64, f32, f64 = ctypes.c_int32, ctypes.c_int64, ctypes.c_float, ctypes.c_double
    sig = {
        "sw_version": ([], ctypes.c_char_p),
        "sw_status_string": ([ctypes.c_int], ctypes.c_char_p),
        "sw_last_cuda_error": ([], ctypes.c_int),
        "sw_geom_make": ([i32, i32, i32, G], ctypes.c_int),
        "sw_cells_padded": ([G], i64),
        "sw_lattice_elems": ([G], i64),
        "sw_tile_count": ([G], i64),
        "sw_dtype_size": ([ctypes.c_int], ctypes.c_size_t),
        "sw_pack_flag": ([G, P, P, P], ctypes.c_int),
        "sw_pack_f": ([G, ctypes.c_int, ctypes.c_int, P, P, P], ctypes.c_int),
        "sw_unpack_f": ([G, ctypes.c_int, ctypes.c_int, P, P, P], ctypes.c_int),
        "sw_unpack_u": ([G, P, P, P], ctypes.c_int),
        "sw_unpack_acc": ([G, P, P, P], ctypes.c_int),
        "sw_build_tiles": ([G, P, P, P], ctypes.c_int),
        "sw_init": ([G, ctypes.c_int, P, P, P, f32, i32, i32, P], ctypes.c_int),
        "sw_step": ([G, ctypes.c_int, P, P, P, P, P, f64, f64, i32, f64, P, i64, P], ctypes.c_int),
        "sw_step_accum": ([G, ctypes.c_int, P, P, P, P, P, f64, f64, i32, f64, P, i64, P, P], ctypes.c_int),
        "sw_step_cfg": ([G, ctypes.c_int, P, P, P, P, P, f64, f64, i32, f64, P, i64, P, ctypes.c_int, P],
                        ctypes.c_int),
        "sw_step_checked": ([G, ctypes.c_int, P, P, P, P, P, f64, f64, i32, f64, P, i64, P, ctypes.c_int, P, P],
                            ctypes.c_int),
        "sw_status_error": ([ctypes.c_uint32], ctypes.c_int),
        "sw_debug_tma_poll_limit": ([i32], i32),
        "sw_debug_aa_tma": ([i32], i32),
        "sw_step_config_count": ([], ctypes.c_int),
        "sw_set_step_config": ([ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "sw_get_step_config": ([ctypes.c_int], ctypes.c_int),
        "sw_set_step_config_accum": ([ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "sw_get_step_config_accum": ([ctypes.c_int], ctypes.c_int),
        "sw_aa_ghost_elems": ([G], i64),
        "sw_step_aa": ([G, ctypes.c_int, P, i32, P, P, P, f64, f64, i32, f64, P, i64, P, P, P, P], ctypes.c_int),
        "sw_macro": ([G, ctypes.c_int, P, P, P, P], ctypes.c_int),
        "sw_accum": ([G, P, P, P], ctypes.c_int),
        "sw_macro_accum": ([G, ctypes.c_int, P, P, P, P, P], ctypes.c_int),
        "sw_force_to_f64": ([P, P, i64, P], ctypes.c_int),
        "sw_coefficients": ([P, i64, i32, f64, f64, i32, P, P], ctypes.c_int),
        "sw_coef_stats": ([P, i64, i64, P, P], ctypes.c_int),
        "sw_recirc_scratch_bytes": ([G, i32, i32], i64),
        "sw_recirc_count": ([G, P, i64, P, i32, i32, f64, P, i64, P, P], ctypes.c_int),
        "sw_pack_box_bytes": ([i32, i32, i32], i64),
        "sw_pack_ellipsoids": ([P, i32, i32, i32, i32, i32, f64, P, P, P], ctypes.c_int),
        "sw_voxelize_stones": ([P, i32, i32, i32, i32, P, P, i32, P], ctypes.c_int),
        "sw_tma_timeouts": ([], i64),
        "sw_slice_xz": ([G, P, i32, P, P], ctypes.c_int),
        "sw_slice_xy": ([G, P, i32, P, P], ctypes.c_int),
        "sw_qcoarse": ([G, P, P, i32, i32, i32, i32, i32, P, P], ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes, fn.restype = args, res
    return L


def check(status, what):
    if status != SW_OK:
        raise StonewallError(status, what, lib().sw_last_cuda_error() if status == SW_ERR_CUDA else 0)


def geom(nx, ny, nz):
    g = SwGeom()
    check(lib().sw_geom_make(int(nx), int(ny), int(nz), ctypes.byref(g)), "sw_geom_make")
    return g


def dtype_code(dtype):
    if isinstance(dtype, int):
        if dtype not in DTYPE_BYTES:
            raise ValueError(f"unknown storage dtype {dtype}")
        return dtype
    try:
        return DTYPE_NAMES[str(dtype).lower()]
    except KeyError:
        raise ValueError(f"unknown storage dtype {dtype!r}; one of {sorted(DTYPE_NAMES)}") from None
