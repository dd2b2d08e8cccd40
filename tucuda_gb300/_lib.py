"""ctypes binding of the C ABI declared in include/tucu_gb300.h.

The shared library is built in-tree (tucuda_gb300/lib/libtucu_gb300.so) by
``__graft_entry__.build()`` / ``make -C tucuda_gb300/csrc``.  There is no CPU
fallback: if the library is missing, importing the filters raises.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libtucu_gb300.so")

# tucu_dtype
U8, F16, BF16, F32, I32 = 0, 1, 2, 3, 4
# tucu_status
OK, NOOP = 0, 1
ERR_ARG, ERR_LOBE, ERR_WINDOW, ERR_DTYPE, ERR_CUDA = -1, -2, -3, -4, -5
ERR_NOMEM, ERR_BUDGET, ERR_TIMEOUT, ERR_STATE, ERR_CANCELLED = -6, -7, -8, -9, -10
# tucu_gauss_op
SMOOTH, DIFF_H, DIFF_V, DIFF_HH, DIFF_HV, DIFF_VV = range(6)
LOBE_MAX = 17
EXTREMA_MIN, EXTREMA_MAX = 0, 1

_c = ctypes
_vp, _sz, _i, _f, _u = _c.c_void_p, _c.c_size_t, _c.c_int, _c.c_float, _c.c_uint
_fp, _ip = _c.POINTER(_c.c_float), _c.POINTER(_c.c_int)
_h = _c.c_void_p

# name -> (restype, argtypes)
PROTOTYPES = {
    "tucu_version": (_i, []),
    "tucu_status_string": (_c.c_char_p, [_i]),
    "tucu_last_error": (_c.c_char_p, []),
    "tucu_device_error": (_i, [_ip]),
    "tucu_debug_tc_wait": (_i, [_c.c_ulonglong, _u]),
    "tucu_fir_create": (_i, [_c.POINTER(_h)]),
    "tucu_fir_initialize": (_i, [_h, _fp, _i, _fp, _i]),
    "tucu_fir_offsets": (_i, [_h, _ip, _ip]),
    "tucu_fir_convolve": (_i, [_h, _vp, _sz, _i, _i, _i, _vp, _sz, _i, _i, _vp]),
    "tucu_fir_destroy": (None, [_h]),
    "tucu_gauss_design": (_i, [_f, _fp, _ip, _fp, _ip, _fp, _ip]),
    "tucu_gauss_design_reference": (_i, [_f, _fp, _ip, _fp, _ip, _fp, _ip]),
    "tucu_gauss_set_reference_lobes": (_i, [_h, _i]),
    "tucu_gauss_create": (_i, [_f, _c.POINTER(_h)]),
    "tucu_gauss_initialize": (_i, [_h, _f]),
    "tucu_gauss_sigma": (_f, [_h]),
    "tucu_gauss_lobes": (_i, [_h, _fp, _ip, _fp, _ip, _fp, _ip]),
    "tucu_gauss_convolve": (_i, [_h, _i, _vp, _sz, _i, _i, _i, _vp, _sz, _i, _i, _vp]),
    "tucu_gauss_convolve_multi": (_i, [_h, _u, _vp, _sz, _i, _i, _i, _c.POINTER(_vp),
                                       _c.POINTER(_sz), _i, _i, _vp]),
    "tucu_gauss_offsets": (_i, [_h, _i, _ip, _ip]),
    "tucu_gauss_destroy": (None, [_h]),
    "tucu_box_create": (_i, [_i, _i, _i, _c.POINTER(_h)]),
    "tucu_box_set_window": (_i, [_h, _i, _i]),
    "tucu_box_offsets": (_i, [_h, _ip, _ip]),
    "tucu_box_convolve": (_i, [_h, _vp, _sz, _i, _i, _i, _vp, _sz, _i, _i, _i, _vp]),
    "tucu_box_convolve_vec": (_i, [_h, _vp, _sz, _i, _i, _i, _vp, _sz, _i, _i, _vp]),
    "tucu_box_stereo": (_i, [_h, _vp, _sz, _vp, _sz, _i, _i, _i, _f, _i, _vp, _sz, _sz, _i, _vp]),
    "tucu_box_destroy": (None, [_h]),
    "tucu_extrema_create": (_i, [_i, _i, _i, _c.POINTER(_h)]),
    "tucu_extrema_set_window": (_i, [_h, _i, _i]),
    "tucu_extrema_offsets": (_i, [_h, _ip, _ip]),
    "tucu_extrema_convolve": (_i, [_h, _i, _vp, _sz, _i, _i, _i, _vp, _sz, _vp, _sz, _i, _vp]),
    "tucu_extrema_destroy": (None, [_h]),
    "tucu_guided_create": (_i, [_i, _i, _f, _i, _c.POINTER(_h)]),
    "tucu_guided_set_window": (_i, [_h, _i, _i]),
    "tucu_guided_set_epsilon": (_i, [_h, _f]),
    "tucu_guided_epsilon": (_f, [_h]),
    "tucu_guided_offsets": (_i, [_h, _ip, _ip]),
    "tucu_guided_convolve": (_i, [_h, _vp, _sz, _vp, _sz, _i, _i, _i, _vp, _sz, _i, _i, _vp]),
    "tucu_guided_destroy": (None, [_h]),
    "tucu_guided_convolve_noalloc": (_i, [_i, _i, _f, _vp, _sz, _vp, _sz, _i, _i, _i, _vp, _sz,
                                         _i, _i, _vp]),
    "tucu_batch_create": (_i, [_c.POINTER(_h)]),
    "tucu_batch_add": (_i, [_h, _vp]),
    "tucu_batch_clear": (_i, [_h]),
    "tucu_batch_set_tensor_cores": (_i, [_h, _i]),
    "tucu_disparity_create": (_i, [_i, _i, _c.POINTER(_h)]),
    "tucu_disparity_select": (_i, [_h, _vp, _sz, _sz, _i, _i, _i, _i, _vp, _sz, _i, _i, _i, _vp]),
    "tucu_disparity_destroy": (None, [_h]),
    "tucu_fir_set_tensor_cores": (_i, [_h, _i]),
    "tucu_gauss_set_tensor_cores": (_i, [_h, _i]),
    "tucu_box_set_tensor_cores": (_i, [_h, _i]),
    "tucu_server_set_tensor_cores": (_i, [_h, _i]),
    "tucu_batch_plan": (_i, [_h, _i, _i]),
    "tucu_batch_launch": (_i, [_h, _vp]),
    "tucu_batch_graph_launch": (_i, [_h, _vp]),
    "tucu_batch_info": (_i, [_h, _ip, _ip, _ip, _c.POINTER(_sz)]),
    "tucu_batch_destroy": (None, [_h]),
    "tucu_pipe_create": (_i, [_i, _c.POINTER(_h)]),
    "tucu_pipe_set_flags": (_i, [_h, _i]),
    "tucu_pipe_add": (_i, [_h, _vp, _vp, _sz, _vp, _sz]),
    "tucu_pipe_plan": (_i, [_h, _i, _i]),
    "tucu_pipe_run": (_i, [_h, _vp]),
    "tucu_pipe_info": (_i, [_h, _ip, _ip, _ip, _c.POINTER(_sz), _c.POINTER(_sz)]),
    "tucu_pipe_destroy": (None, [_h]),
    "tucu_server_create": (_i, [_sz, _i, _i, _c.POINTER(_h)]),
    "tucu_server_submit": (_i, [_h, _vp, _c.POINTER(_c.c_uint64)]),
    "tucu_server_wait": (_i, [_h, _c.c_uint64, _c.c_double, _ip]),
    "tucu_server_cancel": (_i, [_h, _c.c_uint64]),
    "tucu_server_drain": (_i, [_h, _c.c_double]),
    "tucu_server_get_stats": (_i, [_h, _vp]),
    "tucu_server_destroy": (None, [_h]),
}

BATCH_GAUSS, BATCH_BOX = 0, 1
REQ_GAUSS, REQ_BOX, REQ_GUIDED = 0, 1, 2


class BatchJob(ctypes.Structure):
    """tucu_batch_job (include/tucu_gb300.h)."""
    _fields_ = [("op", _i), ("gauss_op", _i), ("sigma", _f), ("winV", _i), ("winH", _i),
                ("normalize", _i), ("in_", _vp), ("in_pitch", _sz), ("in_dtype", _i),
                ("out", _vp), ("out_pitch", _sz), ("out_dtype", _i), ("rows", _i), ("cols", _i),
                ("shift", _i)]

class Request(ctypes.Structure):
    """tucu_request (include/tucu_gb300.h)."""
    _fields_ = [("op", _i), ("sigma", _f), ("radius", _i), ("e", _f), ("normalize", _i),
                ("in_", _vp), ("in_pitch", _sz), ("guide", _vp), ("guide_pitch", _sz),
                ("in_dtype", _i), ("out", _vp), ("out_pitch", _sz), ("out_dtype", _i),
                ("rows", _i), ("cols", _i)]


class ServerStats(ctypes.Structure):
    """tucu_server_stats (include/tucu_gb300.h)."""
    _fields_ = [("submitted", _c.c_uint64), ("completed", _c.c_uint64),
                ("rejected", _c.c_uint64), ("cancelled", _c.c_uint64), ("failed", _c.c_uint64),
                ("p50_ms", _c.c_double), ("p99_ms", _c.c_double), ("max_ms", _c.c_double),
                ("gpix_per_s", _c.c_double), ("wall_s", _c.c_double), ("waves", _c.c_uint64),
                ("mean_wave_requests", _c.c_double), ("budget_bytes", _sz), ("peak_bytes", _sz)]


_lib = None


def load():
    """Loads the library once and declares every prototype.  Raises OSError
    when the library has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise OSError(f"{LIB_PATH} is missing: build it with __graft_entry__.build() "
                      "or `make -C tucuda_gb300/csrc`")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class TucuError(RuntimeError):
    """A C-ABI call returned a negative status (the reference throws
    std::runtime_error or exits in these cases)."""

    def __init__(self, status, msg):
        super().__init__(msg)
        self.status = status


def check(status, what=""):
    """Raises TucuError for a negative status; returns the status otherwise
    (OK or NOOP)."""
    if status < 0:
        lib = load()
        detail = lib.tucu_last_error().decode(errors="replace")
        name = lib.tucu_status_string(status).decode()
        raise TucuError(status, f"{what}: {name}" + (f" ({detail})" if detail else ""))
    return status
