"""Python wrapper of the CPU oracle (oracle/tucu_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as
the checker, and by bench.py's CPU-baseline leg.  Never on the product path.

Functions take and return numpy arrays.  Float results follow the
reference's arithmetic (see tucu_oracle.c); ``*_f64`` variants are the FP64
error oracle; ``box_i64`` gives exact integer window sums.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libtucu_oracle.so")
LOBE_MAX = 17

_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        fp, dp, ip = (ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_double),
                      ctypes.POINTER(ctypes.c_int))
        vp, lg, i, sz = ctypes.c_void_p, ctypes.c_long, ctypes.c_int, ctypes.c_size_t
        L.tuo_lobe_size.restype = sz
        L.tuo_lobe_size.argtypes = [fp, i]
        L.tuo_gauss_lobes.argtypes = [ctypes.c_float, fp, ip, fp, ip, fp, ip]
        L.tuo_gauss_lobes_f64.argtypes = [ctypes.c_float, dp, ip, dp, ip, dp, ip]
        L.tuo_fir_f32.argtypes = [vp, lg, i, i, fp, i, fp, i, vp, lg, i, i]
        L.tuo_fir_f64.argtypes = [vp, lg, i, i, dp, i, dp, i, vp, lg, i, i]
        L.tuo_box_i64.argtypes = [vp, lg, i, i, i, i, vp, lg, i, i]
        L.tuo_box_f32.argtypes = [vp, lg, i, i, i, i, vp, lg, i, i]
        L.tuo_box_pass_f32.argtypes = [vp, lg, i, i, i, vp, lg, i]
        L.tuo_fir_row_nvcc_f32.argtypes = [fp, i, fp, i, fp]
        L.tuo_box_f64.argtypes = [vp, lg, i, i, i, i, vp, lg, i, i]
        L.tuo_guided_f32.argtypes = [vp, lg, vp, lg, i, i, i, i, ctypes.c_float, vp, lg, i, i]
        L.tuo_guided_f64.argtypes = [vp, lg, vp, lg, i, i, i, i, ctypes.c_double, vp, lg, i, i]
        L.tuo_guided_coeffs.argtypes = [i, sz, ctypes.c_float, fp, fp, fp]
        L.tuo_guided_trans.restype = ctypes.c_float
        L.tuo_guided_trans.argtypes = [sz, ctypes.c_float, ctypes.c_float, ctypes.c_float]
        L.tuo_extrema.argtypes = [vp, lg, i, i, i, i, i, vp, lg, vp, lg, i, i]
        L.tuo_stereo.argtypes = [vp, vp, lg, i, i, i, i, ctypes.c_double, i, vp, i]
        L.tuo_select_disparity.argtypes = [vp, i, i, i, i, i, vp, i]
        L.tuo_max_threads.restype = i
        for name in ("tuo_fir_f32", "tuo_fir_f64", "tuo_box_i64", "tuo_box_f32", "tuo_box_f64",
                     "tuo_guided_f32", "tuo_guided_f64", "tuo_extrema", "tuo_stereo",
                     "tuo_select_disparity"):
            getattr(L, name).restype = i
        _lib = L
    return _lib


def max_threads():
    return lib().tuo_max_threads()


def _fptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


# ---- lobes --------------------------------------------------------------------

def lobe_size(lobe, even):
    lb = np.zeros(LOBE_MAX, np.float32)
    lb[:len(lobe)] = lobe
    return int(lib().tuo_lobe_size(_fptr(lb), int(bool(even))))


def gauss_lobes(sigma):
    """Reference-faithful float lobes (lobe0, lobe1, lobe2)."""
    bufs = [np.zeros(LOBE_MAX, np.float32) for _ in range(3)]
    ns = [ctypes.c_int() for _ in range(3)]
    lib().tuo_gauss_lobes(ctypes.c_float(sigma), _fptr(bufs[0]), ctypes.byref(ns[0]),
                          _fptr(bufs[1]), ctypes.byref(ns[1]), _fptr(bufs[2]), ctypes.byref(ns[2]))
    return [b[:n.value].copy() for b, n in zip(bufs, ns)]


def gauss_lobes_f64(sigma):
    bufs = [np.zeros(LOBE_MAX, np.float64) for _ in range(3)]
    ns = [ctypes.c_int() for _ in range(3)]
    lib().tuo_gauss_lobes_f64(ctypes.c_float(sigma), _dptr(bufs[0]), ctypes.byref(ns[0]),
                              _dptr(bufs[1]), ctypes.byref(ns[1]), _dptr(bufs[2]),
                              ctypes.byref(ns[2]))
    return [b[:n.value].copy() for b, n in zip(bufs, ns)]


GAUSS_OP_LOBES = [(0, 0), (1, 0), (0, 1), (2, 0), (1, 1), (0, 2)]  # (H lobe, V lobe)


# ---- FIR --------------------------------------------------------------------------

def fir_f32(img, lobeH, lobeV, shift=True, out=None, nthreads=0):
    """Returns (status, out); out defaults to zeros of img's shape (float32)."""
    a = _c(img, np.float32)
    rows, cols = a.shape
    out = np.zeros((rows, cols), np.float32) if out is None else out
    lh, lv = _c(lobeH, np.float32), _c(lobeV, np.float32)
    st = lib().tuo_fir_f32(a.ctypes.data, cols, rows, cols, _fptr(lh), len(lh), _fptr(lv),
                           len(lv), out.ctypes.data, out.shape[1], int(bool(shift)), nthreads)
    return st, out


def fir_row_nvcc_f32(row, lobe):
    """The reference's tap expression over one row in the order nvcc
    compiles it by default (tucu_oracle.c: tuo_fir_row_nvcc_f32): the
    row.size - 2*(L & ~1) outputs."""
    a = _c(row, np.float32)
    lb = _c(lobe, np.float32)
    out = np.zeros(a.size - 2 * (lb.size & ~1), np.float32)
    st = lib().tuo_fir_row_nvcc_f32(_fptr(a), a.size, _fptr(lb), lb.size, _fptr(out))
    if st != 0:
        raise ValueError(f"tuo_fir_row_nvcc_f32 failed ({st})")
    return out


def fir_f64(img, lobeH, lobeV, shift=True, out=None, nthreads=0):
    a = _c(img, np.float64)
    rows, cols = a.shape
    out = np.zeros((rows, cols), np.float64) if out is None else out
    lh, lv = _c(lobeH, np.float64), _c(lobeV, np.float64)
    st = lib().tuo_fir_f64(a.ctypes.data, cols, rows, cols, _dptr(lh), len(lh), _dptr(lv),
                           len(lv), out.ctypes.data, out.shape[1], int(bool(shift)), nthreads)
    return st, out


# ---- box --------------------------------------------------------------------------

def box_i64(img, wV, wH, shift=True, out=None, nthreads=0):
    a = _c(img, np.int32)
    rows, cols = a.shape
    out = np.zeros((rows, cols), np.int64) if out is None else out
    st = lib().tuo_box_i64(a.ctypes.data, cols, rows, cols, wV, wH, out.ctypes.data,
                           out.shape[1], int(bool(shift)), nthreads)
    return st, out


def box_f32(img, wV, wH, shift=True, out=None, nthreads=0):
    a = _c(img, np.float32)
    rows, cols = a.shape
    out = np.zeros((rows, cols), np.float32) if out is None else out
    st = lib().tuo_box_f32(a.ctypes.data, cols, rows, cols, wV, wH, out.ctypes.data,
                           out.shape[1], int(bool(shift)), nthreads)
    return st, out


def box_pass_f32(img, w, nthreads=0):
    """The vertical pass of box_f32 alone: (rows+1-w, cols) window sums of w
    rows in the reference's 16-row tiles (tucu_oracle.c: tuo_box_pass_f32)."""
    a = _c(img, np.float32)
    rows, cols = a.shape
    out_t = np.zeros((cols, rows + 1 - w), np.float32)
    st = lib().tuo_box_pass_f32(a.ctypes.data, cols, rows, cols, int(w), out_t.ctypes.data,
                                out_t.shape[1], nthreads)
    if st != 0:
        raise ValueError(f"tuo_box_pass_f32 failed ({st})")
    return out_t.T.copy()


def box_f64(img, wV, wH, shift=True, out=None, nthreads=0):
    a = _c(img, np.float64)
    rows, cols = a.shape
    out = np.zeros((rows, cols), np.float64) if out is None else out
    st = lib().tuo_box_f64(a.ctypes.data, cols, rows, cols, wV, wH, out.ctypes.data,
                           out.shape[1], int(bool(shift)), nthreads)
    return st, out


# ---- guided -------------------------------------------------------------------------

def guided_f32(p, g, wV, wH, e, shift=True, out=None, nthreads=0):
    a = _c(p, np.float32)
    rows, cols = a.shape
    gg = None if g is None else _c(g, np.float32)
    out = np.zeros((rows, cols), np.float32) if out is None else out
    st = lib().tuo_guided_f32(a.ctypes.data, cols, None if gg is None else gg.ctypes.data, cols,
                              rows, cols, wV, wH, ctypes.c_float(e), out.ctypes.data,
                              out.shape[1], int(bool(shift)), nthreads)
    return st, out


def guided_f64(p, g, wV, wH, e, shift=True, out=None, nthreads=0):
    a = _c(p, np.float64)
    rows, cols = a.shape
    gg = None if g is None else _c(g, np.float64)
    out = np.zeros((rows, cols), np.float64) if out is None else out
    st = lib().tuo_guided_f64(a.ctypes.data, cols, None if gg is None else gg.ctypes.data, cols,
                              rows, cols, wV, wH, ctypes.c_double(e), out.ctypes.data,
                              out.shape[1], int(bool(shift)), nthreads)
    return st, out


def guided_coeffs(self_guided, n, e, sums):
    s = np.zeros(4, np.float32)
    s[:len(sums)] = sums
    a, b = ctypes.c_float(), ctypes.c_float()
    lib().tuo_guided_coeffs(int(bool(self_guided)), n, ctypes.c_float(e), _fptr(s),
                            ctypes.byref(a), ctypes.byref(b))
    return np.float32(a.value), np.float32(b.value)


def guided_trans(n, A, B, g):
    return np.float32(lib().tuo_guided_trans(n, ctypes.c_float(A), ctypes.c_float(B),
                                             ctypes.c_float(g)))


# ---- storage conversions (the kernels' output rounding) -----------------------------

def to_u8(x):
    """float -> u8 as the reference's implicit float-to-u_char assignment runs
    on a GB300 (pinned by tests/test_oracle_ref_device.py against its own
    device code): truncate toward zero, saturate to the unsigned 32-bit range
    (negative values and NaN give 0), keep the low byte, so values from 256 on
    wrap modulo 256."""
    x = np.nan_to_num(np.asarray(x, np.float64), nan=0.0)
    t = np.clip(np.trunc(x), 0.0, 4294967295.0).astype(np.uint64)
    return (t & 0xFF).astype(np.uint8)


def to_f16(x):
    return np.asarray(x, np.float32).astype(np.float16)


def to_bf16_bits(x):
    """float32 -> bfloat16 bit patterns (uint16), round to nearest even."""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    nan = np.isnan(np.asarray(x, np.float32))
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    r[nan] = 0x7FC0
    return r


def bf16_bits_to_f32(b):
    return (np.asarray(b, np.uint16).astype(np.uint32) << 16).view(np.float32)


def round_to(x, dtype):
    """The value a float32 result takes when stored as `dtype`
    ('u8', 'f16', 'bf16', 'f32'), returned as float32."""
    if dtype == "u8":
        return to_u8(x).astype(np.float32)
    if dtype == "f16":
        return to_f16(x).astype(np.float32)
    if dtype == "bf16":
        return bf16_bits_to_f32(to_bf16_bits(x))
    return np.asarray(x, np.float32)


# ---- sliding-window extrema ---------------------------------------------------------

def extrema(img, wV, wH, is_max=False, shift=True, nthreads=0):
    """Window minima (or maxima) and their input positions, as the
    reference's extrema_finder deque passes give them (tucu_oracle.c:
    tuo_extrema).  Returns (values, positions): float64 (rows, cols) with NaN
    outside the valid region and int32 (rows, cols, 2) (x, y) pairs with -1
    outside it; None, None when the image is smaller than the window."""
    a = _c(img, np.float64)
    rows, cols = a.shape
    val = np.full((rows, cols), np.nan)
    pos = np.full((rows, cols, 2), -1, np.int32)
    rc = lib().tuo_extrema(a.ctypes.data, cols, rows, cols, int(wV), int(wH), int(bool(is_max)),
                           val.ctypes.data, cols, pos.ctypes.data, cols, int(bool(shift)),
                           int(nthreads))
    if rc == 1:
        return None, None
    if rc != 0:
        raise ValueError(f"tuo_extrema failed ({rc})")
    return val, pos


# ---- stereo cost aggregation ---------------------------------------------------------

def stereo(left, right, wV, wH, thresh, ndisp, nthreads=0):
    """Disparity-major window sums of min(|L - R(x+d)|, thresh) (tucu_oracle.c:
    tuo_stereo), float64 (ndisp, rows, cols) with NaN where nothing is
    written; None when the image is smaller than the window."""
    a = _c(left, np.float64)
    b = _c(right, np.float64)
    rows, cols = a.shape
    out = np.full((ndisp, rows, cols), np.nan)
    rc = lib().tuo_stereo(a.ctypes.data, b.ctypes.data, cols, rows, cols, int(wV), int(wH),
                          float(thresh), int(ndisp), out.ctypes.data, int(nthreads))
    if rc == 1:
        return None
    if rc != 0:
        raise ValueError(f"tuo_stereo failed ({rc})")
    return out


def select_disparity(costs, dmax, inc, nthreads=0):
    """DisparitySelector over a (D, rows, cols) cost volume (tucu_oracle.c:
    tuo_select_disparity): float64 (rows, cols) disparities, 0 where the
    left-right check fails."""
    c = _c(costs, np.float64)
    D, rows, cols = c.shape
    out = np.zeros((rows, cols), np.float64)
    rc = lib().tuo_select_disparity(c.ctypes.data, D, rows, cols, int(dmax), int(inc),
                                    out.ctypes.data, int(nthreads))
    if rc != 0:
        raise ValueError("bad cost volume")
    return out
