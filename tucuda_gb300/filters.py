"""The TU::cu filter classes over the C ABI, for torch CUDA tensors.

Same names, constructor arguments, geometry and error behaviour as the
reference's classes:

  FIRFilter2             TU/cu/FIRFilter.h:18-52
  FIRGaussianConvolver2  TU/cu/FIRGaussianConvolver.h:56-90
  BoxFilter2             TU/cu/BoxFilter.h:416-539 (box_convolver)
  GuidedFilter2          TU/cu/GuidedFilter.h:134-214

Images are 2D tensors (rows x cols, row stride may exceed cols) of uint8,
float16, bfloat16, float32 (or int32 for box input/output) on a CUDA device.
``convolve(inp, out, shift=True)`` writes only the valid region of ``out``;
the rest of ``out`` is left as it was, and an image smaller than the filter
support leaves ``out`` untouched, as in the reference.  Bad lobe or window
sizes raise TucuError (the reference throws std::runtime_error).  Work is
queued on torch's current stream.
"""
import ctypes

import torch

from . import _lib
from ._lib import check

_DT = {torch.uint8: _lib.U8, torch.float16: _lib.F16, torch.bfloat16: _lib.BF16,
       torch.float32: _lib.F32, torch.int32: _lib.I32}


def dtype_code(t):
    try:
        return _DT[t.dtype]
    except KeyError:
        raise _lib.TucuError(_lib.ERR_DTYPE, f"unsupported tensor dtype {t.dtype}") from None


def _view(t, what):
    """(pointer, pitch in bytes, rows, cols, dtype code) of a 2D CUDA tensor."""
    if not isinstance(t, torch.Tensor) or t.dim() != 2:
        raise _lib.TucuError(_lib.ERR_ARG, f"{what}: expected a 2D tensor")
    if not t.is_cuda:
        raise _lib.TucuError(_lib.ERR_ARG, f"{what}: tensor must be on a CUDA device")
    if t.stride(1) != 1 and t.size(1) > 1:
        raise _lib.TucuError(_lib.ERR_ARG, f"{what}: rows must be contiguous")
    pitch = t.stride(0) * t.element_size() if t.size(0) > 1 else t.size(1) * t.element_size()
    return ctypes.c_void_p(t.data_ptr()), pitch, t.size(0), t.size(1), dtype_code(t)


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _floats(seq):
    arr = (ctypes.c_float * max(1, len(seq)))(*[float(v) for v in seq])
    return arr, len(seq)


class FIRFilter2:
    """Separable FIR filter (TU/cu/FIRFilter.h:18-52).  Lobes are stored
    outermost tap first; lengths 3,5,9,17 are symmetric, 2,4,8,16
    antisymmetric."""

    LobeSizeMax = _lib.LOBE_MAX

    def __init__(self):
        self._lib = _lib.load()
        self._h = ctypes.c_void_p()
        check(self._lib.tucu_fir_create(ctypes.byref(self._h)), "FIRFilter2")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.tucu_fir_destroy(h)
            self._h = None

    def initialize(self, lobeH, lobeV):
        """FIRFilter2::initialize (TU/cu/FIRFilter.h:245-261)."""
        a, na = _floats(lobeH)
        b, nb = _floats(lobeV)
        check(self._lib.tucu_fir_initialize(self._h, a, na, b, nb), "FIRFilter2::initialize")
        return self

    def offsetV(self):
        v, h = ctypes.c_int(), ctypes.c_int()
        check(self._lib.tucu_fir_offsets(self._h, ctypes.byref(v), ctypes.byref(h)))
        return v.value

    def offsetH(self):
        v, h = ctypes.c_int(), ctypes.c_int()
        check(self._lib.tucu_fir_offsets(self._h, ctypes.byref(v), ctypes.byref(h)))
        return h.value

    def outSizeV(self, n):
        return n - 2 * self.offsetV()

    def outSizeH(self, n):
        return n - 2 * self.offsetH()

    def convolve(self, inp, out, shift=True):
        """FIRFilter2::convolve (TU/cu/FIRFilter.h:298-377).  Returns True when
        something was written (False: image smaller than the support)."""
        ip, ipitch, rows, cols, idt = _view(inp, "input")
        op, opitch, orows, ocols, odt = _view(out, "output")
        if (orows, ocols) != (rows, cols):
            raise _lib.TucuError(_lib.ERR_ARG, "output must have the input's shape")
        st = check(self._lib.tucu_fir_convolve(self._h, ip, ipitch, rows, cols, idt, op, opitch,
                                               odt, int(bool(shift)), _stream()),
                   "FIRFilter2::convolve")
        return st == _lib.OK

    def set_tensor_cores(self, on=True):
        """on: later calls with an f16 input (rows on 16-byte boundaries), an
        f16 or f32 output and at most 33 taps per direction run on the tensor
        cores, FP32-accurate but not bit-equal to the reference arithmetic."""
        check(self._lib.tucu_fir_set_tensor_cores(self._h, int(bool(on))), "tucu_fir_set_tensor_cores")
        return self


class FIRGaussianConvolver2:
    """Gaussian convolver with derivative operators
    (TU/cu/FIRGaussianConvolver.h:56-90)."""

    OPS = ("smooth", "diffH", "diffV", "diffHH", "diffHV", "diffVV")

    def __init__(self, sigma=1.0):
        self._lib = _lib.load()
        self._h = ctypes.c_void_p()
        check(self._lib.tucu_gauss_create(float(sigma), ctypes.byref(self._h)),
              "FIRGaussianConvolver2")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.tucu_gauss_destroy(h)
            self._h = None

    def sigma(self):
        return self._lib.tucu_gauss_sigma(self._h)

    def initialize(self, sigma):
        check(self._lib.tucu_gauss_initialize(self._h, float(sigma)),
              "FIRGaussianConvolver2::initialize")
        return self

    def set_reference_lobes(self, on=True):
        """on: lobes designed in the reference's own float arithmetic (equal
        to the reference's lobes bit for bit) instead of FP64-designed ones
        (tucu_gauss_set_reference_lobes)."""
        check(self._lib.tucu_gauss_set_reference_lobes(self._h, int(bool(on))),
              "FIRGaussianConvolver2::set_reference_lobes")
        return self

    @staticmethod
    def design(sigma, reference=False):
        """Static initialize(sigma, lobe0, lobe1, lobe2): the three lobes as
        lists of floats (outermost tap first); reference=True: designed in the
        reference's float arithmetic (tucu_gauss_design_reference)."""
        lib = _lib.load()
        bufs = [(ctypes.c_float * _lib.LOBE_MAX)() for _ in range(3)]
        ns = [ctypes.c_int() for _ in range(3)]
        fn = lib.tucu_gauss_design_reference if reference else lib.tucu_gauss_design
        check(fn(float(sigma), bufs[0], ctypes.byref(ns[0]), bufs[1], ctypes.byref(ns[1]), bufs[2],
                 ctypes.byref(ns[2])),
              "FIRGaussianConvolver2::initialize")
        return [list(b[:n.value]) for b, n in zip(bufs, ns)]

    def lobes(self):
        bufs = [(ctypes.c_float * _lib.LOBE_MAX)() for _ in range(3)]
        ns = [ctypes.c_int() for _ in range(3)]
        check(self._lib.tucu_gauss_lobes(self._h, bufs[0], ctypes.byref(ns[0]), bufs[1],
                                         ctypes.byref(ns[1]), bufs[2], ctypes.byref(ns[2])))
        return [list(b[:n.value]) for b, n in zip(bufs, ns)]

    def offsets(self, op):
        v, h = ctypes.c_int(), ctypes.c_int()
        check(self._lib.tucu_gauss_offsets(self._h, op, ctypes.byref(v), ctypes.byref(h)))
        return v.value, h.value

    def convolve(self, op, inp, out, shift=True):
        ip, ipitch, rows, cols, idt = _view(inp, "input")
        op_, opitch, orows, ocols, odt = _view(out, "output")
        if (orows, ocols) != (rows, cols):
            raise _lib.TucuError(_lib.ERR_ARG, "output must have the input's shape")
        st = check(self._lib.tucu_gauss_convolve(self._h, int(op), ip, ipitch, rows, cols, idt,
                                                 op_, opitch, odt, int(bool(shift)), _stream()),
                   f"FIRGaussianConvolver2::{self.OPS[op] if 0 <= op < 6 else op}")
        return st == _lib.OK

    def set_tensor_cores(self, on=True):
        """on: later calls with an f16 input (rows on 16-byte boundaries), an
        f16 or f32 output and at most 33 taps per direction run on the tensor
        cores, FP32-accurate but not bit-equal to the reference arithmetic."""
        check(self._lib.tucu_gauss_set_tensor_cores(self._h, int(bool(on))), "tucu_gauss_set_tensor_cores")
        return self

    def smooth(self, inp, out, shift=True):
        return self.convolve(_lib.SMOOTH, inp, out, shift)

    def diffH(self, inp, out, shift=True):
        return self.convolve(_lib.DIFF_H, inp, out, shift)

    def diffV(self, inp, out, shift=True):
        return self.convolve(_lib.DIFF_V, inp, out, shift)

    def diffHH(self, inp, out, shift=True):
        return self.convolve(_lib.DIFF_HH, inp, out, shift)

    def diffHV(self, inp, out, shift=True):
        return self.convolve(_lib.DIFF_HV, inp, out, shift)

    def diffVV(self, inp, out, shift=True):
        return self.convolve(_lib.DIFF_VV, inp, out, shift)

    def convolve_multi(self, inp, outs, shift=True):
        """Several operators in one pass.  ``outs`` maps operator index (or
        name) to an output tensor; all outputs share one dtype."""
        ip, ipitch, rows, cols, idt = _view(inp, "input")
        ptrs = (ctypes.c_void_p * 6)()
        pitches = (ctypes.c_size_t * 6)()
        mask, odt = 0, None
        for key, t in outs.items():
            k = self.OPS.index(key) if isinstance(key, str) else int(key)
            p, pitch, r, c, dt = _view(t, f"output {key}")
            if (r, c) != (rows, cols):
                raise _lib.TucuError(_lib.ERR_ARG, "outputs must have the input's shape")
            if odt is not None and dt != odt:
                raise _lib.TucuError(_lib.ERR_DTYPE, "outputs must share one dtype")
            odt = dt
            ptrs[k], pitches[k] = p, pitch
            mask |= 1 << k
        st = check(self._lib.tucu_gauss_convolve_multi(self._h, mask, ip, ipitch, rows, cols, idt,
                                                       ptrs, pitches, odt, int(bool(shift)),
                                                       _stream()),
                   "FIRGaussianConvolver2 multi")
        return st == _lib.OK


class BoxFilter2:
    """Running-sum box filter with box_convolver (TU/cu/BoxFilter.h:416-539).
    Writes window sums (int32 for integer input, FP32 for float input);
    ``normalize=True`` writes window means instead."""

    def __init__(self, winSizeV, winSizeH, wmax=23):
        self._lib = _lib.load()
        self._h = ctypes.c_void_p()
        check(self._lib.tucu_box_create(int(winSizeV), int(winSizeH), int(wmax),
                                        ctypes.byref(self._h)), "BoxFilter2")
        self._w = (int(winSizeV), int(winSizeH))
        self.WinSizeMax = wmax

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.tucu_box_destroy(h)
            self._h = None

    def winSizeV(self):
        return self._w[0]

    def winSizeH(self):
        return self._w[1]

    def setWinSizeV(self, w):
        check(self._lib.tucu_box_set_window(self._h, int(w), self._w[1]), "setWinSizeV")
        self._w = (int(w), self._w[1])
        return self

    def setWinSizeH(self, w):
        check(self._lib.tucu_box_set_window(self._h, self._w[0], int(w)), "setWinSizeH")
        self._w = (self._w[0], int(w))
        return self

    def outSizeV(self, n):
        return n + 1 - self._w[0]

    def outSizeH(self, n):
        return n + 1 - self._w[1]

    def offsetV(self):
        return self._w[0] // 2

    def offsetH(self):
        return self._w[1] // 2

    def convolve(self, inp, out, shift=True, normalize=False):
        ip, ipitch, rows, cols, idt = _view(inp, "input")
        op, opitch, orows, ocols, odt = _view(out, "output")
        if (orows, ocols) != (rows, cols):
            raise _lib.TucuError(_lib.ERR_ARG, "output must have the input's shape")
        st = check(self._lib.tucu_box_convolve(self._h, ip, ipitch, rows, cols, idt, op, opitch,
                                               odt, int(bool(shift)), int(bool(normalize)),
                                               _stream()), "BoxFilter2::convolve")
        return st == _lib.OK

    def set_tensor_cores(self, on=True):
        """on: later calls with an f16 input (rows on 16-byte boundaries), an
        f16 or f32 output and at most 33 taps per direction run on the tensor
        cores, FP32-accurate but not bit-equal to the reference arithmetic."""
        check(self._lib.tucu_box_set_tensor_cores(self._h, int(bool(on))), "tucu_box_set_tensor_cores")
        return self

    def convolve_vec(self, inp, out, shift=True, normalize=False):
        """Box sums of vector pixels (box_convolver<vec<float, N>>, the
        SuperPixels feature filter): ``inp`` and ``out`` are float32 CUDA
        tensors (rows, cols, N), N = 2, 3 or 4, channels contiguous; input rows
        16-byte aligned."""
        def view3(t, what):
            if (not isinstance(t, torch.Tensor) or not t.is_cuda or t.dim() != 3
                    or t.dtype != torch.float32 or t.stride(2) != 1 or t.stride(1) != t.shape[2]):
                raise _lib.TucuError(_lib.ERR_ARG, f"{what}: float32 CUDA tensor (rows, cols, N), pixels contiguous")
            return ctypes.c_void_p(t.data_ptr()), t.stride(0) * 4
        ip, ipitch = view3(inp, "input")
        op, opitch = view3(out, "output")
        if out.shape != inp.shape:
            raise _lib.TucuError(_lib.ERR_ARG, "output must have the input's shape")
        rows, cols, n = inp.shape
        st = check(self._lib.tucu_box_convolve_vec(self._h, ip, ipitch, rows, cols, n, op, opitch,
                                                   int(bool(shift)), int(bool(normalize)), _stream()),
                   "BoxFilter2::convolve (vector pixels)")
        return st == _lib.OK

    def convolve_stereo(self, left, right, costs, thresh):
        """Stereo cost aggregation (BoxFilter2::convolve(rowL, rowLe, rowR,
        rowO, diff<T>(thresh), D), TU/cu/BoxFilter.h:585-746), disparity-major:
        costs[d, y, x] = window sum at (y, x) of min(|L - R(x + d)|, thresh)
        for d < costs.shape[0].  ``costs``: (D, rows, cols) int32 for u8/int32
        images, float32 for float images."""
        lp, lpitch, rows, cols, dt = _view(left, "left")
        rp, rpitch, rr, rc, rdt = _view(right, "right")
        if (rr, rc) != (rows, cols) or rdt != dt:
            raise _lib.TucuError(_lib.ERR_ARG, "left and right images must match")
        if (not isinstance(costs, torch.Tensor) or not costs.is_cuda or costs.dim() != 3
                or tuple(costs.shape[1:]) != (rows, cols) or costs.stride(2) != 1):
            raise _lib.TucuError(_lib.ERR_ARG, "costs: CUDA tensor (D, rows, cols), rows contiguous")
        es = costs.element_size()
        st = check(self._lib.tucu_box_stereo(self._h, lp, lpitch, rp, rpitch, rows, cols, dt,
                                             float(thresh), costs.shape[0],
                                             ctypes.c_void_p(costs.data_ptr()), costs.stride(1) * es,
                                             costs.stride(0) * es, dtype_code(costs), _stream()),
                   "BoxFilter2::convolve (stereo)")
        return st == _lib.OK


class ExtremaFilter2(BoxFilter2):
    """Sliding-window minimum or maximum with the input position of each: the
    reference's BoxFilter2 with the extrema_finder convolver
    (TU/cu/BoxFilter.h:196-233) over extrema_value / extrema_position /
    extrema_value_position of less (``op="min"``) or greater (``op="max"``).
    Same window geometry as the box filter; among equal values the leftmost
    column wins, and in it the topmost row.  Windows up to 64."""

    OPS = ("min", "max")

    def __init__(self, winSizeV, winSizeH, wmax=23):
        self._lib = _lib.load()
        self._h = ctypes.c_void_p()
        check(self._lib.tucu_extrema_create(int(winSizeV), int(winSizeH), int(wmax),
                                            ctypes.byref(self._h)), "ExtremaFilter2")
        self._w = (int(winSizeV), int(winSizeH))
        self.WinSizeMax = wmax

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.tucu_extrema_destroy(h)
            self._h = None

    def setWinSizeV(self, w):
        check(self._lib.tucu_extrema_set_window(self._h, int(w), self._w[1]), "setWinSizeV")
        self._w = (int(w), self._w[1])
        return self

    def setWinSizeH(self, w):
        check(self._lib.tucu_extrema_set_window(self._h, self._w[0], int(w)), "setWinSizeH")
        self._w = (self._w[0], int(w))
        return self

    def convolve(self, inp, out=None, pos=None, shift=True, op="min"):
        """``out``: window extrema (the input's dtype and shape); ``pos``: int32
        tensor (rows, cols, 2) of (x, y) input positions.  Either may be None,
        not both."""
        ip, ipitch, rows, cols, idt = _view(inp, "input")
        vp, vpitch = None, 0
        if out is not None:
            vp, vpitch, orows, ocols, odt = _view(out, "values")
            if (orows, ocols) != (rows, cols) or odt != idt:
                raise _lib.TucuError(_lib.ERR_ARG, "values must have the input's shape and dtype")
        pp, ppitch = None, 0
        if pos is not None:
            if (not isinstance(pos, torch.Tensor) or not pos.is_cuda or pos.dtype != torch.int32
                    or tuple(pos.shape) != (rows, cols, 2) or pos.stride(2) != 1 or pos.stride(1) != 2):
                raise _lib.TucuError(_lib.ERR_ARG, "positions: int32 CUDA tensor (rows, cols, 2)")
            pp, ppitch = ctypes.c_void_p(pos.data_ptr()), pos.stride(0) * 4
        st = check(self._lib.tucu_extrema_convolve(self._h, self.OPS.index(op), ip, ipitch, rows,
                                                   cols, idt, vp, vpitch, pp, ppitch,
                                                   int(bool(shift)), _stream()),
                   "ExtremaFilter2::convolve")
        return st == _lib.OK


class GuidedFilter2:
    """Guided filter built on box sums (TU/cu/GuidedFilter.h:134-214).  ``e``
    is squared internally, as in the reference."""

    def __init__(self, wrow, wcol, e, wmax=23):
        self._lib = _lib.load()
        self._h = ctypes.c_void_p()
        check(self._lib.tucu_guided_create(int(wrow), int(wcol), float(e), int(wmax),
                                           ctypes.byref(self._h)), "GuidedFilter2")
        self._w = (int(wrow), int(wcol))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.tucu_guided_destroy(h)
            self._h = None

    def winSizeV(self):
        return self._w[0]

    def winSizeH(self):
        return self._w[1]

    def setWinSizeV(self, w):
        check(self._lib.tucu_guided_set_window(self._h, int(w), self._w[1]), "setWinSizeV")
        self._w = (int(w), self._w[1])
        return self

    def setWinSizeH(self, w):
        check(self._lib.tucu_guided_set_window(self._h, self._w[0], int(w)), "setWinSizeH")
        self._w = (self._w[0], int(w))
        return self

    def epsilon(self):
        return self._lib.tucu_guided_epsilon(self._h)

    def setEpsilon(self, e):
        check(self._lib.tucu_guided_set_epsilon(self._h, float(e)), "setEpsilon")
        return self

    def offsetV(self):
        return self._w[0] - 1

    def offsetH(self):
        return self._w[1] - 1

    def outSizeV(self, n):
        return n - 2 * self.offsetV()

    def outSizeH(self, n):
        return n - 2 * self.offsetH()

    def convolve(self, inp, guide, out, shift=True):
        """convolve(ib, ie, gb, ge, out, shift); guide=None selects the
        self-guided overload (TU/cu/GuidedFilter.h:292-344)."""
        ip, ipitch, rows, cols, idt = _view(inp, "input")
        if guide is not None:
            gp, gpitch, gr, gc, gdt = _view(guide, "guide")
            if (gr, gc) != (rows, cols) or gdt != idt:
                raise _lib.TucuError(_lib.ERR_ARG, "guide must match the input's shape and dtype")
        else:
            gp, gpitch = ctypes.c_void_p(0), 0
        op, opitch, orows, ocols, odt = _view(out, "output")
        if (orows, ocols) != (rows, cols):
            raise _lib.TucuError(_lib.ERR_ARG, "output must have the input's shape")
        st = check(self._lib.tucu_guided_convolve(self._h, ip, ipitch, gp, gpitch, rows, cols, idt,
                                                  op, opitch, odt, int(bool(shift)), _stream()),
                   "GuidedFilter2::convolve")
        return st == _lib.OK


class DisparitySelector:
    """TU::cu::DisparitySelector (TU/cu/StereoUtility.h:109-217): winner-take-all
    disparities of a disparity-major cost volume with the left-right
    consistency check (tucu_disparity_select)."""

    def __init__(self, disparity_max, disparity_inconsistency):
        self._lib = _lib.load()
        self._h = ctypes.c_void_p()
        check(self._lib.tucu_disparity_create(int(disparity_max), int(disparity_inconsistency),
                                              ctypes.byref(self._h)), "DisparitySelector")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.tucu_disparity_destroy(h)
            self._h = None

    def select(self, costs, out, rows=None, cols=None, oy=0, ox=0):
        """costs: a (D, H, W) CUDA tensor of int32 or float32 costs (contiguous
        rows; slices rows apart); the rows x cols region at its top left (by
        default all of it) is selected over and written to out at (oy, ox)."""
        import torch
        if costs.dim() != 3 or not costs.is_cuda or costs.stride(2) != 1:
            raise _lib.TucuError(_lib.ERR_ARG, "costs: a 3D CUDA tensor with contiguous rows")
        dt = {torch.int32: _lib.I32, torch.float32: _lib.F32}.get(costs.dtype)
        if dt is None:
            raise _lib.TucuError(_lib.ERR_DTYPE, "costs are int32 or float32")
        D, H, W = costs.shape
        rows = H if rows is None else int(rows)
        cols = W if cols is None else int(cols)
        es = costs.element_size()
        op, opitch, orows, ocols, odt = _view(out, "disparity image")
        if rows > H or cols > W or orows < rows + int(oy) or ocols < cols + int(ox):
            raise _lib.TucuError(_lib.ERR_ARG, "region larger than the costs or the disparity image")
        st = check(self._lib.tucu_disparity_select(
            self._h, ctypes.c_void_p(costs.data_ptr()), costs.stride(1) * es, costs.stride(0) * es,
            D, rows, cols, dt, op, opitch, odt, int(oy), int(ox), _stream()), "DisparitySelector::select")
        return st == _lib.OK
