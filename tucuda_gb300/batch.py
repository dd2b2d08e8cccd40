"""Batched launch over many images (tucu_batch_* of the C ABI).

    b = Batch()
    b.add_gauss(src, dst, sigma=2.0)            # smooth (or op=DIFF_H, ...)
    b.add_box(src2, dst2, 15, 15, normalize=True)
    b.plan()                                    # or b.plan(fir_rows, box_rows)
    b.launch()                                  # one CUDA-graph launch (a kernel per class)

Every output equals the single-image call of the same filter.  The tensors
must stay alive (and at the same addresses) until the batch is re-planned.

HostBatch (tucu_pipe_*) runs the same jobs on host images: each run copies
the inputs in, filters and copies the valid outputs back, in groups whose
copies overlap the filtering of other groups.

    hb = HostBatch(chunks=8)
    hb.add_gauss(host_src, dev_src, host_dst, dev_dst, sigma=2.0)   # pinned CPU + CUDA tensors
    hb.plan()
    hb.run()                                    # ordered on the current stream
"""
import ctypes

import torch

from . import _lib
from ._lib import check
from .filters import _stream, _view


class Batch:
    """tensor=True runs the jobs with f16 inputs (f16 or f32 outputs, at most
    33 taps per direction) on the tensor cores: FP32 accumulation of f16 hi/lo
    products, within a few FP32 ulps of the exact path instead of bit-equal
    to it (tucu_batch_set_tensor_cores)."""

    def __init__(self, tensor=False):
        self._lib = _lib.load()
        self._h = ctypes.c_void_p()
        check(self._lib.tucu_batch_create(ctypes.byref(self._h)), "tucu_batch_create")
        if tensor:
            check(self._lib.tucu_batch_set_tensor_cores(self._h, 1), "tucu_batch_set_tensor_cores")
        self._keep = []
        self.pixels = 0
        self.bytes = 0

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.tucu_batch_destroy(h)
            self._h = None

    def _add(self, job, src, dst):
        idx = check(self._lib.tucu_batch_add(self._h, ctypes.byref(job)), "tucu_batch_add")
        self._keep += [src, dst]
        self.pixels += job.rows * job.cols
        self.bytes += job.rows * job.cols * (src.element_size() + dst.element_size())
        return idx

    @staticmethod
    def _job(src, dst, shift):
        ip, ipitch, rows, cols, idt = _view(src, "input")
        op, opitch, orows, ocols, odt = _view(dst, "output")
        if (rows, cols) != (orows, ocols):
            raise _lib.TucuError(_lib.ERR_ARG, "output must have the input's shape")
        j = _lib.BatchJob()
        j.in_, j.in_pitch, j.in_dtype = ip.value, ipitch, idt
        j.out, j.out_pitch, j.out_dtype = op.value, opitch, odt
        j.rows, j.cols, j.shift = rows, cols, int(bool(shift))
        return j

    def add_gauss(self, src, dst, sigma, op=_lib.SMOOTH, shift=True):
        j = self._job(src, dst, shift)
        j.op, j.gauss_op, j.sigma = _lib.BATCH_GAUSS, int(op), float(sigma)
        return self._add(j, src, dst)

    def add_box(self, src, dst, winV, winH, normalize=False, shift=True):
        j = self._job(src, dst, shift)
        j.op, j.winV, j.winH, j.normalize = _lib.BATCH_BOX, int(winV), int(winH), int(bool(normalize))
        return self._add(j, src, dst)

    def clear(self):
        check(self._lib.tucu_batch_clear(self._h), "tucu_batch_clear")
        self._keep = []
        self.pixels = self.bytes = 0

    def plan(self, fir_rows=0, box_rows=0):
        check(self._lib.tucu_batch_plan(self._h, int(fir_rows), int(box_rows)), "tucu_batch_plan")
        return self

    def launch(self, graph=True):
        fn = self._lib.tucu_batch_graph_launch if graph else self._lib.tucu_batch_launch
        return check(fn(self._h, _stream()), "tucu_batch_launch")

    def info(self):
        nj, ni, g = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        sm = ctypes.c_size_t()
        check(self._lib.tucu_batch_info(self._h, ctypes.byref(nj), ctypes.byref(ni),
                                        ctypes.byref(g), ctypes.byref(sm)))
        return {"jobs": nj.value, "items": ni.value, "kernels": g.value, "smem": sm.value}


class HostBatch:
    """A batch on host images (tucu_pipe_*): every job has a host input and
    output (CPU tensors, page-locked for speed) and the device buffers of the
    same shapes the filters run on."""

    SPANS = 1   # TUCU_PIPE_SPANS
    TENSOR = 2  # TUCU_PIPE_TENSOR

    def __init__(self, chunks=8, spans=False, tensor=False):
        """spans=True: the host images mirror the device layout, and each
        group's images move as one byte range per direction (the bytes
        between images too; see tucu_pipe_set_flags).  tensor=True: the
        groups run as Batch(tensor=True)."""
        self._lib = _lib.load()
        self._h = ctypes.c_void_p()
        check(self._lib.tucu_pipe_create(int(chunks), ctypes.byref(self._h)), "tucu_pipe_create")
        flags = (self.SPANS if spans else 0) | (self.TENSOR if tensor else 0)
        if flags:
            check(self._lib.tucu_pipe_set_flags(self._h, flags), "tucu_pipe_set_flags")
        self._keep = []
        self.pixels = 0

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.tucu_pipe_destroy(h)
            self._h = None

    @staticmethod
    def _host(t, what):
        if t.is_cuda or t.dim() != 2 or t.stride(1) != 1:
            raise _lib.TucuError(_lib.ERR_ARG, f"{what}: 2D CPU tensor with contiguous rows")
        return t.data_ptr(), t.stride(0) * t.element_size()

    def _add(self, j, host_src, dev_src, host_dst, dev_dst):
        if host_src.shape != dev_src.shape or host_dst.shape != dev_dst.shape:
            raise _lib.TucuError(_lib.ERR_ARG, "host and device images must have equal shapes")
        hi, hip = self._host(host_src, "host input")
        ho, hop = self._host(host_dst, "host output")
        idx = check(self._lib.tucu_pipe_add(self._h, ctypes.byref(j), hi, hip, ho, hop),
                    "tucu_pipe_add")
        self._keep += [host_src, dev_src, host_dst, dev_dst]
        self.pixels += j.rows * j.cols
        return idx

    def add_gauss(self, host_src, dev_src, host_dst, dev_dst, sigma, op=_lib.SMOOTH, shift=True):
        j = Batch._job(dev_src, dev_dst, shift)
        j.op, j.gauss_op, j.sigma = _lib.BATCH_GAUSS, int(op), float(sigma)
        return self._add(j, host_src, dev_src, host_dst, dev_dst)

    def add_box(self, host_src, dev_src, host_dst, dev_dst, winV, winH, normalize=False, shift=True):
        j = Batch._job(dev_src, dev_dst, shift)
        j.op, j.winV, j.winH, j.normalize = _lib.BATCH_BOX, int(winV), int(winH), int(bool(normalize))
        return self._add(j, host_src, dev_src, host_dst, dev_dst)

    def plan(self, fir_rows=0, box_rows=0):
        check(self._lib.tucu_pipe_plan(self._h, int(fir_rows), int(box_rows)), "tucu_pipe_plan")
        return self

    def run(self):
        return check(self._lib.tucu_pipe_run(self._h, _stream()), "tucu_pipe_run")

    def info(self):
        nj, ng, nk = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        bi, bo = ctypes.c_size_t(), ctypes.c_size_t()
        check(self._lib.tucu_pipe_info(self._h, ctypes.byref(nj), ctypes.byref(ng), ctypes.byref(nk),
                                       ctypes.byref(bi), ctypes.byref(bo)))
        return {"jobs": nj.value, "groups": ng.value, "kernels": nk.value,
                "h2d_bytes": bi.value, "d2h_bytes": bo.value}
