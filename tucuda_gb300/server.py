"""The request loop of the C ABI (tucu_server_*) for host images.

    with Server(budget_bytes=32 << 30) as srv:
        t = srv.submit_gauss(img, out, sigma=2.0)     # numpy / pinned CPU tensors
        srv.wait(t)
        print(srv.stats())

Requests are admitted while their device buffers fit the budget, batched as
they arrive (continuous batching over several streams) and copied back on
completion; each result equals the single call of the same filter.  The host
arrays must stay alive until their request completes.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import check

_NP_DT = {np.dtype(np.uint8): _lib.U8, np.dtype(np.float16): _lib.F16,
          np.dtype(np.float32): _lib.F32, np.dtype(np.int32): _lib.I32}


def _host_view(a, what):
    """(pointer, pitch, rows, cols, dtype) of a 2D host array (numpy or CPU
    torch tensor, rows contiguous)."""
    try:
        import torch
        if isinstance(a, torch.Tensor):
            if a.is_cuda or a.dim() != 2 or a.stride(1) != 1:
                raise _lib.TucuError(_lib.ERR_ARG, f"{what}: 2D CPU tensor with contiguous rows")
            dt = {torch.uint8: _lib.U8, torch.float16: _lib.F16, torch.bfloat16: _lib.BF16,
                  torch.float32: _lib.F32, torch.int32: _lib.I32}[a.dtype]
            return a.data_ptr(), a.stride(0) * a.element_size(), a.size(0), a.size(1), dt
    except ImportError:
        pass
    if not isinstance(a, np.ndarray) or a.ndim != 2 or a.strides[1] != a.itemsize:
        raise _lib.TucuError(_lib.ERR_ARG, f"{what}: 2D numpy array with contiguous rows")
    return a.ctypes.data, a.strides[0], a.shape[0], a.shape[1], _NP_DT[a.dtype]


class Server:
    def __init__(self, budget_bytes=32 << 30, streams=6, max_wave=16, tensor=False):
        """tensor=True: f16 Gaussian and box requests on the tensor cores
        (tucu_server_set_tensor_cores)."""
        self._lib = _lib.load()
        self._h = ctypes.c_void_p()
        check(self._lib.tucu_server_create(int(budget_bytes), int(streams), int(max_wave),
                                           ctypes.byref(self._h)), "tucu_server_create")
        self._keep = {}
        if tensor:
            check(self._lib.tucu_server_set_tensor_cores(self._h, 1), "tucu_server_set_tensor_cores")

    def close(self):
        if getattr(self, "_h", None):
            self._lib.tucu_server_destroy(self._h)
            self._h = None
            self._keep.clear()

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _submit(self, req, keep):
        t = ctypes.c_uint64()
        check(self._lib.tucu_server_submit(self._h, ctypes.byref(req), ctypes.byref(t)),
              "tucu_server_submit")
        self._keep[t.value] = keep
        return t.value

    def _req(self, op, inp, out, guide=None):
        ip, ipitch, rows, cols, idt = _host_view(inp, "input")
        op_, opitch, orows, ocols, odt = _host_view(out, "output")
        if (rows, cols) != (orows, ocols):
            raise _lib.TucuError(_lib.ERR_ARG, "output must have the input's shape")
        r = _lib.Request()
        r.op, r.in_, r.in_pitch, r.in_dtype = op, ip, ipitch, idt
        r.out, r.out_pitch, r.out_dtype, r.rows, r.cols = op_, opitch, odt, rows, cols
        if guide is not None:
            gp, gpitch, gr, gc, gdt = _host_view(guide, "guide")
            r.guide, r.guide_pitch = gp, gpitch
        return r

    def submit_gauss(self, inp, out, sigma):
        r = self._req(_lib.REQ_GAUSS, inp, out)
        r.sigma = float(sigma)
        return self._submit(r, (inp, out))

    def submit_box(self, inp, out, radius, normalize=False):
        r = self._req(_lib.REQ_BOX, inp, out)
        r.radius, r.normalize = int(radius), int(bool(normalize))
        return self._submit(r, (inp, out))

    def submit_guided(self, inp, guide, out, radius, e):
        r = self._req(_lib.REQ_GUIDED, inp, out, guide)
        r.radius, r.e = int(radius), float(e)
        return self._submit(r, (inp, guide, out))

    def wait(self, ticket, timeout=60.0):
        st = ctypes.c_int()
        rc = self._lib.tucu_server_wait(self._h, ticket, float(timeout), ctypes.byref(st))
        if rc == _lib.ERR_TIMEOUT:
            raise TimeoutError(f"request {ticket} still open after {timeout} s")
        check(rc, "tucu_server_wait")
        self._keep.pop(ticket, None)
        return st.value

    def cancel(self, ticket):
        return self._lib.tucu_server_cancel(self._h, ticket)

    def drain(self, timeout=600.0):
        return check(self._lib.tucu_server_drain(self._h, float(timeout)), "tucu_server_drain")

    def stats(self):
        s = _lib.ServerStats()
        check(self._lib.tucu_server_get_stats(self._h, ctypes.byref(s)), "tucu_server_get_stats")
        return {f: getattr(s, f) for f, _ in s._fields_}
