"""tucu_guided_convolve_noalloc: the guided filter for callers that cannot
allocate device memory (their memory manager owns the GPU, or they cannot
afford cudaMalloc's synchronisation).  Called through the C ABI, its output
must match the allocating entry point's, within the guided-filter tolerance
of the other tests, on two calls in a row (the second must not see the first
call's scratch contents).  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

from helpers import to_device

pytestmark = pytest.mark.gpu

TOL = 0.05  # max abs difference on a 0..255 scale, as in test_guided_gpu.py


def _call_noalloc(lib, w, e, p, g, out, shift=True):
    import torch
    pitch = lambda t: t.stride(0) * t.element_size()  # noqa: E731
    dt = {torch.float32: 3, torch.uint8: 0, torch.float16: 1}
    return lib.tucu_guided_convolve_noalloc(
        w, w, ctypes.c_float(e), ctypes.c_void_p(p.data_ptr()), pitch(p),
        ctypes.c_void_p(g.data_ptr()) if g is not None else None, pitch(g) if g is not None else 0,
        p.size(0), p.size(1), dt[p.dtype], ctypes.c_void_p(out.data_ptr()), pitch(out),
        dt[out.dtype], int(shift), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))


def test_noalloc_matches_allocating_entry_point(cuda):
    import torch
    from tucuda_gb300 import _lib, filters as F
    from tucuda_gb300 import workloads
    lib = _lib.load()
    for call, (rows, cols, w, seed) in enumerate([(1080, 1920, 17, 3), (700, 1300, 9, 8)]):
        p_np, g_np = workloads.guided_pair(rows, cols, seed)
        p, g = to_device(p_np, "f32", cuda), to_device(g_np, "f32", cuda)
        ref = torch.full((rows, cols), -1.0, device=cuda)
        F.GuidedFilter2(w, w, workloads.GUIDED_E).convolve(p, g, ref)
        got = torch.full((rows, cols), -1.0, device=cuda)
        assert _call_noalloc(lib, w, workloads.GUIDED_E, p, g, got) == 0, \
            lib.tucu_last_error()
        torch.cuda.synchronize()
        diff = (got - ref).abs().max().item()
        assert diff <= TOL, (call, diff)
        assert torch.equal(got[: w - 1], ref[: w - 1])   # untouched border stays as it was


def test_noalloc_rejects_images_beyond_the_scratch(cuda):
    import torch
    from tucuda_gb300 import _lib
    lib = _lib.load()
    p = torch.zeros(1100, 2000, device=cuda)
    out = torch.full_like(p, 7.0)
    rc = _call_noalloc(lib, 3, 1.0, p, p, out)
    assert rc == _lib.ERR_ARG
    assert b"16 MiB" in lib.tucu_last_error()
    torch.cuda.synchronize()
    assert (out == 7.0).all()
