"""tucu_guided_convolve_noalloc: the guided filter for callers that cannot
allocate device memory (their memory manager owns the GPU, or they cannot
afford cudaMalloc's synchronisation).  The entry point runs the same kernels
as tucu_guided_convolve with its scratch in a fixed device array instead of
a handle's allocation, so through the C ABI its output must equal the
allocating entry point's bit for bit: guided and self-guided, 8-, 16- and
32-bit input, shifted and unshifted outputs, on two calls in a row whose
inputs differ (the second call must not see the first call's scratch).  This
file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

from helpers import to_device

pytestmark = pytest.mark.gpu


def _call_noalloc(lib, w, e, p, g, out, shift=True):
    import torch
    pitch = lambda t: t.stride(0) * t.element_size()  # noqa: E731
    dt = {torch.uint8: 0, torch.float16: 1, torch.bfloat16: 2, torch.float32: 3}
    return lib.tucu_guided_convolve_noalloc(
        w, w, ctypes.c_float(e), ctypes.c_void_p(p.data_ptr()), pitch(p),
        ctypes.c_void_p(g.data_ptr()) if g is not None else None, pitch(g) if g is not None else 0,
        p.size(0), p.size(1), dt[p.dtype], ctypes.c_void_p(out.data_ptr()), pitch(out),
        dt[out.dtype], int(shift), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))


@pytest.mark.parametrize("dtype", ["f32", "f16", "u8"])
@pytest.mark.parametrize("guided", [True, False])
@pytest.mark.parametrize("shift", [True, False])
def test_noalloc_equals_allocating_entry_point(cuda, dtype, guided, shift):
    import torch
    from tucuda_gb300 import _lib, filters as F
    from tucuda_gb300 import workloads
    lib = _lib.load()
    rows, cols, w = 1080, 1920, 17
    # Two calls in a row on the same size with different data, then a larger
    # window: stale coefficients from the previous call would show.
    for call, (seed, win) in enumerate([(3, w), (8, w), (11, 9)]):
        p_np, g_np = workloads.guided_pair(rows, cols, seed)
        if dtype == "u8":
            p_np, g_np = np.clip(p_np, 0, 255), np.clip(g_np, 0, 255)
        p, g = to_device(p_np, dtype, cuda), to_device(g_np, dtype, cuda)
        gg = g if guided else None
        f = F.GuidedFilter2(win, win, workloads.GUIDED_E)
        ref = torch.full((rows, cols), -1.0, device=cuda)
        f.convolve(p, gg, ref, shift)
        got = torch.full((rows, cols), -1.0, device=cuda)
        assert _call_noalloc(lib, win, workloads.GUIDED_E, p, gg, got, shift) == 0, \
            lib.tucu_last_error()
        torch.cuda.synchronize()
        assert torch.equal(got, ref), (call, (got - ref).abs().max().item())


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
