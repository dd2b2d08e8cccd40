"""The tensor-core kernel's bounded waits (tucu_debug_tc_wait): with each
input stage expecting more bytes than its copies deliver, the first barrier
wait can never complete; after the (shortened) limit the kernel gives up,
waits for its copies and MMAs in flight, frees its tensor memory and reports
code 1 through tucu_device_error.  No fault follows and later launches on the
same context produce correct output.  Nothing here faults a GPU: every copy
stays inside its image and every wait ends at its limit."""
import ctypes

import numpy as np
import pytest

from helpers import to_device

pytestmark = pytest.mark.gpu


def device_error(lib):
    c = ctypes.c_int()
    assert lib.tucu_device_error(ctypes.byref(c)) == 0
    return c.value


def test_wait_that_runs_out_reports_and_leaves_context_usable(F, cuda):
    import torch
    lib = F._lib.load()
    rng = np.random.default_rng(5)
    img = (rng.random((200, 300)) * 255).astype(np.float32)
    src = to_device(img, "f16", cuda, pad=4)
    assert device_error(lib) == 0
    exact = torch.zeros(img.shape, dtype=torch.float16, device=cuda)
    F.FIRGaussianConvolver2(2.0).smooth(src, exact)
    try:
        assert lib.tucu_debug_tc_wait(2_000_000, 1024) == 0   # 2 ms limit, stages never complete
        stuck = torch.full(img.shape, 7.0, dtype=torch.float16, device=cuda)
        F.FIRGaussianConvolver2(2.0).set_tensor_cores(True).smooth(src, stuck)
        torch.cuda.synchronize()
        assert device_error(lib) == 1       # a wait ran out
        # no MMA result ever reached an output: the image keeps its fill value
        assert bool((stuck == 7.0).all())
    finally:
        lib.tucu_debug_tc_wait(0, 0)
    assert device_error(lib) == 0           # the word was cleared by the read
    ok = torch.zeros(img.shape, dtype=torch.float16, device=cuda)
    F.FIRGaussianConvolver2(2.0).set_tensor_cores(True).smooth(src, ok)
    torch.cuda.synchronize()
    assert device_error(lib) == 0
    d = (ok.float() - exact.float()).abs()
    ulp = torch.clamp(exact.float().abs(), min=2.0 ** -14)
    ulp = 2.0 ** (torch.floor(torch.log2(ulp)) - 10)
    assert bool((d <= ulp + 2e-3).all()), d.max().item()
