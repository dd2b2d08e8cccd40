"""u8 outputs outside [0, 256).  The reference's implicit float-to-u_char
assignment, as it runs on a GB300, truncates toward zero, saturates to the
unsigned 32-bit range (negative values give 0) and keeps the low byte
(tests/test_oracle_ref_device.py pins this against its own device code).  The
library's u8 stores do the same, so FIR outputs above 255 and unnormalised box
sums of u8 images wrap modulo 256 as the reference's do, and negative outputs
become 0."""
import numpy as np
import pytest

from helpers import to_device

pytestmark = pytest.mark.gpu


def test_fir_u8_outputs_wrap_like_the_reference(F, oracle, cuda):
    import torch
    rng = np.random.default_rng(3)
    img = np.floor(rng.random((96, 160)) * 255).astype(np.float32)  # exact in u8
    lh = (rng.normal(0, 1.2, 9)).astype(np.float32)  # outputs over about [-2000, 2000]
    lv = (rng.normal(0, 1.2, 5)).astype(np.float32)
    src = to_device(img, "u8", cuda)
    out = torch.zeros(img.shape, dtype=torch.uint8, device=cuda)
    f = F.FIRFilter2()
    f.initialize(lh, lv)
    assert f.convolve(src, out, True)
    torch.cuda.synchronize()
    _, ref = oracle.fir_f32(img, lh, lv, shift=True)
    region = (slice(4, 96 - 4), slice(8, 160 - 8))  # LS_V = 4, LS_H = 8
    r = ref[region]
    assert (r > 255).any() and (r < 0).any() and ((r >= 0) & (r <= 255)).any()
    assert np.array_equal(out.cpu().numpy()[region], oracle.to_u8(r))


@pytest.mark.parametrize("wV,wH", [(5, 7), (1, 2), (15, 15)])
def test_box_u8_sums_wrap_like_the_reference(F, oracle, cuda, wV, wH):
    import torch
    rng = np.random.default_rng(wV * 100 + wH)
    img = rng.integers(0, 256, (120, 300)).astype(np.float32)
    src = to_device(img, "u8", cuda)
    out = torch.zeros(img.shape, dtype=torch.uint8, device=cuda)
    assert F.BoxFilter2(wV, wH, 129).convolve(src, out, True, False)
    torch.cuda.synchronize()
    _, ref = oracle.box_i64(img.astype(np.int32), wV, wH, shift=True)
    region = (slice(wV // 2, wV // 2 + 121 - wV), slice(wH // 2, wH // 2 + 301 - wH))
    assert np.array_equal(out.cpu().numpy()[region], (ref[region] & 0xFF).astype(np.uint8))
