"""The single-image filters with tensor cores switched on
(tucu_fir/gauss/box_set_tensor_cores): every qualifying call (f16 input on
16-byte row boundaries, f16 or f32 output, at most 33 taps per direction) runs
the tcgen05 kernel as one launch, within one f16 ulp (plus the paths' FP32
difference) of the exact call on the same handle; calls that do not qualify
keep the exact kernels, bit for bit."""
import numpy as np
import pytest

from helpers import to_device, torch_dtype

pytestmark = pytest.mark.gpu


def f16_ulp(x):
    a = np.maximum(np.abs(x), 2.0 ** -14)
    return 2.0 ** (np.floor(np.log2(a)) - 10)


def close(a, e, out_dt):
    a, e = a.astype(np.float64), e.astype(np.float64)
    scale = max(float(np.abs(e).max()), 1.0)
    if out_dt == "f16":
        return bool(np.all(np.abs(a - e) <= f16_ulp(e) + 2e-3))
    return float(np.abs(a - e).max()) <= 2e-5 * scale


def pair(cuda, shape, out_dt, fill=5):
    import torch
    return (torch.full(shape, fill, dtype=torch_dtype(out_dt), device=cuda),
            torch.full(shape, fill, dtype=torch_dtype(out_dt), device=cuda))


@pytest.mark.parametrize("sigma", [1.0, 2.0, 3.0, 8.0])
@pytest.mark.parametrize("out_dt", ["f16", "f32"])
def test_gauss_operators(F, cuda, sigma, out_dt):
    import torch
    rng = np.random.default_rng(int(sigma * 10) + len(out_dt))
    img = (rng.random((517, 1000)) * 255).astype(np.float32)
    src = to_device(img, "f16", cuda, pad=8)
    exact = F.FIRGaussianConvolver2(sigma)
    tc = F.FIRGaussianConvolver2(sigma).set_tensor_cores(True)
    for op in range(6):
        o1, o2 = pair(cuda, img.shape, out_dt)
        exact.convolve(op, src, o1)
        tc.convolve(op, src, o2, True)
        torch.cuda.synchronize()
        a, e = o2.float().cpu().numpy(), o1.float().cpu().numpy()
        # whole images: pixels outside the valid region keep the fill value in both
        assert close(a, e, out_dt), (sigma, op, np.abs(a - e).max())


def test_fir_unequal_lobes(F, oracle, cuda):
    """FIRFilter2 with a 33-tap horizontal and a 9-tap vertical lobe: unequal
    radii on the tensor cores (the exact path pads them to one radius)."""
    import torch
    l0 = oracle.gauss_lobes(4.0)[0]      # 17 taps: radius 16
    l1 = oracle.gauss_lobes(1.0)[0]      # 5 taps: radius 4
    rng = np.random.default_rng(3)
    img = (rng.random((300, 700)) * 255).astype(np.float32)
    src = to_device(img, "f16", cuda, pad=4)
    exact = F.FIRFilter2().initialize(l0, l1)
    tc = F.FIRFilter2().initialize(l0, l1).set_tensor_cores(True)
    o1, o2 = pair(cuda, img.shape, "f32")
    exact.convolve(src, o1)
    tc.convolve(src, o2)
    torch.cuda.synchronize()
    assert close(o2.cpu().numpy(), o1.cpu().numpy(), "f32")


@pytest.mark.parametrize("w", [(1, 1), (3, 3), (7, 7), (2, 5), (15, 15), (31, 31), (33, 33), (8, 31)])
def test_box_windows(F, cuda, w):
    import torch
    rng = np.random.default_rng(w[0] * 100 + w[1])
    img = (rng.random((400, 900)) * 255).astype(np.float32)
    src = to_device(img, "f16", cuda, pad=4)
    exact = F.BoxFilter2(w[0], w[1], 64)
    tc = F.BoxFilter2(w[0], w[1], 64).set_tensor_cores(True)
    for out_dt, norm in [("f16", True), ("f32", False)]:
        o1, o2 = pair(cuda, img.shape, out_dt)
        exact.convolve(src, o1, True, norm)
        tc.convolve(src, o2, True, norm)
        torch.cuda.synchronize()
        a, e = o2.float().cpu().numpy(), o1.float().cpu().numpy()
        assert close(a, e, out_dt), (w, out_dt, np.abs(a - e).max())


@pytest.mark.parametrize("shape,shift", [((9000, 300), True), ((700, 520), False)])
def test_tall_images_and_unshifted_outputs(F, cuda, shape, shift):
    """A 9000-row image spans several row bands of the single launch; with
    shift off the valid region sits at (0, 0), as on the exact path."""
    import torch
    rng = np.random.default_rng(shape[0])
    img = (rng.random(shape) * 255).astype(np.float32)
    src = to_device(img, "f16", cuda, pad=4)
    for f_exact, f_tc in [(F.FIRGaussianConvolver2(8.0), F.FIRGaussianConvolver2(8.0).set_tensor_cores(True)),
                          (F.BoxFilter2(15, 9, 64), F.BoxFilter2(15, 9, 64).set_tensor_cores(True))]:
        o1, o2 = pair(cuda, img.shape, "f32")
        if isinstance(f_exact, F.BoxFilter2):
            f_exact.convolve(src, o1, shift, False)
            f_tc.convolve(src, o2, shift, False)
        else:
            f_exact.smooth(src, o1, shift)
            f_tc.smooth(src, o2, shift)
        torch.cuda.synchronize()
        assert close(o2.cpu().numpy(), o1.cpu().numpy(), "f32"), (shape, shift)


def test_calls_that_do_not_qualify_stay_exact(F, cuda):
    """u8 input, unaligned f16 rows, a bf16 output and a 35-wide box window keep
    the exact kernels: bit-equal to a handle without tensor cores."""
    import torch
    rng = np.random.default_rng(9)
    img = (rng.random((200, 333)) * 255).astype(np.float32)
    cases = [(to_device(img, "u8", cuda, pad=3), "f32", "gauss"),
             (to_device(img, "f16", cuda), "f16", "gauss"),           # 666-byte rows
             (to_device(img, "f16", cuda, pad=3), "bf16", "gauss"),
             (to_device(img, "f16", cuda, pad=3), "f32", "box35")]
    for src, out_dt, what in cases:
        o1, o2 = pair(cuda, img.shape, out_dt)
        if what == "gauss":
            F.FIRGaussianConvolver2(2.0).smooth(src, o1)
            F.FIRGaussianConvolver2(2.0).set_tensor_cores(True).smooth(src, o2)
        else:
            F.BoxFilter2(35, 35, 64).convolve(src, o1)
            F.BoxFilter2(35, 35, 64).set_tensor_cores(True).convolve(src, o2)
        torch.cuda.synchronize()
        assert torch.equal(o1, o2), (what, out_dt)
