"""Windows wider than a 4-column warp tile holds (126..129 columns), which
run the window-sum strip at 8 columns per lane, and large images (4 Mpixel,
several rounds of warp tasks).  Integer sums are bit-exact against the
oracle, float sums within the FP64 tolerance of the box filter, and a batched
image gets the same bits as the single call (both pick the strip width by the
same rule)."""
import numpy as np
import pytest

from helpers import quantise_input, to_device, to_numpy_f32, torch_dtype

pytestmark = pytest.mark.gpu
SENTINEL = -7
BIG = (2048, 2112)       # 4.3 Mpixel


def run_box(F, img, in_dt, out_dt, wV, wH, dev, shift=True, normalize=False, pad=0, offset=0):
    import torch
    src = to_device(img, in_dt, dev, pad=pad, offset=offset)
    out = torch.full(img.shape, SENTINEL, dtype=torch_dtype(out_dt), device=dev)
    wrote = F.BoxFilter2(wV, wH, 129).convolve(src, out, shift, normalize)
    torch.cuda.synchronize()
    return wrote, out


def valid_mask(shape, wV, wH, shift):
    rows, cols = shape
    m = np.zeros(shape, bool)
    oy, ox = (wV // 2, wH // 2) if shift else (0, 0)
    m[oy:oy + rows + 1 - wV, ox:ox + cols + 1 - wH] = True
    return m


@pytest.mark.parametrize("wV,wH", [(3, 126), (5, 127), (1, 128), (129, 129), (17, 125)])
@pytest.mark.parametrize("pad,offset", [(0, 0), (0, 1)])
def test_wide_windows_u8_bit_exact(F, oracle, cuda, wV, wH, pad, offset):
    rng = np.random.default_rng(wH * 7 + wV)
    img = rng.integers(0, 256, (301, 917)).astype(np.float32)
    wrote, out = run_box(F, img, "u8", "i32", wV, wH, cuda, pad=pad, offset=offset)
    st, ref = oracle.box_i64(img.astype(np.int32), wV, wH)
    assert wrote and st == 0
    m = valid_mask(img.shape, wV, wH, True)
    got = out.cpu().numpy().astype(np.int64)
    assert np.array_equal(got[m], ref[m])
    assert (got[~m] == SENTINEL).all()


@pytest.mark.parametrize("in_dt", ["f16", "bf16", "f32"])
@pytest.mark.parametrize("wV,wH", [(9, 129), (129, 127)])
def test_wide_windows_float_vs_fp64(F, oracle, cuda, in_dt, wV, wH):
    rng = np.random.default_rng(wV + wH)
    img = (rng.random((400, 1100)) * 255).astype(np.float32)
    wrote, out = run_box(F, img, in_dt, "f32", wV, wH, cuda)
    q = quantise_input(img, in_dt)
    _, ref = oracle.box_f64(q.astype(np.float64), wV, wH)
    m = valid_mask(img.shape, wV, wH, True)
    got = to_numpy_f32(out)
    # FP32 sums of 8-pixel lane groups and 256-column warp prefixes: relative
    # error per pixel below 1e-5 of the FP64 sums of the stored input.
    assert np.max(np.abs(got[m] - ref[m]) / np.abs(ref[m]).clip(1.0)) < 1e-5


@pytest.mark.parametrize("wV,wH", [(15, 15), (3, 31), (31, 3)])
@pytest.mark.parametrize("shift", [True, False])
def test_large_u8_int32_bit_exact(F, oracle, cuda, wV, wH, shift):
    rng = np.random.default_rng(wV * 31 + wH)
    img = rng.integers(0, 256, BIG).astype(np.float32)
    wrote, out = run_box(F, img, "u8", "i32", wV, wH, cuda, shift)
    _, ref = oracle.box_i64(img.astype(np.int32), wV, wH, shift=shift)
    m = valid_mask(img.shape, wV, wH, shift)
    got = out.cpu().numpy().astype(np.int64)
    assert np.array_equal(got[m], ref[m])
    assert (got[~m] == SENTINEL).all()


def test_large_i32_bit_exact(F, oracle, cuda):
    rng = np.random.default_rng(3)
    img = rng.integers(-100000, 100000, BIG).astype(np.int64)
    import torch
    src = torch.from_numpy(img.astype(np.int32)).to(cuda)
    out = torch.full(BIG, SENTINEL, dtype=torch.int32, device=cuda)
    F.BoxFilter2(15, 15, 129).convolve(src, out, True, False)
    torch.cuda.synchronize()
    _, ref = oracle.box_i64(img.astype(np.int32), 15, 15)
    m = valid_mask(BIG, 15, 15, True)
    assert np.array_equal(out.cpu().numpy().astype(np.int64)[m], ref[m])


@pytest.mark.parametrize("out_dt", ["u8", "f16"])
@pytest.mark.parametrize("shift", [True, False])
def test_large_u8_means_exact(F, oracle, cuda, out_dt, shift):
    rng = np.random.default_rng(9)
    img = rng.integers(0, 256, BIG).astype(np.float32)
    wrote, out = run_box(F, img, "u8", out_dt, 15, 15, cuda, shift, normalize=True)
    _, ref = oracle.box_i64(img.astype(np.int32), 15, 15, shift=shift)
    m = valid_mask(BIG, 15, 15, shift)
    inv = np.float32(1.0) / np.float32(225)
    want = oracle.round_to((ref[m].astype(np.float32) * inv).astype(np.float32), out_dt)
    assert np.array_equal(to_numpy_f32(out)[m], want)


@pytest.mark.parametrize("dt", ["f16", "bf16", "f32"])
@pytest.mark.parametrize("pad", [0, 4, 1])
def test_large_float_vs_fp64(F, oracle, cuda, dt, pad):
    # pad 0 and 4: asynchronous row copies; pad 1: synchronous loads.
    rng = np.random.default_rng(17 + pad)
    img = (rng.random(BIG) * 255).astype(np.float32)
    wrote, out = run_box(F, img, dt, dt, 15, 15, cuda, pad=pad, normalize=True)
    q = quantise_input(img, dt)
    _, ref = oracle.box_f64(q.astype(np.float64), 15, 15)
    m = valid_mask(BIG, 15, 15, True)
    mean = ref[m] / 225.0
    got = to_numpy_f32(out)[m].astype(np.float64)
    # the FP32 mean within 1e-5 relative, then one rounding to the output type
    ulp = {"f16": 2.0 ** -10, "bf16": 2.0 ** -7, "f32": 2.0 ** -23}[dt]
    assert np.max(np.abs(got - mean) / np.abs(mean).clip(1.0)) < 1e-5 + ulp


@pytest.mark.parametrize("dt,out_dt,norm", [("f16", "f16", True), ("f32", "f32", False),
                                            ("u8", "i32", False), ("bf16", "bf16", True)])
def test_batch_equals_single_large_and_wide(F, cuda, dt, out_dt, norm):
    import torch
    from tucuda_gb300.batch import Batch
    rng = np.random.default_rng(23)
    shapes = [BIG, (2200, 1980), (300, 700)]
    wins = [(15, 15), (7, 129), (9, 5)]
    b = Batch()
    singles, batched = [], []
    for (rows, cols), (wV, wH) in zip(shapes, wins):
        img = (rng.random((rows, cols)) * 255).astype(np.float32)
        src = to_device(img, dt, cuda)
        o1 = torch.full((rows, cols), 5, dtype=torch_dtype(out_dt), device=cuda)
        o2 = torch.full((rows, cols), 5, dtype=torch_dtype(out_dt), device=cuda)
        F.BoxFilter2(wV, wH, 129).convolve(src, o1, True, norm)
        b.add_box(src, o2, wV, wH, norm, True)
        singles.append(o1)
        batched.append(o2)
    b.plan(256, 128)
    b.launch(graph=False)
    torch.cuda.synchronize()
    for o1, o2 in zip(singles, batched):
        assert torch.equal(o1, o2)
