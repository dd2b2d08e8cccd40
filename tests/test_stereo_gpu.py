"""Stereo cost aggregation (BoxFilter2's stereo overload with diff<T>,
disparity-major) against the oracle: int32 sums of u8 images bit-exact, float
sums within the box filter's float tolerance; disparities that reach past the
right edge, ragged and pitched images, every (wH-1) mod 4 and d mod 4."""
import numpy as np
import pytest

from helpers import to_device, torch_dtype

pytestmark = pytest.mark.gpu
SENT = -9


def run(F, L, R, dt, wV, wH, thresh, ndisp, dev, pad=0, wmax=64):
    import torch
    left, right = to_device(L, dt, dev, pad=pad), to_device(R, dt, dev, pad=pad)
    cdt = torch.int32 if dt in ("u8", "i32") else torch.float32
    costs = torch.full((ndisp,) + L.shape, SENT, dtype=cdt, device=dev)
    b = F.BoxFilter2(wV, wH, wmax)
    wrote = b.convolve_stereo(left, right, costs, thresh)
    torch.cuda.synchronize()
    return wrote, costs.cpu().numpy().astype(np.float64)


@pytest.mark.parametrize("wV,wH", [(1, 1), (3, 3), (5, 7), (9, 9), (15, 15), (4, 6), (21, 2)])
@pytest.mark.parametrize("ndisp", [1, 7, 64])
def test_u8_int32_bit_exact(F, oracle, cuda, wV, wH, ndisp):
    rng = np.random.default_rng(wV * 100 + wH + ndisp)
    L = rng.integers(0, 256, (97, 301)).astype(np.float32)
    R = np.roll(L, 5, axis=1) + rng.integers(-10, 11, L.shape)
    R = np.clip(R, 0, 255).astype(np.float32)
    wrote, got = run(F, L, R, "u8", wV, wH, 50, ndisp, cuda)
    ref = oracle.stereo(L, R, wV, wH, 50, ndisp)
    assert wrote
    m = ~np.isnan(ref)
    assert np.array_equal(got[m], ref[m])
    assert np.all(got[~m] == SENT)


@pytest.mark.parametrize("dt", ["f32", "f16", "bf16"])
def test_float_within_tolerance(F, oracle, cuda, dt):
    import torch
    rng = np.random.default_rng(len(dt))
    L = (rng.random((150, 260)) * 255).astype(np.float32)
    R = (rng.random((150, 260)) * 255).astype(np.float32)
    if dt != "f32":
        L = torch.from_numpy(L).to(torch_dtype(dt)).float().numpy()
        R = torch.from_numpy(R).to(torch_dtype(dt)).float().numpy()
    wrote, got = run(F, L, R, dt, 11, 13, 40.5, 9, cuda, pad=3)
    ref = oracle.stereo(L, R, 11, 13, 40.5, 9)
    m = ~np.isnan(ref)
    assert wrote
    # FP32 window sums of at most 143 values <= 40.5 each: relative 1e-5
    assert np.max(np.abs(got[m] - ref[m]) / np.maximum(ref[m], 1.0)) < 1e-5
    assert np.all(got[~m] == SENT)


@pytest.mark.parametrize("shape", [(16, 16), (40, 129), (300, 1000), (1, 200)])
def test_shapes_and_pitches(F, oracle, cuda, shape):
    rng = np.random.default_rng(shape[0] + shape[1])
    L = rng.integers(0, 256, shape).astype(np.float32)
    R = rng.integers(0, 256, shape).astype(np.float32)
    wV = min(7, shape[0])
    wrote, got = run(F, L, R, "u8", wV, 7, 30, 13, cuda, pad=5)
    ref = oracle.stereo(L, R, wV, 7, 30, 13)
    m = ~np.isnan(ref)
    assert wrote and np.array_equal(got[m], ref[m])


def test_errors_and_noop(F, cuda):
    import torch
    from tucuda_gb300 import _lib
    b = F.BoxFilter2(5, 5)
    L = torch.zeros(4, 40, dtype=torch.uint8, device=cuda)
    c = torch.full((3, 4, 40), 7, dtype=torch.int32, device=cuda)
    assert b.convolve_stereo(L, L, c, 10) is False and torch.all(c == 7)
    L = torch.zeros(40, 40, dtype=torch.uint8, device=cuda)
    with pytest.raises(_lib.TucuError) as e:
        b.convolve_stereo(L, L, torch.zeros(3, 40, 40, dtype=torch.float32, device=cuda), 10)
    assert e.value.status == _lib.ERR_DTYPE
    with pytest.raises(_lib.TucuError):
        b.convolve_stereo(L, L, torch.zeros(3, 40, 40, dtype=torch.int32, device=cuda), -1)


@pytest.mark.parametrize("dt", ["u8", "f16", "f32", "i32"])
@pytest.mark.parametrize("ndisp", [5, 32])
def test_aligned_rows_async_path(F, oracle, cuda, dt, ndisp):
    # rows 4-pixel aligned: the lanes copy both images with cp.async, the right
    # one as two aligned groups shifted by d mod 4
    rng = np.random.default_rng(ndisp + len(dt))
    L = rng.integers(0, 200, (130, 512)).astype(np.float32)
    R = rng.integers(0, 200, (130, 512)).astype(np.float32)
    wrote, got = run(F, L, R, dt, 9, 11, 25, ndisp, cuda)
    ref = oracle.stereo(L, R, 9, 11, 25, ndisp)
    m = ~np.isnan(ref)
    assert wrote
    if dt in ("u8", "i32"):
        assert np.array_equal(got[m], ref[m])
    else:
        assert np.max(np.abs(got[m] - ref[m]) / np.maximum(ref[m], 1.0)) < 1e-5


@pytest.mark.parametrize("wV,wH", [(3, 126), (2, 129), (5, 127)])
@pytest.mark.parametrize("pad", [0, 3])
def test_wide_windows_u8_bit_exact(F, oracle, cuda, wV, wH, pad):
    # Windows wider than a 4-column warp tile holds run 8 columns per lane;
    # 13 disparities cover every d mod 8 of the right-row shift.
    rng = np.random.default_rng(wH + pad)
    L = rng.integers(0, 256, (41, 700)).astype(np.float32)
    R = np.clip(np.roll(L, 3, axis=1) + rng.integers(-10, 11, L.shape), 0, 255).astype(np.float32)
    wrote, got = run(F, L, R, "u8", wV, wH, 50, 13, cuda, pad=pad, wmax=129)
    ref = oracle.stereo(L, R, wV, wH, 50, 13)
    m = ~np.isnan(ref)
    assert wrote and np.array_equal(got[m], ref[m])
    assert np.all(got[~m] == SENT)


@pytest.mark.parametrize("dt", ["f32", "f16"])
def test_wide_windows_float_within_tolerance(F, oracle, cuda, dt):
    import torch
    rng = np.random.default_rng(7)
    L = (rng.random((30, 520)) * 255).astype(np.float32)
    R = (rng.random((30, 520)) * 255).astype(np.float32)
    if dt != "f32":
        L = torch.from_numpy(L).to(torch_dtype(dt)).float().numpy()
        R = torch.from_numpy(R).to(torch_dtype(dt)).float().numpy()
    wrote, got = run(F, L, R, dt, 3, 128, 40.5, 11, cuda, wmax=129)
    ref = oracle.stereo(L, R, 3, 128, 40.5, 11)
    m = ~np.isnan(ref)
    assert wrote
    assert np.max(np.abs(got[m] - ref[m]) / np.maximum(ref[m], 1.0)) < 1e-5
    assert np.all(got[~m] == SENT)


@pytest.mark.parametrize("thresh,held", [(300, 44), (256, 0), (255.7, 255), (511, 255), (50.9, 50)])
def test_u8_threshold_is_held_as_u_char(F, oracle, cuda, thresh, held):
    """diff<u_char>(thresh) holds the threshold as a u_char (functional.h:
    385-398): its integer part modulo 256, so thresholds from 256 on wrap."""
    rng = np.random.default_rng(int(thresh * 10))
    L = rng.integers(0, 256, (40, 120)).astype(np.float32)
    R = rng.integers(0, 256, (40, 120)).astype(np.float32)
    wrote, got = run(F, L, R, "u8", 3, 3, thresh, 5, cuda)
    ref = oracle.stereo(L, R, 3, 3, held, 5)
    assert wrote
    m = ~np.isnan(ref)
    assert np.array_equal(got[m], ref[m])
