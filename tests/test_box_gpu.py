"""Parity of the one-pass box filter with the CPU oracle: integer sums are
bit-exact (int32 against the oracle's int64); float sums are checked
against the FP64 oracle with a stated tolerance."""
import numpy as np
import pytest

from helpers import quantise_input, to_device, to_numpy_f32, torch_dtype

pytestmark = pytest.mark.gpu
SENTINEL = -7


def run_box(F, img, in_dt, out_dt, wV, wH, dev, shift=True, normalize=False, pad=0, offset=0,
            wmax=129):
    import torch
    src = to_device(img, in_dt, dev, pad=pad, offset=offset)
    out = torch.full(img.shape, SENTINEL, dtype=torch_dtype(out_dt), device=dev)
    b = F.BoxFilter2(wV, wH, wmax)
    wrote = b.convolve(src, out, shift, normalize)
    torch.cuda.synchronize()
    return wrote, out


def valid_mask(shape, wV, wH, shift):
    rows, cols = shape
    m = np.zeros(shape, bool)
    oy, ox = (wV // 2, wH // 2) if shift else (0, 0)
    m[oy:oy + rows + 1 - wV, ox:ox + cols + 1 - wH] = True
    return m


@pytest.mark.parametrize("wV,wH", [(1, 1), (3, 3), (15, 15), (7, 31), (31, 7), (23, 23),
                                   (2, 64), (64, 2), (129, 3)])
@pytest.mark.parametrize("shift", [True, False])
def test_u8_int32_sums_bit_exact(F, oracle, cuda, wV, wH, shift):
    rng = np.random.default_rng(wV * 1000 + wH)
    img = rng.integers(0, 256, (203, 1301)).astype(np.float32)
    wrote, out = run_box(F, img, "u8", "i32", wV, wH, cuda, shift)
    st, ref = oracle.box_i64(img.astype(np.int32), wV, wH, shift=shift)
    assert wrote == (st == 0)
    m = valid_mask(img.shape, wV, wH, shift)
    got = out.cpu().numpy().astype(np.int64)
    assert np.array_equal(got[m], ref[m])
    assert (got[~m] == SENTINEL).all()


@pytest.mark.parametrize("shape", [(15, 15), (16, 40), (100, 1), (1, 100), (37, 1025), (1100, 37),
                                   (14, 20)])
def test_ragged_and_smaller_than_window(F, oracle, cuda, shape):
    rng = np.random.default_rng(shape[0] + shape[1])
    img = rng.integers(0, 256, shape).astype(np.float32)
    wrote, out = run_box(F, img, "u8", "i32", 15, 15, cuda)
    st, ref = oracle.box_i64(img.astype(np.int32), 15, 15)
    assert wrote == (st == 0)
    got = out.cpu().numpy().astype(np.int64)
    if st == 0:
        m = valid_mask(shape, 15, 15, True)
        assert np.array_equal(got[m], ref[m])
    else:
        assert (got == SENTINEL).all()      # BoxFilter.h:551-557: silent no-op


@pytest.mark.parametrize("pad,offset", [(0, 1), (1, 0), (3, 2)])
def test_unaligned_rows(F, oracle, cuda, pad, offset):
    rng = np.random.default_rng(pad + offset)
    img = rng.integers(0, 256, (90, 333)).astype(np.float32)
    wrote, out = run_box(F, img, "u8", "i32", 9, 5, cuda, pad=pad, offset=offset)
    st, ref = oracle.box_i64(img.astype(np.int32), 9, 5)
    m = valid_mask(img.shape, 9, 5, True)
    assert np.array_equal(out.cpu().numpy().astype(np.int64)[m], ref[m])


def test_config2_box15_planes_bit_exact(F, oracle, cuda):
    # 1920x1080x3 planar u8, U{0..255}, 15x15 int32 sums, bit-exact.
    rng = np.random.default_rng(2)
    planes = rng.integers(0, 256, (3, 1080, 1920)).astype(np.float32)
    for p in planes:
        wrote, out = run_box(F, p, "u8", "i32", 15, 15, cuda)
        _, ref = oracle.box_i64(p.astype(np.int32), 15, 15)
        m = valid_mask(p.shape, 15, 15, True)
        assert np.array_equal(out.cpu().numpy().astype(np.int64)[m], ref[m])


@pytest.mark.parametrize("in_dt", ["f16", "bf16", "f32"])
@pytest.mark.parametrize("wV,wH", [(7, 7), (31, 31)])
def test_float_sums_vs_fp64(F, oracle, cuda, in_dt, wV, wH):
    # FP32 accumulation with compensated vertical updates: relative error
    # per pixel below 1e-5 against the FP64 sums of the stored input.
    rng = np.random.default_rng(wV)
    img = (rng.random((517, 1200)) * 255).astype(np.float32)
    wrote, out = run_box(F, img, in_dt, "f32", wV, wH, cuda)
    q = quantise_input(img, in_dt)
    _, ref = oracle.box_f64(q.astype(np.float64), wV, wH)
    m = valid_mask(img.shape, wV, wH, True)
    got = to_numpy_f32(out)
    assert np.max(np.abs(got[m] - ref[m]) / np.abs(ref[m]).clip(1.0)) < 1e-5


@pytest.mark.parametrize("out_dt", ["f16", "u8", "f32"])
def test_normalized_means(F, oracle, cuda, out_dt):
    rng = np.random.default_rng(5)
    img = rng.integers(0, 256, (200, 300)).astype(np.float32)
    wrote, out = run_box(F, img, "u8", out_dt, 31, 31, cuda, normalize=True)
    _, ref = oracle.box_i64(img.astype(np.int32), 31, 31)
    m = valid_mask(img.shape, 31, 31, True)
    # mean = sum * fl(1/n): the reciprocal rounded to float, one float multiply
    inv = np.float32(1.0) / np.float32(961)
    want = oracle.round_to((ref[m].astype(np.float32) * inv).astype(np.float32), out_dt)
    assert np.array_equal(to_numpy_f32(out)[m], want)


def test_window_above_wmax_raises(F, cuda):
    with pytest.raises(F._lib.TucuError):
        F.BoxFilter2(24, 3)          # WMAX = 23 by default (BoxFilter.h:417)


@pytest.mark.parametrize("in_dt,out_dt", [("f16", "f16"), ("f32", "f32"), ("u8", "i32"), ("bf16", "f32")])
def test_load_paths_bit_identical(F, cuda, in_dt, out_dt):
    # Aligned rows (asynchronous vector copies) and unaligned ones
    # (synchronous element loads) give bit-identical window sums and means.
    import torch
    rng = np.random.default_rng(12)
    img = (rng.random((150, 517)) * 255).astype(np.float32)
    for normalize in (False, True):
        outs = []
        for pad, offset in [(0, 0), (5, 0), (1, 3), (128, 0)]:
            src = to_device(img, in_dt, cuda, pad=pad, offset=offset)
            out = torch.full(img.shape, SENTINEL, dtype=torch_dtype(out_dt), device=cuda)
            F.BoxFilter2(15, 31, 129).convolve(src, out, True, normalize)
            torch.cuda.synchronize()
            outs.append(out.cpu().numpy().view(np.uint8))
        for o in outs[1:]:
            assert np.array_equal(outs[0], o)
