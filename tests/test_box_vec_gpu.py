"""Box sums of vector pixels (box_convolver<vec<float, N>>, the filter
SuperPixels runs over its feature vectors): every channel equals the FP32 box
filter of that channel plane bit for bit, and the FP64 oracle within the box
filter's float tolerance; pixels outside the valid region are untouched."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
SENT = -3.0


def planes_box(F, img, wV, wH, shift, normalize, dev):
    import torch
    outs = []
    b = F.BoxFilter2(wV, wH, 129)
    for c in range(img.shape[2]):
        src = torch.from_numpy(np.ascontiguousarray(img[:, :, c])).to(dev)
        o = torch.full(src.shape, SENT, dtype=torch.float32, device=dev)
        b.convolve(src, o, shift, normalize)
        outs.append(o)
    torch.cuda.synchronize()
    return torch.stack(outs, dim=2).cpu().numpy()


@pytest.mark.parametrize("n", [2, 3, 4])
@pytest.mark.parametrize("wV,wH", [(1, 1), (3, 5), (7, 7), (15, 15), (31, 9), (8, 33)])
@pytest.mark.parametrize("shift,normalize", [(True, False), (False, True)])
def test_channels_equal_plane_box(F, oracle, cuda, n, wV, wH, shift, normalize):
    import torch
    rng = np.random.default_rng(n * 1000 + wV * 40 + wH)
    rows, cols = 203, 517
    img = (rng.random((rows, cols, n)) * 255).astype(np.float32)
    # rows padded so that every row starts on a 16-byte boundary
    pc = (cols * n + 3) // 4 * 4 + 4
    store = torch.zeros(rows, pc, dtype=torch.float32, device=cuda)
    src = store[:, :cols * n].view(rows, cols, n)
    src.copy_(torch.from_numpy(img).to(cuda))
    out = torch.full((rows, cols, n), SENT, dtype=torch.float32, device=cuda)
    b = F.BoxFilter2(wV, wH, 129)
    assert b.convolve_vec(src, out, shift, normalize)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    want = planes_box(F, img, wV, wH, shift, normalize, cuda)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    for c in range(n):
        _, ref = oracle.box_f64(img[:, :, c].astype(np.float64), wV, wH, shift=shift)
        oy, ox = (wV // 2, wH // 2) if shift else (0, 0)
        v = (slice(oy, oy + rows + 1 - wV), slice(ox, ox + cols + 1 - wH))
        r = ref[v] / (wV * wH) if normalize else ref[v]
        # FP32 window sums are differences of prefix sums over a warp's 128
        # columns of column sums (<= 128 * wV * 255): a few ulp of that.
        tol = 2.0 ** -20 * 128 * wV * 255 / ((wV * wH) if normalize else 1)
        assert np.max(np.abs(got[:, :, c][v] - r)) < tol


def test_alignment_and_noop(F, cuda):
    import torch
    from tucuda_gb300 import _lib
    b = F.BoxFilter2(5, 5)
    x = torch.zeros(40, 41, 3, dtype=torch.float32, device=cuda)  # 492-byte rows
    with pytest.raises(_lib.TucuError):
        b.convolve_vec(x, torch.zeros_like(x))
    x = torch.zeros(4, 40, 4, dtype=torch.float32, device=cuda)
    o = torch.full_like(x, 2.0)
    assert b.convolve_vec(x, o) is False and torch.all(o == 2.0)


@pytest.mark.parametrize("n", [2, 3, 4])
@pytest.mark.parametrize("wV,wH", [(3, 129), (9, 126)])
def test_wide_window_channels_equal_plane_box(F, oracle, cuda, n, wV, wH):
    # Windows wider than a 4-column warp tile holds: vector pixels and the
    # plane filter both run 8 pixels per lane, so they still agree bit for bit.
    import torch
    rng = np.random.default_rng(n * 7 + wH)
    rows, cols = 61, 430
    img = (rng.random((rows, cols, n)) * 255).astype(np.float32)
    pc = (cols * n + 3) // 4 * 4 + 4
    store = torch.zeros(rows, pc, dtype=torch.float32, device=cuda)
    src = store[:, :cols * n].view(rows, cols, n)
    src.copy_(torch.from_numpy(img).to(cuda))
    out = torch.full((rows, cols, n), SENT, dtype=torch.float32, device=cuda)
    assert F.BoxFilter2(wV, wH, 129).convolve_vec(src, out, True, False)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    want = planes_box(F, img, wV, wH, True, False, cuda)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    for c in range(n):
        _, ref = oracle.box_f64(img[:, :, c].astype(np.float64), wV, wH)
        v = (slice(wV // 2, wV // 2 + rows + 1 - wV), slice(wH // 2, wH // 2 + cols + 1 - wH))
        # prefix sums over a warp's 256 columns of column sums
        assert np.max(np.abs(got[:, :, c][v] - ref[v])) < 2.0 ** -20 * 256 * wV * 255
