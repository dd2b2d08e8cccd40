"""Guided filter against the CPU oracles: error vs FP64 with a stated
bound, and agreement with the reference-faithful float oracle."""
import numpy as np
import pytest

from helpers import quantise_input, rel_rms, to_device, to_numpy_f32, torch_dtype

pytestmark = pytest.mark.gpu
SENTINEL = -3.0


def guide_pair(rows, cols, seed):
    from tucuda_gb300 import workloads
    return workloads.guided_pair(rows, cols, seed)


def run_guided(F, p, g, w, e, in_dt, out_dt, dev, shift=True):
    import torch
    sp = to_device(p, in_dt, dev)
    sg = None if g is None else to_device(g, in_dt, dev)
    out = torch.full(p.shape, SENTINEL, dtype=torch_dtype(out_dt), device=dev)
    gf = F.GuidedFilter2(w, w, e, wmax=129)
    wrote = gf.convolve(sp, sg, out, shift)
    torch.cuda.synchronize()
    return wrote, out


def mask(shape, w, shift):
    m = np.zeros(shape, bool)
    o = w - 1 if shift else 0
    m[o:o + shape[0] - 2 * (w - 1), o:o + shape[1] - 2 * (w - 1)] = True
    return m


def test_config3_guided_1080p(F, oracle, cuda):
    # 1920x1080 f32; guide = 8 sinusoids + 128 + N(0,10); input = guide +
    # N(0,25); radius 8 (w=17); eps = 0.01*255^2 -> e = 25.5 (squared inside).
    p, g = guide_pair(1080, 1920, 3)
    wrote, out = run_guided(F, p, g, 17, 25.5, "f32", "f32", cuda)
    assert wrote
    m = mask(p.shape, 17, True)
    _, r64 = oracle.guided_f64(p.astype(np.float64), g.astype(np.float64), 17, 17, 25.5)
    _, r32 = oracle.guided_f32(p, g, 17, 17, 25.5)
    got = to_numpy_f32(out)
    err_gpu = rel_rms(got[m], r64[m])
    err_ref = rel_rms(r32[m], r64[m])
    assert err_gpu < 1e-5, err_gpu
    # the mean-shifted sums are at least as accurate as the reference's
    assert err_gpu <= max(err_ref, 1e-6), (err_gpu, err_ref)
    assert np.abs(got[m] - r32[m]).max() < 0.05
    assert (got[~m] == SENTINEL).all()


@pytest.mark.parametrize("storage,bound", [("f16", 1e-3), ("bf16", 4e-3)])
def test_guided_reduced_storage(F, oracle, cuda, storage, bound):
    p, g = guide_pair(300, 500, 4)
    wrote, out = run_guided(F, p, g, 17, 25.5, storage, storage, cuda)
    m = mask(p.shape, 17, True)
    _, r64 = oracle.guided_f64(p.astype(np.float64), g.astype(np.float64), 17, 17, 25.5)
    assert rel_rms(to_numpy_f32(out)[m], r64[m]) < bound


@pytest.mark.parametrize("w", [3, 9, 33])
@pytest.mark.parametrize("shift", [True, False])
def test_guided_windows_u8_input(F, oracle, cuda, w, shift):
    rng = np.random.default_rng(w)
    g = rng.integers(0, 256, (120, 1100)).astype(np.float32)
    p = np.clip(g + rng.normal(0, 20, g.shape), 0, 255).astype(np.float32)
    pq, gq = quantise_input(p, "u8"), quantise_input(g, "u8")
    wrote, out = run_guided(F, pq, gq, w, 2.0, "u8", "f32", cuda, shift)
    m = mask(p.shape, w, shift)
    _, r64 = oracle.guided_f64(pq.astype(np.float64), gq.astype(np.float64), w, w, 2.0,
                               shift=shift)
    got = to_numpy_f32(out)
    assert np.abs(got[m] - r64[m]).max() < 0.02
    assert (got[~m] == SENTINEL).all()


def test_self_guided_matches_reference_formula(F, oracle, cuda):
    # The self-guided overload reproduces the reference's offset term
    # b = (Sp - a*Spp)/n (GuidedFilter.h:97).
    rng = np.random.default_rng(9)
    p = (rng.random((64, 80)) * 4).astype(np.float32)
    wrote, out = run_guided(F, p, None, 5, 0.5, "f32", "f32", cuda)
    m = mask(p.shape, 5, True)
    _, r64 = oracle.guided_f64(p.astype(np.float64), None, 5, 5, 0.5)
    got = to_numpy_f32(out)
    np.testing.assert_allclose(got[m], r64[m], rtol=1e-4, atol=1e-3)


def test_guided_too_small_is_noop(F, oracle, cuda):
    p = np.ones((20, 200), np.float32)
    wrote, out = run_guided(F, p, p, 11, 1.0, "f32", "f32", cuda)
    assert not wrote and (to_numpy_f32(out) == SENTINEL).all()


@pytest.mark.parametrize("self_guided", [False, True])
@pytest.mark.parametrize("in_dt", ["f16", "u8", "f32"])
def test_load_paths_bit_identical(F, cuda, in_dt, self_guided):
    # Rows aligned for asynchronous vector copies and rows that are not
    # (odd pitch, shifted base) take different load paths; the sums and the
    # coefficient arithmetic are the same, so the outputs agree bit for bit.
    import torch
    rng = np.random.default_rng(11)
    p = (rng.random((96, 233)) * 255).astype(np.float32)
    g = None if self_guided else (rng.random((96, 233)) * 255).astype(np.float32)
    outs = []
    for pad, offset in [(0, 0), (3, 0), (1, 1), (64, 0)]:
        sp = to_device(p, in_dt, cuda, pad=pad, offset=offset)
        sg = None if g is None else to_device(g, in_dt, cuda, pad=pad, offset=offset)
        out = torch.full(p.shape, SENTINEL, dtype=torch.float32, device=cuda)
        F.GuidedFilter2(13, 13, 25.5, wmax=129).convolve(sp, sg, out, True)
        torch.cuda.synchronize()
        outs.append(out.cpu().numpy().view(np.uint32))
    for o in outs[1:]:
        assert np.array_equal(outs[0], o)


@pytest.mark.parametrize("wV,wH", [(9, 129), (127, 126)])
def test_guided_wide_windows(F, oracle, cuda, wV, wH):
    # Windows wider than a 4-column warp tile holds run 8 columns per lane.
    import torch
    p, g = guide_pair(300, 640, 6)
    sp, sg = to_device(p, "f32", cuda), to_device(g, "f32", cuda)
    out = torch.full(p.shape, SENTINEL, dtype=torch.float32, device=cuda)
    assert F.GuidedFilter2(wV, wH, 25.5, wmax=129).convolve(sp, sg, out, True)
    torch.cuda.synchronize()
    m = np.zeros(p.shape, bool)
    m[wV - 1:p.shape[0] - (wV - 1), wH - 1:p.shape[1] - (wH - 1)] = True
    _, r64 = oracle.guided_f64(p.astype(np.float64), g.astype(np.float64), wV, wH, 25.5)
    got = to_numpy_f32(out)
    assert rel_rms(got[m], r64[m]) < 1e-5
    assert (got[~m] == SENTINEL).all()


@pytest.mark.parametrize("in_dt", ["f16", "u8", "f32"])
def test_wide_window_load_paths_bit_identical(F, cuda, in_dt):
    import torch
    rng = np.random.default_rng(13)
    p = (rng.random((70, 400)) * 255).astype(np.float32)
    g = (rng.random((70, 400)) * 255).astype(np.float32)
    outs = []
    for pad, offset in [(0, 0), (4, 0), (1, 1)]:
        sp, sg = to_device(p, in_dt, cuda, pad=pad, offset=offset), to_device(g, in_dt, cuda, pad=pad, offset=offset)
        out = torch.full(p.shape, SENTINEL, dtype=torch.float32, device=cuda)
        F.GuidedFilter2(5, 128, 25.5, wmax=129).convolve(sp, sg, out, True)
        torch.cuda.synchronize()
        outs.append(out.cpu().numpy().view(np.uint32))
    for o in outs[1:]:
        assert np.array_equal(outs[0], o)
