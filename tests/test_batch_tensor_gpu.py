"""The batch's tensor-core path (tucu_batch_set_tensor_cores): FIR and box
jobs of f16 images as banded matrix products on tcgen05.  Its results are
checked against the exact FP32-pipe path of the same batch (which equals the
oracle bit for bit): f16 outputs within one f16 ulp, f32 outputs within a few
FP32 ulps of the image's scale; against the FP64 oracle at the f16 storage
floor; jobs it cannot take keep the exact kernels; an intermediate beyond the
f16 range is reported as device error 2."""
import ctypes

import numpy as np
import pytest

from helpers import rel_rms, to_device, torch_dtype

pytestmark = pytest.mark.gpu


def device_error(F):
    c = ctypes.c_int()
    assert F._lib.load().tucu_device_error(ctypes.byref(c)) == 0
    return c.value


def f16_ulp(x):
    """Spacing of f16 values at |x| (subnormal spacing below the normal range)."""
    a = np.maximum(np.abs(x), 2.0 ** -14)
    return 2.0 ** (np.floor(np.log2(a)) - 10)


def make_jobs(rng):
    jobs = []
    for i in range(22):
        rows = int(rng.integers(40, 900))
        cols = int(rng.integers(40, 1700))
        out = "f32" if i % 3 == 0 else "f16"
        if i % 2:
            w = int(rng.choice([1, 3, 5, 7, 15, 31, 33]))
            jobs.append(dict(op="box", rows=rows, cols=cols, out=out, w=w, norm=out == "f16" or i % 4 == 1,
                             shift=bool(i % 5 != 0)))
        else:
            sigma = float(rng.choice([1.0, 2.0, 3.0, 4.0, 8.0]))
            jobs.append(dict(op="gauss", rows=rows, cols=cols, out=out, sigma=sigma, gop=int(i // 2) % 6,
                             shift=bool(i % 5 != 0)))
    return jobs


def run_batch(F, jobs, srcs, tensor, cuda, fir_rows=0):
    import torch
    from tucuda_gb300.batch import Batch
    b = Batch(tensor=tensor)
    outs = []
    for j, src in zip(jobs, srcs):
        o = torch.full(src.shape, 5, dtype=torch_dtype(j["out"]), device=cuda)
        if j["op"] == "gauss":
            b.add_gauss(src, o, j["sigma"], j["gop"], j["shift"])
        else:
            b.add_box(src, o, j["w"], j["w"], j["norm"], j["shift"])
        outs.append(o)
    b.plan(fir_rows, 0)
    b.launch()
    torch.cuda.synchronize()
    return b, [o.float().cpu().numpy() for o in outs]


@pytest.mark.parametrize("fir_rows", [0, 96, 1024])
def test_tensor_batch_matches_exact_path(F, cuda, fir_rows):
    rng = np.random.default_rng(21 + fir_rows)
    jobs = make_jobs(rng)
    srcs = []
    for j in jobs:
        img = (rng.random((j["rows"], j["cols"])) * 255).astype(np.float32)
        pad = (-j["cols"]) % 8 + 8 * int(rng.integers(0, 3))  # rows on 16-byte boundaries
        srcs.append(to_device(img, "f16", cuda, pad=pad))
    bt, tc_out = run_batch(F, jobs, srcs, True, cuda, fir_rows)
    assert bt.info()["kernels"] == 2  # one tensor-core class per output type, nothing else
    _, ex_out = run_batch(F, jobs, srcs, False, cuda, fir_rows)
    assert device_error(F) == 0
    for j, a, e in zip(jobs, tc_out, ex_out):
        # whole images: pixels outside the valid region keep the fill value 5 in both
        scale = max(float(np.abs(e).max()), 1.0)
        if j["out"] == "f16":
            # one output rounding apart, plus the paths' difference before it:
            # FP32 rounding of partial sums of the size of the pixels (255),
            # which matters for the small values of derivative outputs
            assert np.all(np.abs(a - e) <= f16_ulp(e) + 2e-3), (j, np.abs(a - e).max())
            if j["op"] == "box" or j["gop"] == 0:
                assert np.mean(a != e) < 0.02, j
        else:
            assert np.abs(a - e).max() <= 2e-5 * scale, (j, np.abs(a - e).max(), scale)


@pytest.mark.parametrize("shape,op", [
    ((33, 33), ("gauss", 8.0)),      # one output pixel (33 taps each way)
    ((40, 4000), ("gauss", 1.0)),    # one strip row band, 32 column strips
    ((3000, 40), ("box", 33)),       # a single partial column strip, tall
    ((200, 300), ("box", 1)),        # 1 x 1 windows (one tap)
    ((129, 136), ("box", 2)),        # even window
    ((257, 520), ("gauss", 3.0)),
])
def test_tensor_batch_edge_shapes(F, cuda, shape, op):
    """Edge geometries on the tensor-core path against the exact path:
    single-pixel outputs, strips narrower than 128 columns, one tap, even
    windows, bands that end inside a 64-row chunk."""
    rng = np.random.default_rng(sum(shape))
    img = (rng.random(shape) * 255).astype(np.float32)
    src = to_device(img, "f16", cuda, pad=(-shape[1]) % 8)
    if op[0] == "gauss":
        jobs = [dict(op="gauss", out="f32", sigma=op[1], gop=0, shift=True)]
    else:
        jobs = [dict(op="box", out="f32", w=op[1], norm=False, shift=True)]
    bt, tc_out = run_batch(F, jobs, [src], True, cuda, 64)
    assert bt.info()["kernels"] == 1
    _, ex_out = run_batch(F, jobs, [src], False, cuda, 64)
    assert device_error(F) == 0
    scale = max(float(np.abs(ex_out[0]).max()), 1.0)
    assert np.abs(tc_out[0] - ex_out[0]).max() <= 2e-5 * scale
    assert np.array_equal(tc_out[0] == 5, ex_out[0] == 5)


def test_tensor_batch_error_vs_fp64(F, oracle, cuda):
    """Gaussian smooth sigma 8 and 15x15 box means of a 1080 x 1920 f16 image
    of U[0,255): the tensor path's error against the FP64 oracle is the f16
    output rounding (relative RMS ~2.2e-4, bar 1e-3), like the exact path's."""
    import torch
    rng = np.random.default_rng(5)
    img = (rng.random((1080, 1920)) * 255).astype(np.float16)
    src = torch.from_numpy(img).to(cuda)
    x = img.astype(np.float64)
    jobs = [dict(op="gauss", out="f16", sigma=8.0, gop=0, shift=True),
            dict(op="box", out="f16", w=15, norm=True, shift=True)]
    _, tc_out = run_batch(F, jobs, [src, src], True, cuda)
    _, ex_out = run_batch(F, jobs, [src, src], False, cuda)
    l0 = oracle.gauss_lobes_f64(8.0)[0]
    _, g_ref = oracle.fir_f64(x, l0, l0)
    r = len(l0) & ~1
    _, b_ref = oracle.box_f64(x, 15, 15)
    b_ref = b_ref / 225.0
    for out_tc, out_ex, ref, v in [(tc_out[0], ex_out[0], g_ref, (slice(r, 1080 - r), slice(r, 1920 - r))),
                                   (tc_out[1], ex_out[1], b_ref, (slice(7, 1073), slice(7, 1913)))]:
        e_tc, e_ex = rel_rms(out_tc[v], ref[v]), rel_rms(out_ex[v], ref[v])
        assert e_tc < 1e-3 and abs(e_tc - e_ex) < 1e-5, (e_tc, e_ex)
        assert np.abs(out_tc[v] - ref[v]).max() < 0.07


def test_tensor_batch_leaves_unaligned_jobs_exact(F, cuda):
    """A job whose rows are not on 16-byte boundaries cannot be described by
    the tensor-core path's TMA map: it keeps the FP32-pipe kernel (bit-equal)."""
    rng = np.random.default_rng(8)
    img = (rng.random((300, 517)) * 255).astype(np.float32)
    src = to_device(img, "f16", cuda)  # 1034-byte rows
    jobs = [dict(op="gauss", out="f16", sigma=2.0, gop=0, shift=True)]
    bt, tc_out = run_batch(F, jobs, [src], True, cuda)
    _, ex_out = run_batch(F, jobs, [src], False, cuda)
    assert np.array_equal(tc_out[0], ex_out[0])
    assert bt.info()["kernels"] == 1


def test_tensor_batch_reports_f16_overflow(F, cuda):
    """31 x 31 window sums of pixels near the f16 maximum: each horizontal sum
    exceeds 65504, so the f16 hi/lo pair cannot carry it; the kernel flags
    device error 2 instead of writing silently wrong sums unreported."""
    import torch
    device_error(F)  # clear
    src = torch.full((256, 512), 60000.0, dtype=torch.float16, device=cuda)
    jobs = [dict(op="box", out="f32", w=31, norm=False, shift=True)]
    run_batch(F, jobs, [src], True, cuda)
    assert device_error(F) == 2
    assert device_error(F) == 0
