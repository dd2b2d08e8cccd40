"""Parity of the fused FIR / Gaussian kernels with the CPU oracle.

The oracle evaluates each output in the kernel's order (pairs outermost
first, FMA-fused, centre last -- the reference's device::convolve with its
sums contracted to FMAs), so float32 outputs must be BIT-EXACT, and outputs
stored as u8/f16/bf16 must equal the oracle's float result rounded the same
way.  Error against the FP64 oracle is checked with stated bounds.
"""
import numpy as np
import pytest

from helpers import quantise_input, rel_rms, to_device, to_numpy_f32

pytestmark = pytest.mark.gpu

SENTINEL = 77


def run_fir(F, lh, lv, img, in_dt, out_dt, dev, shift=True, pad=0, offset=0):
    import torch
    from helpers import torch_dtype
    src = to_device(img, in_dt, dev, pad=pad, offset=offset)
    out = torch.full(img.shape, SENTINEL, dtype=torch_dtype(out_dt), device=dev)
    f = F.FIRFilter2().initialize(lh, lv)
    wrote = f.convolve(src, out, shift)
    torch.cuda.synchronize()
    return wrote, out


def expected(oracle, img, lh, lv, in_dt, out_dt, shift=True):
    q = quantise_input(img, in_dt)
    st, ref = oracle.fir_f32(q, lh, lv, shift=shift)
    return st, ref


def check_region(oracle, got, ref, lh, lv, out_dt, shift, shape):
    rows, cols = shape
    rv, rh = len(lv) & ~1, len(lh) & ~1
    oy, ox = (rv, rh) if shift else (0, 0)
    orows, ocols = rows - 2 * rv, cols - 2 * rh
    g = to_numpy_f32(got)
    mask = np.zeros(shape, bool)
    mask[oy:oy + orows, ox:ox + ocols] = True
    want = oracle.round_to(ref, out_dt)
    if out_dt == "f32":
        assert np.array_equal(g[mask].view(np.uint32), want[mask].view(np.uint32)), \
            np.abs(g[mask] - want[mask]).max()
    else:
        assert np.array_equal(g[mask], want[mask]), np.abs(g[mask] - want[mask]).max()
    assert (g[~mask] == SENTINEL).all(), "pixels outside the valid region were written"


LOBE_LENS = [2, 3, 4, 5, 8, 9, 16, 17]


@pytest.mark.parametrize("LH", LOBE_LENS)
@pytest.mark.parametrize("LV", [3, 8, 17])
def test_all_lobe_lengths_f32_bit_exact(F, oracle, cuda, LH, LV):
    rng = np.random.default_rng(LH * 100 + LV)
    lh = rng.normal(0, 0.3, LH).astype(np.float32)
    lv = rng.normal(0, 0.3, LV).astype(np.float32)
    img = (rng.random((157, 203)) * 255).astype(np.float32)
    wrote, out = run_fir(F, lh, lv, img, "f32", "f32", cuda)
    assert wrote
    st, ref = expected(oracle, img, lh, lv, "f32", "f32")
    check_region(oracle, out, ref, lh, lv, "f32", True, img.shape)


@pytest.mark.parametrize("in_dt", ["u8", "f16", "bf16", "f32"])
@pytest.mark.parametrize("out_dt", ["u8", "f16", "bf16", "f32"])
def test_dtypes_gaussian_smooth(F, oracle, cuda, in_dt, out_dt):
    rng = np.random.default_rng(7)
    img = (rng.random((130, 300)) * 255).astype(np.float32)
    g = F.FIRGaussianConvolver2(2.0)
    l0, _, _ = g.lobes()
    wrote, out = run_fir(F, l0, l0, img, in_dt, out_dt, cuda)
    assert wrote
    st, ref = expected(oracle, img, l0, l0, in_dt, out_dt)
    check_region(oracle, out, ref, l0, l0, out_dt, True, img.shape)


@pytest.mark.parametrize("shape", [(33, 35), (34, 34), (40, 65), (97, 63), (64, 64), (300, 129),
                                   (1, 1), (2, 500), (500, 2)])
@pytest.mark.parametrize("shift", [True, False])
def test_ragged_shapes_and_noop(F, oracle, cuda, shape, shift):
    rng = np.random.default_rng(sum(shape))
    img = (rng.random(shape) * 255).astype(np.float32)
    l0, l1, _ = F.FIRGaussianConvolver2(4.0).lobes()    # radius 16 both ways
    wrote, out = run_fir(F, l1, l0, img, "f32", "f32", cuda, shift=shift)
    st, ref = expected(oracle, img, l1, l0, "f32", "f32", shift=shift)
    assert wrote == (st == 0)
    if st == 0:
        check_region(oracle, out, ref, l1, l0, "f32", shift, shape)
    else:
        assert (to_numpy_f32(out) == SENTINEL).all()


@pytest.mark.parametrize("pad,offset", [(0, 1), (3, 0), (5, 3), (16, 0)])
@pytest.mark.parametrize("in_dt", ["u8", "f32"])
def test_unaligned_pitch_and_base(F, oracle, cuda, pad, offset, in_dt):
    # Rows that are not 16-byte aligned cannot be described to TMA; the
    # kernel then stages with plain loads.  Results must not change.
    rng = np.random.default_rng(pad * 10 + offset)
    img = (rng.random((77, 91)) * 255).astype(np.float32)
    l0, l1, l2 = F.FIRGaussianConvolver2(1.5).lobes()
    wrote, out = run_fir(F, l2, l1, img, in_dt, "f32", cuda, pad=pad, offset=offset)
    assert wrote
    st, ref = expected(oracle, img, l2, l1, in_dt, "f32")
    check_region(oracle, out, ref, l2, l1, "f32", True, img.shape)


@pytest.mark.parametrize("sigma", [1.0, 2.0, 2.25, 3.0, 8.0])
def test_six_gaussian_operators_and_multi(F, oracle, cuda, sigma):
    import torch
    rng = np.random.default_rng(int(sigma * 100))
    img = (rng.random((150, 170)) * 255).astype(np.float32)
    g = F.FIRGaussianConvolver2(sigma)
    lobes = g.lobes()
    src = to_device(img, "f32", cuda)
    singles = {}
    for op, name in enumerate(F.FIRGaussianConvolver2.OPS):
        out = torch.full(img.shape, SENTINEL, dtype=torch.float32, device=cuda)
        assert getattr(g, name)(src, out)
        lh, lv = (lobes[i] for i in oracle.GAUSS_OP_LOBES[op])
        st, ref = oracle.fir_f32(img, lh, lv)
        torch.cuda.synchronize()
        check_region(oracle, out, ref, lh, lv, "f32", True, img.shape)
        singles[op] = to_numpy_f32(out)
    outs = {op: torch.full(img.shape, SENTINEL, dtype=torch.float32, device=cuda)
            for op in range(6)}
    assert g.convolve_multi(src, outs)
    torch.cuda.synchronize()
    for op in range(6):
        # equal to the single-operator result (zero padding of shorter lobes
        # can only change the sign of an exactly-zero result)
        assert np.array_equal(to_numpy_f32(outs[op]), singles[op]), op


def test_reference_lobes_bit_exact_for_golden_sigmas(F, oracle, cuda):
    # With the reference-lobe switch the handle designs its lobes in the
    # reference's float arithmetic: they equal the oracle's restatement of
    # FIRGaussianConvolver2::initialize (pinned bit for bit to the
    # reference's own output in test_oracle_golden / test_capi), and every
    # operator's f32 output equals the oracle's FP32 convolution with those
    # lobes bit for bit: the whole Gaussian path, lobes included, matches the
    # reference arithmetic.
    import json
    import os
    import struct
    import torch
    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "ref_vectors.json")))
    f = lambda h: struct.unpack(">f", bytes.fromhex(h))[0]  # noqa: E731
    rng = np.random.default_rng(26)
    img = (rng.random((80, 96)) * 255).astype(np.float32)
    src = to_device(img, "f32", cuda)
    for case in gold["lobes"]:
        sigma = f(case["sigma"])
        g = F.FIRGaussianConvolver2(sigma).set_reference_lobes(True)
        lobes = g.lobes()
        ref_lobes = oracle.gauss_lobes(sigma)
        for mine, ref in zip(lobes, ref_lobes):
            assert np.array(mine, np.float32).tobytes() == np.array(ref, np.float32).tobytes(), sigma
        for op, name in enumerate(F.FIRGaussianConvolver2.OPS):
            lh, lv = (lobes[i] for i in oracle.GAUSS_OP_LOBES[op])
            if img.shape[0] <= 2 * (len(lv) & ~1) or img.shape[1] <= 2 * (len(lh) & ~1):
                continue
            out = torch.full(img.shape, SENTINEL, dtype=torch.float32, device=cuda)
            assert getattr(g, name)(src, out)
            st, ref = oracle.fir_f32(img, lh, lv)
            torch.cuda.synchronize()
            check_region(oracle, out, ref, lh, lv, "f32", True, img.shape)


def test_config1_plain_smooth_640x480(F, oracle, cuda):
    # Plain Gaussian smoothing of one 640x480 float32 image, U[0,255), sigma=2
    # (radius 8, 17 taps): bit-exact with the oracle; error vs FP64 <= 1e-6.
    rng = np.random.default_rng(1)
    img = (rng.random((480, 640), dtype=np.float32) * 255).astype(np.float32)
    g = F.FIRGaussianConvolver2(2.0)
    l0 = g.lobes()[0]
    assert len(l0) == 9
    wrote, out = run_fir(F, l0, l0, img, "f32", "f32", cuda)
    st, ref = expected(oracle, img, l0, l0, "f32", "f32")
    check_region(oracle, out, ref, l0, l0, "f32", True, img.shape)
    d0 = oracle.gauss_lobes_f64(2.0)[0]
    _, ref64 = oracle.fir_f64(img.astype(np.float64), d0, d0)
    v = slice(8, 472), slice(8, 632)
    assert rel_rms(to_numpy_f32(out)[v], ref64[v]) < 1e-6


@pytest.mark.parametrize("storage,bound", [("f32", 1e-6), ("f16", 1e-3)])
def test_config2_derivatives_error_vs_fp64(F, oracle, cuda, storage, bound):
    # 1920x1080 planes, sigma=3 (radius 16 by the reference's rule), six
    # operators; relative RMS error against the FP64 oracle per output.
    import torch
    rng = np.random.default_rng(2)
    img = rng.integers(0, 256, (1080, 1920)).astype(np.float32)
    g = F.FIRGaussianConvolver2(3.0)
    src = to_device(img, "u8", cuda)
    outs = {op: torch.zeros(img.shape, dtype=torch.float32 if storage == "f32" else torch.float16,
                            device=cuda) for op in range(6)}
    g.convolve_multi(src, outs)
    torch.cuda.synchronize()
    d = oracle.gauss_lobes_f64(3.0)
    v = slice(16, 1064), slice(16, 1904)
    for op in range(6):
        lh, lv = (d[i] for i in oracle.GAUSS_OP_LOBES[op])
        _, ref = oracle.fir_f64(img.astype(np.float64), lh, lv)
        err = rel_rms(to_numpy_f32(outs[op])[v], ref[v])
        assert err < bound, (op, err)
