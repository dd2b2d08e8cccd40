"""The library's kernels against the reference's own device code run on a
GB300 (tests/golden/ref_device_vectors.json, made by
tests/golden/make_ref_device.py from oracle/ref_device.cu), on the fixture's
inputs through the public API:

- FIR (FIRFilter2, float32): each row of taps within one float epsilon of the
  sum of |tap x pair| of the reference's (nvcc fuses the first two terms the
  other way round), and bit-equal to the oracle's;
- integer box sums (BoxFilter2, int32 input): bit-equal down a 16-row tile
  (window wV x 1); float box sums: both within the box filter's general bar
  against FP64;
- window minima and maxima (ExtremaFilter2): bit-equal, ties included, and
  the row each one came from equal to the reference's (the earliest of tied
  values)."""
import json
import os
import sys

import numpy as np
import pytest

from helpers import to_device

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "ref_device_vectors.json")


@pytest.fixture(scope="module")
def ref():
    sys.path.insert(0, os.path.join(HERE, "golden"))
    from make_ref_device import unpack
    with open(FIXTURE) as f:
        data = json.load(f)
    return data, {k: unpack(v) for k, v in data["inputs"].items()}, unpack


def test_fir_rows_against_the_reference(F, oracle, cuda, ref):
    import torch
    data, inputs, unpack = ref
    eps = float(np.finfo(np.float32).eps)
    for c in (c for c in data["cases"] if c["kind"] == "fir"):
        lobe, row = unpack(c["lobe"]), inputs[c["in"]]
        LS = lobe.size & ~1
        img = np.zeros((5, row.size), np.float32)
        img[2] = row
        src = to_device(img, "f32", cuda)
        out = torch.full(img.shape, -7.0, device=cuda)
        f = F.FIRFilter2()
        f.initialize(lobe, np.array([0, 0, 1], np.float32))  # identity vertical lobe
        assert f.convolve(src, out, False)
        torch.cuda.synchronize()
        got = out.cpu().numpy()[0, : row.size - 2 * LS].astype(np.float64)
        want = unpack(c["fma"]).astype(np.float64)
        r = row.astype(np.float64)
        n = row.size - 2 * LS
        scale = np.zeros(n)
        for k in range(LS):
            pair = (r[k:k + n] + r[2 * LS - k:2 * LS - k + n]) if lobe.size % 2 else \
                   (r[k:k + n] - r[2 * LS - k:2 * LS - k + n])
            scale += np.abs(float(lobe[k]) * pair)
        if lobe.size % 2:
            scale += np.abs(float(lobe[LS]) * r[LS:LS + n])
        assert np.all(np.abs(got - want) <= eps * scale), (c["name"], c["sigma"])
        _, mine = oracle.fir_f32(img, lobe, np.array([0, 0, 1], np.float32), shift=False)
        assert np.array_equal(got, mine[0, :n].astype(np.float64)), (c["name"], c["sigma"])


def test_box_tiles_against_the_reference(F, cuda, ref):
    import torch
    data, inputs, unpack = ref
    for c in (c for c in data["cases"] if c["kind"] == "box"):
        tile = inputs[c["in"]][: c["rows"]]
        integral = c["kernel"].endswith("i32")
        src = to_device(tile, "i32" if integral else "f32", cuda)
        out = torch.full(tile.shape, -7, dtype=torch.int32 if integral else torch.float32, device=cuda)
        assert F.BoxFilter2(c["w"], 1, 129).convolve(src, out, False, False)
        torch.cuda.synchronize()
        got = out.cpu().numpy()[:16]
        want = unpack(c["out"])
        if integral:
            assert np.array_equal(got, want), (c["in"], c["w"])
        else:
            exact = np.array([[tile[y:y + c["w"], x].astype(np.float64).sum() for x in range(32)]
                              for y in range(16)])
            # Both within the box filter's general bar against FP64 (a few ulp
            # of prefix sums of at most 128 column sums); they need not agree
            # bit for bit: the reference's running sums take a rounding per row
            # of its tile, this library's window one column wide is the
            # difference of two prefix sums across the warp (both about 1e-4
            # relative on the small sums here; the 1e-5 relative bar is for
            # windows of 7 x 7 and more).
            bound = 2.0 ** -20 * 128 * c["w"] * 255
            assert np.max(np.abs(want - exact)) <= bound, c["w"]
            assert np.max(np.abs(got - exact)) <= bound, c["w"]


def test_extrema_tiles_against_the_reference(F, cuda, ref):
    import torch
    data, inputs, unpack = ref
    for c in (c for c in data["cases"] if c["kind"] == "ext"):
        tile = inputs[c["in"]][: c["rows"]]
        src = to_device(tile, "f32", cuda)
        val = torch.full(tile.shape, 7.0, device=cuda)
        op = "max" if "max" in c["kernel"] else "min"
        assert F.ExtremaFilter2(c["w"], 1, 64).convolve(src, val, None, False, op)
        torch.cuda.synchronize()
        assert np.array_equal(val.cpu().numpy()[:16], unpack(c["out"])), (c["in"], op, c["w"])
    for c in (c for c in data["cases"] if c["kind"] == "arg"):
        tile = inputs[c["in"]][: c["rows"]]
        src = to_device(tile, "f32", cuda)
        pos = torch.full(tile.shape + (2,), -5, dtype=torch.int32, device=cuda)
        op = "max" if "max" in c["kernel"] else "min"
        assert F.ExtremaFilter2(c["w"], 1, 64).convolve(src, None, pos, False, op)
        torch.cuda.synchronize()
        p = pos.cpu().numpy()[:16]
        assert np.array_equal(p[..., 1], unpack(c["row"])), (c["in"], op, c["w"])
        assert np.array_equal(p[..., 0], np.broadcast_to(np.arange(32), (16, 32)))
