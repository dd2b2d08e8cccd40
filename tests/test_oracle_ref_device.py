"""The oracle against the reference's own device code run on a GB300
(tests/golden/ref_device_vectors.json: tests/golden/make_ref_device.py ran
oracle/ref_device.cu, whose kernels call the reference's TU/cu/FIRFilter.h and
TU/cu/BoxFilter.h device functions compiled where they lie):

- FIR taps (FIRFilter.h:66-176) for random lobes of every accepted length and
  for the reference's own Gaussian lobes.  As nvcc compiles the expressions by
  default (FMA contraction), they equal the oracle's restatement of that order
  (fir_row_nvcc_f32: the second pair's product rounded, the outermost pair
  fused into it, then FMAs) bit for bit, which pins the pairing of the taps,
  the sign of the odd (antisymmetric) lobes and the order of the sums.  The
  oracle's FIR (fir_f32), which the FP32 kernels equal bit for bit, rounds the
  outermost product first and fuses the second pair into it: one rounding of
  that first step apart, within one float epsilon of the sum of |tap x pair|
  (1.3% of the outputs differ for the Gaussian lobes).  Built with -fmad=false
  the expressions land within a few epsilons of the same sum;
- the u8 store of fir_filterV (FIRFilter.h:207-231): the compiler's float ->
  unsigned char assignment of those taps equals the oracle's to_u8;
- box_convolver (BoxFilter.h:175-194) down the columns of one 16-row tile:
  int32 sums exact, float32 sums bit for bit with the oracle's box pass;
- extrema_finder with extrema_value (BoxFilter.h:196-233): the window minima
  and maxima equal the oracle's deque pass, ties included; with
  extrema_position, the row each one came from equals the oracle's, so the
  earliest of tied values wins as in the oracle."""
import json
import os

import numpy as np
import pytest

from oracle import oracle as orc

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "ref_device_vectors.json")


def _load():
    if not os.path.exists(FIXTURE):
        pytest.skip("tests/golden/ref_device_vectors.json not generated")
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    from make_ref_device import unpack
    with open(FIXTURE) as f:
        data = json.load(f)
    inputs = {k: unpack(v) for k, v in data["inputs"].items()}
    return data, inputs, unpack


def oracle_taps(row, lobe):
    """The oracle's FIR taps over one row: the H pass of a 5-row image whose
    middle row is `row`, through the identity V lobe (0, 0, 1), which passes
    each H result on unchanged."""
    img = np.zeros((5, row.size), np.float32)
    img[2] = row
    _, out = orc.fir_f32(img, lobe, np.array([0, 0, 1], np.float32), shift=False)
    return out[0, : row.size - 2 * (lobe.size & ~1)]


def cases(data, kind):
    return [c for c in data["cases"] if c["kind"] == kind]


def term_scale(row, lobe):
    """Per output, the sum of |tap x pair| (and |centre tap x centre|): the
    scale one rounding of a partial sum is measured against."""
    L = lobe.size
    LS, sym = L & ~1, L & 1
    n = row.size - 2 * LS
    r = row.astype(np.float64)
    s = np.zeros(n)
    for k in range(LS):
        pair = r[k:k + n] + r[2 * LS - k:2 * LS - k + n] if sym else r[k:k + n] - r[2 * LS - k:2 * LS - k + n]
        s += np.abs(float(lobe[k]) * pair)
    if sym:
        s += np.abs(float(lobe[LS]) * r[LS:LS + n])
    return s


def test_fir_taps_equal_the_reference_expressions():
    data, inputs, unpack = _load()
    fir = cases(data, "fir")
    assert len(fir) >= 8 + 15
    for c in fir:
        lobe = unpack(c["lobe"])
        got = unpack(c["fma"])
        assert np.array_equal(got, orc.fir_row_nvcc_f32(inputs[c["in"]], lobe)), (c["name"], c["sigma"])


def test_oracle_fir_within_one_rounding_of_the_reference():
    data, inputs, unpack = _load()
    eps = float(np.finfo(np.float32).eps)
    differ = total = 0
    for c in cases(data, "fir"):
        lobe, row = unpack(c["lobe"]), inputs[c["in"]]
        got = unpack(c["fma"]).astype(np.float64)
        mine = oracle_taps(row, lobe).astype(np.float64)
        assert np.all(np.abs(mine - got) <= eps * term_scale(row, lobe)), (c["name"], c["sigma"])
        if c["lobes"] == "gauss":
            differ += int((mine != got).sum())
            total += got.size
    assert differ < 0.05 * total


def test_fir_taps_without_contraction_within_ulps():
    data, inputs, unpack = _load()
    eps = float(np.finfo(np.float32).eps)
    for c in cases(data, "fir"):
        a, b = unpack(c["fma"]).astype(np.float64), unpack(c["nofma"]).astype(np.float64)
        # different roundings of the same sum of at most 17 products
        assert np.all(np.abs(a - b) <= 4 * eps * term_scale(inputs[c["in"]], unpack(c["lobe"]))), c["name"]


def test_odd_lobes_are_antisymmetric():
    """A sign error would flip every odd-lobe output: the reference's taps of
    an even-length lobe change sign when the row is mirrored."""
    data, inputs, unpack = _load()
    row = inputs["px"]
    for c in cases(data, "fir"):
        lobe = unpack(c["lobe"])
        if lobe.size % 2:
            continue
        fwd = orc.fir_row_nvcc_f32(row, lobe)
        rev = orc.fir_row_nvcc_f32(row[::-1].copy(), lobe)[::-1]
        scale = term_scale(row, lobe)
        assert np.all(np.abs(fwd + rev) <= 4 * np.finfo(np.float32).eps * scale), c["name"]
        assert np.array_equal(unpack(c["fma"]), fwd)


def test_u8_store_equals_the_oracle_rule():
    data, inputs, unpack = _load()
    u8 = cases(data, "fir_u8")
    assert u8
    seen = np.zeros(3, bool)  # negative, in range, above 255
    for c in u8:
        for var in ("fma", "nofma"):
            f, u = unpack(c[var]), unpack(c[var + "_u8"])
            assert np.array_equal(u, orc.to_u8(f)), (c["name"], var)
            seen |= [bool((f < 0).any()), bool(((f >= 0) & (f <= 255)).any()), bool((f > 255).any())]
        assert np.array_equal(unpack(c["fma"]), orc.fir_row_nvcc_f32(inputs[c["in"]], unpack(c["lobe"])))
    assert seen.all()


def test_box_convolver_sums():
    data, inputs, unpack = _load()
    box = cases(data, "box")
    assert len(box) == 18
    for c in box:
        tile = inputs[c["in"]][: c["rows"]]
        got = unpack(c["out"])
        assert c["builds_agree"], c
        if c["kernel"].endswith("i32"):
            _, want = orc.box_i64(tile, c["w"], 1, shift=False)
            assert np.array_equal(got.astype(np.int64), want[:16]), (c["in"], c["w"])
        else:
            want = orc.box_pass_f32(tile, c["w"])
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), c["w"]


def test_extrema_finder_values():
    data, inputs, unpack = _load()
    ext = cases(data, "ext")
    assert len(ext) == 20
    for c in ext:
        tile = inputs[c["in"]][: c["rows"]]
        is_max = "max" in c["kernel"]
        val, _ = orc.extrema(tile, c["w"], 1, is_max=is_max, shift=False)
        got = unpack(c["out"])
        assert c["builds_agree"], c
        assert np.array_equal(got.astype(np.float64), val[:16]), (c["in"], c["kernel"], c["w"])


def test_extrema_finder_positions():
    data, inputs, unpack = _load()
    arg = cases(data, "arg")
    assert len(arg) == 20
    ties = 0
    for c in arg:
        tile = inputs[c["in"]][: c["rows"]]
        is_max = "max" in c["kernel"]
        val, pos = orc.extrema(tile, c["w"], 1, is_max=is_max, shift=False)
        assert np.array_equal(unpack(c["val"]).astype(np.float64), val[:16]), (c["in"], c["w"])
        assert np.array_equal(unpack(c["row"]), pos[:16, :, 1]), (c["in"], c["kernel"], c["w"])
        if c["in"] == "ext_ties":
            win = np.lib.stride_tricks.sliding_window_view(tile, c["w"], axis=0)[:16]
            best = win.max(-1) if is_max else win.min(-1)
            ties += int(((win == best[..., None]).sum(-1) > 1).sum())
    assert ties > 1000  # windows holding the extremum more than once


def test_fixture_matches_the_harness_build():
    """When the harness has been built here, its cubins are the ones that made
    the fixture (a changed harness needs the fixture regenerated)."""
    import hashlib
    data, _, _ = _load()
    root = os.path.dirname(HERE)
    for var, name in (("fma", "ref_device.cubin"), ("nofma", "ref_device_nofma.cubin")):
        p = os.path.join(root, "oracle", "_ref", name)
        if not os.path.exists(p):
            pytest.skip("the device harness is not built here")
        assert hashlib.sha256(open(p, "rb").read()).hexdigest() == data["cubin_sha256"][var], name
