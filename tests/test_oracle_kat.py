"""Known-answer checks of the CPU oracle (no reference fixture involved)."""
import numpy as np
import pytest


@pytest.mark.parametrize("sigma", [0.5, 1.0, 2.0, 3.0, 4.0, 8.0])
def test_lobe0_normalised(oracle, sigma):
    l0, l1, l2 = oracle.gauss_lobes(sigma)
    assert abs(2 * l0[:-1].astype(np.float64).sum() + l0[-1] - 1.0) < 1e-6
    assert len(l0) % 2 == 1 and len(l1) % 2 == 0 and len(l2) % 2 == 1


def test_sigma_radii_match_reference_rule(oracle):
    # sigma=2 -> 9 taps per side incl. centre (radius 8); sigma=3 -> radius 16
    # (the reference's rule, not the radius 12 a continuous 4-sigma cut gives)
    assert [len(x) for x in oracle.gauss_lobes(1.0)] == [5, 4, 5]
    assert [len(x) for x in oracle.gauss_lobes(2.0)] == [9, 8, 9]
    assert [len(x) for x in oracle.gauss_lobes(3.0)] == [17, 16, 17]
    assert [len(x) for x in oracle.gauss_lobes(8.0)] == [17, 16, 17]


def test_fir_impulse_response_is_outer_product(oracle):
    l0, l1, _ = oracle.gauss_lobes(2.0)
    img = np.zeros((41, 43), np.float32)
    img[20, 21] = 1.0
    st, out = oracle.fir_f32(img, l1, l0, shift=True)
    assert st == 0
    # full kernels: symmetric lobe0, antisymmetric lobe1 (kernel tap d = lobe1[R-d])
    k0 = np.concatenate([l0, l0[-2::-1]])
    k1 = np.concatenate([l1, [0.0], -l1[::-1]])
    # correlation of an impulse gives the flipped kernel
    ref = np.outer(k0[::-1], k1[::-1])
    np.testing.assert_allclose(out[12:29, 13:30], ref, rtol=1e-6, atol=1e-9)


def test_fir_constant_and_ramp(oracle):
    l0, l1, l2 = oracle.gauss_lobes(2.0)
    const = np.full((50, 60), 100.0, np.float32)
    _, s = oracle.fir_f32(const, l0, l0)
    np.testing.assert_allclose(s[8:42, 8:52], 100.0, rtol=1e-6)
    _, d = oracle.fir_f32(const, l1, l0)
    assert np.abs(d[8:42, 8:52]).max() < 1e-4
    ramp = np.tile(np.arange(60, dtype=np.float32), (50, 1))
    _, d = oracle.fir_f32(ramp, l1, l0)
    # the reference's lobe1 norm leaves lb1[L] out of the sum, so the slope is
    # slightly above 1
    v = d[8:42, 8:52]
    assert np.allclose(v, v[0, 0]) and 0.99 < v[0, 0] < 1.05


def test_fir_noop_and_unsupported(oracle):
    l0, _, _ = oracle.gauss_lobes(2.0)
    st, out = oracle.fir_f32(np.ones((16, 100), np.float32), l0, l0)
    assert st == 1 and not out.any()            # rows <= 2*LS
    st, _ = oracle.fir_f32(np.ones((40, 40), np.float32), np.ones(6, np.float32), l0)
    assert st == -1


def test_box_known_answers(oracle):
    ones = np.ones((30, 40), np.int32)
    st, out = oracle.box_i64(ones, 7, 5, shift=True)
    assert st == 0
    assert (out[3:27, 2:38] == 35).all() and not out[:3].any() and not out[:, :2].any()
    rng = np.random.default_rng(0)
    img = rng.integers(0, 256, (33, 47)).astype(np.int32)
    _, out = oracle.box_i64(img, 4, 6, shift=False)
    ref = np.zeros_like(out)
    for y in range(30):
        for x in range(42):
            ref[y, x] = img[y:y + 4, x:x + 6].sum()
    assert np.array_equal(out, ref)
    _, f = oracle.box_f32(img.astype(np.float32), 4, 6, shift=False)
    np.testing.assert_allclose(f[:30, :42], ref[:30, :42], rtol=1e-6)
    st, _ = oracle.box_i64(img, 40, 3)
    assert st == 1


def test_guided_constant_and_fp64_agreement(oracle):
    const = np.full((40, 40), 77.0, np.float32)
    _, out = oracle.guided_f64(const, const, 5, 5, 2.0)
    np.testing.assert_allclose(out[4:36, 4:36], 77.0, rtol=1e-12)
    rng = np.random.default_rng(3)
    g = (rng.random((64, 70)) * 255).astype(np.float32)
    p = g + rng.normal(0, 25, g.shape).astype(np.float32)
    _, a = oracle.guided_f32(p, g, 7, 7, 25.5)
    _, b = oracle.guided_f64(p, g, 7, 7, 25.5)
    np.testing.assert_allclose(a[6:58, 6:64], b[6:58, 6:64], rtol=1e-4, atol=1e-2)
