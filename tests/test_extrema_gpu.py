"""Parity of the sliding-window extrema kernel (BoxFilter2 with
extrema_finder) with the oracle's restatement of the reference's deque
passes: values and (x, y) positions bit-exact for every storage type, both
operators, shift on and off, windows 1..64, ragged and pitched images."""
import numpy as np
import pytest

from helpers import to_device, torch_dtype

pytestmark = pytest.mark.gpu
SENT = 7


def run(F, img, dt, wV, wH, dev, op="min", shift=True, pad=0, want=("val", "pos"), wmax=64):
    import torch
    src = to_device(img, dt, dev, pad=pad)
    rows, cols = img.shape
    val = torch.full((rows, cols), SENT, dtype=torch_dtype(dt), device=dev) if "val" in want else None
    pos = torch.full((rows, cols, 2), -5, dtype=torch.int32, device=dev) if "pos" in want else None
    f = F.ExtremaFilter2(wV, wH, wmax)
    wrote = f.convolve(src, val, pos, shift, op)
    torch.cuda.synchronize()
    return wrote, val, pos


def image(rng, shape, dt, ties=False):
    if ties:
        return rng.integers(0, 3, shape).astype(np.float32)
    if dt == "u8":
        return rng.integers(0, 256, shape).astype(np.float32)
    if dt == "i32":
        return rng.integers(-(1 << 30), 1 << 30, shape).astype(np.float64)
    x = (rng.random(shape) * 510 - 255).astype(np.float32)
    if dt == "f16":
        return x.astype(np.float16).astype(np.float32)
    if dt == "bf16":
        import torch
        return torch.from_numpy(x).to(torch.bfloat16).float().numpy()
    return x


def check(oracle, img, wV, wH, op, shift, val, pos, dt):
    import torch
    rv, rp = oracle.extrema(img.astype(np.float64), wV, wH, op == "max", shift)
    m = ~np.isnan(rv)
    if val is not None:
        got = val.to(torch.float64 if dt != "i32" else torch.int64).cpu().numpy().astype(np.float64)
        assert np.array_equal(got[m], rv[m])
        assert np.all(got[~m] == SENT)  # nothing outside the valid region
    if pos is not None:
        gp = pos.cpu().numpy()
        assert np.array_equal(gp[m], rp[m])
        assert np.all(gp[~m] == -5)


@pytest.mark.parametrize("dt", ["u8", "f16", "bf16", "f32", "i32"])
@pytest.mark.parametrize("op", ["min", "max"])
def test_types_bit_exact(F, oracle, cuda, dt, op):
    rng = np.random.default_rng(len(dt) * 10 + (op == "max"))
    img = image(rng, (211, 389), dt)
    wrote, val, pos = run(F, img, dt, 15, 15, cuda, op)
    assert wrote
    check(oracle, img, 15, 15, op, True, val, pos, dt)


@pytest.mark.parametrize("wV,wH", [(1, 1), (1, 9), (9, 1), (2, 2), (3, 3), (7, 31), (31, 7),
                                   (33, 33), (17, 64), (64, 17), (64, 64)])
@pytest.mark.parametrize("shift", [True, False])
def test_windows_with_ties(F, oracle, cuda, wV, wH, shift):
    rng = np.random.default_rng(wV * 100 + wH)
    img = image(rng, (160, 300), "u8", ties=True)  # ties everywhere: position rule matters
    for op in ("min", "max"):
        wrote, val, pos = run(F, img, "u8", wV, wH, cuda, op, shift)
        assert wrote
        check(oracle, img, wV, wH, op, shift, val, pos, "u8")


@pytest.mark.parametrize("shape", [(32, 128), (46, 142), (33, 129), (95, 191), (1, 64), (64, 1),
                                   (500, 1000), (1080, 1920)])
def test_ragged_and_tile_edges(F, oracle, cuda, shape):
    rng = np.random.default_rng(shape[0] + shape[1])
    img = image(rng, shape, "f32")
    wV, wH = min(15, shape[0]), min(15, shape[1])
    wrote, val, pos = run(F, img, "f32", wV, wH, cuda, "min", True, pad=3)
    assert wrote
    check(oracle, img, wV, wH, "min", True, val, pos, "f32")


def test_single_outputs_and_pitches(F, oracle, cuda):
    rng = np.random.default_rng(5)
    img = image(rng, (77, 131), "f16", ties=True)
    for want in (("val",), ("pos",)):
        wrote, val, pos = run(F, img, "f16", 5, 6, cuda, "max", False, pad=5, want=want)
        assert wrote
        check(oracle, img, 5, 6, "max", False, val, pos, "f16")


def test_errors_and_noop(F, cuda):
    import torch
    from tucuda_gb300 import _lib
    with pytest.raises(_lib.TucuError) as e:
        F.ExtremaFilter2(3, 3, 65)
    assert e.value.status == _lib.ERR_WINDOW
    with pytest.raises(_lib.TucuError) as e:
        F.ExtremaFilter2(24, 3)  # above the default WMAX of 23
    assert e.value.status == _lib.ERR_WINDOW
    f = F.ExtremaFilter2(5, 5)
    x = torch.zeros(4, 40, dtype=torch.float32, device=cuda)
    out = torch.full_like(x, 3)
    assert f.convolve(x, out) is False  # smaller than the window: nothing written
    assert torch.all(out == 3)
    x = torch.zeros(40, 40, dtype=torch.float32, device=cuda)
    with pytest.raises(_lib.TucuError):
        f.convolve(x, None, None)
    with pytest.raises(ValueError):
        f.convolve(x, torch.zeros_like(x), op="median")
    code = ctypes_code(F)
    assert code == 0


def ctypes_code(F):
    import ctypes
    c = ctypes.c_int(-1)
    assert F._lib.load().tucu_device_error(ctypes.byref(c)) == 0
    return c.value


@pytest.mark.parametrize("op", ["min", "max"])
@pytest.mark.parametrize("wV,wH", [(15, 15), (1, 64), (64, 3), (7, 33)])
@pytest.mark.parametrize("ties", [False, True])
def test_u8_values_only(F, oracle, cuda, op, wV, wH, ties):
    # Values without positions run an instantiation that tracks no rows or
    # columns; its values equal the oracle's (and the positions run's).
    rng = np.random.default_rng(wV * 100 + wH + ties)
    img = image(rng, (157, 421), "u8", ties=ties)
    wrote, val, pos = run(F, img, "u8", wV, wH, cuda, op, True, pad=3, want=("val",))
    assert wrote and pos is None
    check(oracle, img, wV, wH, op, True, val, None, "u8")
    wrote2, val2, pos2 = run(F, img, "u8", wV, wH, cuda, op, True, pad=3)
    assert wrote2 and bool((val2 == val).all())
