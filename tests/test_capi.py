"""C-ABI boundary checks that need no GPU: the library loads, exports every
symbol include/*.h declares, and its host-only logic (lobe design, argument
and window checks, status text) behaves as the reference does."""
import ctypes
import glob
import json
import os
import re
import struct

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from tucuda_gb300 import _lib
    return _lib.load()


def declared_symbols():
    names = set()
    for path in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(path).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"\b(tucu_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_every_declared_symbol_is_exported(lib):
    names = declared_symbols()
    assert len(names) >= 30
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_python_prototypes_cover_the_header():
    from tucuda_gb300 import _lib
    assert declared_symbols() <= set(_lib.PROTOTYPES), declared_symbols() - set(_lib.PROTOTYPES)


def test_status_strings(lib):
    assert lib.tucu_status_string(0) == b"ok"
    assert b"window" in lib.tucu_status_string(-3)
    assert lib.tucu_version() >= 10000


def _design(lib, sigma):
    bufs = [(ctypes.c_float * 17)() for _ in range(3)]
    ns = [ctypes.c_int() for _ in range(3)]
    rc = lib.tucu_gauss_design(sigma, bufs[0], ctypes.byref(ns[0]), bufs[1], ctypes.byref(ns[1]),
                               bufs[2], ctypes.byref(ns[2]))
    return rc, [np.array(b[:n.value], np.float32) for b, n in zip(bufs, ns)]


def test_fp64_lobe_design_against_reference_fixture(lib):
    # The product designs coefficients in FP64 and rounds once; the lengths
    # must equal the reference's exactly and the values agree to 16 float ulps
    # of the lobe's largest coefficient: the reference's float normalisation
    # sums (17 terms for sigma >= 3) carry relative errors near 1e-6, and far
    # taps of small sigmas differ by more ulps of their own because the
    # reference's float exp argument is itself rounded (those taps are ~1e-20
    # of the peak).
    gold = json.load(open(os.path.join(ROOT, "tests", "golden", "ref_vectors.json")))
    f = lambda h: struct.unpack(">f", bytes.fromhex(h))[0]  # noqa: E731
    for case in gold["lobes"]:
        rc, mine = _design(lib, f(case["sigma"]))
        assert rc == 0
        for k in range(3):
            ref = np.array([f(h) for h in case[f"lobe{k}"]], np.float32)
            assert len(mine[k]) == len(ref)
            tol = 16 * np.finfo(np.float32).eps * np.abs(ref).max()
            assert np.abs(mine[k] - ref).max() <= tol, (case["sigma"], k, mine[k] - ref)


def test_reference_lobe_design_is_bit_exact(lib):
    # tucu_gauss_design_reference restates the reference's float design: every
    # length and every coefficient equals the lobes the reference's own
    # FIRGaussianConvolver2::initialize produced (the fixture), bit for bit.
    gold = json.load(open(os.path.join(ROOT, "tests", "golden", "ref_vectors.json")))
    f = lambda h: struct.unpack(">f", bytes.fromhex(h))[0]  # noqa: E731
    for case in gold["lobes"]:
        bufs = [(ctypes.c_float * 17)() for _ in range(3)]
        ns = [ctypes.c_int() for _ in range(3)]
        assert lib.tucu_gauss_design_reference(f(case["sigma"]), bufs[0], ctypes.byref(ns[0]), bufs[1],
                                               ctypes.byref(ns[1]), bufs[2], ctypes.byref(ns[2])) == 0
        for k in range(3):
            ref = np.array([f(h) for h in case[f"lobe{k}"]], np.float32)
            mine = np.array(bufs[k][:ns[k].value], np.float32)
            assert mine.tobytes() == ref.tobytes(), (case["sigma"], k)


def test_design_rejects_bad_sigma(lib):
    rc, _ = _design(lib, 0.0)
    assert rc == -1
    rc, _ = _design(lib, float("nan"))
    assert rc == -1


def test_fir_lobe_limits(lib):
    h = ctypes.c_void_p()
    assert lib.tucu_fir_create(ctypes.byref(h)) == 0
    lobe = (ctypes.c_float * 18)(*([0.1] * 18))
    # FIRFilter.h:250-251: more than 17 taps throws
    assert lib.tucu_fir_initialize(h, lobe, 18, lobe, 9) == -2
    assert b"too large lobe size" in lib.tucu_last_error()
    assert lib.tucu_fir_initialize(h, lobe, 9, lobe, 4) == 0
    v, hh = ctypes.c_int(), ctypes.c_int()
    assert lib.tucu_fir_offsets(h, ctypes.byref(v), ctypes.byref(hh)) == 0
    assert (v.value, hh.value) == (4, 8)
    lib.tucu_fir_destroy(h)


def test_box_and_guided_window_limits(lib):
    h = ctypes.c_void_p()
    # BoxFilter.h:464-480: WMAX=23 by default
    assert lib.tucu_box_create(24, 3, 0, ctypes.byref(h)) == -3
    assert lib.tucu_box_create(23, 23, 0, ctypes.byref(h)) == 0
    assert lib.tucu_box_set_window(h, 31, 31) == -3
    v, hh = ctypes.c_int(), ctypes.c_int()
    assert lib.tucu_box_offsets(h, ctypes.byref(v), ctypes.byref(hh)) == 0
    assert (v.value, hh.value) == (11, 11)
    lib.tucu_box_destroy(h)
    assert lib.tucu_box_create(31, 31, 64, ctypes.byref(h)) == 0
    lib.tucu_box_destroy(h)
    g = ctypes.c_void_p()
    assert lib.tucu_guided_create(17, 17, 25.5, 0, ctypes.byref(g)) == 0
    assert lib.tucu_guided_offsets(g, ctypes.byref(v), ctypes.byref(hh)) == 0
    assert (v.value, hh.value) == (16, 16)
    assert abs(lib.tucu_guided_epsilon(g) - 25.5) < 1e-6
    lib.tucu_guided_destroy(g)


def test_null_arguments_are_rejected(lib):
    assert lib.tucu_fir_create(None) == -1
    assert lib.tucu_fir_convolve(None, None, 0, 1, 1, 3, None, 0, 3, 1, None) == -1
    h = ctypes.c_void_p()
    assert lib.tucu_box_create(3, 3, 0, ctypes.byref(h)) == 0
    assert lib.tucu_box_convolve(h, None, 16, 4, 4, 0, None, 16, 4, 1, 0, None) == -1
    assert lib.tucu_box_convolve(h, ctypes.c_void_p(16), 16, 4, 4, 9, ctypes.c_void_p(16), 16, 4,
                                 1, 0, None) == -4
    lib.tucu_box_destroy(h)
