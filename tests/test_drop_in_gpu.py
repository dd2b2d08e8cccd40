"""The C++ drop-in classes (include/TU/cu/*.h, the reference's TU::cu class
names over the C ABI), driven by tests/cpp/drop_in_test.cpp the way code
written for the reference calls them: each output equals the Python path's
output for the same input bit for bit (same kernels; the C++ layer only has
to get the geometry, pitches, types and flags right), pixels outside the
valid region are untouched, and the error behaviour holds (checked inside
the program)."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "tucuda_gb300", "lib", "tucu_drop_in_test")
NP = {0: np.uint8, 1: np.float16, 3: np.float32, 4: np.int32}


def load(d, name):
    with open(os.path.join(d, name + ".bin"), "rb") as f:
        rows, cols, dt = np.frombuffer(f.read(12), np.int32)
        a = np.frombuffer(f.read(), NP[int(dt)]).reshape(rows, cols, -1)
        return (a[..., 0] if a.shape[-1] == 1 else a).copy()


@pytest.fixture(scope="module")
def outputs(tmp_path_factory):
    if not os.path.exists(EXE):
        pytest.fail("tucu_drop_in_test is not built (run __graft_entry__.build())")
    d = str(tmp_path_factory.mktemp("drop_in"))
    r = subprocess.run([EXE, d], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    return d


def run_py(F, cuda, fn, inp, out_dtype, fill):
    import torch
    src = torch.from_numpy(inp).to(cuda)
    out = torch.full(inp.shape, fill, dtype=out_dtype, device=cuda)
    fn(src, out)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_gaussian(F, cuda, outputs):
    import torch
    g_in = load(outputs, "g_in")
    g = F.FIRGaussianConvolver2(2.0)
    sm = run_py(F, cuda, lambda s, o: g.smooth(s, o), g_in, torch.float32, -1.0)
    dh = run_py(F, cuda, lambda s, o: g.diffH(s, o, False), g_in, torch.float32, -1.0)
    assert np.array_equal(load(outputs, "g_smooth").view(np.uint32), sm.view(np.uint32))
    assert np.array_equal(load(outputs, "g_diffh_noshift").view(np.uint32), dh.view(np.uint32))


def test_fir_filter(F, cuda, outputs):
    import torch
    f_in = load(outputs, "f_in")
    f = F.FIRFilter2()
    f.initialize([0.05, 0.1, 0.2, 0.25, 0.4], [-0.1, -0.2, -0.3, -0.4])
    out = run_py(F, cuda, lambda s, o: f.convolve(s, o), f_in, torch.float32, -1.0)
    got = load(outputs, "f_out")
    assert np.array_equal(got.view(np.uint32), out.view(np.uint32))
    assert (got[:4] == -1.0).all() and (got[:, :4] == -1.0).all()


def test_box_sums(F, cuda, oracle, outputs):
    import torch
    b_in = load(outputs, "b_in")
    got = load(outputs, "b_out")
    b = F.BoxFilter2(15, 15, 31)
    out = run_py(F, cuda, lambda s, o: b.convolve(s, o), b_in, torch.int32, -7)
    assert np.array_equal(got, out)
    _, ref = oracle.box_i64(b_in.astype(np.int32), 15, 15)
    m = np.zeros(b_in.shape, bool)
    m[7:7 + 286, 7:7 + 387] = True
    assert np.array_equal(got[m].astype(np.int64), ref[m]) and (got[~m] == -7).all()


def test_guided(F, cuda, outputs):
    import torch
    p, gd = load(outputs, "p"), load(outputs, "gd")
    gf = F.GuidedFilter2(17, 17, 25.5, wmax=23)
    g_t = torch.from_numpy(gd).to(cuda)
    o1 = run_py(F, cuda, lambda s, o: gf.convolve(s, g_t, o), p, torch.float32, -3.0)
    o2 = run_py(F, cuda, lambda s, o: gf.convolve(s, None, o), p, torch.float32, -3.0)
    assert np.array_equal(load(outputs, "o_guided").view(np.uint32), o1.view(np.uint32))
    assert np.array_equal(load(outputs, "o_self").view(np.uint32), o2.view(np.uint32))


def test_extrema(F, cuda, oracle, outputs):
    import torch
    b_in = load(outputs, "b_in")
    val, pos = load(outputs, "e_val"), load(outputs, "e_pos")
    assert pos.shape == b_in.shape + (2,)
    f = F.ExtremaFilter2(7, 9)
    src = torch.from_numpy(b_in).to(cuda)
    v = torch.full(b_in.shape, 200, dtype=torch.uint8, device=cuda)
    p = torch.full(b_in.shape + (2,), -5, dtype=torch.int32, device=cuda)
    f.convolve(src, v, p)
    torch.cuda.synchronize()
    assert np.array_equal(val, v.cpu().numpy()) and np.array_equal(pos, p.cpu().numpy())
    rv, rp = oracle.extrema(b_in.astype(np.float64), 7, 9)
    m = ~np.isnan(rv)
    assert np.array_equal(val[m].astype(np.float64), rv[m]) and np.array_equal(pos[m], rp[m])
    assert (val[~m] == 200).all() and (pos[~m] == -5).all()
    # BoxFilter2<extrema_finder<extrema_value<less>>>: the same minima alone
    assert np.array_equal(load(outputs, "e_val2"), val)


def test_stereo_costs(F, cuda, oracle, outputs):
    import torch
    L, R = load(outputs, "b_in"), load(outputs, "s_right")
    got = load(outputs, "s_costs").reshape(16, 300, 401)
    b = F.BoxFilter2(7, 7, 31)
    c = torch.zeros(16, 300, 401, dtype=torch.int32, device=cuda)
    b.convolve_stereo(torch.from_numpy(L).to(cuda), torch.from_numpy(R).to(cuda), c, 50)
    torch.cuda.synchronize()
    assert np.array_equal(got, c.cpu().numpy())
    ref = oracle.stereo(L.astype(np.float64), R.astype(np.float64), 7, 7, 50, 16)
    m = ~np.isnan(ref)
    assert np.array_equal(got[m].astype(np.float64), ref[m]) and (got[~m] == 0).all()


def test_tensor_core_switch(F, cuda, outputs):
    """FIRGaussianConvolver2<float>(8).setTensorCores(true).smooth on an f16
    Array2 (rows of 1280 bytes): the tensor-core kernel, within a few FP32 ulps
    of the image's scale of the exact call, the same pixels written."""
    import torch
    t_in, t_out = load(outputs, "t_in"), load(outputs, "t_out")
    ref = run_py(F, cuda, lambda s, o: F.FIRGaussianConvolver2(8.0).smooth(s, o), t_in,
                 torch.float32, -1.0)
    assert np.array_equal(t_out == -1.0, ref == -1.0)
    assert np.abs(t_out - ref).max() <= 2e-5 * np.abs(ref).max()


def test_disparity_selector(oracle, outputs):
    """TU::cu::DisparitySelector<int32_t>(40, 2) over the drop-in stereo costs
    (294 x 395 valid region) into a 300 x 401 image from (3, 3)."""
    costs = load(outputs, "s_costs").reshape(16, 300, 401)
    got = load(outputs, "s_disp")
    ref = oracle.select_disparity(costs[:, :294, :395].astype(np.float64), 40, 2)
    assert np.array_equal(got[3:297, 3:398], ref.astype(np.int32))
    assert (got[:3] == 0).all() and (got[:, :3] == 0).all() and (got[297:] == 0).all()


def test_vector_box(F, cuda, outputs):
    import torch
    vin, vout = load(outputs, "v_in"), load(outputs, "v_out")
    assert vin.shape == (120, 333, 4)
    b = F.BoxFilter2(5, 9)
    x = torch.from_numpy(vin).to(cuda)
    y = torch.full_like(x, -1.0)
    b.convolve_vec(x, y)
    torch.cuda.synchronize()
    assert np.array_equal(vout.view(np.uint32), y.cpu().numpy().view(np.uint32))
    assert (vout[:2] == -1.0).all() and (vout[:, :4] == -1.0).all()
