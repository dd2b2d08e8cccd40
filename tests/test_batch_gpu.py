"""The batched persistent launch: every output equals the single-image call
of the same filter (bit for bit) and the oracle; the CUDA-graph replay gives
the same result as the direct launch."""
import numpy as np
import pytest

from helpers import to_device, to_numpy_f32, torch_dtype

pytestmark = pytest.mark.gpu


def make_jobs(rng):
    jobs = []
    dts = ["u8", "f16", "bf16", "f32"]
    for i in range(24):
        rows = int(rng.integers(20, 700))
        cols = int(rng.integers(20, 1500))
        dt = dts[i % 4]
        if i % 3 == 2:
            w = int(rng.choice([3, 7, 15, 31]))
            jobs.append(dict(op="box", rows=rows, cols=cols, in_dt=dt,
                             out_dt="i32" if dt == "u8" and i % 2 else dt, w=w,
                             norm=not (dt == "u8" and i % 2), shift=bool(i % 2)))
        else:
            sigma = float(rng.choice([1.0, 2.0, 4.0, 8.0]))
            op = int(rng.choice([0, 3, 5])) if sigma != 2.25 else 0
            jobs.append(dict(op="gauss", rows=rows, cols=cols, in_dt=dt, out_dt=dt if dt != "u8" else "f32",
                             sigma=sigma, gop=op, shift=bool(i % 2)))
    return jobs


def test_batch_equals_single_calls(F, oracle, cuda):
    import torch
    from tucuda_gb300.batch import Batch
    rng = np.random.default_rng(11)
    jobs = make_jobs(rng)
    b = Batch()
    singles, batched = [], []
    for j in jobs:
        img = (rng.random((j["rows"], j["cols"])) * 255).astype(np.float32)
        src = to_device(img, j["in_dt"], cuda, pad=int(rng.integers(0, 9)))
        o1 = torch.full(img.shape, 5, dtype=torch_dtype(j["out_dt"]), device=cuda)
        o2 = torch.full(img.shape, 5, dtype=torch_dtype(j["out_dt"]), device=cuda)
        if j["op"] == "gauss":
            g = F.FIRGaussianConvolver2(j["sigma"])
            g.convolve(j["gop"], src, o1, j["shift"])
            b.add_gauss(src, o2, j["sigma"], j["gop"], j["shift"])
        else:
            f = F.BoxFilter2(j["w"], j["w"], 64)
            f.convolve(src, o1, j["shift"], j["norm"])
            b.add_box(src, o2, j["w"], j["w"], j["norm"], j["shift"])
        singles.append(o1)
        batched.append(o2)
    for fr, br in [(64, 32), (256, 128)]:
        for o in batched:
            o.fill_(5)
        b.plan(fr, br)
        b.launch(graph=False)
        torch.cuda.synchronize()
        for j, o1, o2 in zip(jobs, singles, batched):
            assert torch.equal(o1, o2), (j, fr, br)
        for o in batched:
            o.fill_(5)
        b.launch(graph=True)
        b.launch(graph=True)
        torch.cuda.synchronize()
        for j, o1, o2 in zip(jobs, singles, batched):
            assert torch.equal(o1, o2), ("graph", j)
    info = b.info()
    assert info["jobs"] == len(jobs) and info["items"] > len(jobs)
    code = F._lib.load()
    import ctypes
    c = ctypes.c_int(-1)
    assert code.tucu_device_error(ctypes.byref(c)) == 0 and c.value == 0


def test_batched_workload_spec_sample_matches_oracle(F, oracle, cuda):
    # a few images of the benchmark workload, FP16 storage, against the oracle
    import torch
    from tucuda_gb300 import workloads
    from tucuda_gb300.batch import Batch
    jobs = workloads.batched_spec(seed=4, n=256)[:10]
    b = Batch()
    srcs, outs = [], []
    for j in jobs:
        src = torch.empty(j.rows, j.cols, dtype=torch.float16, device=cuda)
        workloads.fill_uniform_(src, j.seed)
        out = torch.zeros_like(src)
        if j.op == "gauss":
            b.add_gauss(src, out, j.sigma)
        else:
            b.add_box(src, out, j.window, j.window, normalize=True)
        srcs.append(src)
        outs.append(out)
    b.plan()
    b.launch()
    torch.cuda.synchronize()
    for j, src, out in zip(jobs, srcs, outs):
        img = src.float().cpu().numpy()
        got = out.float().cpu().numpy()
        if j.op == "gauss":
            l0 = F.FIRGaussianConvolver2(j.sigma).lobes()[0]
            _, ref = oracle.fir_f32(img, l0, l0)
            r = len(l0) - 1
            v = (slice(r, j.rows - r), slice(r, j.cols - r))
            assert np.array_equal(got[v], oracle.round_to(ref, "f16")[v])
        else:
            w = j.window
            _, ref = oracle.box_f64(img.astype(np.float64), w, w)
            v = (slice(w // 2, w // 2 + j.rows + 1 - w), slice(w // 2, w // 2 + j.cols + 1 - w))
            want = (ref[v] / (w * w))
            assert np.max(np.abs(got[v] - want) / np.maximum(np.abs(want), 1)) < 2e-3


@pytest.mark.parametrize("chunks", [1, 3, 8])
def test_host_batch_equals_single_calls(F, cuda, chunks):
    # Jobs on host images (page-locked): copies in, filtering and copies out
    # overlap across groups; every valid output equals the single-image call
    # bit for bit, pixels outside the valid region keep the caller's values,
    # and a second run gives the same bits.
    import torch
    from tucuda_gb300.batch import HostBatch
    rng = np.random.default_rng(13)
    jobs = make_jobs(rng)[:14]
    hb = HostBatch(chunks=chunks)
    refs, houts = [], []
    for j in jobs:
        img = (rng.random((j["rows"], j["cols"])) * 255).astype(np.float32)
        src = to_device(img, j["in_dt"], cuda)
        ref = torch.full(img.shape, 5, dtype=torch_dtype(j["out_dt"]), device=cuda)
        hsrc = src.cpu().pin_memory()
        dsrc = torch.zeros_like(src)
        hdst = torch.full(img.shape, 5, dtype=torch_dtype(j["out_dt"])).pin_memory()
        ddst = torch.zeros(img.shape, dtype=torch_dtype(j["out_dt"]), device=cuda)
        if j["op"] == "gauss":
            F.FIRGaussianConvolver2(j["sigma"]).convolve(j["gop"], src, ref, j["shift"])
            hb.add_gauss(hsrc, dsrc, hdst, ddst, j["sigma"], j["gop"], j["shift"])
        else:
            F.BoxFilter2(j["w"], j["w"], 64).convolve(src, ref, j["shift"], j["norm"])
            hb.add_box(hsrc, dsrc, hdst, ddst, j["w"], j["w"], j["norm"], j["shift"])
        refs.append(ref)
        houts.append(hdst)
    hb.plan()
    info = hb.info()
    assert info["jobs"] == len(jobs) and info["groups"] == min(chunks, len(jobs))
    first = None
    for run in range(2):
        hb.run()
        torch.cuda.synchronize()
        got = [h.view(torch.uint8).numpy().copy() for h in houts]
        for j, ref, g in zip(jobs, refs, got):
            assert np.array_equal(ref.cpu().view(torch.uint8).numpy(), g), j
        if first is not None:
            assert all(np.array_equal(a, b) for a, b in zip(first, got))
        first = got


@pytest.mark.parametrize("chunks", [1, 4])
def test_host_batch_spans(F, cuda, chunks):
    # Host slabs that mirror the device slabs (same offsets and pitches): with
    # span copies each group moves as one range per direction, every valid
    # output still equals the single-image call, the info reports the span
    # bytes, and jobs whose host images lie elsewhere fall back to pitched
    # copies of their own.
    import torch
    from tucuda_gb300.batch import HostBatch
    rng = np.random.default_rng(17)
    jobs = [j for j in make_jobs(rng) if j["in_dt"] == "f16" and j["out_dt"] == "f16"][:6]
    jobs += [dict(op="gauss", rows=300, cols=410, in_dt="f16", out_dt="f16", sigma=2.0, gop=0, shift=True)]
    layout, off = [], 0
    for j in jobs:
        pitch = (j["cols"] * 2 + 127) // 128 * 128
        layout.append((off, pitch))
        off += (pitch * j["rows"] + 255) // 256 * 256
    d_in = torch.zeros(off // 2, dtype=torch.float16, device=cuda)
    d_out = torch.zeros(off // 2, dtype=torch.float16, device=cuda)
    h_in = torch.zeros(off // 2, dtype=torch.float16).pin_memory()
    h_out = torch.full((off // 2,), 7, dtype=torch.float16).pin_memory()

    def view(buf, o, pitch, j):
        return buf[o // 2:o // 2 + pitch // 2 * j["rows"]].view(j["rows"], pitch // 2)[:, :j["cols"]]

    hb = HostBatch(chunks=chunks, spans=True)
    refs, houts = [], []
    for k, (j, (o, pitch)) in enumerate(zip(jobs, layout)):
        img = (rng.random((j["rows"], j["cols"])) * 255).astype(np.float32)
        src = to_device(img, "f16", cuda)
        ref = torch.zeros(img.shape, dtype=torch.float16, device=cuda)
        ds, dd = view(d_in, o, pitch, j), view(d_out, o, pitch, j)
        if k == len(jobs) - 1:  # host images outside the slabs
            hs = torch.zeros(img.shape, dtype=torch.float16).pin_memory()
            hd = torch.full(img.shape, 7, dtype=torch.float16).pin_memory()
        else:
            hs, hd = view(h_in, o, pitch, j), view(h_out, o, pitch, j)
        hs.copy_(src.cpu())
        if j["op"] == "gauss":
            F.FIRGaussianConvolver2(j["sigma"]).convolve(j["gop"], src, ref, j["shift"])
            hb.add_gauss(hs, ds, hd, dd, j["sigma"], j["gop"], j["shift"])
        else:
            F.BoxFilter2(j["w"], j["w"], 64).convolve(src, ref, j["shift"], j["norm"])
            hb.add_box(hs, ds, hd, dd, j["w"], j["w"], j["norm"], j["shift"])
        refs.append(ref)
        houts.append(hd)
    hb.plan()
    info = hb.info()
    img_bytes = sum(j["rows"] * j["cols"] * 2 for j in jobs)
    assert info["h2d_bytes"] > img_bytes  # spans carry the row padding too
    hb.run()
    torch.cuda.synchronize()
    for j, ref, hd in zip(jobs, refs, houts):
        if j["op"] == "gauss":
            oy, ox = F.FIRGaussianConvolver2(j["sigma"]).offsets(j["gop"])
            v = (slice(oy, j["rows"] - oy), slice(ox, j["cols"] - ox))
        else:
            w = j["w"]
            v = (slice(w // 2, w // 2 + j["rows"] + 1 - w), slice(w // 2, w // 2 + j["cols"] + 1 - w))
        if not j["shift"]:
            v = (slice(0, v[0].stop - v[0].start), slice(0, v[1].stop - v[1].start))
        want = ref.cpu()[v].view(torch.int16).numpy()
        got = hd[v].view(torch.int16).numpy()
        assert np.array_equal(want, got), j
    # the job outside the slabs kept its border (pitched copy of its own)
    last = houts[-1].view(torch.int16).numpy()
    assert (last[0, :] == torch.tensor(7, dtype=torch.float16).view(torch.int16).item()).all()
