"""The serving loop: results of a mixed stream of requests (continuous
batching over several streams) equal the single calls bit for bit; admission
refusal, malformed requests, cancellation and injected admission failures are
reported per request."""
import os

import numpy as np
import pytest

from helpers import torch_dtype

pytestmark = pytest.mark.gpu


def _single(F, job, img, guide, dev):
    import torch
    src = torch.from_numpy(img).to(dev)
    out = torch.full(img.shape, 7, dtype=torch_dtype(job["out_dt"]), device=dev)
    if job["op"] == "gauss":
        F.FIRGaussianConvolver2(job["sigma"]).smooth(src, out)
    elif job["op"] == "box":
        F.BoxFilter2(2 * job["r"] + 1, 2 * job["r"] + 1, 129).convolve(src, out, True, job["norm"])
    else:
        g = torch.from_numpy(guide).to(dev) if guide is not None else None
        F.GuidedFilter2(2 * job["r"] + 1, 2 * job["r"] + 1, job["e"], 129).convolve(src, g, out)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _jobs(rng, n):
    jobs = []
    for i in range(n):
        dt = "u8" if i % 2 else "f16"
        rows, cols = int(rng.integers(40, 600)), int(rng.integers(40, 900))
        u = rng.random()
        if u < 0.5:
            jobs.append(dict(op="gauss", sigma=float(rng.uniform(1, 8)), dt=dt, out_dt=dt,
                             rows=rows, cols=cols))
        elif u < 0.8:
            norm = bool(i % 3)
            jobs.append(dict(op="box", r=int(rng.integers(1, 16)), dt=dt, norm=norm,
                             out_dt=dt if norm else ("i32" if dt == "u8" else "f32"),
                             rows=rows, cols=cols))
        else:
            jobs.append(dict(op="guided", r=int(rng.integers(2, 9)), e=25.5, dt=dt, out_dt="f32",
                             rows=rows, cols=cols, self_guided=bool(i % 4 == 0)))
    return jobs


NP = {"u8": np.uint8, "f16": np.float16, "f32": np.float32, "i32": np.int32}


def _image(rng, job):
    a = rng.random((job["rows"], job["cols"])) * 255
    return a.astype(NP[job["dt"]])


def test_server_results_equal_single_calls(F, cuda):
    from tucuda_gb300.server import Server
    rng = np.random.default_rng(21)
    jobs = _jobs(rng, 48)
    imgs = [_image(rng, j) for j in jobs]
    guides = [(_image(rng, j) if j["op"] == "guided" and not j["self_guided"] else None)
              for j in jobs]
    refs = [_single(F, j, im, g, cuda) for j, im, g in zip(jobs, imgs, guides)]
    outs = [np.full(im.shape, 7, dtype=NP[j["out_dt"]]) for j, im in zip(jobs, imgs)]
    with Server(budget_bytes=64 << 20, streams=3, max_wave=16) as srv:
        tickets = []
        for j, im, g, o in zip(jobs, imgs, guides, outs):
            if j["op"] == "gauss":
                tickets.append(srv.submit_gauss(im, o, j["sigma"]))
            elif j["op"] == "box":
                tickets.append(srv.submit_box(im, o, j["r"], j["norm"]))
            else:
                tickets.append(srv.submit_guided(im, g, o, j["r"], j["e"]))
        status = [srv.wait(t) for t in tickets]
        st = srv.stats()
    assert all(s in (0, 1) for s in status), status
    for j, ref, got in zip(jobs, refs, outs):
        assert np.array_equal(ref.view(np.uint8), got.view(np.uint8)), j
    assert st["completed"] == len(jobs)
    assert st["waves"] >= 2 and st["mean_wave_requests"] > 1.0
    assert st["peak_bytes"] <= st["budget_bytes"]
    assert st["p99_ms"] >= st["p50_ms"] > 0


def test_server_tensor_cores_close_to_single_calls(F, cuda):
    """With tensor cores on, f16 Gaussian and box requests run on the tcgen05
    kernel: within one f16 ulp (plus the paths' FP32 difference) of the exact
    single calls; u8 and guided requests keep their kernels and stay bit-equal."""
    from tucuda_gb300.server import Server
    rng = np.random.default_rng(23)
    jobs = _jobs(rng, 32)
    imgs = [_image(rng, j) for j in jobs]
    guides = [(_image(rng, j) if j["op"] == "guided" and not j["self_guided"] else None)
              for j in jobs]
    refs = [_single(F, j, im, g, cuda) for j, im, g in zip(jobs, imgs, guides)]
    outs = [np.full(im.shape, 7, dtype=NP[j["out_dt"]]) for j, im in zip(jobs, imgs)]
    with Server(budget_bytes=64 << 20, streams=3, max_wave=16, tensor=True) as srv:
        tickets = []
        for j, im, g, o in zip(jobs, imgs, guides, outs):
            if j["op"] == "gauss":
                tickets.append(srv.submit_gauss(im, o, j["sigma"]))
            elif j["op"] == "box":
                tickets.append(srv.submit_box(im, o, j["r"], j["norm"]))
            else:
                tickets.append(srv.submit_guided(im, g, o, j["r"], j["e"]))
        status = [srv.wait(t) for t in tickets]
    assert all(s in (0, 1) for s in status), status
    for j, ref, got in zip(jobs, refs, outs):
        if j["dt"] == "f16" and j["op"] != "guided":
            r, g_ = ref.astype(np.float64), got.astype(np.float64)
            scale = max(float(np.abs(r).max()), 1.0)
            if j["out_dt"] == "f16":
                ulp = 2.0 ** (np.floor(np.log2(np.maximum(np.abs(r), 2.0 ** -14))) - 10)
                assert np.all(np.abs(g_ - r) <= ulp + 2e-3), j
            else:
                assert np.abs(g_ - r).max() <= 2e-5 * scale, j
        else:
            assert np.array_equal(ref.view(np.uint8), got.view(np.uint8)), j


def test_server_admission_cancel_and_malformed(cuda):
    from tucuda_gb300 import _lib
    from tucuda_gb300.server import Server
    big = np.zeros((2000, 2000), np.float32)
    out = np.zeros_like(big)
    small = np.ones((300, 400), np.float32)
    with Server(budget_bytes=4 << 20, streams=1, max_wave=1) as srv:
        with pytest.raises(_lib.TucuError) as ei:
            srv.submit_box(big, out, 3)                  # never fits 4 MiB
        assert ei.value.status == _lib.ERR_BUDGET
        with pytest.raises(_lib.TucuError) as ei:
            srv.submit_gauss(small, np.zeros_like(small), sigma=0.0)   # malformed
        assert ei.value.status == _lib.ERR_ARG
        outs = [np.zeros_like(small) for _ in range(12)]
        tickets = [srv.submit_gauss(small, o, 3.0) for o in outs]
        # the last ones queue behind a one-request budget; cancel one of them
        rc = srv.cancel(tickets[-1])
        assert rc in (0, _lib.ERR_STATE)
        res = [srv.wait(t) for t in tickets]
        if rc == 0:
            assert res[-1] == _lib.ERR_CANCELLED
        assert all(r == 0 for r in res[:-1])
        st = srv.stats()
        assert st["rejected"] == 2


def test_server_injected_admission_failures(cuda):
    from tucuda_gb300 import _lib
    from tucuda_gb300.server import Server
    os.environ["TUCU_SERVER_FAIL_ADMIT_EVERY"] = "3"
    try:
        srv = Server(budget_bytes=64 << 20, streams=2, max_wave=4)
    finally:
        del os.environ["TUCU_SERVER_FAIL_ADMIT_EVERY"]
    img = np.ones((128, 160), np.uint8)
    outs = [np.zeros((128, 160), np.int32) for _ in range(9)]
    tickets = [srv.submit_box(img, o, 2) for o in outs]
    res = [srv.wait(t) for t in tickets]
    st = srv.stats()
    srv.close()
    assert res.count(_lib.ERR_NOMEM) >= 1 and res.count(0) >= 1
    assert st["failed"] == res.count(_lib.ERR_NOMEM)
    for r, o in zip(res, outs):
        if r == 0:
            assert (o[2:-2, 2:-2] == 25).all()
