"""Single-kernel cases for profiling: runs one filter call on a seeded
synthetic image a few times, so that a profiler can capture one launch of
one kernel in isolation.

    python cases.py CASE [REPS] [ROWS COLS]

CASE is one of
    fir<sigma>_<dt>      Gaussian smooth, dt in u8, f16, bf16, f32 (out = in)
    box<w>_u8            w x w window sums, u8 -> int32
    box<w>_f16           w x w window means, f16 -> f16
    guided<w>_<dt>       guided filter, w x w windows, e = 25.5, out f32
    multi<sigma>_<dt>    all six Gaussian operators in one pass, out f32
    ext<w>_<dt>          w x w window minima and their positions
    vec<n>box<w>         box sums of n-channel float feature vectors
    stereo<w>_d<D>       stereo cost aggregation of a 1920x1080 u8 pair
                         (w x w windows, D disparities, int32 costs)
    select<D>            stereo costs (7 x 7, D disparities) of a 1920x1080 u8
                         pair, then DisparitySelector over them (the case
                         times the selection)
    tcfir<sigma>         Gaussian smooth of an f16 image on the tensor cores
                         (a one-job tensor-core batch, 1024-row strips)
    tcbox<w>             w x w window means of an f16 image, tensor cores
Default size 6480 x 11520 (74.6 Mpix: an f16 image is 149 MB, more than
the 129 MB L2, so DRAM counters mean something).
"""
import sys


def run(case, reps=3, rows=6480, cols=11520):
    import torch
    from tucuda_gb300 import filters as F

    dev = torch.device("cuda:0")
    gen = torch.Generator(device=dev)
    gen.manual_seed(7)
    dts = {"u8": torch.uint8, "f16": torch.float16, "bf16": torch.bfloat16, "f32": torch.float32}

    def image(dt):
        x = torch.rand(rows, cols, device=dev, generator=gen) * 255
        return x.to(torch.uint8) if dt == torch.uint8 else x.to(dt)

    if case.startswith("select"):
        from tucuda_gb300 import workloads
        D = int(case[6:])
        sl, sr = (torch.from_numpy(a).to(dev) for a in workloads.stereo_pair())
        costs = torch.empty((D,) + tuple(sl.shape), dtype=torch.int32, device=dev)
        F.BoxFilter2(7, 7, 23).convolve_stereo(sl, sr, costs, 50)
        sel = F.DisparitySelector(80, 2)
        disp = torch.zeros(sl.shape, dtype=torch.int32, device=dev)
        fn = lambda: sel.select(costs, disp, sl.shape[0] - 6, sl.shape[1] - 6, 3, 3)
    elif case.startswith("tc"):
        from tucuda_gb300.batch import Batch
        x = image(torch.float16)
        y = torch.zeros_like(x)
        b = Batch(tensor=True)
        if case.startswith("tcfir"):
            b.add_gauss(x, y, float(case[5:]))
        else:
            w = int(case[5:])
            b.add_box(x, y, w, w, normalize=True)
        b.plan(1024, 0)
        fn = lambda: b.launch(graph=False)
    elif case.startswith("fir"):
        sigma, dt = case[3:].split("_")
        x = image(dts[dt])
        y = torch.zeros_like(x)
        g = F.FIRGaussianConvolver2(float(sigma))
        fn = lambda: g.smooth(x, y)
    elif case.startswith("box"):
        w, dt = case[3:].split("_")
        b = F.BoxFilter2(int(w), int(w), 129)
        x = image(dts[dt])
        if dt == "u8":
            y = torch.zeros(rows, cols, device=dev, dtype=torch.int32)
            fn = lambda: b.convolve(x, y)
        else:
            y = torch.zeros_like(x)
            fn = lambda: b.convolve(x, y, True, True)
    elif case.startswith("guided"):
        w, dt = case[6:].split("_")
        p, g = image(dts[dt]), image(dts[dt])
        o = torch.zeros(rows, cols, device=dev, dtype=torch.float32)
        gf = F.GuidedFilter2(int(w), int(w), 25.5, 129)
        fn = lambda: gf.convolve(p, g, o)
    elif case.startswith("multi"):
        sigma, dt = case[5:].split("_")
        x = image(dts[dt])
        outs = {k: torch.zeros(rows, cols, device=dev, dtype=torch.float32) for k in range(6)}
        g = F.FIRGaussianConvolver2(float(sigma))
        fn = lambda: g.convolve_multi(x, outs)
    elif case.startswith("vec"):
        n, w = case[3:].split("box")
        x = torch.rand(rows, cols, int(n), device=dev, generator=gen) * 255
        y = torch.zeros_like(x)
        b = F.BoxFilter2(int(w), int(w), 64)
        fn = lambda: b.convolve_vec(x, y)
    elif case.startswith("stereo"):
        w, d = case[6:].split("_d")
        from tucuda_gb300 import workloads
        sl, sr = (torch.from_numpy(a).to(dev) for a in workloads.stereo_pair())
        c = torch.zeros((int(d),) + tuple(sl.shape), device=dev, dtype=torch.int32)
        b = F.BoxFilter2(int(w), int(w), 64)
        fn = lambda: b.convolve_stereo(sl, sr, c, 50)
    elif case.startswith("ext"):
        w, dt = case[3:].split("_")
        x = image(dts[dt])
        v = torch.zeros_like(x)
        p = torch.zeros(rows, cols, 2, device=dev, dtype=torch.int32)
        f = F.ExtremaFilter2(int(w), int(w), 64)
        fn = lambda: f.convolve(x, v, p)
    else:
        raise SystemExit(f"unknown case {case!r}")
    for _ in range(reps):
        fn()
    torch.cuda.synchronize()
    print("ok", case, rows, cols, flush=True)


if __name__ == "__main__":
    a = sys.argv[1:]
    if not a:
        raise SystemExit(__doc__)
    run(a[0], int(a[1]) if len(a) > 1 else 3, *(int(v) for v in a[2:4]))
