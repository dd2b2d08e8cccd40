"""Seeded synthetic inputs with the shapes and value distributions of the
five benchmark configurations (no dataset is involved):

  1. plain_image      one 640x480 float32 image, i.i.d. U[0,255)
  2. planes_u8        1920x1080x3 planar uint8, i.i.d. U{0..255}
  3. guided_pair      1920x1080 guide = 128 + 8 random sinusoids + N(0,10^2),
                      input = guide + N(0,25^2)
  4. batched_spec     256 images, W~U[320,4096], H~U[240,2160], FP16 storage of
                      U[0,255); op drawn from {Gaussian sigma 1,2,4,8; box
                      radius 3,7,15}
  5. serving_trace    Poisson arrivals; sizes log-uniform from 640x480 to
                      3840x2160; u8/f16 50/50; 50% smooth sigma~U[1,8], 30% box
                      radius~U{3..15}, 20% guided radius~U{4..16}
"""
import math
from dataclasses import dataclass, field

import numpy as np

GUIDED_E = 25.5  # eps = 0.01*255^2 as a variance; the filters square e internally


def plain_image(seed=1, rows=480, cols=640):
    rng = np.random.default_rng(seed)
    return (rng.random((rows, cols), dtype=np.float32) * 255).astype(np.float32)


def planes_u8(seed=2, rows=1080, cols=1920, planes=3):
    rng = np.random.default_rng(seed)
    return rng.integers(0, 256, (planes, rows, cols), dtype=np.uint8)


def feature_image(rows=2160, cols=3840, seed=7):
    """Per-pixel feature vectors of the kind SuperPixels box-filters
    (colour and position terms): float32 (rows, cols, 4) with three smooth
    colour-like channels and the column coordinate."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:rows, 0:cols].astype(np.float32)
    f = np.empty((rows, cols, 4), np.float32)
    for c in range(3):
        a, b = rng.uniform(0.002, 0.02, 2)
        f[:, :, c] = 128 + 100 * np.sin(a * x + b * y + c) + rng.normal(0, 5, (rows, cols))
    f[:, :, 3] = x
    return f


def stereo_pair(rows=1080, cols=1920, seed=6, shift=9):
    """A u8 stereo pair: a textured left image and the right one equal to it
    shifted by `shift` columns, plus noise (so the costs have a clear
    minimum at d = shift)."""
    rng = np.random.default_rng(seed)
    left = rng.integers(0, 256, (rows, cols)).astype(np.int32)
    right = np.roll(left, shift, axis=1) + rng.integers(-6, 7, (rows, cols))
    return left.astype(np.uint8), np.clip(right, 0, 255).astype(np.uint8)


def guided_pair(rows=1080, cols=1920, seed=3):
    """(input, guide) as float32 arrays."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:rows, 0:cols].astype(np.float64)
    guide = np.full((rows, cols), 128.0)
    for _ in range(8):
        amp = rng.uniform(0, 60)
        period = math.exp(rng.uniform(math.log(8), math.log(256)))
        theta, phi = rng.uniform(0, 2 * math.pi, 2)
        guide += amp * np.sin(2 * math.pi * (x * math.cos(theta) + y * math.sin(theta)) / period
                              + phi)
    guide += rng.normal(0, 10, (rows, cols))
    inp = guide + rng.normal(0, 25, (rows, cols))
    return inp.astype(np.float32), guide.astype(np.float32)


@dataclass
class Job:
    """One image of a batched or served workload."""
    op: str             # "gauss" (smooth), "box" or "guided"
    rows: int
    cols: int
    dtype: str          # storage: "u8", "f16", ...
    sigma: float = 0.0  # Gaussian
    radius: int = 0     # box / guided: window = 2*radius+1
    arrival: float = 0.0
    seed: int = 0
    extra: dict = field(default_factory=dict)

    @property
    def window(self):
        return 2 * self.radius + 1

    @property
    def pixels(self):
        return self.rows * self.cols


BATCH_OPS = [("gauss", 1.0), ("gauss", 2.0), ("gauss", 4.0), ("gauss", 8.0),
             ("box", 3), ("box", 7), ("box", 15)]


def batched_spec(seed=4, n=256, dtype="f16"):
    rng = np.random.default_rng(seed)
    jobs = []
    for i in range(n):
        cols = int(rng.integers(320, 4097))
        rows = int(rng.integers(240, 2161))
        op, arg = BATCH_OPS[int(rng.integers(0, len(BATCH_OPS)))]
        if op == "gauss":
            jobs.append(Job("gauss", rows, cols, dtype, sigma=float(arg), seed=seed * 100000 + i))
        else:
            jobs.append(Job("box", rows, cols, dtype, radius=int(arg), seed=seed * 100000 + i))
    return jobs


def serving_trace(seed=5, n=100000, rate=10000.0):
    rng = np.random.default_rng(seed)
    t = 0.0
    jobs = []
    for i in range(n):
        t += rng.exponential(1.0 / rate)
        s = rng.random()
        cols = int(round(640 * (3840 / 640) ** s))
        rows = int(round(480 * (2160 / 480) ** s))
        dtype = "u8" if rng.random() < 0.5 else "f16"
        u = rng.random()
        if u < 0.5:
            job = Job("gauss", rows, cols, dtype, sigma=float(rng.uniform(1.0, 8.0)))
        elif u < 0.8:
            job = Job("box", rows, cols, dtype, radius=int(rng.integers(3, 16)))
        else:
            job = Job("guided", rows, cols, dtype, radius=int(rng.integers(4, 17)))
        job.arrival = t
        job.seed = seed * 1000000 + i
        jobs.append(job)
    return jobs


def fill_uniform_(t, seed, lo=0.0, hi=255.0):
    """Fills a torch tensor (any device, float or uint8) with seeded uniform
    pixels in [lo, hi) (integers 0..255 for uint8)."""
    import torch
    gen = torch.Generator(device=t.device)
    gen.manual_seed(int(seed))
    if t.dtype == torch.uint8:
        t.copy_(torch.randint(0, 256, t.shape, generator=gen, device=t.device, dtype=torch.uint8))
    else:
        tmp = torch.rand(t.shape, generator=gen, device=t.device, dtype=torch.float32)
        t.copy_(tmp * (hi - lo) + lo)
    return t
