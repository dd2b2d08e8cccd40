"""Autotuner for the batched launch's tile shapes (strip heights).

Times the planned batch for each candidate (FIR strip rows, box strip rows)
with CUDA events and keeps the fastest; results are cached in a JSON file
keyed by GPU name and a signature of the batch (operators, sizes, types), so
a serving process tunes once per workload class.
"""
import hashlib
import json
import os

import torch

CANDIDATES = [(128, 64), (256, 128), (512, 128), (512, 256), (768, 128), (1024, 128), (1024, 256),
              (1536, 128), (2048, 128), (1024, 96), (1024, 160)]
# Tensor-core batches: only the FIR/box strip height matters (all jobs are
# 128-column strips of one kernel).
TENSOR_CANDIDATES = [(256, 128), (512, 128), (768, 128), (1024, 128), (1280, 128), (1536, 128),
                     (2048, 128), (3072, 128), (4096, 128)]
CACHE = os.environ.get("TUCU_AUTOTUNE_CACHE",
                       os.path.join(os.path.expanduser("~"), ".cache", "tucuda_gb300", "autotune.json"))


def signature(desc):
    return hashlib.sha1(json.dumps(desc, sort_keys=True).encode()).hexdigest()[:16]


def _load():
    try:
        with open(CACHE) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(data):
    try:
        os.makedirs(os.path.dirname(CACHE), exist_ok=True)
        tmp = CACHE + ".tmp"
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1)
        os.replace(tmp, CACHE)
    except OSError:
        pass


def time_batch(batch, reps=3):
    batch.launch()
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(reps):
        batch.launch()
    e.record()
    torch.cuda.synchronize()
    return s.elapsed_time(e) / reps


def tune(batch, desc, candidates=CANDIDATES, force=False):
    """Plans `batch` with the best tile shapes for the workload `desc` (a
    JSON-able description).  Returns (fir_rows, box_rows, table)."""
    key = f"{torch.cuda.get_device_name()}|{signature(desc)}"
    data = _load()
    if not force and key in data:
        fr, br = data[key]["best"]
        batch.plan(fr, br)
        return fr, br, data[key]
    table = {}
    for fr, br in candidates:
        batch.plan(fr, br)
        table[f"{fr},{br}"] = time_batch(batch)
    best = min(table, key=table.get)
    fr, br = (int(v) for v in best.split(","))
    batch.plan(fr, br)
    data[key] = {"best": [fr, br], "ms": table}
    _store(data)
    return fr, br, data[key]
