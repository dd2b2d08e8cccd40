"""DisparitySelector on the GPU (tucu_disparity_select) against the oracle's
restatement on the same cost volume, bit for bit: costs from the stereo box
filter (int32, u8 images) and float volumes; output types, offsets, the
selected region, the smallest and largest search widths."""
import numpy as np
import pytest

from helpers import torch_dtype

pytestmark = pytest.mark.gpu


def run(F, costs, dmax, inc, out_dt="i32", rows=None, cols=None, oy=0, ox=0, fill=-7):
    import torch
    D, H, W = costs.shape
    rows = H if rows is None else rows
    cols = W if cols is None else cols
    out = torch.full((rows + oy + 2, cols + ox + 3), fill, dtype=torch_dtype(out_dt), device=costs.device)
    F.DisparitySelector(dmax, inc).select(costs, out, rows, cols, oy, ox)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_stereo_pipeline_u8(F, oracle, cuda):
    """Box-aggregated costs of a shifted u8 pair (7 x 7 windows, 64
    disparities), then selection over the valid cost region."""
    import torch
    from tucuda_gb300 import workloads
    left, right = workloads.stereo_pair(rows=240, cols=320)
    L, R = torch.from_numpy(left).to(cuda), torch.from_numpy(right).to(cuda)
    D = 64
    costs = torch.zeros((D, 240, 320), dtype=torch.int32, device=cuda)
    F.BoxFilter2(7, 7).convolve_stereo(L, R, costs, 50)
    rows, cols = 240 - 6, 320 - 6
    got = run(F, costs, 80, 2, "i32", rows, cols, 3, 3)
    ref = oracle.select_disparity(costs[:, :rows, :cols].cpu().numpy().astype(np.float64), 80, 2)
    assert np.array_equal(got[3:3 + rows, 3:3 + cols], ref.astype(np.int32))
    # untouched outside the region
    assert (got[:3] == -7).all() and (got[:, :3] == -7).all() and (got[3 + rows:] == -7).all()
    # the pair is shifted by 9 columns: most consistent pixels find it
    assert np.mean(got[3:3 + rows, 3:3 + cols] == 80 - 9) > 0.5


@pytest.mark.parametrize("D", [1, 5, 37, 256])
@pytest.mark.parametrize("out_dt", ["i32", "f32", "u8"])
@pytest.mark.parametrize("W", [700, 701])  # rows on 16-byte boundaries (4 columns a thread) or not
def test_float_volumes(F, oracle, cuda, D, out_dt, W):
    import torch
    rng = np.random.default_rng(D)
    H = 23
    vol = rng.integers(0, 6, (D, H, W)).astype(np.float32)  # ties on purpose
    costs = torch.from_numpy(vol).to(cuda)
    dmax = 200 if out_dt == "u8" else 300
    got = run(F, costs, dmax, 3, out_dt, fill=0)
    ref = oracle.select_disparity(vol.astype(np.float64), dmax, 3)
    assert np.array_equal(got[:H, :W].astype(np.float64), ref)


def test_rejects_bad_arguments(F, cuda):
    import torch
    from tucuda_gb300 import _lib
    sel = F.DisparitySelector(10, 1)
    out = torch.zeros((8, 8), dtype=torch.int32, device=cuda)
    with pytest.raises(_lib.TucuError):
        sel.select(torch.zeros((2, 8, 8), dtype=torch.float16, device=cuda), out)
    with pytest.raises(_lib.TucuError):
        sel.select(torch.zeros((257, 8, 8), dtype=torch.int32, device=cuda), out)
    with pytest.raises(_lib.TucuError):  # the output too small for region + offset
        sel.select(torch.zeros((2, 8, 8), dtype=torch.int32, device=cuda), out, 8, 8, 1, 0)
