"""Shared helpers of the GPU parity tests."""
import numpy as np

NP_OF = {"u8": np.uint8, "f16": np.float16, "f32": np.float32, "i32": np.int32}


def torch_dtype(name):
    import torch
    return {"u8": torch.uint8, "f16": torch.float16, "bf16": torch.bfloat16,
            "f32": torch.float32, "i32": torch.int32}[name]


def to_device(arr, dtype, dev, pad=0, offset=0):
    """Copies a float/int numpy image to the GPU in `dtype`; pad > 0 leaves
    extra elements at the end of each row (a pitch larger than the width) and
    offset > 0 shifts the base pointer by that many elements (unaligned)."""
    import torch
    rows, cols = arr.shape
    t = torch.from_numpy(np.ascontiguousarray(arr)).to(torch.float32 if dtype not in ("u8", "i32")
                                                       else torch.int64)
    t = t.to(torch_dtype(dtype))
    store = torch.zeros(rows * (cols + pad) + offset, dtype=torch_dtype(dtype), device=dev)
    view = store[offset:offset + rows * (cols + pad)].view(rows, cols + pad)[:, :cols]
    view.copy_(t.to(dev))
    return view


def to_numpy_f32(t):
    import torch
    return t.to(torch.float32).cpu().numpy()


def quantise_input(img, dtype):
    """The float32 values a stored input of `dtype` holds."""
    from oracle import oracle as orc
    if dtype == "u8":
        return np.clip(np.floor(img), 0, 255).astype(np.float32)
    return orc.round_to(img, dtype)


def rel_rms(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.sqrt(np.mean((a - b) ** 2)) / max(np.sqrt(np.mean(b ** 2)), 1e-30))
