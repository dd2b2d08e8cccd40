"""Regenerates tests/golden/ref_device_vectors.json: outputs of the reference's
own device code, run on a GPU.

oracle/ref_device.cu wraps the reference's FIRFilter.h tap expressions
(device::convolve) and BoxFilter.h column convolvers (box_convolver, and
extrema_finder with extrema_value and extrema_position) in small kernels; `make -C oracle
ref_device REF=<checkout>` compiles them where the reference's headers lie
into oracle/_ref/ref_device.cubin (nvcc's default device flags: FMA
contraction on) and oracle/_ref/ref_device_nofma.cubin (-fmad=false).  This
script loads the cubins with the CUDA driver API, runs every case on seeded
inputs and writes the inputs and outputs (little-endian arrays, zlib, base64)
to the JSON file named by the first argument.  It needs a GPU and the cubins,
not the reference checkout, so the cubins are built where the checkout is and
run where the GPU is:

    make -C oracle ref_device REF=<checkout>
    python tests/golden/make_ref_device.py tests/golden/ref_device_vectors.json

Cases (each kernel checks its sizes before any access):
  fir   device::convolve over a row of 192 samples, for random lobes of every
        length FIRFilter2 accepts and for the reference's own Gaussian lobes
        (tests/golden/ref_vectors.json), both cubins; also the taps assigned to
        unsigned char (fir_filterV's u8 store) on inputs spanning [-200, 500)
  box   box_convolver down the 32 columns of one tile of the reference's box
        kernel (16 output rows: rows = w + 15), int32 and float32
  ext   extrema_finder minima and maxima down 32 columns of w + 15 rows
  arg   the same with extrema_position: each extremum's value and row
"""
import base64
import ctypes
import hashlib
import json
import os
import sys
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
CUBINS = {"fma": os.path.join(ROOT, "oracle", "_ref", "ref_device.cubin"),
          "nofma": os.path.join(ROOT, "oracle", "_ref", "ref_device_nofma.cubin")}
LOBE_LENGTHS = (2, 3, 4, 5, 8, 9, 16, 17)
N_ROW = 192
TILE_COLS = 32
TILE_OUT_ROWS = 16  # BoxFilter2::BlockDim output rows per block
BOX_WINDOWS = (1, 2, 3, 7, 15, 31)
EXT_WINDOWS = (2, 3, 7, 15, 21)


def pack(a):
    a = np.ascontiguousarray(a)
    a = a.astype(a.dtype.newbyteorder("<"), copy=False)
    return {"dtype": a.dtype.str, "shape": list(a.shape),
            "data": base64.b64encode(zlib.compress(a.tobytes(), 9)).decode()}


def unpack(d):
    raw = zlib.decompress(base64.b64decode(d["data"]))
    return np.frombuffer(raw, dtype=np.dtype(d["dtype"])).reshape(d["shape"]).copy()


def ref_gauss_lobes():
    """The reference's own float Gaussian lobes for a few sigmas (lobe0,
    lobe1, lobe2 of FIRGaussianConvolver2), from the committed fixture."""
    with open(os.path.join(HERE, "ref_vectors.json")) as f:
        lobes = json.load(f)["lobes"]
    out = []
    for e in lobes[::6]:
        sigma = np.frombuffer(bytes.fromhex(e["sigma"]), ">f4")[0]
        for k in ("lobe0", "lobe1", "lobe2"):
            lobe = np.array([np.frombuffer(bytes.fromhex(h), ">f4")[0] for h in e[k]], np.float32)
            out.append((float(sigma), k, lobe))
    return out


class Driver:
    """The CUDA driver calls this script needs, on torch's primary context."""

    def __init__(self):
        import torch
        self.torch = torch
        torch.zeros(1, device="cuda")  # makes the primary context current
        self.cu = ctypes.CDLL("libcuda.so.1")
        self.cu.cuModuleLoad.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p]
        self.cu.cuModuleGetFunction.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p,
                                                ctypes.c_char_p]
        self.cu.cuLaunchKernel.argtypes = [ctypes.c_void_p] + [ctypes.c_uint] * 6 + [
            ctypes.c_uint, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p]
        self.cu.cuModuleUnload.argtypes = [ctypes.c_void_p]

    def check(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{what}: CUDA driver error {rc}")

    def load(self, path):
        mod = ctypes.c_void_p()
        self.check(self.cu.cuModuleLoad(ctypes.byref(mod), path.encode()), f"cuModuleLoad {path}")
        return mod

    def launch(self, mod, name, grid, block, *args):
        fn = ctypes.c_void_p()
        self.check(self.cu.cuModuleGetFunction(ctypes.byref(fn), mod, name.encode()), name)
        ptrs = (ctypes.c_void_p * len(args))(*[ctypes.cast(ctypes.pointer(a), ctypes.c_void_p)
                                               for a in args])
        self.check(self.cu.cuLaunchKernel(fn, grid, 1, 1, block, 1, 1, 0, None, ptrs, None), name)
        self.check(self.cu.cuCtxSynchronize(), name)

    def dev(self, a):
        return self.torch.from_numpy(np.ascontiguousarray(a)).cuda()

    @staticmethod
    def ptr(t):
        return ctypes.c_void_p(t.data_ptr())


def fir_cases(drv, mods):
    torch = drv.torch
    rng = np.random.default_rng(11)
    px = rng.uniform(0.0, 255.0, N_ROW).astype(np.float32)
    wide = rng.uniform(-200.0, 500.0, N_ROW).astype(np.float32)
    lobes = [("random", 0.0, f"L{L}", (rng.standard_normal(L) * 0.3).astype(np.float32))
             for L in LOBE_LENGTHS]
    lobes += [("gauss", s, k, lb) for s, k, lb in ref_gauss_lobes()]
    cases = []
    for kind, sigma, name, lobe in lobes:
        L = len(lobe)
        n_out = N_ROW - 2 * (L & ~1)
        case = {"kind": "fir", "lobes": kind, "sigma": sigma, "name": name,
                "lobe": pack(lobe), "in": "px"}
        for var, mod in mods.items():
            out = torch.full((N_ROW,), float("nan"), dtype=torch.float32, device="cuda")
            d_in, d_lobe = drv.dev(px), drv.dev(lobe)
            drv.launch(mod, "ref_fir_row", (N_ROW + 127) // 128, 128, drv.ptr(d_in),
                       ctypes.c_int(N_ROW), drv.ptr(d_lobe), ctypes.c_int(L), drv.ptr(out))
            case[var] = pack(out.cpu().numpy()[:n_out])
        cases.append(case)
        if kind == "random" or name == "lobe0":
            case = {"kind": "fir_u8", "lobes": kind, "sigma": sigma, "name": name,
                    "lobe": pack(lobe), "in": "wide"}
            for var, mod in mods.items():
                f = torch.full((N_ROW,), float("nan"), dtype=torch.float32, device="cuda")
                u = torch.zeros(N_ROW, dtype=torch.uint8, device="cuda")
                d_in, d_lobe = drv.dev(wide), drv.dev(lobe)
                drv.launch(mod, "ref_fir_row", (N_ROW + 127) // 128, 128, drv.ptr(d_in),
                           ctypes.c_int(N_ROW), drv.ptr(d_lobe), ctypes.c_int(L), drv.ptr(f))
                drv.launch(mod, "ref_fir_row_u8", (N_ROW + 127) // 128, 128, drv.ptr(d_in),
                           ctypes.c_int(N_ROW), drv.ptr(d_lobe), ctypes.c_int(L), drv.ptr(u))
                case[var] = pack(f.cpu().numpy()[:n_out])
                case[var + "_u8"] = pack(u.cpu().numpy()[:n_out])
            cases.append(case)
    return {"px": pack(px), "wide": pack(wide)}, cases


def tile_cases(drv, mods):
    torch = drv.torch
    rng = np.random.default_rng(23)
    inputs, cases = {}, []
    rows_max = TILE_OUT_ROWS + max(max(BOX_WINDOWS), max(EXT_WINDOWS)) - 1
    inputs["box_u8"] = rng.integers(0, 256, (rows_max, TILE_COLS)).astype(np.int32)
    inputs["box_wide"] = rng.integers(-10 ** 6, 10 ** 6, (rows_max, TILE_COLS)).astype(np.int32)
    inputs["box_f32"] = rng.uniform(0.0, 255.0, (rows_max, TILE_COLS)).astype(np.float32)
    inputs["ext_ties"] = rng.integers(0, 6, (rows_max, TILE_COLS)).astype(np.float32)
    inputs["ext_f32"] = rng.uniform(0.0, 1.0, (rows_max, TILE_COLS)).astype(np.float32)
    jobs = [("box", "ref_box_cols_i32", "box_u8", w) for w in BOX_WINDOWS]
    jobs += [("box", "ref_box_cols_i32", "box_wide", w) for w in BOX_WINDOWS]
    jobs += [("box", "ref_box_cols_f32", "box_f32", w) for w in BOX_WINDOWS]
    for src in ("ext_ties", "ext_f32"):
        for kern in ("ref_min_cols_f32", "ref_max_cols_f32"):
            jobs += [("ext", kern, src, w) for w in EXT_WINDOWS]
    for kind, kern, src, w in jobs:
        rows = TILE_OUT_ROWS + w - 1
        tile = np.ascontiguousarray(inputs[src][:rows])
        case = {"kind": kind, "kernel": kern, "in": src, "w": w, "rows": rows}
        got = {}
        for var, mod in mods.items():
            d_in = drv.dev(tile)
            out = torch.full((rows, TILE_COLS), -7, dtype=d_in.dtype, device="cuda")
            drv.launch(mod, kern, 1, TILE_COLS, drv.ptr(d_in), ctypes.c_int(rows), ctypes.c_int(w),
                       drv.ptr(out))
            got[var] = out.cpu().numpy()[:TILE_OUT_ROWS]
        # no multiplies in these convolvers: both builds must agree
        case["builds_agree"] = bool(np.array_equal(got["fma"].view(np.uint32),
                                                   got["nofma"].view(np.uint32)))
        case["out"] = pack(got["fma"])
        cases.append(case)
    for src in ("ext_ties", "ext_f32"):
        for kern in ("ref_argmin_cols_f32", "ref_argmax_cols_f32"):
            for w in EXT_WINDOWS:
                rows = TILE_OUT_ROWS + w - 1
                tile = np.ascontiguousarray(inputs[src][:rows])
                d_in = drv.dev(tile)
                val = torch.full((rows, TILE_COLS), -7.0, dtype=torch.float32, device="cuda")
                row = torch.full((rows, TILE_COLS), -7, dtype=torch.int32, device="cuda")
                drv.launch(mods["fma"], kern, 1, TILE_COLS, drv.ptr(d_in), ctypes.c_int(rows),
                           ctypes.c_int(w), drv.ptr(val), drv.ptr(row))
                cases.append({"kind": "arg", "kernel": kern, "in": src, "w": w, "rows": rows,
                              "val": pack(val.cpu().numpy()[:TILE_OUT_ROWS]),
                              "row": pack(row.cpu().numpy()[:TILE_OUT_ROWS])})
    return {k: pack(v) for k, v in inputs.items()}, cases


def main() -> int:
    out_path = sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "ref_device_vectors.json")
    for p in CUBINS.values():
        if not os.path.exists(p):
            print(f"{p} is missing: make -C oracle ref_device REF=<reference checkout>",
                  file=sys.stderr)
            return 1
    drv = Driver()
    mods = {k: drv.load(p) for k, p in CUBINS.items()}
    fir_inputs, fir = fir_cases(drv, mods)
    tile_inputs, tiles = tile_cases(drv, mods)
    data = {"_generated_by": "tests/golden/make_ref_device.py (oracle/ref_device.cu)",
            "device": drv.torch.cuda.get_device_name(0),
            "cubin_sha256": {k: hashlib.sha256(open(p, "rb").read()).hexdigest()
                             for k, p in CUBINS.items()},
            "inputs": {**fir_inputs, **tile_inputs},
            "cases": fir + tiles}
    with open(out_path, "w") as f:
        json.dump(data, f, separators=(",", ":"))
        f.write("\n")
    print("wrote", out_path, len(data["cases"]), "cases")
    return 0


if __name__ == "__main__":
    sys.exit(main())
