"""float64 numpy restatement of the pixel stage of JPEG decoding — test
infrastructure: the oracle for zig_ornament_gb300/csrc/jpeg.cu.

From quantised coefficient planes (natural order, as the entropy decoder
returns them and as tests/golden/make_jpeg.py wrote them): dequantise, exact
8x8 inverse DCT (ITU-T T.81 A.3.3), level shift, round to nearest, clamp;
chroma upsampled by replication (output column x reads component column
x * h / hmax); JFIF YCbCr -> RGB; alpha 255; rows flipped when asked — the
zstbi setFlipVerticallyOnLoad(true) convention of the reference's example
app (glfw_example/app_no_interop.zig:17).

Parity with the reference's own decoder (stb_image through zstbi, a git
submodule absent from the reference tree) is unpinned: stb_image uses a
fixed-point IDCT and a triangle chroma filter, this restatement the exact
transform and replication.  The GPU kernel is pinned against this oracle
(within one level for FP32 rounding) and against nvJPEG.
"""
from __future__ import annotations

import numpy as np


def _basis():
    m = np.zeros((8, 8))
    for u in range(8):
        c = np.sqrt(0.5) if u == 0 else 1.0
        for x in range(8):
            m[u, x] = 0.5 * c * np.cos((2 * x + 1) * u * np.pi / 16)
    return m


BASIS = _basis()   # BASIS[u, x]


def idct_plane(coef: np.ndarray, quant: np.ndarray) -> np.ndarray:
    """coef [bh][bw][64] int, quant [64] -> uint8 plane [bh*8][bw*8]."""
    bh, bw = coef.shape[:2]
    F = coef.astype(np.float64).reshape(bh, bw, 8, 8) * quant.astype(np.float64).reshape(8, 8)
    f = np.einsum("vy,abvu,ux->abyx", BASIS, F, BASIS)
    s = np.clip(np.rint(f) + 128, 0, 255).astype(np.uint8)
    return s.transpose(0, 2, 1, 3).reshape(bh * 8, bw * 8)


def to_rgba(planes, sampling, width, height, ycbcr=True, flip_y=True) -> np.ndarray:
    """planes: uint8 sample planes; sampling: [(h, v)] per component."""
    hmax = max(s[0] for s in sampling)
    vmax = max(s[1] for s in sampling)
    ys = np.arange(height)
    src_rows = height - 1 - ys if flip_y else ys
    xs = np.arange(width)
    comps = []
    for p, (h, v) in zip(planes, sampling):
        comps.append(p[(src_rows * v // vmax)[:, None], (xs * h // hmax)[None, :]].astype(np.float64))
    out = np.empty((height, width, 4), np.uint8)
    out[..., 3] = 255
    if len(comps) == 1:
        out[..., 0] = out[..., 1] = out[..., 2] = comps[0]
    elif ycbcr:
        y, cb, cr = comps[0], comps[1] - 128.0, comps[2] - 128.0
        for i, val in enumerate((y + 1.402 * cr, y - 0.344136 * cb - 0.714136 * cr, y + 1.772 * cb)):
            out[..., i] = np.clip(np.rint(val), 0, 255)
    else:
        for i in range(3):
            out[..., i] = comps[i]
    return out


def decode_fixture(fx: dict, name: str, flip_y=True) -> np.ndarray:
    """RGBA8 of one tests/golden/jpeg_fixtures.npz entry."""
    w, h, n = (int(v) for v in fx[f"{name}/size"])
    sampling = [tuple(int(a) for a in s) for s in fx[f"{name}/sampling"]]
    if n == 1:
        sampling = [(1, 1)]
    planes = [idct_plane(fx[f"{name}/coef{c}"], fx[f"{name}/quant{c}"]) for c in range(n)]
    return to_rgba(planes, sampling, w, h, bool(fx[f"{name}/ycbcr"]), flip_y)
