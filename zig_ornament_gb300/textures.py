"""JPEG texture loading for the scene API — the texture path of the
reference's example app: ``loadTexture(name, 4)`` reads the file with zstbi
(stb_image) as RGBA8, flipped vertically on load
(glfw_example/examples.zig:492-503, glfw_example/app_no_interop.zig:17), and
``Scene.createTexture(data, w, h, 4, 1, false, 1.0)`` (src/scene.zig:339-351)
makes the texture.

Decoding goes through libornament_cuda's orn_jpeg_* calls: entropy decoding
on the host, the inverse DCT, chroma upsampling, colour conversion and the
flip on the GPU.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path
from typing import Tuple, Union

import numpy as np

from . import _lib

Source = Union[str, Path, bytes, bytearray, memoryview]


def _bytes(src: Source) -> bytes:
    if isinstance(src, (bytes, bytearray, memoryview)):
        return bytes(src)
    return Path(src).read_bytes()


def _check(status: int) -> None:
    if status != _lib.ORN_OK:
        lib = _lib.load()
        msg = lib.orn_jpeg_last_error().decode() or lib.orn_status_string(status).decode()
        raise _lib.OrnamentError(status, msg)


def jpeg_info(src: Source) -> Tuple[int, int, int]:
    """(width, height, components) from the frame header."""
    data = _bytes(src)
    w, h, n = C.c_uint32(), C.c_uint32(), C.c_uint32()
    _check(_lib.load().orn_jpeg_info(data, len(data), C.byref(w), C.byref(h), C.byref(n)))
    return w.value, h.value, n.value


def read_jpeg(src: Source, flip_y: bool = True, device: int = -1) -> np.ndarray:
    """RGBA8 pixels, shape (height, width, 4); flip_y=True is zstbi's
    flip-on-load (first row = bottom of the image)."""
    data = _bytes(src)
    w, h, _ = jpeg_info(data)
    out = np.empty((h, w, 4), np.uint8)
    _check(_lib.load().orn_jpeg_decode(data, len(data), device, 1 if flip_y else 0,
                                       out.ctypes.data_as(C.c_void_p), out.nbytes))
    return out


def jpeg_coefficients(src: Source, component: int) -> Tuple[np.ndarray, np.ndarray]:
    """The entropy decoder's quantised coefficients of one component,
    [blocks_h][blocks_w][64] in natural order, and its quantisation table."""
    data = _bytes(src)
    lib = _lib.load()
    bw, bh = C.c_uint32(), C.c_uint32()
    quant = np.zeros(64, np.uint16)
    _check(lib.orn_jpeg_coefficients(data, len(data), component, None, 0, C.byref(bw), C.byref(bh),
                                     quant.ctypes.data_as(C.c_void_p)))
    coef = np.zeros((bh.value, bw.value, 64), np.int16)
    _check(lib.orn_jpeg_coefficients(data, len(data), component, coef.ctypes.data_as(C.c_void_p), coef.size,
                                     None, None, None))
    return coef, quant


def load_texture(scene, src: Source, device: int = -1):
    """examples.zig loadTexture(name, 4) + Scene.createTexture(..., 4, 1,
    false, 1.0)."""
    rgba = read_jpeg(src, flip_y=True, device=device)
    h, w = rgba.shape[:2]
    return scene.createTexture(rgba, w, h, 4, 1, False, 1.0)
