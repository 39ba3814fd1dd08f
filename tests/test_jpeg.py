"""The JPEG texture loader's host stage (CPU): the entropy decoder returns
exactly the quantised coefficients the fixture encoder wrote
(tests/golden/make_jpeg.py: 4:4:4, 4:2:0, 4:2:2, 4:4:0, 4:1:1, grayscale,
16-bit tables, restart intervals, one scan per component, Adobe RGB, fill
bytes and comments), headers parse, unsupported and corrupt streams fail
with a status — including every truncation and random byte damage — and
decoding without a device fails loudly."""
from pathlib import Path

import numpy as np
import pytest

from zig_ornament_gb300 import _lib, textures

GOLDEN = Path(__file__).resolve().parent / "golden"
FIX = np.load(GOLDEN / "jpeg_fixtures.npz")
NAMES = sorted({k.split("/")[0] for k in FIX.files})


def _data(name):
    return (GOLDEN / "jpeg" / f"{name}.jpg").read_bytes()


@pytest.mark.parametrize("name", NAMES)
def test_header(name):
    w, h, n = (int(v) for v in FIX[f"{name}/size"])
    assert textures.jpeg_info(_data(name)) == (w, h, n)


@pytest.mark.parametrize("name", NAMES)
def test_coefficients_are_the_encoders(name):
    n = int(FIX[f"{name}/size"][2])
    for c in range(n):
        coef, quant = textures.jpeg_coefficients(_data(name), c)
        want = FIX[f"{name}/coef{c}"]
        assert coef.shape == want.shape
        assert np.array_equal(coef, want), (name, c, np.argwhere(coef != want)[:5])
        assert np.array_equal(quant, FIX[f"{name}/quant{c}"])


def test_bad_component_and_small_buffer():
    data = _data("gray_64x48")
    with pytest.raises(_lib.OrnamentError, match="INVALID_ARGUMENT"):
        textures.jpeg_coefficients(data, 1)
    lib = _lib.load()
    buf = np.zeros(10, np.int16)
    assert lib.orn_jpeg_coefficients(data, len(data), 0, buf.ctypes.data, buf.size, None, None, None) == 8


def _status(data):
    lib = _lib.load()
    bw, bh = _lib.C.c_uint32(), _lib.C.c_uint32()
    return lib.orn_jpeg_coefficients(bytes(data), len(data), 0, None, 0, _lib.C.byref(bw), _lib.C.byref(bh), None)


def test_unsupported_kinds():
    data = bytearray(_data("rgb444_q1"))
    i = data.index(b"\xff\xc0")
    prog = data[:]
    prog[i + 1] = 0xC2                      # progressive
    assert _status(prog) == 10
    arith = data[:]
    arith[i + 1] = 0xC9                     # arithmetic coding
    assert _status(arith) == 10
    twelve = data[:]
    twelve[i + 4] = 12                      # 12-bit samples
    assert _status(twelve) == 10
    assert _status(b"not a jpeg at all") == 11
    assert _status(b"") == 11


def test_every_truncation_fails_cleanly():
    data = _data("rgb420_restart")
    for cut in range(0, len(data) - 2):
        st = _status(data[:cut])
        assert st in (11, 10), (cut, st)


def test_random_damage_never_crashes():
    rs = np.random.default_rng(7)
    for name in ("rgb444_q1", "rgb420_restart", "rgb422_multiscan", "gray_q16"):
        data = _data(name)
        for _ in range(300):
            d = bytearray(data)
            for _ in range(rs.integers(1, 6)):
                d[rs.integers(0, len(d))] = rs.integers(0, 256)
            assert _status(d) in (0, 10, 11)


def test_decode_without_a_device_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    with pytest.raises(_lib.OrnamentError, match="NO_DEVICE"):
        textures.read_jpeg(_data("gray_64x48"))
