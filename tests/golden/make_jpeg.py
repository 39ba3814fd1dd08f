"""Writes the JPEG fixtures of tests/test_jpeg.py and tests/test_gpu_jpeg.py:
small sequential-Huffman JPEG files (tests/golden/jpeg/*.jpg) made by the
baseline encoder below, and tests/golden/jpeg_fixtures.npz with, per file,
the quantised coefficients the encoder wrote (the entropy decoder must give
them back exactly) and the quantisation tables and sampling factors (the
pixel oracle needs them).

The encoder follows ITU-T T.81: JFIF colour transform, box-filtered chroma
subsampling, float64 forward DCT, quantisation by rounding, DC differences
and AC run/size symbols (F.1.2), Huffman tables built from the symbol counts
with lengths limited to 16 bits and the all-ones code reserved (the Annex K.2
procedure), byte stuffing, restart markers.  Quantisation tables are this
project's own ramps, not the standard's example tables.

    python tests/golden/make_jpeg.py      # rewrites the fixtures
"""
from __future__ import annotations

import heapq
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
OUT_DIR = HERE / "jpeg"


def zigzag_natural():
    order = []
    for s in range(15):
        lo, hi = max(0, s - 7), min(s, 7)
        rows = range(lo, hi + 1) if s & 1 else range(hi, lo - 1, -1)
        order.extend(r * 8 + (s - r) for r in rows)
    return np.array(order)


ZZ = zigzag_natural()


def dct_matrix():
    m = np.zeros((8, 8))
    for u in range(8):
        c = np.sqrt(0.5) if u == 0 else 1.0
        for x in range(8):
            m[u, x] = 0.5 * c * np.cos((2 * x + 1) * u * np.pi / 16)
    return m


DCT = dct_matrix()


def quant_table(step: float, base: int = 1, limit: int = 255):
    u, v = np.meshgrid(np.arange(8), np.arange(8))
    return np.clip(np.round(base + step * (u + v)), 1, limit).astype(np.int64).reshape(64)


# ------------------------------------------------------------------ image

def synthetic_rgb(w, h, seed):
    rs = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w].astype(np.float64)
    img = np.zeros((h, w, 3))
    img[..., 0] = 128 + 100 * np.sin(x / 5.0 + seed)
    img[..., 1] = 255 * x / max(w - 1, 1)
    img[..., 2] = 255 * y / max(h - 1, 1)
    img += rs.normal(0, 18, img.shape)
    for _ in range(6):   # hard-edged rectangles: large coefficients
        x0, y0 = rs.integers(0, w), rs.integers(0, h)
        img[y0:y0 + rs.integers(2, 12), x0:x0 + rs.integers(2, 12)] = rs.choice([0, 255], 3)
    return np.clip(np.round(img), 0, 255).astype(np.uint8)


def rgb_to_ycbcr(rgb):
    r, g, b = [rgb[..., i].astype(np.float64) for i in range(3)]
    y = 0.299 * r + 0.587 * g + 0.114 * b
    cb = -0.168736 * r - 0.331264 * g + 0.5 * b + 128
    cr = 0.5 * r - 0.418688 * g - 0.081312 * b + 128
    return [y, cb, cr]


def component_plane(full, w, h, hs, vs, hmax, vmax, bw, bh):
    """Box-subsampled, edge-padded plane of bh*8 x bw*8 samples."""
    cw, ch = -(-w * hs // hmax), -(-h * vs // vmax)
    fx, fy = hmax // hs, vmax // vs
    padded = np.pad(full, ((0, ch * fy - h), (0, cw * fx - w)), mode="edge")
    sub = padded.reshape(ch, fy, cw, fx).mean(axis=(1, 3))
    return np.pad(sub, ((0, bh * 8 - ch), (0, bw * 8 - cw)), mode="edge")


def forward_blocks(plane, q):
    bh, bw = plane.shape[0] // 8, plane.shape[1] // 8
    blocks = (plane - 128.0).reshape(bh, 8, bw, 8).transpose(0, 2, 1, 3)
    coef = np.einsum("ux,abxy,vy->abuv", DCT, blocks, DCT).reshape(bh, bw, 64)
    return np.round(coef / q).astype(np.int64)


# ------------------------------------------------------------------ entropy coding

def category(v):
    v = abs(int(v))
    return v.bit_length()


def block_symbols(zz_coef, pred):
    """(dc_symbols, ac_symbols) for one block: lists of (symbol, bits, nbits)."""
    dc = []
    diff = int(zz_coef[0]) - pred
    s = category(diff)
    dc.append((s, diff if diff >= 0 else diff + (1 << s) - 1, s))
    ac = []
    run = 0
    last = np.nonzero(zz_coef[1:])[0]
    end = last[-1] + 1 if len(last) else 0
    for k in range(1, 64):
        v = int(zz_coef[k])
        if k > end:
            break
        if v == 0:
            run += 1
            continue
        while run > 15:
            ac.append((0xF0, 0, 0))
            run -= 16
        s = category(v)
        ac.append(((run << 4) | s, v if v >= 0 else v + (1 << s) - 1, s))
        run = 0
    if end < 63:
        ac.append((0x00, 0, 0))   # EOB
    return dc, ac


def huffman_table(freq):
    """(BITS[16], HUFFVAL) from symbol counts; lengths <= 16, all-ones code
    reserved by a dummy symbol of count 1 that is dropped at the end."""
    freq = dict(freq)
    freq[256] = 1
    heap = [(f, i, [s]) for i, (s, f) in enumerate(sorted(freq.items()))]
    heapq.heapify(heap)
    length = {s: 0 for s in freq}
    tick = len(heap)
    if len(heap) == 1:
        length[heap[0][2][0]] = 1
    while len(heap) > 1:
        f1, _, s1 = heapq.heappop(heap)
        f2, _, s2 = heapq.heappop(heap)
        for s in s1 + s2:
            length[s] += 1
        heapq.heappush(heap, (f1 + f2, tick, s1 + s2))
        tick += 1
    bits = [0] * 300
    for s, l in length.items():
        bits[l] += 1
    for i in range(299, 16, -1):   # limit to 16 bits (Figure K.3)
        while bits[i] > 0:
            j = i - 2
            while bits[j] == 0:
                j -= 1
            bits[i] -= 2
            bits[i - 1] += 1
            bits[j + 1] += 2
            bits[j] -= 1
    # symbols by original length (the dummy last among the longest), refilled
    order = sorted(freq, key=lambda s: (length[s], s))
    longest = max(i for i in range(17) if bits[i])
    bits[longest] -= 1            # the dummy's code (all ones) is dropped
    order.remove(256)
    return bits[1:17], order


def canonical_codes(bits, vals):
    codes, code, k = {}, 0, 0
    for l in range(1, 17):
        for _ in range(bits[l - 1]):
            codes[vals[k]] = (code, l)
            code += 1
            k += 1
        code <<= 1
    return codes


class BitWriter:
    def __init__(self):
        self.out = bytearray()
        self.acc = 0
        self.n = 0

    def put(self, value, nbits):
        for i in range(nbits - 1, -1, -1):
            self.acc = (self.acc << 1) | ((value >> i) & 1)
            self.n += 1
            if self.n == 8:
                self.out.append(self.acc)
                if self.acc == 0xFF:
                    self.out.append(0x00)
                self.acc, self.n = 0, 0

    def flush(self):
        if self.n:
            self.put((1 << (8 - self.n)) - 1, 8 - self.n)


def segment(marker, payload):
    return bytes([0xFF, marker]) + (len(payload) + 2).to_bytes(2, "big") + bytes(payload)


# ------------------------------------------------------------------ encoder

def encode(img, sampling, qsteps, restart=0, scans="interleaved", q16=False, adobe_rgb=False,
           extras=False):
    """img: (h, w) gray or (h, w, 3) RGB uint8.  sampling: [(h, v)] per
    component.  Returns (jpeg bytes, coefficient planes, quant tables)."""
    h, w = img.shape[:2]
    ncomp = 1 if img.ndim == 2 else 3
    if ncomp == 1:
        fulls = [img.astype(np.float64)]
    elif adobe_rgb:
        fulls = [img[..., i].astype(np.float64) for i in range(3)]
    else:
        fulls = rgb_to_ycbcr(img)
    hmax = max(s[0] for s in sampling)
    vmax = max(s[1] for s in sampling)
    mcux, mcuy = -(-w // (8 * hmax)), -(-h // (8 * vmax))
    qtabs = [quant_table(*qs) for qs in qsteps]
    planes, quants, tq = [], [], []
    for c in range(ncomp):
        hs, vs = sampling[c]
        bw, bh = mcux * hs, mcuy * vs
        plane = component_plane(fulls[c], w, h, hs, vs, hmax, vmax, bw, bh)
        t = min(c, len(qtabs) - 1)
        tq.append(t)
        coef = forward_blocks(plane, qtabs[t])
        dc = np.clip(coef[..., 0], -1024, 1023)   # DC differences stay within 11 bits
        coef = np.clip(coef, -1023, 1023)          # AC values within 10 bits
        coef[..., 0] = dc
        planes.append(coef)                  # [bh][bw][64] natural order
        quants.append(qtabs[t])

    # the block sequence of each scan
    def scan_units(comps):
        units = []   # list of MCUs; each a list of (component, row, col)
        if len(comps) == 1:
            c = comps[0]
            hs, vs = sampling[c]
            cw, ch = -(-w * hs // hmax), -(-h * vs // vmax)
            for r in range(-(-ch // 8)):
                for col in range(-(-cw // 8)):
                    units.append([(c, r, col)])
        else:
            for my in range(mcuy):
                for mx in range(mcux):
                    mcu = []
                    for c in comps:
                        hs, vs = sampling[c]
                        for by in range(vs):
                            for bx in range(hs):
                                mcu.append((c, my * vs + by, mx * hs + bx))
                    units.append(mcu)
        return units

    scan_list = [list(range(ncomp))] if scans == "interleaved" else [[c] for c in range(ncomp)]
    if scans != "interleaved":
        # a non-interleaved scan codes only the blocks that hold samples:
        # the MCU padding is never written, and decoders leave it zero
        for c in range(ncomp):
            hs, vs = sampling[c]
            cw, ch = -(-w * hs // hmax), -(-h * vs // vmax)
            planes[c][-(-ch // 8):, :] = 0
            planes[c][:, -(-cw // 8):] = 0
    # symbol statistics: table 0 for component 0, table 1 for the chroma
    tid = [0] + [1] * (ncomp - 1)
    dcf = [dict(), dict()]
    acf = [dict(), dict()]
    scan_syms = []
    for comps in scan_list:
        units = scan_units(comps)
        syms = []
        pred = {c: 0 for c in comps}
        for m, mcu in enumerate(units):
            if restart and m and m % restart == 0:
                pred = {c: 0 for c in comps}
                syms.append(None)          # restart boundary
            for c, r, col in mcu:
                zz = planes[c][r, col][ZZ]
                dc, ac = block_symbols(zz, pred[c])
                pred[c] = int(zz[0])
                syms.append((c, dc, ac))
                for s, _, _ in dc:
                    dcf[tid[c]][s] = dcf[tid[c]].get(s, 0) + 1
                for s, _, _ in ac:
                    acf[tid[c]][s] = acf[tid[c]].get(s, 0) + 1
        scan_syms.append((comps, syms))

    out = bytearray([0xFF, 0xD8])
    if adobe_rgb:
        out += segment(0xEE, b"Adobe" + bytes([0, 100, 0, 0, 0, 0, 0]))
    else:
        out += segment(0xE0, b"JFIF\0" + bytes([1, 1, 0, 0, 1, 0, 1, 0, 0]))
    if extras:
        out += segment(0xFE, b"fixture comment")
    for t, q in enumerate(qtabs):
        if q16:
            out += segment(0xDB, bytes([0x10 | t]) + b"".join(int(v).to_bytes(2, "big") for v in q[ZZ]))
        else:
            out += segment(0xDB, bytes([t]) + bytes(int(v) for v in q[ZZ]))
    sof = [8] + list(h.to_bytes(2, "big")) + list(w.to_bytes(2, "big")) + [ncomp]
    for c in range(ncomp):
        sof += [c + 1, (sampling[c][0] << 4) | sampling[c][1], tq[c]]
    out += segment(0xC1 if q16 else 0xC0, sof)
    tables = {}
    for t in range(1 if ncomp == 1 else 2):
        for cls, freq in ((0, dcf[t]), (1, acf[t])):
            bits, vals = huffman_table(freq)
            tables[(cls, t)] = canonical_codes(bits, vals)
            out += segment(0xC4, [(cls << 4) | t] + bits + vals)
    if restart:
        out += segment(0xDD, list(restart.to_bytes(2, "big")))
    for comps, syms in scan_syms:
        sos = [len(comps)]
        for c in comps:
            sos += [c + 1, (tid[c] << 4) | tid[c]]
        sos += [0, 63, 0]
        out += segment(0xDA, sos)
        bw_ = BitWriter()
        rst = 0
        for item in syms:
            if item is None:
                bw_.flush()
                out += bw_.out
                out += bytes([0xFF, 0xD0 + rst])
                rst = (rst + 1) & 7
                bw_ = BitWriter()
                continue
            c, dc, ac = item
            for s, v, n in dc:
                code, l = tables[(0, tid[c])][s]
                bw_.put(code, l)
                bw_.put(v, n)
            for s, v, n in ac:
                code, l = tables[(1, tid[c])][s]
                bw_.put(code, l)
                bw_.put(v, n)
        bw_.flush()
        out += bw_.out
        if extras:
            out += bytes([0xFF, 0xFF])   # fill bytes before the next marker
    out += bytes([0xFF, 0xD9])
    return bytes(out), planes, quants


FIXTURES = {
    # name: (width, height, gray, sampling, qsteps, restart, scans, q16, adobe_rgb, extras)
    "rgb444_q1": (45, 29, False, [(1, 1)] * 3, [(0.0, 1), (0.0, 1)], 0, "interleaved", False, False, False),
    "rgb420_restart": (61, 37, False, [(2, 2), (1, 1), (1, 1)], [(1.5, 2), (2.5, 3)], 3, "interleaved", False,
                       False, True),
    "rgb422_multiscan": (50, 20, False, [(2, 1), (1, 1), (1, 1)], [(1.0, 2), (2.0, 4)], 0, "separate", False,
                         False, False),
    "rgb440": (30, 35, False, [(1, 2), (1, 1), (1, 1)], [(2.0, 3), (3.0, 3)], 2, "interleaved", False, False,
               False),
    "rgb411": (70, 18, False, [(4, 1), (1, 1), (1, 1)], [(1.0, 2), (2.0, 2)], 0, "interleaved", False, False,
               False),
    "gray_q16": (33, 17, True, [(1, 1)], [(40.0, 3, 1000)], 0, "interleaved", True, False, False),
    "rgb_adobe": (24, 16, False, [(1, 1)] * 3, [(1.0, 2)], 0, "interleaved", False, True, False),
    "rgb444_128x96": (128, 96, False, [(1, 1)] * 3, [(1.2, 2), (2.0, 3)], 0, "interleaved", False, False, False),
    "rgb420_128x96": (128, 96, False, [(2, 2), (1, 1), (1, 1)], [(1.2, 2), (2.0, 3)], 0, "interleaved", False,
                      False, False),
    "gray_64x48": (64, 48, True, [(1, 1)], [(1.0, 2)], 4, "interleaved", False, False, False),
}


def main():
    OUT_DIR.mkdir(exist_ok=True)
    arrays = {}
    for i, (name, (w, h, gray, sampling, qsteps, restart, scans, q16, adobe, extras)) in enumerate(FIXTURES.items()):
        rgb = synthetic_rgb(w, h, seed=100 + i)
        img = (0.299 * rgb[..., 0] + 0.587 * rgb[..., 1] + 0.114 * rgb[..., 2]).round().astype(np.uint8) \
            if gray else rgb
        data, planes, quants = encode(img, sampling, qsteps, restart, scans, q16, adobe, extras)
        (OUT_DIR / f"{name}.jpg").write_bytes(data)
        arrays[f"{name}/size"] = np.array([w, h, len(planes)])
        arrays[f"{name}/sampling"] = np.array(sampling[:len(planes)])
        arrays[f"{name}/ycbcr"] = np.array(0 if (adobe or gray) else 1)
        for c, (p, q) in enumerate(zip(planes, quants)):
            arrays[f"{name}/coef{c}"] = p.astype(np.int16)
            arrays[f"{name}/quant{c}"] = q.astype(np.uint16)
        print(f"{name}: {w}x{h}, {len(data)} bytes")
    np.savez_compressed(HERE / "jpeg_fixtures.npz", **arrays)


if __name__ == "__main__":
    main()
