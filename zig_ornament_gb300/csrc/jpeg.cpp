// jpeg.cpp — JPEG (ITU-T T.81) sequential Huffman decoding on the host: the
// marker parser and the entropy decoder, which produce one plane of
// quantised DCT coefficients per component.  The arithmetic stages run on
// the GPU (jpeg.cu).
//
// Handled: SOF0 / SOF1 (8-bit samples), 1 or 3 components with sampling
// factors 1..4, interleaved and non-interleaved scans (several scans per
// frame), 8- and 16-bit quantisation tables, restart intervals, APP14 Adobe
// colour transform and 'R','G','B' component ids (no YCbCr conversion).
// Rejected with ORN_ERR_UNSUPPORTED: progressive, lossless, hierarchical and
// arithmetic-coded frames, 12-bit samples, 2- and 4-component images, DNL
// heights.  Corrupt streams give ORN_ERR_BAD_IMAGE; nothing is read outside
// the input buffer.
//
// Procedures follow the standard: Huffman tables from BITS/HUFFVAL (Annex C),
// DECODE with MAXCODE/VALPTR (F.2.2.3, here behind a 9-bit lookup),
// RECEIVE/EXTEND (F.2.2.1), the zig-zag sequence (Figure A.6), MCU order
// (A.2).
#include <algorithm>
#include <cstring>
#include <string>

#include "jpeg.h"
#include "ornament_cuda.h"

namespace orn {
namespace jpeg {
namespace {

// natural index of the k-th coefficient in zig-zag order
struct Zigzag {
    uint8_t natural[64];
    Zigzag() {
        int k = 0;
        for (int s = 0; s <= 14; ++s) {
            const int lo = std::max(0, s - 7), hi = std::min(s, 7);
            if (s & 1)
                for (int r = lo; r <= hi; ++r) natural[k++] = (uint8_t)(r * 8 + (s - r));
            else
                for (int r = hi; r >= lo; --r) natural[k++] = (uint8_t)(r * 8 + (s - r));
        }
    }
};
const Zigzag kZigzag;

constexpr int kFastBits = 9;

struct Huffman {
    bool present = false;
    uint8_t vals[256] = {};
    int32_t maxcode[17] = {};   // by code length, -1 when no code has that length
    int32_t mincode[17] = {};
    int32_t valptr[17] = {};
    uint16_t fast[1 << kFastBits] = {};   // (length << 8) | symbol; 0: longer than kFastBits

    bool build(const uint8_t counts[16], const uint8_t* symbols, int total) {
        std::memset(fast, 0, sizeof(fast));
        std::memcpy(vals, symbols, (size_t)total);
        int32_t code = 0;
        int j = 0;
        for (int l = 1; l <= 16; ++l) {
            const int n = counts[l - 1];
            if (n == 0) {
                maxcode[l] = -1;
            } else {
                valptr[l] = j;
                mincode[l] = code;
                for (int i = 0; i < n; ++i, ++j, ++code) {
                    if (code >= (1 << l)) return false;   // more codes than fit in l bits
                    if (l <= kFastBits) {
                        const int shift = kFastBits - l;
                        for (int f = 0; f < (1 << shift); ++f)
                            fast[(code << shift) | f] = (uint16_t)((l << 8) | vals[j]);
                    }
                }
                maxcode[l] = code - 1;
            }
            if (code > (1 << l)) return false;   // more codes than fit in l bits
            code <<= 1;
        }
        present = true;
        return true;
    }
};

// Entropy-coded segment reader: byte stuffing (FF 00) removed, fill bytes
// before a marker skipped, zeros fed once a marker or the end is reached.
struct Bits {
    const uint8_t* p;
    const uint8_t* end;
    uint64_t buf = 0;      // MSB-aligned
    int cnt = 0;
    bool at_marker = false;
    uint32_t zeros_fed = 0;

    void fill() {
        while (cnt <= 56) {
            uint32_t b = 0;
            bool real = false;
            if (!at_marker && p < end) {
                if (*p != 0xFF) {
                    b = *p++;
                    real = true;
                } else if (p + 1 >= end) {
                    at_marker = true;          // truncated: treated as the end
                } else if (p[1] == 0x00) {
                    b = 0xFF;                  // stuffed byte
                    p += 2;
                    real = true;
                } else if (p[1] == 0xFF) {
                    ++p;                       // fill byte before a marker
                    continue;
                } else {
                    at_marker = true;          // p stays on the marker
                }
            }
            if (!real) ++zeros_fed;
            buf |= (uint64_t)b << (56 - cnt);
            cnt += 8;
        }
    }
    uint32_t peek(int n) const { return (uint32_t)(buf >> (64 - n)); }
    void skip(int n) {
        buf <<= n;
        cnt -= n;
    }
    // Moves to the next marker (dropping buffered bits and any garbage).
    void resync() {
        buf = 0;
        cnt = 0;
        at_marker = false;
        zeros_fed = 0;
        while (p + 1 < end && !(p[0] == 0xFF && p[1] != 0x00 && p[1] != 0xFF)) ++p;
        if (p + 1 >= end) p = end;
    }
};

inline int decode_symbol(Bits& br, const Huffman& h) {
    br.fill();
    const uint16_t f = h.fast[br.peek(kFastBits)];
    if (f) {
        br.skip(f >> 8);
        return f & 0xFF;
    }
    const uint32_t code16 = br.peek(16);
    for (int l = kFastBits + 1; l <= 16; ++l) {
        const int32_t c = (int32_t)(code16 >> (16 - l));
        if (c <= h.maxcode[l]) {
            br.skip(l);
            return h.vals[h.valptr[l] + c - h.mincode[l]];
        }
    }
    return -1;
}

// RECEIVE(s) followed by EXTEND (F.2.2.1); the caller has filled the buffer.
inline int receive_extend(Bits& br, int s) {
    if (s == 0) return 0;
    const int v = (int)br.peek(s);
    br.skip(s);
    return v < (1 << (s - 1)) ? v - (1 << s) + 1 : v;
}

bool decode_block(Bits& br, const Huffman& dc, const Huffman& ac, int* pred, int16_t* out) {
    std::memset(out, 0, 64 * sizeof(int16_t));
    const int t = decode_symbol(br, dc);
    if (t < 0 || t > 11) return false;
    br.fill();
    const int dcv = *pred + receive_extend(br, t);
    if (dcv < -32768 || dcv > 32767) return false;
    *pred = dcv;
    out[0] = (int16_t)dcv;
    for (int k = 1; k < 64;) {
        const int rs = decode_symbol(br, ac);
        if (rs < 0) return false;
        const int r = rs >> 4, s = rs & 15;
        if (s == 0) {
            if (r != 15) break;   // EOB
            k += 16;              // ZRL
            if (k > 64) return false;
            continue;
        }
        if (s > 10) return false;
        k += r;
        if (k > 63) return false;
        br.fill();
        out[kZigzag.natural[k]] = (int16_t)receive_extend(br, s);
        ++k;
    }
    return true;
}

struct Parser {
    const uint8_t* data = nullptr;
    size_t len = 0;
    size_t pos = 0;
    Image* img = nullptr;
    std::string* err = nullptr;
    Huffman dc[4], ac[4];
    uint32_t restart = 0;
    bool have_frame = false;
    bool adobe = false;
    int adobe_transform = -1;

    int fail(int status, const char* msg) {
        if (err) *err = msg;
        return status;
    }
    bool need(size_t n) const { return pos + n <= len; }
    uint32_t u8(size_t at) const { return data[at]; }
    uint32_t u16(size_t at) const { return ((uint32_t)data[at] << 8) | data[at + 1]; }

    int read_dqt(size_t seg, size_t seg_len) {
        size_t at = seg, end = seg + seg_len;
        while (at < end) {
            const uint32_t pq = u8(at) >> 4, tq = u8(at) & 15;
            ++at;
            if (pq > 1 || tq > 3) return fail(ORN_ERR_BAD_IMAGE, "bad DQT table");
            const size_t bytes = pq ? 128 : 64;
            if (at + bytes > end) return fail(ORN_ERR_BAD_IMAGE, "short DQT segment");
            for (int k = 0; k < 64; ++k) {
                const uint32_t q = pq ? u16(at + 2 * k) : u8(at + k);
                if (q == 0) return fail(ORN_ERR_BAD_IMAGE, "zero quantisation step");
                img->quant[tq][kZigzag.natural[k]] = (uint16_t)q;
            }
            img->quant_present[tq] = true;
            at += bytes;
        }
        return ORN_OK;
    }

    int read_dht(size_t seg, size_t seg_len) {
        size_t at = seg, end = seg + seg_len;
        while (at < end) {
            if (at + 17 > end) return fail(ORN_ERR_BAD_IMAGE, "short DHT segment");
            const uint32_t tc = u8(at) >> 4, th = u8(at) & 15;
            if (tc > 1 || th > 3) return fail(ORN_ERR_BAD_IMAGE, "bad DHT table");
            uint8_t counts[16];
            int total = 0;
            for (int i = 0; i < 16; ++i) {
                counts[i] = data[at + 1 + i];
                total += counts[i];
            }
            at += 17;
            if (total > 256 || at + (size_t)total > end) return fail(ORN_ERR_BAD_IMAGE, "bad DHT counts");
            Huffman& h = tc ? ac[th] : dc[th];
            if (!h.build(counts, data + at, total)) return fail(ORN_ERR_BAD_IMAGE, "bad Huffman code lengths");
            at += (size_t)total;
        }
        return ORN_OK;
    }

    int read_sof(size_t seg, size_t seg_len, bool header_only) {
        if (have_frame) return fail(ORN_ERR_BAD_IMAGE, "second frame header");
        if (seg_len < 6) return fail(ORN_ERR_BAD_IMAGE, "short SOF segment");
        if (u8(seg) != 8) return fail(ORN_ERR_UNSUPPORTED, "only 8-bit samples are supported");
        img->height = u16(seg + 1);
        img->width = u16(seg + 3);
        img->ncomp = u8(seg + 5);
        if (img->height == 0) return fail(ORN_ERR_UNSUPPORTED, "DNL-defined heights are not supported");
        if (img->width == 0) return fail(ORN_ERR_BAD_IMAGE, "zero width");
        if (img->ncomp != 1 && img->ncomp != 3)
            return fail(ORN_ERR_UNSUPPORTED, "only 1- and 3-component images are supported");
        if (seg_len < 6 + 3 * (size_t)img->ncomp) return fail(ORN_ERR_BAD_IMAGE, "short SOF segment");
        img->hmax = img->vmax = 1;
        for (uint32_t i = 0; i < img->ncomp; ++i) {
            Component& c = img->comp[i];
            c.id = u8(seg + 6 + 3 * i);
            c.h = u8(seg + 7 + 3 * i) >> 4;
            c.v = u8(seg + 7 + 3 * i) & 15;
            c.tq = u8(seg + 8 + 3 * i);
            if (c.h < 1 || c.h > 4 || c.v < 1 || c.v > 4 || c.tq > 3)
                return fail(ORN_ERR_BAD_IMAGE, "bad component sampling or table");
            for (uint32_t k = 0; k < i; ++k)
                if (img->comp[k].id == c.id) return fail(ORN_ERR_BAD_IMAGE, "duplicate component id");
            if (img->ncomp == 1) c.h = c.v = 1;   // one component: the factors have no meaning
            img->hmax = std::max(img->hmax, c.h);
            img->vmax = std::max(img->vmax, c.v);
        }
        if ((uint64_t)img->width * img->height > (1ull << 28))
            return fail(ORN_ERR_UNSUPPORTED, "image larger than 2^28 pixels");
        img->mcux = (img->width + 8 * img->hmax - 1) / (8 * img->hmax);
        img->mcuy = (img->height + 8 * img->vmax - 1) / (8 * img->vmax);
        if (img->ncomp == 3 && img->comp[0].id == 'R' && img->comp[1].id == 'G' && img->comp[2].id == 'B')
            img->ycbcr = false;
        if (!header_only) {
            for (uint32_t i = 0; i < img->ncomp; ++i) {
                Component& c = img->comp[i];
                c.bw = img->mcux * c.h;
                c.bh = img->mcuy * c.v;
                try {
                    c.coef.assign((size_t)c.bw * c.bh * 64, 0);
                } catch (...) {
                    return fail(ORN_ERR_OUT_OF_MEMORY, "out of host memory for the coefficients");
                }
            }
        }
        have_frame = true;
        return ORN_OK;
    }

    int read_sos(size_t seg, size_t seg_len) {
        if (!have_frame) return fail(ORN_ERR_BAD_IMAGE, "scan before the frame header");
        if (seg_len < 1) return fail(ORN_ERR_BAD_IMAGE, "short SOS segment");
        const uint32_t ns = u8(seg);
        if (ns < 1 || ns > img->ncomp || seg_len < 4 + 2 * (size_t)ns) return fail(ORN_ERR_BAD_IMAGE, "bad SOS");
        int idx[kMaxComponents];
        uint32_t td[kMaxComponents], ta[kMaxComponents];
        uint32_t blocks_per_mcu = 0;
        for (uint32_t i = 0; i < ns; ++i) {
            const uint32_t cs = u8(seg + 1 + 2 * i);
            idx[i] = -1;
            for (uint32_t k = 0; k < img->ncomp; ++k)
                if (img->comp[k].id == cs) idx[i] = (int)k;
            if (idx[i] < 0) return fail(ORN_ERR_BAD_IMAGE, "scan names an unknown component");
            for (uint32_t k = 0; k < i; ++k)
                if (idx[k] == idx[i]) return fail(ORN_ERR_BAD_IMAGE, "component twice in a scan");
            td[i] = u8(seg + 2 + 2 * i) >> 4;
            ta[i] = u8(seg + 2 + 2 * i) & 15;
            if (td[i] > 3 || ta[i] > 3 || !dc[td[i]].present || !ac[ta[i]].present)
                return fail(ORN_ERR_BAD_IMAGE, "scan uses an undefined Huffman table");
            if (!img->quant_present[img->comp[idx[i]].tq])
                return fail(ORN_ERR_BAD_IMAGE, "component uses an undefined quantisation table");
            blocks_per_mcu += ns == 1 ? 1 : img->comp[idx[i]].h * img->comp[idx[i]].v;
        }
        if (blocks_per_mcu > 10) return fail(ORN_ERR_BAD_IMAGE, "more than 10 blocks per MCU");
        const size_t p = seg + 1 + 2 * ns;
        if (u8(p) != 0 || u8(p + 1) != 63 || u8(p + 2) != 0)
            return fail(ORN_ERR_UNSUPPORTED, "spectral selection / successive approximation (progressive)");
        pos = seg + seg_len;

        Bits br{data + pos, data + len};
        int pred[kMaxComponents] = {0, 0, 0};
        uint32_t mcus_x, mcus_y;
        if (ns == 1) {
            const Component& c = img->comp[idx[0]];
            const uint32_t cw = (img->width * c.h + img->hmax - 1) / img->hmax;
            const uint32_t ch = (img->height * c.v + img->vmax - 1) / img->vmax;
            mcus_x = (cw + 7) / 8;
            mcus_y = (ch + 7) / 8;
        } else {
            mcus_x = img->mcux;
            mcus_y = img->mcuy;
        }
        const uint64_t total = (uint64_t)mcus_x * mcus_y;
        uint64_t left_in_interval = restart;
        for (uint64_t m = 0; m < total; ++m) {
            if (restart && left_in_interval == 0) {
                br.resync();
                if (br.p + 1 >= br.end || br.p[1] < 0xD0 || br.p[1] > 0xD7)
                    return fail(ORN_ERR_BAD_IMAGE, "missing restart marker");
                br.p += 2;
                pred[0] = pred[1] = pred[2] = 0;
                left_in_interval = restart;
            }
            const uint32_t mx = (uint32_t)(m % mcus_x), my = (uint32_t)(m / mcus_x);
            for (uint32_t i = 0; i < ns; ++i) {
                Component& c = img->comp[idx[i]];
                const uint32_t nh = ns == 1 ? 1 : c.h, nv = ns == 1 ? 1 : c.v;
                for (uint32_t by = 0; by < nv; ++by)
                    for (uint32_t bx = 0; bx < nh; ++bx) {
                        const uint32_t col = mx * nh + bx, row = my * nv + by;
                        int16_t* out = c.coef.data() + ((size_t)row * c.bw + col) * 64;
                        if (!decode_block(br, dc[td[i]], ac[ta[i]], &pred[i], out))
                            return fail(ORN_ERR_BAD_IMAGE, "corrupt entropy-coded data");
                    }
            }
            if (br.zeros_fed > 64) return fail(ORN_ERR_BAD_IMAGE, "entropy-coded data ends early");
            if (restart) --left_in_interval;
        }
        for (uint32_t i = 0; i < ns; ++i) img->comp[idx[i]].decoded = true;
        br.resync();
        pos = (size_t)(br.p - data);
        return ORN_OK;
    }

    int run(bool header_only) {
        if (len < 4 || data[0] != 0xFF || data[1] != 0xD8) return fail(ORN_ERR_BAD_IMAGE, "not a JPEG stream");
        pos = 2;
        for (;;) {
            // next marker (fill bytes allowed)
            while (pos < len && data[pos] != 0xFF) ++pos;
            while (pos + 1 < len && data[pos + 1] == 0xFF) ++pos;
            if (pos + 1 >= len) return fail(ORN_ERR_BAD_IMAGE, "no end-of-image marker");
            const uint32_t m = data[pos + 1];
            pos += 2;
            if (m == 0xD9) break;                          // EOI
            if (m >= 0xD0 && m <= 0xD7) continue;          // stray RSTn
            if (m == 0x01) continue;                       // TEM
            if (!need(2)) return fail(ORN_ERR_BAD_IMAGE, "truncated marker segment");
            const size_t seg_len = u16(pos);
            if (seg_len < 2 || pos + seg_len > len) return fail(ORN_ERR_BAD_IMAGE, "truncated marker segment");
            const size_t seg = pos + 2, body = seg_len - 2;
            int st = ORN_OK;
            switch (m) {
                case 0xC0:
                case 0xC1:
                    st = read_sof(seg, body, header_only);
                    if (st == ORN_OK && header_only) return ORN_OK;
                    break;
                case 0xC2: case 0xC3: case 0xC5: case 0xC6: case 0xC7:
                case 0xC9: case 0xCA: case 0xCB: case 0xCD: case 0xCE: case 0xCF:
                    return fail(ORN_ERR_UNSUPPORTED, "progressive, lossless, hierarchical or arithmetic-coded JPEG");
                case 0xC4: st = read_dht(seg, body); break;
                case 0xDB: st = read_dqt(seg, body); break;
                case 0xDD:
                    if (body < 2) return fail(ORN_ERR_BAD_IMAGE, "short DRI segment");
                    restart = u16(seg);
                    break;
                case 0xDA:
                    st = read_sos(seg, body);
                    if (st != ORN_OK) return st;
                    continue;                               // pos already past the scan
                case 0xEE:
                    if (body >= 12 && std::memcmp(data + seg, "Adobe", 5) == 0) {
                        adobe = true;
                        adobe_transform = (int)u8(seg + 11);
                    }
                    break;
                case 0xDC:
                    return fail(ORN_ERR_UNSUPPORTED, "DNL marker");
                default:
                    break;                                  // APPn, COM, others: skipped
            }
            if (st != ORN_OK) return st;
            pos += seg_len;
        }
        if (!have_frame) return fail(ORN_ERR_BAD_IMAGE, "no frame header");
        if (header_only) return ORN_OK;
        for (uint32_t i = 0; i < img->ncomp; ++i)
            if (!img->comp[i].decoded) return fail(ORN_ERR_BAD_IMAGE, "a component has no scan");
        if (adobe && img->ncomp == 3) img->ycbcr = adobe_transform != 0;
        return ORN_OK;
    }
};

}  // namespace

std::string& last_error() {
    static thread_local std::string msg;
    return msg;
}

int parse(const uint8_t* data, size_t len, bool header_only, Image* out, std::string* err) {
    if (!data || !out) return ORN_ERR_INVALID_ARGUMENT;
    *out = Image{};
    Parser ps;
    ps.data = data;
    ps.len = len;
    ps.img = out;
    ps.err = err;
    return ps.run(header_only);
}

}  // namespace jpeg
}  // namespace orn

extern "C" {

int orn_jpeg_info(const void* data, size_t len, uint32_t* width, uint32_t* height, uint32_t* components) {
    using namespace orn::jpeg;
    if (!data || !width || !height || !components) return ORN_ERR_INVALID_ARGUMENT;
    Image img;
    last_error().clear();
    const int st = parse((const uint8_t*)data, len, true, &img, &last_error());
    if (st != ORN_OK) return st;
    *width = img.width;
    *height = img.height;
    *components = img.ncomp;
    return ORN_OK;
}

int orn_jpeg_coefficients(const void* data, size_t len, uint32_t component, int16_t* out, size_t out_len,
                          uint32_t* blocks_w, uint32_t* blocks_h, uint16_t* quant) {
    using namespace orn::jpeg;
    if (!data) return ORN_ERR_INVALID_ARGUMENT;
    Image img;
    last_error().clear();
    const int st = parse((const uint8_t*)data, len, false, &img, &last_error());
    if (st != ORN_OK) return st;
    if (component >= img.ncomp) {
        last_error() = "component index out of range";
        return ORN_ERR_INVALID_ARGUMENT;
    }
    const Component& c = img.comp[component];
    if (blocks_w) *blocks_w = c.bw;
    if (blocks_h) *blocks_h = c.bh;
    if (quant) std::memcpy(quant, img.quant[c.tq], 64 * sizeof(uint16_t));
    if (out) {
        if (out_len < c.coef.size()) {
            last_error() = "coefficient buffer too small";
            return ORN_ERR_BUFFER_TOO_SMALL;
        }
        std::memcpy(out, c.coef.data(), c.coef.size() * sizeof(int16_t));
    }
    return ORN_OK;
}

const char* orn_jpeg_last_error(void) { return orn::jpeg::last_error().c_str(); }

}  // extern "C"
