// npz.cpp -- .npz (zip of .npy) reader with a small DEFLATE decoder.
//
// The zip structures (end-of-central-directory, central directory, local
// headers, ZIP64 extra field 0x0001) follow PKWARE's APPNOTE.TXT; the .npy
// header follows numpy's format spec (magic \x93NUMPY, version, little-endian
// header length, Python-literal dict with descr / fortran_order / shape);
// inflate follows RFC 1951 (stored, fixed and dynamic Huffman blocks, decoded
// with canonical code counts).  The length / distance base tables are the
// ones the RFC defines.
#include "npz.h"

#include <cstdio>
#include <cstring>

#include "common.h"

namespace cnncrf {

namespace {

struct Bits {
    const uint8_t *p;
    size_t n, pos = 0; // bit position
    bool err = false;
    int bit()
    {
        if ((pos >> 3) >= n) {
            err = true;
            return 0;
        }
        int b = (p[pos >> 3] >> (pos & 7)) & 1;
        ++pos;
        return b;
    }
    uint32_t get(int k)
    {
        uint32_t v = 0;
        for (int i = 0; i < k; ++i) v |= (uint32_t)bit() << i;
        return v;
    }
};

struct Huff {
    uint16_t count[16];
    std::vector<uint16_t> sym;
};

// canonical code from code lengths (RFC 1951 3.2.2)
bool build(Huff &h, const uint8_t *len, int n)
{
    std::memset(h.count, 0, sizeof h.count);
    for (int i = 0; i < n; ++i) h.count[len[i]]++;
    h.count[0] = 0;
    uint16_t offs[16];
    offs[1] = 0;
    for (int l = 1; l < 15; ++l) offs[l + 1] = offs[l] + h.count[l];
    h.sym.assign(n, 0);
    for (int i = 0; i < n; ++i)
        if (len[i]) h.sym[offs[len[i]]++] = (uint16_t)i;
    return true;
}

int decode(Bits &b, const Huff &h)
{
    int code = 0, first = 0, index = 0;
    for (int l = 1; l < 16; ++l) {
        code |= b.bit();
        int c = h.count[l];
        if (code - first < c) return h.sym[index + (code - first)];
        index += c;
        first += c;
        first <<= 1;
        code <<= 1;
        if (b.err) return -1;
    }
    return -1;
}

const uint16_t LBASE[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                            31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t LEXT[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t DBASE[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                            193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t DEXT[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

bool codes(Bits &b, const Huff &lit, const Huff &dist, std::vector<uint8_t> &out, size_t cap)
{
    for (;;) {
        int s = decode(b, lit);
        if (s < 0 || b.err) return false;
        if (s < 256) {
            if (out.size() >= cap) return false;
            out.push_back((uint8_t)s);
        } else if (s == 256) {
            return true;
        } else {
            s -= 257;
            if (s >= 29) return false;
            size_t len = LBASE[s] + b.get(LEXT[s]);
            int ds = decode(b, dist);
            if (ds < 0 || ds >= 30) return false;
            size_t d = DBASE[ds] + b.get(DEXT[ds]);
            if (d > out.size() || out.size() + len > cap || b.err) return false;
            size_t from = out.size() - d;
            for (size_t i = 0; i < len; ++i) out.push_back(out[from + i]);
        }
    }
}

uint16_t rd16(const uint8_t *p) { return (uint16_t)(p[0] | (p[1] << 8)); }
uint32_t rd32(const uint8_t *p) { return (uint32_t)rd16(p) | ((uint32_t)rd16(p + 2) << 16); }
uint64_t rd64(const uint8_t *p) { return (uint64_t)rd32(p) | ((uint64_t)rd32(p + 4) << 32); }

// parse the .npy header of a decompressed member
int parse_npy(const std::vector<uint8_t> &b, const std::string &what, NpyArray *out)
{
    if (b.size() < 10 || b[0] != 0x93 || std::memcmp(&b[1], "NUMPY", 5) != 0)
        return fail(CNNCRF_EIO, "%s: not a .npy member", what.c_str());
    int major = b[6];
    size_t hl, off;
    if (major == 1) {
        hl = rd16(&b[8]);
        off = 10;
    } else {
        if (b.size() < 12) return fail(CNNCRF_EIO, "%s: truncated .npy header", what.c_str());
        hl = rd32(&b[8]);
        off = 12;
    }
    if (off + hl > b.size()) return fail(CNNCRF_EIO, "%s: truncated .npy header", what.c_str());
    std::string hdr((const char *)&b[off], hl);
    if (hdr.find("'<f4'") == std::string::npos)
        return fail(CNNCRF_ESHAPE, "%s: dtype is not little-endian float32 (%s)", what.c_str(), hdr.c_str());
    if (hdr.find("'fortran_order': True") != std::string::npos)
        return fail(CNNCRF_ESHAPE, "%s: Fortran-ordered arrays are not supported", what.c_str());
    size_t sp = hdr.find("'shape'");
    size_t lp = hdr.find('(', sp), rp = hdr.find(')', lp);
    if (sp == std::string::npos || lp == std::string::npos || rp == std::string::npos)
        return fail(CNNCRF_EIO, "%s: no shape in .npy header", what.c_str());
    out->shape.clear();
    int64_t n = 1;
    const char *s = hdr.c_str() + lp + 1, *e = hdr.c_str() + rp;
    while (s < e) {
        while (s < e && (*s == ' ' || *s == ',')) ++s;
        if (s >= e) break;
        char *end;
        long long v = strtoll(s, &end, 10);
        if (end == s) return fail(CNNCRF_EIO, "%s: bad shape", what.c_str());
        out->shape.push_back(v);
        n *= v;
        s = end;
    }
    size_t data = off + hl;
    if (b.size() - data < (size_t)n * 4) return fail(CNNCRF_EIO, "%s: truncated data", what.c_str());
    out->data.resize((size_t)n);
    std::memcpy(out->data.data(), &b[data], (size_t)n * 4);
    return CNNCRF_OK;
}

} // namespace

bool inflate_raw(const uint8_t *in, size_t in_size, std::vector<uint8_t> *out, size_t out_size)
{
    Bits b{in, in_size};
    out->clear();
    out->reserve(out_size);
    int last;
    do {
        last = b.bit();
        int type = (int)b.get(2);
        if (b.err) return false;
        if (type == 0) {
            b.pos = (b.pos + 7) & ~(size_t)7;
            size_t byte = b.pos >> 3;
            if (byte + 4 > in_size) return false;
            uint16_t len = rd16(in + byte), nlen = rd16(in + byte + 2);
            if ((uint16_t)~nlen != len || byte + 4 + len > in_size || out->size() + len > out_size) return false;
            out->insert(out->end(), in + byte + 4, in + byte + 4 + len);
            b.pos = (byte + 4 + len) * 8;
        } else if (type == 1) {
            uint8_t l[288], d[30];
            for (int i = 0; i < 144; ++i) l[i] = 8;
            for (int i = 144; i < 256; ++i) l[i] = 9;
            for (int i = 256; i < 280; ++i) l[i] = 7;
            for (int i = 280; i < 288; ++i) l[i] = 8;
            for (int i = 0; i < 30; ++i) d[i] = 5;
            Huff lit, dist;
            build(lit, l, 288);
            build(dist, d, 30);
            if (!codes(b, lit, dist, *out, out_size)) return false;
        } else if (type == 2) {
            int nlen = (int)b.get(5) + 257, ndist = (int)b.get(5) + 1, ncode = (int)b.get(4) + 4;
            static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19] = {0};
            for (int i = 0; i < ncode; ++i) cl[order[i]] = (uint8_t)b.get(3);
            Huff lencode;
            build(lencode, cl, 19);
            uint8_t lens[320] = {0};
            int idx = 0;
            while (idx < nlen + ndist) {
                int s = decode(b, lencode);
                if (s < 0 || b.err) return false;
                if (s < 16) {
                    lens[idx++] = (uint8_t)s;
                } else {
                    int rep;
                    uint8_t val = 0;
                    if (s == 16) {
                        if (idx == 0) return false;
                        val = lens[idx - 1];
                        rep = 3 + (int)b.get(2);
                    } else if (s == 17) {
                        rep = 3 + (int)b.get(3);
                    } else {
                        rep = 11 + (int)b.get(7);
                    }
                    if (idx + rep > nlen + ndist) return false;
                    while (rep--) lens[idx++] = val;
                }
            }
            Huff lit, dist;
            build(lit, lens, nlen);
            build(dist, lens + nlen, ndist);
            if (!codes(b, lit, dist, *out, out_size)) return false;
        } else {
            return false;
        }
    } while (!last);
    return out->size() == out_size;
}

int npz_load(const std::string &path, const std::string &key, NpyArray *out)
{
    FILE *f = fopen(path.c_str(), "rb");
    if (!f) return fail(CNNCRF_EIO, "cannot open %s", path.c_str());
    std::vector<uint8_t> buf;
    fseek(f, 0, SEEK_END);
    long sz = ftell(f);
    fseek(f, 0, SEEK_SET);
    if (sz > 0) {
        buf.resize((size_t)sz);
        if (fread(buf.data(), 1, (size_t)sz, f) != (size_t)sz) buf.clear();
    }
    fclose(f);
    if (buf.size() < 22) return fail(CNNCRF_EIO, "%s: not a zip archive", path.c_str());
    // end of central directory: scan back over a possible comment
    long eocd = -1;
    for (long i = (long)buf.size() - 22; i >= 0 && i >= (long)buf.size() - 22 - 65535; --i)
        if (rd32(&buf[i]) == 0x06054b50u) {
            eocd = i;
            break;
        }
    if (eocd < 0) return fail(CNNCRF_EIO, "%s: no end of central directory", path.c_str());
    uint64_t nent = rd16(&buf[eocd + 10]);
    uint64_t cd = rd32(&buf[eocd + 16]);
    if (cd == 0xFFFFFFFFull || nent == 0xFFFF) { // ZIP64 end record via its locator
        long loc = eocd - 20;
        if (loc < 0 || rd32(&buf[loc]) != 0x07064b50u) return fail(CNNCRF_EIO, "%s: bad ZIP64 locator", path.c_str());
        uint64_t z64 = rd64(&buf[loc + 8]);
        if (z64 + 56 > buf.size() || rd32(&buf[z64]) != 0x06064b50u)
            return fail(CNNCRF_EIO, "%s: bad ZIP64 end record", path.c_str());
        nent = rd64(&buf[z64 + 32]);
        cd = rd64(&buf[z64 + 48]);
    }
    std::string want = key + ".npy";
    uint64_t p = cd;
    for (uint64_t e = 0; e < nent; ++e) {
        if (p + 46 > buf.size() || rd32(&buf[p]) != 0x02014b50u)
            return fail(CNNCRF_EIO, "%s: corrupt central directory", path.c_str());
        uint16_t method = rd16(&buf[p + 10]);
        uint64_t csize = rd32(&buf[p + 20]), usize = rd32(&buf[p + 24]);
        uint16_t nl = rd16(&buf[p + 28]), xl = rd16(&buf[p + 30]), cl = rd16(&buf[p + 32]);
        uint64_t lho = rd32(&buf[p + 42]);
        if (p + 46 + nl + xl > buf.size()) return fail(CNNCRF_EIO, "%s: corrupt central directory", path.c_str());
        std::string name((const char *)&buf[p + 46], nl);
        // ZIP64 extra: the 0xFFFFFFFF fields in order usize, csize, offset
        const uint8_t *x = &buf[p + 46 + nl], *xe = x + xl;
        while (x + 4 <= xe) {
            uint16_t tag = rd16(x), len = rd16(x + 2);
            const uint8_t *d = x + 4;
            if (tag == 0x0001) {
                if (usize == 0xFFFFFFFFull && d + 8 <= x + 4 + len) usize = rd64(d), d += 8;
                if (csize == 0xFFFFFFFFull && d + 8 <= x + 4 + len) csize = rd64(d), d += 8;
                if (lho == 0xFFFFFFFFull && d + 8 <= x + 4 + len) lho = rd64(d), d += 8;
            }
            x += 4 + len;
        }
        p += 46 + nl + xl + cl;
        if (name != want) continue;
        if (lho + 30 > buf.size() || rd32(&buf[lho]) != 0x04034b50u)
            return fail(CNNCRF_EIO, "%s: corrupt local header of %s", path.c_str(), name.c_str());
        uint64_t data = lho + 30 + rd16(&buf[lho + 26]) + rd16(&buf[lho + 28]);
        if (data + csize > buf.size()) return fail(CNNCRF_EIO, "%s: truncated member %s", path.c_str(), name.c_str());
        std::vector<uint8_t> raw;
        if (method == 0) {
            raw.assign(buf.begin() + data, buf.begin() + data + csize);
        } else if (method == 8) {
            if (!inflate_raw(&buf[data], csize, &raw, usize))
                return fail(CNNCRF_EIO, "%s: bad deflate stream in %s", path.c_str(), name.c_str());
        } else {
            return fail(CNNCRF_EIO, "%s: compression method %d of %s not supported", path.c_str(), method,
                        name.c_str());
        }
        return parse_npy(raw, path + ":" + name, out);
    }
    return fail(CNNCRF_EIO, "%s: no array %s", path.c_str(), key.c_str());
}

} // namespace cnncrf
