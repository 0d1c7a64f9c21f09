// npz.cpp -- .npz (zip of .npy) reader with a small DEFLATE decoder, and a
// writer of uncompressed archives (training checkpoints).
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
#include <string>

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

namespace {

// CRC-32 of the zip format (reflected polynomial 0xEDB88320, initial and
// final XOR 0xFFFFFFFF; APPNOTE.TXT 4.4.7), table-driven
struct Crc32Table {
    uint32_t t[256];
    Crc32Table()
    {
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t c = i;
            for (int k = 0; k < 8; ++k) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            t[i] = c;
        }
    }
};

uint32_t crc32_update(uint32_t crc, const uint8_t *p, size_t n)
{
    static const Crc32Table table; // initialised once, thread-safe
    crc = ~crc;
    for (size_t i = 0; i < n; ++i) crc = table.t[(crc ^ p[i]) & 0xffu] ^ (crc >> 8);
    return ~crc;
}

void put16(std::vector<uint8_t> &b, uint32_t v)
{
    b.push_back((uint8_t)v);
    b.push_back((uint8_t)(v >> 8));
}
void put32(std::vector<uint8_t> &b, uint32_t v)
{
    put16(b, v & 0xffffu);
    put16(b, v >> 16);
}

// .npy format 1.0 header: magic, version, header length, the dict padded
// with spaces and ended by '\n' so that the data starts 64-byte aligned
std::vector<uint8_t> npy_header(const std::vector<int64_t> &shape)
{
    std::string dict = "{'descr': '<f4', 'fortran_order': False, 'shape': (";
    for (size_t i = 0; i < shape.size(); ++i) {
        dict += std::to_string((long long)shape[i]);
        if (shape.size() == 1 || i + 1 < shape.size()) dict += ",";
        if (i + 1 < shape.size()) dict += " ";
    }
    dict += "), }";
    size_t total = 10 + dict.size() + 1;
    dict.append((64 - total % 64) % 64, ' ');
    dict += '\n';
    std::vector<uint8_t> h = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
    put16(h, (uint32_t)dict.size());
    h.insert(h.end(), dict.begin(), dict.end());
    return h;
}

} // namespace

int npz_save(const std::string &path, const std::vector<NpzMember> &members)
{
    if (members.size() > 0xFFFEu) return fail(CNNCRF_EUNSUPPORTED, "npz_save: %zu members", members.size());
    const std::string tmp = path + ".tmp";
    FILE *f = fopen(tmp.c_str(), "wb");
    if (!f) return fail(CNNCRF_EIO, "npz_save: cannot create %s", tmp.c_str());
    std::vector<uint8_t> cdir;
    uint64_t off = 0;
    bool ok = true;
    for (const NpzMember &m : members) {
        int64_t n = 1;
        for (int64_t s : m.shape) {
            if (s < 0) ok = false;
            n *= s;
        }
        if (!ok || (n > 0 && !m.data)) {
            fclose(f);
            remove(tmp.c_str());
            return fail(CNNCRF_EINVAL, "npz_save: member %s has a bad shape or no data", m.key.c_str());
        }
        const std::string name = m.key + ".npy";
        const std::vector<uint8_t> hdr = npy_header(m.shape);
        const uint64_t size = hdr.size() + (uint64_t)n * 4;
        if (off + 30 + name.size() + size >= 0xFFFFFFFFull) {
            fclose(f);
            remove(tmp.c_str());
            return fail(CNNCRF_EUNSUPPORTED, "npz_save: archive above 4 GiB at member %s", m.key.c_str());
        }
        uint32_t crc = crc32_update(0, hdr.data(), hdr.size());
        crc = crc32_update(crc, (const uint8_t *)m.data, (size_t)n * 4);
        // local file header (APPNOTE 4.3.7): version 2.0, no flags, STORED, 1980-01-01 00:00
        std::vector<uint8_t> lh;
        put32(lh, 0x04034b50u);
        put16(lh, 20), put16(lh, 0), put16(lh, 0), put16(lh, 0), put16(lh, 0x21);
        put32(lh, crc), put32(lh, (uint32_t)size), put32(lh, (uint32_t)size);
        put16(lh, (uint32_t)name.size()), put16(lh, 0);
        lh.insert(lh.end(), name.begin(), name.end());
        ok = fwrite(lh.data(), 1, lh.size(), f) == lh.size() && fwrite(hdr.data(), 1, hdr.size(), f) == hdr.size() &&
             (n == 0 || fwrite(m.data, 4, (size_t)n, f) == (size_t)n);
        if (!ok) break;
        // its central directory entry (APPNOTE 4.3.12)
        put32(cdir, 0x02014b50u);
        put16(cdir, 20), put16(cdir, 20), put16(cdir, 0), put16(cdir, 0), put16(cdir, 0), put16(cdir, 0x21);
        put32(cdir, crc), put32(cdir, (uint32_t)size), put32(cdir, (uint32_t)size);
        put16(cdir, (uint32_t)name.size()), put16(cdir, 0), put16(cdir, 0), put16(cdir, 0), put16(cdir, 0);
        put32(cdir, 0), put32(cdir, (uint32_t)off);
        cdir.insert(cdir.end(), name.begin(), name.end());
        off += lh.size() + size;
    }
    if (ok) {
        // end of central directory record (APPNOTE 4.3.16)
        std::vector<uint8_t> end;
        put32(end, 0x06054b50u);
        put16(end, 0), put16(end, 0), put16(end, (uint32_t)members.size()), put16(end, (uint32_t)members.size());
        put32(end, (uint32_t)cdir.size()), put32(end, (uint32_t)off), put16(end, 0);
        ok = off + cdir.size() < 0xFFFFFFFFull && fwrite(cdir.data(), 1, cdir.size(), f) == cdir.size() &&
             fwrite(end.data(), 1, end.size(), f) == end.size();
    }
    ok = (fclose(f) == 0) && ok;
    if (!ok || rename(tmp.c_str(), path.c_str()) != 0) {
        remove(tmp.c_str());
        return fail(CNNCRF_EIO, "npz_save: cannot write %s", path.c_str());
    }
    return CNNCRF_OK;
}

} // namespace cnncrf

extern "C" {

int cnncrf_npz_read(const char *npz_path, const char *key, int64_t shape[4], int *ndim, float *h_data,
                    size_t capacity)
{
    using namespace cnncrf;
    clear_error();
    if (!npz_path || !key || !shape || !ndim) return fail(CNNCRF_EINVAL, "null argument");
    NpyArray a;
    CNNCRF_TRY(npz_load(npz_path, key, &a));
    if (a.shape.size() > 4) return fail(CNNCRF_ESHAPE, "npz_read: %s has %zu dimensions", key, a.shape.size());
    *ndim = (int)a.shape.size();
    for (size_t i = 0; i < a.shape.size(); ++i) shape[i] = a.shape[i];
    if (h_data) {
        if (capacity < a.data.size())
            return fail(CNNCRF_ESHAPE, "npz_read: %s has %zu values, the buffer %zu", key, a.data.size(), capacity);
        std::memcpy(h_data, a.data.data(), a.data.size() * sizeof(float));
    }
    return CNNCRF_OK;
}

int cnncrf_npz_write(const char *npz_path, int count, const char *const *keys, const float *const *h_data,
                     const int64_t *shapes, const int *ndims)
{
    using namespace cnncrf;
    clear_error();
    if (!npz_path || count < 0 || (count > 0 && (!keys || !h_data || !shapes || !ndims)))
        return fail(CNNCRF_EINVAL, "null argument");
    std::vector<NpzMember> m((size_t)count);
    for (int i = 0; i < count; ++i) {
        if (!keys[i] || ndims[i] < 0 || ndims[i] > 4) return fail(CNNCRF_EINVAL, "npz_write: member %d", i);
        m[i].key = keys[i];
        m[i].data = h_data[i];
        m[i].shape.assign(shapes + 4 * i, shapes + 4 * i + ndims[i]);
    }
    return npz_save(npz_path, m);
}

} // extern "C"
