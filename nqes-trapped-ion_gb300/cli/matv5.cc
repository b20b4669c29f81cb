// MAT v5 (MATLAB Level 5) reader/writer; see matv5.h.
//
// Layout: a 128-byte header (116 bytes of text, 8 bytes subsystem offset,
// version 0x0100, endian mark "IM" for little-endian files), then data
// elements. Each element is an 8-byte tag (u32 type, u32 byte count) followed
// by its data padded to 8 bytes; a tag whose upper 16 bits are non-zero is a
// "small" element: type in the low 16 bits, byte count in the high 16 bits,
// up to 4 data bytes in the tag's second word. A variable is an miMATRIX (14)
// element holding, in order, array flags (miUINT32), dimensions (miINT32), the
// name (miINT8), the real part and, for complex arrays, the imaginary part.
#include "matv5.h"

#include <cstdio>
#include <cstring>
#include <ctime>

namespace nqes_cli {

namespace {

enum : uint32_t {
    miINT8 = 1, miUINT8 = 2, miINT16 = 3, miUINT16 = 4, miINT32 = 5, miUINT32 = 6,
    miSINGLE = 7, miDOUBLE = 9, miINT64 = 12, miUINT64 = 13, miMATRIX = 14, miCOMPRESSED = 15,
};
constexpr uint32_t mxDOUBLE_CLASS = 6;
constexpr uint32_t kComplexFlag = 0x0800;

uint32_t rd32(const unsigned char *p) {
    return uint32_t(p[0]) | uint32_t(p[1]) << 8 | uint32_t(p[2]) << 16 | uint32_t(p[3]) << 24;
}

struct Elem {
    uint32_t type = 0, nbytes = 0;
    const unsigned char *data = nullptr;
    size_t total = 0;  // bytes consumed including tag and padding
};

bool next_elem(const unsigned char *p, size_t avail, Elem &e) {
    if (avail < 8) return false;
    const uint32_t w0 = rd32(p), w1 = rd32(p + 4);
    if (w0 >> 16) {  // small data element
        e.type = w0 & 0xffff;
        e.nbytes = w0 >> 16;
        e.data = p + 4;
        e.total = 8;
        return e.nbytes <= 4;
    }
    e.type = w0;
    e.nbytes = w1;
    e.data = p + 8;
    e.total = 8 + ((size_t(w1) + 7) / 8) * 8;
    return e.total <= avail || (e.type == miMATRIX && 8 + size_t(w1) <= avail);
}

bool to_doubles(const Elem &e, std::vector<double> &out, size_t n) {
    out.assign(n, 0.0);
    size_t w = 0;
    switch (e.type) {
    case miINT8: w = 1; break;
    case miUINT8: w = 1; break;
    case miINT16: w = 2; break;
    case miUINT16: w = 2; break;
    case miINT32: w = 4; break;
    case miUINT32: w = 4; break;
    case miSINGLE: w = 4; break;
    case miDOUBLE: w = 8; break;
    case miINT64: w = 8; break;
    case miUINT64: w = 8; break;
    default: return false;
    }
    if (size_t(e.nbytes) < n * w) return false;
    for (size_t t = 0; t < n; t++) {
        const unsigned char *q = e.data + t * w;
        switch (e.type) {
        case miINT8: out[t] = double(int8_t(q[0])); break;
        case miUINT8: out[t] = double(q[0]); break;
        case miINT16: { int16_t v; std::memcpy(&v, q, 2); out[t] = v; break; }
        case miUINT16: { uint16_t v; std::memcpy(&v, q, 2); out[t] = v; break; }
        case miINT32: { int32_t v; std::memcpy(&v, q, 4); out[t] = v; break; }
        case miUINT32: { uint32_t v; std::memcpy(&v, q, 4); out[t] = v; break; }
        case miSINGLE: { float v; std::memcpy(&v, q, 4); out[t] = v; break; }
        case miDOUBLE: { double v; std::memcpy(&v, q, 8); out[t] = v; break; }
        case miINT64: { int64_t v; std::memcpy(&v, q, 8); out[t] = double(v); break; }
        case miUINT64: { uint64_t v; std::memcpy(&v, q, 8); out[t] = double(v); break; }
        }
    }
    return true;
}

void put32(std::vector<unsigned char> &b, uint32_t v) {
    for (int s = 0; s < 32; s += 8) b.push_back((v >> s) & 0xff);
}
void pad8(std::vector<unsigned char> &b) {
    while (b.size() % 8) b.push_back(0);
}
void put_elem(std::vector<unsigned char> &b, uint32_t type, const void *data, uint32_t nbytes) {
    put32(b, type);
    put32(b, nbytes);
    const unsigned char *p = static_cast<const unsigned char *>(data);
    b.insert(b.end(), p, p + nbytes);
    pad8(b);
}

}  // namespace

bool mat_read(const std::string &path, std::map<std::string, MatArray> &vars, std::string &err) {
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) {
        err = "cannot open " + path;
        return false;
    }
    std::vector<unsigned char> buf;
    unsigned char chunk[1 << 16];
    size_t n;
    while ((n = std::fread(chunk, 1, sizeof chunk, f)) > 0) buf.insert(buf.end(), chunk, chunk + n);
    std::fclose(f);
    if (buf.size() < 128 || buf[126] != 'I' || buf[127] != 'M') {
        err = path + " is not a little-endian MAT v5 file";
        return false;
    }
    size_t pos = 128;
    while (pos + 8 <= buf.size()) {
        Elem top;
        if (!next_elem(buf.data() + pos, buf.size() - pos, top)) break;
        if (top.type == miCOMPRESSED) {
            err = path + ": compressed MAT elements are not supported";
            return false;
        }
        if (top.type == miMATRIX) {
            const unsigned char *p = top.data, *end = top.data + top.nbytes;
            Elem flags, dims, name;
            bool ok = next_elem(p, end - p, flags);
            p += ok ? flags.total : 0;
            ok = ok && next_elem(p, end - p, dims);
            p += ok ? dims.total : 0;
            ok = ok && next_elem(p, end - p, name);
            p += ok ? name.total : 0;
            if (ok && flags.nbytes >= 4) {
                MatArray a;
                const uint32_t fl = rd32(flags.data);
                const uint32_t cls = fl & 0xff;
                a.is_complex = (fl & kComplexFlag) != 0;
                a.is_double = cls == mxDOUBLE_CLASS;
                for (uint32_t t = 0; t + 4 <= dims.nbytes; t += 4) a.dims.push_back(size_t(int32_t(rd32(dims.data + t))));
                const std::string nm(reinterpret_cast<const char *>(name.data), name.nbytes);
                Elem rpart, ipart;
                const bool numeric = cls >= 6 && cls <= 15;
                if (numeric && next_elem(p, end - p, rpart) && to_doubles(rpart, a.re, a.numel())) {
                    p += rpart.total;
                    if (a.is_complex) {
                        if (!next_elem(p, end - p, ipart) || !to_doubles(ipart, a.im, a.numel())) {
                            err = path + ": variable " + nm + " has a malformed imaginary part";
                            return false;
                        }
                    }
                    vars[nm] = std::move(a);
                }
            }
        }
        pos += top.total;
    }
    return true;
}

bool mat_write(const std::string &path, const std::vector<std::pair<std::string, MatArray>> &vars, std::string &err) {
    std::vector<unsigned char> b(128, ' ');
    char text[117];
    std::time_t now = std::time(nullptr);
    char tbuf[64];
    std::strftime(tbuf, sizeof tbuf, "%a %b %d %H:%M:%S %Y", std::gmtime(&now));
    std::snprintf(text, sizeof text, "MATLAB 5.0 MAT-file, Platform: GB300, Created by: nqes-gb300 on %s", tbuf);
    std::memcpy(b.data(), text, std::strlen(text));
    for (int t = 116; t < 124; t++) b[t] = 0;
    b[124] = 0x00;
    b[125] = 0x01;
    b[126] = 'I';
    b[127] = 'M';
    for (const auto &[name, a] : vars) {
        std::vector<unsigned char> m;
        uint32_t fl[2] = {mxDOUBLE_CLASS | (a.is_complex ? kComplexFlag : 0u), 0};
        put_elem(m, miUINT32, fl, 8);
        std::vector<int32_t> d(a.dims.begin(), a.dims.end());
        put_elem(m, miINT32, d.data(), uint32_t(d.size() * 4));
        put_elem(m, miINT8, name.data(), uint32_t(name.size()));
        put_elem(m, miDOUBLE, a.re.data(), uint32_t(a.re.size() * 8));
        if (a.is_complex) put_elem(m, miDOUBLE, a.im.data(), uint32_t(a.im.size() * 8));
        put32(b, miMATRIX);
        put32(b, uint32_t(m.size()));
        b.insert(b.end(), m.begin(), m.end());
    }
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) {
        err = "cannot create " + path;
        return false;
    }
    const bool ok = std::fwrite(b.data(), 1, b.size(), f) == b.size();
    std::fclose(f);
    if (!ok) err = "short write to " + path;
    return ok;
}

}  // namespace nqes_cli
