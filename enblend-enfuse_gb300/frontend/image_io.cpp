// image_io.cpp -- baseline TIFF and .npy reading and writing (see image_io.hpp).
#include "image_io.hpp"

#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <stdexcept>

namespace enbfront {

namespace {

[[noreturn]] void fail(const std::string& path, const std::string& why)
{
    throw std::runtime_error(path + ": " + why);
}

std::vector<uint8_t> slurp(const std::string& path)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        fail(path, "cannot open");
    }
    return std::vector<uint8_t>((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
}

bool ends_with(const std::string& s, const std::string& e)
{
    if (s.size() < e.size()) {
        return false;
    }
    std::string t = s.substr(s.size() - e.size());
    for (char& c : t) {
        c = (char)std::tolower((unsigned char)c);
    }
    return t == e;
}

// ---- TIFF ---------------------------------------------------------------------

struct TiffReader {
    const std::vector<uint8_t>& b;
    bool big;
    std::string path;
    uint32_t u16(size_t o) const
    {
        if (o + 2 > b.size()) {
            fail(path, "truncated TIFF");
        }
        return big ? (uint32_t)(b[o] << 8 | b[o + 1]) : (uint32_t)(b[o] | b[o + 1] << 8);
    }
    uint32_t u32(size_t o) const
    {
        if (o + 4 > b.size()) {
            fail(path, "truncated TIFF");
        }
        return big ? ((uint32_t)b[o] << 24 | (uint32_t)b[o + 1] << 16 | (uint32_t)b[o + 2] << 8 | b[o + 3])
                   : ((uint32_t)b[o] | (uint32_t)b[o + 1] << 8 | (uint32_t)b[o + 2] << 16 | (uint32_t)b[o + 3] << 24);
    }
    // values of a tag entry (SHORT or LONG), count n
    std::vector<uint32_t> values(size_t entry) const
    {
        const uint32_t type = u16(entry + 2), n = u32(entry + 4);
        const size_t sz = type == 3 ? 2 : 4;
        if (type != 3 && type != 4) {
            return {};
        }
        size_t off = entry + 8;
        if (n * sz > 4) {
            off = u32(entry + 8);
        }
        std::vector<uint32_t> v(n);
        for (uint32_t i = 0; i < n; ++i) {
            v[i] = sz == 2 ? u16(off + i * 2) : u32(off + i * 4);
        }
        return v;
    }
};

Image read_tiff(const std::string& path)
{
    const std::vector<uint8_t> b = slurp(path);
    if (b.size() < 8 || !((b[0] == 'I' && b[1] == 'I') || (b[0] == 'M' && b[1] == 'M'))) {
        fail(path, "not a TIFF file");
    }
    TiffReader r{b, b[0] == 'M', path};
    if (r.u16(2) != 42) {
        fail(path, "not a classic TIFF file");
    }
    const size_t ifd = r.u32(4);
    const uint32_t n = r.u16(ifd);
    std::map<uint32_t, std::vector<uint32_t>> tag;
    for (uint32_t i = 0; i < n; ++i) {
        const size_t e = ifd + 2 + 12 * i;
        tag[r.u16(e)] = r.values(e);
    }
    const auto one = [&](uint32_t t, uint32_t dflt) { return tag.count(t) && !tag[t].empty() ? tag[t][0] : dflt; };
    if (one(259, 1) != 1) {
        fail(path, "compressed TIFF is not supported (uncompressed baseline TIFF only)");
    }
    if (one(284, 1) != 1) {
        fail(path, "planar TIFF is not supported (chunky samples only)");
    }
    Image img;
    img.width = (int)one(256, 0);
    img.height = (int)one(257, 0);
    img.samples = (int)one(277, 1);
    img.extra = tag.count(338) ? (int)tag[338].size() : 0;
    const uint32_t bits = one(258, 8), fmt = one(339, 1);
    if (bits == 8 && fmt == 1) {
        img.type = SampleType::U8;
    } else if (bits == 16 && fmt == 1) {
        img.type = SampleType::U16;
    } else if (bits == 32 && fmt == 3) {
        img.type = SampleType::F32;
    } else {
        fail(path, "sample format not supported (8/16-bit unsigned or 32-bit float)");
    }
    if (img.width <= 0 || img.height <= 0 || img.samples < 1 || img.samples > 4 || img.extra > 1) {
        fail(path, "image layout not supported");
    }
    const std::vector<uint32_t> offs = tag[273], counts = tag[279];
    if (offs.empty() || offs.size() != counts.size()) {
        fail(path, "missing strips");
    }
    img.data.resize(img.row_bytes() * img.height);
    size_t pos = 0;
    for (size_t s = 0; s < offs.size() && pos < img.data.size(); ++s) {
        const size_t len = std::min<size_t>(counts[s], img.data.size() - pos);
        if ((size_t)offs[s] + len > b.size()) {
            fail(path, "truncated strip");
        }
        std::memcpy(&img.data[pos], &b[offs[s]], len);
        pos += len;
    }
    if (pos != img.data.size()) {
        fail(path, "short image data");
    }
    if (r.big && img.sample_bytes() > 1) {
        const size_t sb = img.sample_bytes();
        for (size_t i = 0; i < img.data.size(); i += sb) {
            for (size_t j = 0; j < sb / 2; ++j) {
                std::swap(img.data[i + j], img.data[i + sb - 1 - j]);
            }
        }
    }
    return img;
}

void put16(std::vector<uint8_t>& v, uint32_t x)
{
    v.push_back((uint8_t)(x & 0xff));
    v.push_back((uint8_t)(x >> 8));
}

void put32(std::vector<uint8_t>& v, uint32_t x)
{
    put16(v, x & 0xffff);
    put16(v, x >> 16);
}

void write_tiff(const std::string& path, const Image& img)
{
    const uint32_t bits = (uint32_t)img.sample_bytes() * 8;
    const size_t nbytes = img.data.size();
    if (nbytes > 0xfff00000u) {
        fail(path, "image too large for a classic TIFF file");
    }
    // header, then the IFD, then the out-of-line values, then the pixels
    struct Entry {
        uint16_t tag, type;
        std::vector<uint32_t> v;
    };
    const uint32_t photometric = img.samples - img.extra >= 3 ? 2 : 1;
    std::vector<Entry> e = {
        {256, 4, {(uint32_t)img.width}},
        {257, 4, {(uint32_t)img.height}},
        {258, 3, std::vector<uint32_t>((size_t)img.samples, bits)},
        {259, 3, {1}},
        {262, 3, {photometric}},
        {273, 4, {0}},  // strip offset, filled below
        {277, 3, {(uint32_t)img.samples}},
        {278, 4, {(uint32_t)img.height}},
        {279, 4, {(uint32_t)nbytes}},
        {284, 3, {1}},
    };
    if (img.extra) {
        e.push_back({338, 3, {2}});  // unassociated alpha
    }
    e.push_back({339, 3, std::vector<uint32_t>((size_t)img.samples, img.type == SampleType::F32 ? 3u : 1u)});
    const uint32_t ifd = 8, ifd_size = 2 + 12 * (uint32_t)e.size() + 4;
    uint32_t extra_off = ifd + ifd_size;
    std::vector<uint8_t> extra;
    const uint32_t data_off_guess = 0;  // computed after the out-of-line values
    (void)data_off_guess;
    // out-of-line arrays
    std::vector<uint32_t> ool(e.size(), 0);
    for (size_t i = 0; i < e.size(); ++i) {
        const size_t sz = e[i].type == 3 ? 2 : 4;
        if (e[i].v.size() * sz > 4) {
            ool[i] = extra_off + (uint32_t)extra.size();
            for (uint32_t x : e[i].v) {
                if (sz == 2) {
                    put16(extra, x);
                } else {
                    put32(extra, x);
                }
            }
        }
    }
    const uint32_t data_off = (extra_off + (uint32_t)extra.size() + 15u) & ~15u;
    for (Entry& x : e) {
        if (x.tag == 273) {
            x.v[0] = data_off;
        }
    }
    std::vector<uint8_t> head = {'I', 'I', 42, 0};
    put32(head, ifd);
    put16(head, (uint32_t)e.size());
    for (size_t i = 0; i < e.size(); ++i) {
        put16(head, e[i].tag);
        put16(head, e[i].type);
        put32(head, (uint32_t)e[i].v.size());
        const size_t sz = e[i].type == 3 ? 2 : 4;
        if (e[i].v.size() * sz > 4) {
            put32(head, ool[i]);
        } else if (sz == 2) {
            put16(head, e[i].v[0]);
            put16(head, e[i].v.size() > 1 ? e[i].v[1] : 0);
        } else {
            put32(head, e[i].v[0]);
        }
    }
    put32(head, 0);  // no next IFD
    head.insert(head.end(), extra.begin(), extra.end());
    head.resize(data_off, 0);
    std::ofstream f(path, std::ios::binary);
    if (!f) {
        fail(path, "cannot create");
    }
    f.write(reinterpret_cast<const char*>(head.data()), (std::streamsize)head.size());
    f.write(reinterpret_cast<const char*>(img.data.data()), (std::streamsize)img.data.size());
    if (!f) {
        fail(path, "write failed");
    }
}

// ---- .npy ---------------------------------------------------------------------

Image read_npy(const std::string& path)
{
    const std::vector<uint8_t> b = slurp(path);
    if (b.size() < 10 || std::memcmp(b.data(), "\x93NUMPY", 6) != 0) {
        fail(path, "not a .npy file");
    }
    const int major = b[6];
    size_t hlen, hoff;
    if (major == 1) {
        hlen = (size_t)b[8] | (size_t)b[9] << 8;
        hoff = 10;
    } else {
        hlen = (size_t)b[8] | (size_t)b[9] << 8 | (size_t)b[10] << 16 | (size_t)b[11] << 24;
        hoff = 12;
    }
    if (hoff + hlen > b.size()) {
        fail(path, "truncated .npy header");
    }
    const std::string h(reinterpret_cast<const char*>(&b[hoff]), hlen);
    Image img;
    if (h.find("'<u1'") != std::string::npos || h.find("'|u1'") != std::string::npos) {
        img.type = SampleType::U8;
    } else if (h.find("'<u2'") != std::string::npos) {
        img.type = SampleType::U16;
    } else if (h.find("'<f4'") != std::string::npos) {
        img.type = SampleType::F32;
    } else {
        fail(path, "array type not supported (uint8, uint16 or float32, little-endian)");
    }
    if (h.find("'fortran_order': True") != std::string::npos) {
        fail(path, "Fortran-ordered arrays are not supported");
    }
    const size_t sp = h.find("'shape': (");
    if (sp == std::string::npos) {
        fail(path, "no shape in the .npy header");
    }
    std::vector<long> dims;
    std::istringstream ss(h.substr(sp + 10, h.find(')', sp) - sp - 10));
    std::string tok;
    while (std::getline(ss, tok, ',')) {
        if (tok.find_first_not_of(" ") != std::string::npos) {
            dims.push_back(std::stol(tok));
        }
    }
    if (dims.size() == 2) {
        dims.push_back(1);
    }
    if (dims.size() != 3 || dims[2] < 1 || dims[2] > 4) {
        fail(path, "expected an (H, W) or (H, W, S) array with S <= 4");
    }
    img.height = (int)dims[0];
    img.width = (int)dims[1];
    img.samples = (int)dims[2];
    img.extra = (img.samples == 2 || img.samples == 4) ? 1 : 0;
    const size_t off = hoff + hlen, n = img.row_bytes() * img.height;
    if (off + n > b.size()) {
        fail(path, "truncated .npy data");
    }
    img.data.assign(b.begin() + (long)off, b.begin() + (long)(off + n));
    return img;
}

void write_npy(const std::string& path, const Image& img)
{
    const char* descr = img.type == SampleType::U8 ? "|u1" : (img.type == SampleType::U16 ? "<u2" : "<f4");
    std::ostringstream h;
    h << "{'descr': '" << descr << "', 'fortran_order': False, 'shape': (" << img.height << ", " << img.width;
    if (img.samples > 1) {
        h << ", " << img.samples;
    }
    h << "), }";
    std::string hs = h.str();
    const size_t total = 10 + hs.size() + 1;
    hs.append((64 - total % 64) % 64, ' ');
    hs.push_back('\n');
    std::ofstream f(path, std::ios::binary);
    if (!f) {
        fail(path, "cannot create");
    }
    const uint8_t pre[10] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0, (uint8_t)(hs.size() & 0xff), (uint8_t)(hs.size() >> 8)};
    f.write(reinterpret_cast<const char*>(pre), 10);
    f.write(hs.data(), (std::streamsize)hs.size());
    f.write(reinterpret_cast<const char*>(img.data.data()), (std::streamsize)img.data.size());
    if (!f) {
        fail(path, "write failed");
    }
}

}  // namespace

Image read_image(const std::string& path)
{
    if (ends_with(path, ".npy")) {
        return read_npy(path);
    }
    if (ends_with(path, ".tif") || ends_with(path, ".tiff")) {
        return read_tiff(path);
    }
    fail(path, "unknown image format (TIFF or .npy)");
}

void write_image(const std::string& path, const Image& img)
{
    if (ends_with(path, ".npy")) {
        write_npy(path, img);
    } else if (ends_with(path, ".tif") || ends_with(path, ".tiff")) {
        write_tiff(path, img);
    } else {
        fail(path, "unknown output format (TIFF or .npy)");
    }
}

std::string sample_type_name(SampleType t)
{
    return t == SampleType::U8 ? "UINT8" : (t == SampleType::U16 ? "UINT16" : "FLOAT");
}

}  // namespace enbfront
