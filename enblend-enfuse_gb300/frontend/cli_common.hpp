// cli_common.hpp -- pieces shared by the enfuse and enblend front ends:
// option values in the reference's formats (src/common.h, src/enfuse.cc),
// conversions between image files and enb_image descriptors, and errors.
#pragma once

#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <regex>
#include <stdexcept>
#include <string>
#include <vector>

#include "enbgpu.h"
#include "image_io.hpp"

namespace enbfront {

struct UsageError : std::runtime_error {
    explicit UsageError(const std::string& m) : std::runtime_error(m) {}
};

inline std::string lower(std::string s)
{
    for (char& c : s) {
        c = (char)std::tolower((unsigned char)c);
    }
    return s;
}

// Tokens of a numeric option argument, split at the reference's delimiters
// ";:/" (NUMERIC_OPTION_DELIMITERS, src/common.h:45).
inline std::vector<std::string> split_numeric(const std::string& a)
{
    std::vector<std::string> out;
    const std::regex delim("[;:/]");
    for (std::sregex_token_iterator t(a.begin(), a.end(), delim, -1), e; t != e; ++t) {
        out.push_back(t->str());
    }
    return out;
}

inline double number(const std::string& opt, const std::string& v)
{
    size_t tail = 0;
    double x = 0.0;
    try {
        x = std::stod(v, &tail);
    } catch (const std::exception&) {
        throw UsageError("illegal numeric format \"" + v + "\" of " + opt);
    }
    if (tail != v.size()) {
        throw UsageError("trailing characters \"" + v.substr(tail) + "\" in the argument of " + opt);
    }
    return x;
}

inline int integer(const std::string& opt, const std::string& v)
{
    size_t tail = 0;
    long x = 0;
    try {
        x = std::stol(v, &tail);
    } catch (const std::exception&) {
        throw UsageError(opt + " requires an integer argument, not \"" + v + "\"");
    }
    if (tail != v.size()) {
        throw UsageError(opt + " requires an integer argument, not \"" + v + "\"");
    }
    return (int)x;
}

// A cutoff value: a number, a percentage when it ends in '%'
// (AlternativePercentage, src/enfuse.cc:1225-1258).
inline void cutoff_value(const std::string& opt, const std::string& tok, double& value, int32_t& pct)
{
    size_t tail = 0;
    try {
        value = std::stod(tok, &tail);
    } catch (const std::exception&) {
        throw UsageError("illegal numeric format \"" + tok + "\" in " + opt);
    }
    if (tail == tok.size()) {
        pct = 0;
    } else if (tok.substr(tail) == "%") {
        pct = 1;
    } else {
        throw UsageError("unrecognized cutoff \"" + tok.substr(tail) + "\" in \"" + tok + "\" of " + opt);
    }
}

// Gray projector names of MultiGrayscaleAccessor (src/mga.h:78-123); the
// channel mixer takes its weights as "channel-mixer:R:G:B".
inline int gray_projector(const std::string& name, double mixer[3])
{
    const std::string n = lower(name);
    if (n.empty() || n == "average") return ENB_GRAY_AVERAGE;
    if (n == "value") return ENB_GRAY_VALUE;
    if (n == "anti-value") return ENB_GRAY_ANTI_VALUE;
    if (n == "lightness") return ENB_GRAY_LIGHTNESS;
    if (n == "luminance") return ENB_GRAY_LUMINANCE;
    if (n == "l-star" || n == "pl-star") {
        throw UsageError("grayscale projector \"" + name + "\" (CIE L*) is not supported by this build");
    }
    if (n.compare(0, 13, "channel-mixer") == 0) {
        const std::vector<std::string> t = split_numeric(n.substr(13));
        std::vector<std::string> w;
        for (const std::string& s : t) {
            if (!s.empty()) {
                w.push_back(s);
            }
        }
        if (w.size() != 3) {
            throw UsageError("\"channel-mixer\" is a grayscale projector requiring arguments like "
                             "\"channel-mixer:0.30:0.59:0.11\"");
        }
        for (int i = 0; i < 3; ++i) {
            mixer[i] = number("--gray-projector", w[i]);
            if (mixer[i] < 0.0) {
                throw UsageError("nonsensical channel weight " + w[i]);
            }
        }
        if (mixer[0] + mixer[1] + mixer[2] == 0.0) {
            throw UsageError("sum of channel weights is zero");
        }
        return ENB_GRAY_MIXER;
    }
    throw UsageError("unknown grayscale projector \"" + name + "\"");
}

// wraparoundOfString (src/common.h:305-316).  The reference's pyramids know
// only the periodic x direction: every mode but none wraps horizontally.
inline int wrap_mode(const std::string& a)
{
    const std::string m = lower(a);
    if (m.empty() || m == "horizontal") return 1;
    if (m == "none" || m == "open") return 0;
    if (m == "vertical" || m == "both" || m == "horizontal+vertical" || m == "vertical+horizontal") return 1;
    throw UsageError("unrecognized wrap-around mode \"" + a + "\"");
}

// --levels: an integer or "auto" (src/enfuse.cc:1696-1725).
inline int levels_arg(const std::string& a)
{
    const std::string u = lower(a);
    if (u == "auto" || u == "automatic") return 0;
    if (a.find_first_not_of("+-0123456789") != std::string::npos || a.empty()) {
        throw UsageError("options \"-l\" or \"--levels\" require an integer argument or \"auto\"");
    }
    int n = integer("--levels", a);
    if (n == 0) n = 1;
    return n > 29 ? 29 : n;
}

// expandFilenameTemplate's "%n" / "%i" / "%%" (src/common.h:710-790) for the
// mask files: %n the one-based image number, %i the zero-based one, both
// zero-padded to the digits of the image count unless a width is given.
inline std::string expand_template(const std::string& t, unsigned count, unsigned number)
{
    std::string out;
    for (size_t i = 0; i < t.size(); ++i) {
        if (t[i] != '%' || i + 1 >= t.size()) {
            out.push_back(t[i]);
            continue;
        }
        size_t j = i + 1;
        char pad = '0';
        while (j < t.size() && (t[j] == '0' || std::ispunct((unsigned char)t[j])) && t[j] != '%') {
            pad = t[j++];
        }
        std::string width;
        while (j < t.size() && std::isdigit((unsigned char)t[j])) {
            width.push_back(t[j++]);
        }
        if (j >= t.size()) {
            out.push_back('%');
            break;
        }
        const char c = t[j];
        if (c == '%') {
            out.push_back('%');
        } else if (c == 'n' || c == 'i') {
            const unsigned n = c == 'n' ? number + 1 : number, total = c == 'n' ? count + 1 : count;
            unsigned digits = 1;
            for (unsigned v = total - 1; v >= 10; v /= 10) {
                ++digits;
            }
            const unsigned wdt = width.empty() ? digits : (unsigned)std::atoi(width.c_str());
            std::string s = std::to_string(n);
            while (s.size() < wdt) {
                s.insert(s.begin(), pad);
            }
            out += s;
        } else {
            throw UsageError(std::string("unsupported conversion \"%") + c + "\" in the mask template \"" + t + "\"");
        }
        i = j;
    }
    return out;
}

inline int dtype_of(SampleType t)
{
    return t == SampleType::U8 ? ENB_U8 : (t == SampleType::U16 ? ENB_U16 : ENB_F32);
}

// Descriptor of an interleaved host image (colour samples without the alpha).
inline enb_image pixel_desc(Image& img)
{
    enb_image d{};
    d.data = img.data.data();
    d.pitch = (int64_t)img.row_bytes();
    d.width = img.width;
    d.height = img.height;
    d.channels = img.samples - img.extra >= 3 ? 3 : 1;
    d.pix_stride = img.samples;
    d.dtype = dtype_of(img.type);
    d.planar = 0;
    return d;
}

inline enb_image plane_desc(void* p, int w, int h, int64_t pitch, int dtype)
{
    enb_image d{};
    d.data = p;
    d.pitch = pitch;
    d.width = w;
    d.height = h;
    d.channels = 1;
    d.pix_stride = 1;
    d.dtype = dtype;
    return d;
}

// The output image as the reference writes it (checkpoint, src/assemble.h:
// 133-225): the colour samples and an alpha band of the union alpha (0 or the
// type's maximum, 1.0 for float).
inline Image with_alpha(const Image& colour, int C, const std::vector<uint8_t>& alpha)
{
    Image o;
    o.width = colour.width;
    o.height = colour.height;
    o.samples = C + 1;
    o.extra = 1;
    o.type = colour.type;
    const size_t sb = colour.sample_bytes(), npx = (size_t)colour.width * colour.height;
    o.data.resize(npx * o.samples * sb);
    for (size_t p = 0; p < npx; ++p) {
        std::memcpy(&o.data[p * o.samples * sb], &colour.data[p * colour.samples * sb], (size_t)C * sb);
        uint8_t* a = &o.data[(p * o.samples + C) * sb];
        if (colour.type == SampleType::U8) {
            a[0] = alpha[p] ? 255 : 0;
        } else if (colour.type == SampleType::U16) {
            const uint16_t v = alpha[p] ? 65535 : 0;
            std::memcpy(a, &v, 2);
        } else {
            const float v = alpha[p] ? 1.0f : 0.0f;
            std::memcpy(a, &v, 4);
        }
    }
    return o;
}

// The alpha plane of an image as the library thresholds it (the 4th sample
// of RGBA pixels between half the type's maximum and the maximum,
// src/assemble.h:240-253; [0.5, 1] for float), 255 or 0; opaque otherwise.
inline std::vector<uint8_t> alpha_plane(const Image& img)
{
    const size_t npx = (size_t)img.width * img.height;
    std::vector<uint8_t> a(npx, 255);
    if (img.samples != 4) {
        return a;  // the library reads a footprint from the 4th sample of RGBA pixels only
    }
    const int ai = 3;
    for (size_t p = 0; p < npx; ++p) {
        const size_t i = p * img.samples + ai;
        bool on;
        if (img.type == SampleType::U8) {
            on = img.data[i] >= 127;
        } else if (img.type == SampleType::U16) {
            uint16_t v;
            std::memcpy(&v, &img.data[i * 2], 2);
            on = v >= 32767;
        } else {
            float v;
            std::memcpy(&v, &img.data[i * 4], 4);
            on = v >= 0.5f && v <= 1.0f;
        }
        a[p] = on ? 255 : 0;
    }
    return a;
}

inline void check(enb_ctx* ctx, enb_status st, const char* what)
{
    if (st != ENB_OK) {
        throw std::runtime_error(std::string(what) + ": " + (ctx ? enb_last_error(ctx) : "no context"));
    }
}

}  // namespace enbfront
