// image_io.hpp -- image files of the enfuse / enblend front ends: baseline
// TIFF (uncompressed, chunky, 8/16-bit unsigned or 32-bit float samples,
// gray / gray + alpha / RGB / RGBA, strips) and NumPy .npy arrays (uint8,
// uint16 or float32, (H, W) or (H, W, S)).  The reference reads and writes
// its images through VIGRA's impex (src/assemble.h:133-295); this is the
// subset its hot path needs, without libtiff.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace enbfront {

enum class SampleType { U8, U16, F32 };

struct Image {
    int width = 0, height = 0;
    int samples = 0;        // samples a pixel (1 gray, 2 gray + alpha, 3 RGB, 4 RGBA)
    int extra = 0;          // of which extra (alpha) samples: 0 or 1
    SampleType type = SampleType::U8;
    std::vector<uint8_t> data;  // interleaved rows, no padding
    size_t sample_bytes() const { return type == SampleType::U8 ? 1 : (type == SampleType::U16 ? 2 : 4); }
    size_t row_bytes() const { return (size_t)width * samples * sample_bytes(); }
};

// Reads a .tif/.tiff or .npy file; throws std::runtime_error with the reason.
Image read_image(const std::string& path);
// Writes by the file name's extension (.tif/.tiff or .npy).
void write_image(const std::string& path, const Image& img);

std::string sample_type_name(SampleType t);

}  // namespace enbfront
