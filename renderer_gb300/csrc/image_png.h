// image_png.h — PNG decoding for texture and environment images, written for
// this library (no codec library is linked).
//
// The renderer reads texture images with cv::imread(file) (IMREAD_COLOR,
// src/texturematerial.cpp:50) and environment images with
// cv::imread(file, ANYDEPTH | COLOR) (src/environmentmap.cpp:22). IMREAD_COLOR
// yields 8-bit BGR: grey is replicated to three channels, palette indices are
// expanded, alpha is dropped and 16-bit samples keep their high byte. The
// decoder here returns that image as floats 0..255 in BGR order, row 0 at the
// top, like the repository's PPM reader.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace gbrt_img {

// zlib stream (RFC 1950) around DEFLATE data (RFC 1951): appends the
// inflated bytes to out. Returns false with a reason on malformed input, a
// bad Adler-32 checksum or output beyond max_out bytes.
bool zlib_inflate(const uint8_t* in, size_t n, std::vector<uint8_t>& out, size_t max_out, std::string& why);

// True when the bytes start with the PNG signature.
bool is_png(const std::string& data);

// PNG (ISO/IEC 15948): bit depths 1-16, colour types grey, RGB, palette,
// grey+alpha and RGBA, non-interlaced and Adam7, chunk CRCs checked.
bool decode_png(const std::string& data, std::vector<float>& bgr, int& W, int& H, std::string& why);

}  // namespace gbrt_img
