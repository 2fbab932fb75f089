// image_jpeg.h — JPEG decoding for texture and environment images, written
// for this library (no codec library is linked).
//
// Sequential (baseline and extended) Huffman-coded JPEG, ITU-T T.81: 8-bit
// samples, one (grey) or three (YCbCr, or RGB under an Adobe marker)
// components, any sampling factors, interleaved and single-component scans,
// restart intervals. Progressive, lossless, hierarchical and arithmetic-coded
// files and four-component (CMYK) images are refused with a reason. The
// image comes back as cv::imread(IMREAD_COLOR) returns it: 8-bit BGR, grey
// replicated, as floats 0..255, row 0 at the top. Chroma of 2x1 and 2x2
// subsampled images is upsampled by the triangle filter (each output sample
// 3/4 of the nearer and 1/4 of the farther input sample), other factors by
// replication; the inverse DCT is evaluated exactly (double precision) and
// rounded, so samples can differ from libjpeg's integer arithmetic by about
// one unit.
#pragma once
#include <string>
#include <vector>

namespace gbrt_img {

// True when the bytes start with a JPEG start-of-image marker.
bool is_jpeg(const std::string& data);

bool decode_jpeg(const std::string& data, std::vector<float>& bgr, int& W, int& H, std::string& why);

}  // namespace gbrt_img
