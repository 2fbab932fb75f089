// image_out.cu — the step after the film: the tonemapper on the GPU and the
// film writers of the renderer's command line, behind the C ABI.
//
//   gbrt_tonemap(_device)  Tonemapper::map (src/tonemapper.cpp:31-56): per
//                          channel clamp(255 * c^(1/gamma)) truncated to 8
//                          bits, BGR film -> RGB bytes.
//   gbrt_write_image       --save-exr / --save-img / --save-mat
//                          (src/main.cpp:223-265): OpenEXR (uncompressed,
//                          32-bit float B,G,R channels), PFM, Radiance HDR
//                          (flat RGBE), MATLAB function (.m), and 8-bit
//                          PNG (stored deflate blocks), PPM or BMP through the
//                          tonemapper.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "gbrt_internal.h"

namespace gbrt {

// 255 * c^(1/gamma) clamped to [0, 255] and truncated, as Tonemapper::clamp
// does with its float argument. The power is evaluated in double like the
// renderer's pow(float, double).
__host__ __device__ inline unsigned char tonemap_channel(float c, double inv_gamma) {
  float x = float(255.0 * pow(double(c), inv_gamma));
  if (!(x > 0.f)) return 0;  // also NaN (the renderer converts it undefined)
  if (x >= 255.f) return 255;
  return static_cast<unsigned char>(int(x));
}

__global__ void k_tonemap(const float* __restrict__ film, unsigned char* __restrict__ rgb, size_t npix,
                          double inv_gamma) {
  size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= npix) return;
  const float* p = film + 3 * i;
  unsigned char* o = rgb + 3 * i;
  o[0] = tonemap_channel(p[2], inv_gamma);
  o[1] = tonemap_channel(p[1], inv_gamma);
  o[2] = tonemap_channel(p[0], inv_gamma);
}

namespace {

void tonemap_host(const float* film, unsigned char* rgb, size_t npix, float gamma) {
  double ig = 1.0 / double(gamma);
  for (size_t i = 0; i < npix; ++i) {
    rgb[3 * i + 0] = tonemap_channel(film[3 * i + 2], ig);
    rgb[3 * i + 1] = tonemap_channel(film[3 * i + 1], ig);
    rgb[3 * i + 2] = tonemap_channel(film[3 * i + 0], ig);
  }
}

std::string lowerExt(const std::string& p) {
  size_t d = p.find_last_of('.');
  std::string e = d == std::string::npos ? "" : p.substr(d + 1);
  for (char& c : e) c = char(::tolower(c));
  return e;
}

template <typename T>
void put(std::vector<unsigned char>& b, T v) {
  unsigned char tmp[sizeof(T)];
  std::memcpy(tmp, &v, sizeof(T));  // little-endian hosts (x86-64, aarch64)
  b.insert(b.end(), tmp, tmp + sizeof(T));
}
void putStr(std::vector<unsigned char>& b, const char* s) { b.insert(b.end(), s, s + std::strlen(s) + 1); }
void putAttr(std::vector<unsigned char>& b, const char* name, const char* type, const std::vector<unsigned char>& v) {
  putStr(b, name);
  putStr(b, type);
  put<int32_t>(b, int32_t(v.size()));
  b.insert(b.end(), v.begin(), v.end());
}

// OpenEXR 2.0 single-part scan-line file, NO_COMPRESSION, FLOAT channels
// B, G, R (alphabetical order), one scan line per block.
std::vector<unsigned char> encodeEXR(const float* film, int W, int H) {
  std::vector<unsigned char> b;
  put<uint32_t>(b, 20000630u);  // magic 0x762f3101
  put<uint32_t>(b, 2u);         // version 2, no flags
  std::vector<unsigned char> ch;
  for (const char* n : {"B", "G", "R"}) {
    putStr(ch, n);
    put<int32_t>(ch, 2);  // FLOAT
    ch.push_back(0);      // pLinear
    ch.push_back(0); ch.push_back(0); ch.push_back(0);
    put<int32_t>(ch, 1);
    put<int32_t>(ch, 1);
  }
  ch.push_back(0);
  putAttr(b, "channels", "chlist", ch);
  putAttr(b, "compression", "compression", {0});
  std::vector<unsigned char> box;
  put<int32_t>(box, 0); put<int32_t>(box, 0); put<int32_t>(box, W - 1); put<int32_t>(box, H - 1);
  putAttr(b, "dataWindow", "box2i", box);
  putAttr(b, "displayWindow", "box2i", box);
  putAttr(b, "lineOrder", "lineOrder", {0});
  std::vector<unsigned char> f1;
  put<float>(f1, 1.f);
  putAttr(b, "pixelAspectRatio", "float", f1);
  std::vector<unsigned char> v2;
  put<float>(v2, 0.f); put<float>(v2, 0.f);
  putAttr(b, "screenWindowCenter", "v2f", v2);
  putAttr(b, "screenWindowWidth", "float", f1);
  b.push_back(0);  // end of header
  const size_t lineBytes = size_t(W) * 3 * 4;
  uint64_t off = b.size() + uint64_t(H) * 8;
  for (int y = 0; y < H; ++y) {
    put<uint64_t>(b, off);
    off += 8 + lineBytes;
  }
  for (int y = 0; y < H; ++y) {
    put<int32_t>(b, y);
    put<int32_t>(b, int32_t(lineBytes));
    for (int c : {0, 1, 2})  // B G R in the film's channel order
      for (int x = 0; x < W; ++x) put<float>(b, film[(size_t(y) * W + x) * 3 + c]);
  }
  return b;
}

uint32_t crc32(const unsigned char* p, size_t n, uint32_t c = 0) {
  static uint32_t table[256];
  static bool init = false;
  if (!init) {
    for (uint32_t i = 0; i < 256; ++i) {
      uint32_t v = i;
      for (int k = 0; k < 8; ++k) v = (v & 1) ? 0xEDB88320u ^ (v >> 1) : v >> 1;
      table[i] = v;
    }
    init = true;
  }
  c = ~c;
  for (size_t i = 0; i < n; ++i) c = table[(c ^ p[i]) & 0xff] ^ (c >> 8);
  return ~c;
}

void putBE(std::vector<unsigned char>& b, uint32_t v) {
  b.push_back((v >> 24) & 0xff); b.push_back((v >> 16) & 0xff); b.push_back((v >> 8) & 0xff); b.push_back(v & 0xff);
}

// PNG, 8-bit RGB, zlib stream of stored (uncompressed) deflate blocks.
std::vector<unsigned char> encodePNG(const unsigned char* rgb, int W, int H) {
  std::vector<unsigned char> raw;
  raw.reserve(size_t(H) * (size_t(W) * 3 + 1));
  for (int y = 0; y < H; ++y) {
    raw.push_back(0);
    raw.insert(raw.end(), rgb + size_t(y) * W * 3, rgb + size_t(y + 1) * W * 3);
  }
  std::vector<unsigned char> z = {0x78, 0x01};
  uint32_t a = 1, bsum = 0;
  for (unsigned char c : raw) { a = (a + c) % 65521u; bsum = (bsum + a) % 65521u; }
  size_t pos = 0;
  do {
    size_t len = std::min<size_t>(65535, raw.size() - pos);
    bool last = pos + len == raw.size();
    z.push_back(last ? 1 : 0);
    z.push_back(len & 0xff); z.push_back((len >> 8) & 0xff);
    z.push_back(~len & 0xff); z.push_back((~len >> 8) & 0xff);
    z.insert(z.end(), raw.begin() + pos, raw.begin() + pos + len);
    pos += len;
  } while (pos < raw.size());
  putBE(z, (bsum << 16) | a);
  std::vector<unsigned char> out = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};
  auto chunk = [&](const char* type, const std::vector<unsigned char>& data) {
    putBE(out, uint32_t(data.size()));
    size_t start = out.size();
    out.insert(out.end(), type, type + 4);
    out.insert(out.end(), data.begin(), data.end());
    putBE(out, crc32(out.data() + start, out.size() - start));
  };
  std::vector<unsigned char> ihdr;
  putBE(ihdr, uint32_t(W)); putBE(ihdr, uint32_t(H));
  ihdr.push_back(8); ihdr.push_back(2); ihdr.push_back(0); ihdr.push_back(0); ihdr.push_back(0);
  chunk("IHDR", ihdr);
  chunk("IDAT", z);
  chunk("IEND", {});
  return out;
}

std::vector<unsigned char> encodeBMP(const unsigned char* rgb, int W, int H) {
  const int row = (W * 3 + 3) & ~3;
  std::vector<unsigned char> b;
  b.push_back('B'); b.push_back('M');
  put<uint32_t>(b, uint32_t(54 + row * H));
  put<uint32_t>(b, 0); put<uint32_t>(b, 54);
  put<uint32_t>(b, 40); put<int32_t>(b, W); put<int32_t>(b, H);
  put<uint16_t>(b, 1); put<uint16_t>(b, 24); put<uint32_t>(b, 0); put<uint32_t>(b, uint32_t(row * H));
  put<int32_t>(b, 2835); put<int32_t>(b, 2835); put<uint32_t>(b, 0); put<uint32_t>(b, 0);
  for (int y = H - 1; y >= 0; --y) {  // bottom-up rows, BGR bytes
    for (int x = 0; x < W; ++x) {
      const unsigned char* p = rgb + (size_t(y) * W + x) * 3;
      b.push_back(p[2]); b.push_back(p[1]); b.push_back(p[0]);
    }
    for (int k = W * 3; k < row; ++k) b.push_back(0);
  }
  return b;
}

bool writeFile(const std::string& path, const std::vector<unsigned char>& data) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) return false;
  bool ok = std::fwrite(data.data(), 1, data.size(), f) == data.size();
  return std::fclose(f) == 0 && ok;
}

// Flat RGBE (no run-length coding): shared exponent of the largest channel.
std::vector<unsigned char> encodeHDR(const float* film, int W, int H) {
  std::string head = "#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y " + std::to_string(H) + " +X " + std::to_string(W) + "\n";
  std::vector<unsigned char> b(head.begin(), head.end());
  for (size_t i = 0; i < size_t(W) * H; ++i) {
    float B = film[3 * i], G = film[3 * i + 1], R = film[3 * i + 2];
    float m = std::max(R, std::max(G, B));
    if (!(m > 1e-32f)) { b.push_back(0); b.push_back(0); b.push_back(0); b.push_back(0); continue; }
    int e;
    float f = std::frexp(m, &e) * 256.f / m;
    b.push_back((unsigned char)std::max(0.f, R * f));
    b.push_back((unsigned char)std::max(0.f, G * f));
    b.push_back((unsigned char)std::max(0.f, B * f));
    b.push_back((unsigned char)(e + 128));
  }
  return b;
}

std::vector<unsigned char> encodePFM(const float* film, int W, int H) {
  std::string head = "PF\n" + std::to_string(W) + " " + std::to_string(H) + "\n-1.0\n";
  std::vector<unsigned char> b(head.begin(), head.end());
  for (int y = H - 1; y >= 0; --y)  // bottom-up, RGB
    for (int x = 0; x < W; ++x)
      for (int c : {2, 1, 0}) put<float>(b, film[(size_t(y) * W + x) * 3 + c]);
  return b;
}

// The MATLAB dump of --save-mat (src/main.cpp:238-265): a function returning
// an H x W x 3 RGB array, written channel by channel.
std::vector<unsigned char> encodeM(const float* film, int W, int H, const std::string& path) {
  size_t s = path.find_last_of('/');
  std::string base = path.substr(s == std::string::npos ? 0 : s + 1);
  size_t d = base.find('.');
  if (d != std::string::npos) base = base.substr(0, d);
  std::string out = "function im = " + base + "()\n  im = zeros(" + std::to_string(H) + "," + std::to_string(W) + ",3);\n";
  char buf[64];
  for (int c = 0; c < 3; ++c) {
    out += "  im(:, :, " + std::to_string(3 - c) + ")=[";
    for (int y = 0; y < H; ++y) {
      for (int x = 0; x < W; ++x) {
        std::snprintf(buf, sizeof buf, "%10f,", double(film[(size_t(y) * W + x) * 3 + c]));
        out += buf;
      }
      out += ";";
    }
    out += "];\n";
  }
  out += "end\n";
  return std::vector<unsigned char>(out.begin(), out.end());
}

}  // namespace
}  // namespace gbrt

using namespace gbrt;

extern "C" {

gbrt_status gbrt_tonemap(const float* film_bgr, int32_t width, int32_t height, float gamma, uint8_t* rgb) {
  if (!film_bgr || !rgb || width <= 0 || height <= 0 || !(gamma > 0.f))
    return fail(nullptr, GBRT_ERR_INVALID_ARG, "gbrt_tonemap: bad argument");
  tonemap_host(film_bgr, rgb, size_t(width) * height, gamma);
  return GBRT_OK;
}

gbrt_status gbrt_tonemap_device(gbrt_ctx* ctx, const float* d_film_bgr, int32_t width, int32_t height, float gamma,
                                uint8_t* d_rgb, void* stream) {
  if (!ctx || !d_film_bgr || !d_rgb || width <= 0 || height <= 0 || !(gamma > 0.f))
    return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_tonemap_device: bad argument");
  GBRT_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  size_t npix = size_t(width) * height;
  k_tonemap<<<unsigned((npix + 255) / 256), 256, 0, st>>>(d_film_bgr, d_rgb, npix, 1.0 / double(gamma));
  GBRT_CUDA_TRY(ctx, cudaGetLastError());
  return GBRT_OK;
}

gbrt_status gbrt_write_image(const char* path, const float* film_bgr, int32_t width, int32_t height, float gamma) {
  if (!path || !film_bgr || width <= 0 || height <= 0)
    return fail(nullptr, GBRT_ERR_INVALID_ARG, "gbrt_write_image: bad argument");
  std::string p(path), e = lowerExt(p);
  std::vector<unsigned char> data;
  if (e == "exr") data = encodeEXR(film_bgr, width, height);
  else if (e == "pfm") data = encodePFM(film_bgr, width, height);
  else if (e == "hdr") data = encodeHDR(film_bgr, width, height);
  else if (e == "m") data = encodeM(film_bgr, width, height, p);
  else if (e == "png" || e == "ppm" || e == "bmp") {
    if (!(gamma > 0.f)) return fail(nullptr, GBRT_ERR_INVALID_ARG, "gbrt_write_image: gamma must be positive");
    std::vector<unsigned char> rgb(size_t(width) * height * 3);
    tonemap_host(film_bgr, rgb.data(), size_t(width) * height, gamma);
    if (e == "png") data = encodePNG(rgb.data(), width, height);
    else if (e == "bmp") data = encodeBMP(rgb.data(), width, height);
    else {
      std::string h = "P6\n" + std::to_string(width) + " " + std::to_string(height) + "\n255\n";
      data.assign(h.begin(), h.end());
      data.insert(data.end(), rgb.begin(), rgb.end());
    }
  } else {
    return fail(nullptr, GBRT_ERR_UNSUPPORTED, "gbrt_write_image: unknown file type '" + e + "'");
  }
  if (!writeFile(p, data)) return fail(nullptr, GBRT_ERR_IO, "gbrt_write_image: cannot write " + p);
  return GBRT_OK;
}

}  // extern "C"
