// image_png.cpp — inflate (RFC 1950/1951) and PNG decoding (ISO/IEC 15948)
// for texture and environment images; replaces the PNG path of cv::imread in
// TextureMaterial::load (src/texturematerial.cpp:48-60) and
// EnvironmentMap::load (src/environmentmap.cpp:20-33).
//
// Inflate: an LSB-first bit reader and, per Huffman alphabet, a table indexed
// by the next 15 input bits (bit-reversed canonical codes, RFC 1951 3.2.2),
// so each symbol costs one lookup. PNG: chunks with CRC-32, IDAT
// concatenated and inflated once, per-row filters (None, Sub, Up, Average,
// Paeth), Adam7 passes scattered into the image, then IMREAD_COLOR's
// conversion to 8-bit BGR.
#include "image_png.h"

#include <cstring>

namespace gbrt_img {
namespace {

// ------------------------------------------------------------- bit input ---
struct Bits {
  const uint8_t* p;
  size_t n, pos = 0;  // pos: next byte to load into acc
  uint64_t acc = 0;
  int cnt = 0;        // valid bits in acc
  size_t over = 0;    // zero bytes supplied past the end
  void fill() {
    while (cnt <= 56) {
      uint64_t b = 0;
      if (pos < n) b = p[pos];
      else ++over;
      ++pos;
      acc |= b << cnt;
      cnt += 8;
    }
  }
  uint32_t peek(int k) {
    if (cnt < k) fill();
    return uint32_t(acc & ((uint64_t(1) << k) - 1));
  }
  void drop(int k) { acc >>= k; cnt -= k; }
  uint32_t get(int k) {
    if (k == 0) return 0;
    uint32_t v = peek(k);
    drop(k);
    return v;
  }
  // Bytes consumed from the input, counting only whole bytes not held back.
  bool overrun() const { return over * 8 > size_t(cnt); }
  void align() { drop(cnt & 7); }
};

// A canonical Huffman code as a 2^15-entry table: entry = symbol << 4 | length,
// 0 where no code of up to 15 bits begins with those bits.
struct Huff {
  std::vector<uint16_t> tab;
  bool build(const uint8_t* len, int n) {
    int count[16] = {0};
    for (int i = 0; i < n; ++i) count[len[i]]++;
    count[0] = 0;
    int left = 1;  // over-subscription check
    for (int l = 1; l < 16; ++l) {
      left <<= 1;
      left -= count[l];
      if (left < 0) return false;
    }
    int next[16];
    int code = 0;
    for (int l = 1; l < 16; ++l) {
      code = (code + count[l - 1]) << 1;
      next[l] = code;
    }
    tab.assign(1u << 15, 0);
    for (int s = 0; s < n; ++s) {
      int l = len[s];
      if (!l) continue;
      uint32_t c = uint32_t(next[l]++), r = 0;
      for (int b = 0; b < l; ++b) r |= ((c >> b) & 1u) << (l - 1 - b);
      for (uint32_t f = r; f < (1u << 15); f += (1u << l)) tab[f] = uint16_t(s << 4 | l);
    }
    return true;
  }
  // Symbol, or -1 for bits that start no code.
  int decode(Bits& b) const {
    uint16_t e = tab[b.peek(15)];
    if (!e) return -1;
    b.drop(e & 15);
    return e >> 4;
  }
};

// Length and distance symbol bases and extra bits (RFC 1951 3.2.5).
const uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
// Order in which code-length code lengths are sent (RFC 1951 3.2.7).
const uint8_t kClOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

bool inflate_codes(Bits& b, const Huff& lit, const Huff& dist, std::vector<uint8_t>& out, size_t base,
                   size_t max_out, std::string& why) {
  for (;;) {
    int s = lit.decode(b);
    if (s < 0) { why = "invalid literal/length code"; return false; }
    if (s < 256) {
      if (out.size() - base >= max_out) { why = "image data larger than the image"; return false; }
      out.push_back(uint8_t(s));
      continue;
    }
    if (s == 256) return true;
    s -= 257;
    if (s >= 29) { why = "invalid length symbol"; return false; }
    size_t len = kLenBase[s] + b.get(kLenExtra[s]);
    int d = dist.decode(b);
    if (d < 0 || d >= 30) { why = "invalid distance code"; return false; }
    size_t dst = kDistBase[d] + b.get(kDistExtra[d]);
    if (dst > out.size() - base) { why = "distance before the start of the stream"; return false; }
    if (out.size() - base + len > max_out) { why = "image data larger than the image"; return false; }
    size_t from = out.size() - dst;
    for (size_t i = 0; i < len; ++i) out.push_back(out[from + i]);  // overlapping copies repeat
    if (b.overrun()) { why = "truncated deflate stream"; return false; }
  }
}

bool inflate_raw(Bits& b, std::vector<uint8_t>& out, size_t max_out, std::string& why) {
  const size_t base = out.size();
  static Huff fixLit, fixDist;
  static bool fixed_ready = [] {
    uint8_t l[288];
    for (int i = 0; i < 144; ++i) l[i] = 8;
    for (int i = 144; i < 256; ++i) l[i] = 9;
    for (int i = 256; i < 280; ++i) l[i] = 7;
    for (int i = 280; i < 288; ++i) l[i] = 8;
    fixLit.build(l, 288);
    uint8_t d[30];
    for (int i = 0; i < 30; ++i) d[i] = 5;
    fixDist.build(d, 30);
    return true;
  }();
  (void)fixed_ready;
  Huff lit, dist;
  for (;;) {
    const uint32_t last = b.get(1), type = b.get(2);
    if (type == 0) {
      b.align();
      uint32_t len = b.get(16), nlen = b.get(16);
      if ((len ^ 0xffffu) != nlen) { why = "stored block length check failed"; return false; }
      if (out.size() - base + len > max_out) { why = "image data larger than the image"; return false; }
      for (uint32_t i = 0; i < len; ++i) out.push_back(uint8_t(b.get(8)));
      if (b.overrun()) { why = "truncated stored block"; return false; }
    } else if (type == 1) {
      if (!inflate_codes(b, fixLit, fixDist, out, base, max_out, why)) return false;
    } else if (type == 2) {
      const int hlit = int(b.get(5)) + 257, hdist = int(b.get(5)) + 1, hclen = int(b.get(4)) + 4;
      if (hlit > 286 || hdist > 30) { why = "too many length or distance codes"; return false; }
      uint8_t cl[19] = {0};
      for (int i = 0; i < hclen; ++i) cl[kClOrder[i]] = uint8_t(b.get(3));
      Huff clh;
      if (!clh.build(cl, 19)) { why = "bad code-length code"; return false; }
      uint8_t lens[286 + 30] = {0};
      int k = 0;
      while (k < hlit + hdist) {
        int s = clh.decode(b);
        if (s < 0) { why = "invalid code-length symbol"; return false; }
        if (s < 16) { lens[k++] = uint8_t(s); continue; }
        int rep;
        uint8_t val = 0;
        if (s == 16) {
          if (k == 0) { why = "length repeat with no previous length"; return false; }
          val = lens[k - 1];
          rep = 3 + int(b.get(2));
        } else if (s == 17) {
          rep = 3 + int(b.get(3));
        } else {
          rep = 11 + int(b.get(7));
        }
        if (k + rep > hlit + hdist) { why = "code lengths overrun"; return false; }
        while (rep--) lens[k++] = val;
      }
      if (lens[256] == 0) { why = "no end-of-block code"; return false; }
      if (!lit.build(lens, hlit) || !dist.build(lens + hlit, hdist)) { why = "over-subscribed code"; return false; }
      if (!inflate_codes(b, lit, dist, out, base, max_out, why)) return false;
    } else {
      why = "reserved deflate block type";
      return false;
    }
    if (b.overrun()) { why = "truncated deflate stream"; return false; }
    if (last) return true;
  }
}

uint32_t crc32_of(const uint8_t* p, size_t n, uint32_t crc = 0) {
  static uint32_t table[256];
  static bool ready = [] {
    for (uint32_t i = 0; i < 256; ++i) {
      uint32_t c = i;
      for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xedb88320u ^ (c >> 1) : c >> 1;
      table[i] = c;
    }
    return true;
  }();
  (void)ready;
  crc = ~crc;
  for (size_t i = 0; i < n; ++i) crc = table[(crc ^ p[i]) & 0xffu] ^ (crc >> 8);
  return ~crc;
}

uint32_t be32(const uint8_t* p) { return uint32_t(p[0]) << 24 | uint32_t(p[1]) << 16 | uint32_t(p[2]) << 8 | p[3]; }

int paeth(int a, int b, int c) {
  int p = a + b - c;
  int pa = p > a ? p - a : a - p, pb = p > b ? p - b : b - p, pc = p > c ? p - c : c - p;
  if (pa <= pb && pa <= pc) return a;
  return pb <= pc ? b : c;
}

// Undoes the filters of h rows of rowBytes bytes (each preceded by its filter
// type byte) in place; bpp = bytes per complete pixel, at least 1.
bool unfilter(uint8_t* d, size_t rowBytes, size_t h, size_t bpp, std::string& why) {
  uint8_t* prev = nullptr;
  for (size_t y = 0; y < h; ++y) {
    uint8_t* row = d + y * (rowBytes + 1);
    const uint8_t f = row[0];
    uint8_t* x = row + 1;
    switch (f) {
      case 0: break;
      case 1:
        for (size_t i = bpp; i < rowBytes; ++i) x[i] = uint8_t(x[i] + x[i - bpp]);
        break;
      case 2:
        if (prev)
          for (size_t i = 0; i < rowBytes; ++i) x[i] = uint8_t(x[i] + prev[i]);
        break;
      case 3:
        for (size_t i = 0; i < rowBytes; ++i) {
          int a = i >= bpp ? x[i - bpp] : 0, b = prev ? prev[i] : 0;
          x[i] = uint8_t(x[i] + ((a + b) >> 1));
        }
        break;
      case 4:
        for (size_t i = 0; i < rowBytes; ++i) {
          int a = i >= bpp ? x[i - bpp] : 0, b = prev ? prev[i] : 0, c = (prev && i >= bpp) ? prev[i - bpp] : 0;
          x[i] = uint8_t(x[i] + paeth(a, b, c));
        }
        break;
      default:
        why = "unknown PNG filter type";
        return false;
    }
    prev = x;
  }
  return true;
}

}  // namespace

bool zlib_inflate(const uint8_t* in, size_t n, std::vector<uint8_t>& out, size_t max_out, std::string& why) {
  if (n < 6) { why = "zlib stream too short"; return false; }
  const uint8_t cmf = in[0], flg = in[1];
  if ((cmf & 15) != 8 || (cmf >> 4) > 7) { why = "not a deflate zlib stream"; return false; }
  if ((uint32_t(cmf) * 256 + flg) % 31 != 0) { why = "zlib header check failed"; return false; }
  if (flg & 0x20) { why = "zlib preset dictionary not allowed"; return false; }
  const size_t start = out.size();
  Bits b{in + 2, n - 2};
  if (!inflate_raw(b, out, max_out, why)) return false;
  b.align();
  // Adler-32 of the uncompressed data follows, big-endian.
  uint32_t want = 0;
  for (int i = 0; i < 4; ++i) want = want << 8 | b.get(8);
  if (b.overrun()) { why = "zlib stream missing its checksum"; return false; }
  uint32_t s1 = 1, s2 = 0;
  for (size_t i = start; i < out.size(); ++i) {
    s1 = (s1 + out[i]) % 65521u;
    s2 = (s2 + s1) % 65521u;
  }
  if ((s2 << 16 | s1) != want) { why = "zlib Adler-32 mismatch"; return false; }
  return true;
}

bool is_png(const std::string& data) {
  static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', 0x0d, 0x0a, 0x1a, 0x0a};
  return data.size() >= 8 && std::memcmp(data.data(), sig, 8) == 0;
}

bool decode_png(const std::string& data, std::vector<float>& bgr, int& W, int& H, std::string& why) {
  if (!is_png(data)) { why = "not a PNG file"; return false; }
  const uint8_t* p = reinterpret_cast<const uint8_t*>(data.data());
  const size_t n = data.size();
  size_t pos = 8;
  uint32_t w = 0, h = 0;
  int depth = 0, ctype = -1, interlace = 0;
  std::vector<uint8_t> idat, plte;
  bool seenHdr = false, seenEnd = false;
  while (pos + 12 <= n) {
    const uint32_t len = be32(p + pos);
    const uint8_t* type = p + pos + 4;
    if (len > n - pos - 12) { why = "truncated PNG chunk"; return false; }
    const uint8_t* body = p + pos + 8;
    if (crc32_of(type, size_t(len) + 4) != be32(body + len)) { why = "PNG chunk CRC mismatch"; return false; }
    const std::string t(reinterpret_cast<const char*>(type), 4);
    if (!seenHdr && t != "IHDR") { why = "PNG does not start with IHDR"; return false; }
    if (t == "IHDR") {
      if (len != 13 || seenHdr) { why = "bad IHDR"; return false; }
      seenHdr = true;
      w = be32(body);
      h = be32(body + 4);
      depth = body[8];
      ctype = body[9];
      interlace = body[12];
      if (body[10] != 0 || body[11] != 0 || interlace > 1) { why = "unsupported PNG compression/filter/interlace"; return false; }
    } else if (t == "PLTE") {
      plte.assign(body, body + len);
    } else if (t == "IDAT") {
      idat.insert(idat.end(), body, body + len);
    } else if (t == "IEND") {
      seenEnd = true;
      break;
    } else if (!(type[0] & 0x20)) {
      why = "unknown critical PNG chunk " + t;
      return false;
    }
    pos += size_t(len) + 12;
  }
  if (!seenHdr || !seenEnd) { why = "PNG without IHDR or IEND"; return false; }
  int chans;
  switch (ctype) {
    case 0: chans = 1; if (depth != 1 && depth != 2 && depth != 4 && depth != 8 && depth != 16) chans = 0; break;
    case 2: chans = 3; if (depth != 8 && depth != 16) chans = 0; break;
    case 3: chans = 1; if (depth != 1 && depth != 2 && depth != 4 && depth != 8) chans = 0; break;
    case 4: chans = 2; if (depth != 8 && depth != 16) chans = 0; break;
    case 6: chans = 4; if (depth != 8 && depth != 16) chans = 0; break;
    default: chans = 0;
  }
  if (!chans) { why = "unsupported PNG colour type / bit depth"; return false; }
  if (w == 0 || h == 0 || w > 65536 || h > 65536 || uint64_t(w) * h > (uint64_t(1) << 28)) {
    why = "unsupported PNG size";
    return false;
  }
  if (ctype == 3 && (plte.empty() || plte.size() % 3 != 0)) { why = "palette image without a valid PLTE"; return false; }
  const size_t bitsPP = size_t(chans) * depth;
  const size_t bpp = bitsPP >= 8 ? bitsPP / 8 : 1;

  // Pass geometry: Adam7 (origin, step) per pass, or the whole image.
  static const int a7[7][4] = {{0, 0, 8, 8}, {4, 0, 8, 8}, {0, 4, 4, 8}, {2, 0, 4, 4},
                               {0, 2, 2, 4}, {1, 0, 2, 2}, {0, 1, 1, 2}};
  const int passes = interlace ? 7 : 1;
  size_t total = 0;
  for (int k = 0; k < passes; ++k) {
    const int x0 = interlace ? a7[k][0] : 0, y0 = interlace ? a7[k][1] : 0;
    const int dx = interlace ? a7[k][2] : 1, dy = interlace ? a7[k][3] : 1;
    const size_t pw = w > uint32_t(x0) ? (w - x0 + dx - 1) / dx : 0, ph = h > uint32_t(y0) ? (h - y0 + dy - 1) / dy : 0;
    if (pw && ph) total += ph * ((pw * bitsPP + 7) / 8 + 1);
  }
  std::vector<uint8_t> raw;
  raw.reserve(total);
  if (!zlib_inflate(idat.data(), idat.size(), raw, total, why)) return false;
  if (raw.size() != total) { why = "PNG image data shorter than the image"; return false; }

  // Each pixel as 8-bit samples (IMREAD_COLOR's reductions), then BGR.
  W = int(w);
  H = int(h);
  bgr.assign(size_t(w) * h * 3, 0.f);
  size_t off = 0;
  for (int k = 0; k < passes; ++k) {
    const int x0 = interlace ? a7[k][0] : 0, y0 = interlace ? a7[k][1] : 0;
    const int dx = interlace ? a7[k][2] : 1, dy = interlace ? a7[k][3] : 1;
    const size_t pw = w > uint32_t(x0) ? (w - x0 + dx - 1) / dx : 0, ph = h > uint32_t(y0) ? (h - y0 + dy - 1) / dy : 0;
    if (!pw || !ph) continue;
    const size_t rowBytes = (pw * bitsPP + 7) / 8;
    if (!unfilter(raw.data() + off, rowBytes, ph, bpp, why)) return false;
    for (size_t py = 0; py < ph; ++py) {
      const uint8_t* row = raw.data() + off + py * (rowBytes + 1) + 1;
      for (size_t px = 0; px < pw; ++px) {
        // sample c of this pixel, reduced to 8 bits
        auto sample = [&](int c) -> int {
          const size_t idx = px * chans + c;
          if (depth == 8) return row[idx];
          if (depth == 16) return row[idx * 2];  // high byte
          const size_t bit = idx * depth;
          const int v = (row[bit >> 3] >> (8 - depth - int(bit & 7))) & ((1 << depth) - 1);
          return v;
        };
        int r, g, b;
        if (ctype == 3) {
          const size_t i = size_t(sample(0));
          if (3 * i + 2 >= plte.size()) { why = "palette index out of range"; return false; }
          r = plte[3 * i]; g = plte[3 * i + 1]; b = plte[3 * i + 2];
        } else if (ctype == 0 || ctype == 4) {
          int v = sample(0);
          if (depth < 8) v = v * (255 / ((1 << depth) - 1));  // 1/2/4-bit grey scaled to 0..255
          r = g = b = v;
        } else {
          r = sample(0); g = sample(1); b = sample(2);
        }
        const size_t X = x0 + px * dx, Y = y0 + py * dy;
        float* o = bgr.data() + (Y * w + X) * 3;
        o[0] = float(b); o[1] = float(g); o[2] = float(r);
      }
    }
    off += ph * (rowBytes + 1);
  }
  return true;
}

}  // namespace gbrt_img
