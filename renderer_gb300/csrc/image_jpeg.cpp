// image_jpeg.cpp — sequential Huffman JPEG decoding (ITU-T T.81) for texture
// and environment images; replaces the JPEG path of cv::imread in
// TextureMaterial::load (src/texturematerial.cpp:48-60) and
// EnvironmentMap::load (src/environmentmap.cpp:20-33).
//
// Markers are read in order; DQT / DHT / DRI / SOF set up the tables and the
// frame; each SOS scan is entropy-decoded into per-component coefficient
// planes (dequantised, natural order); after the last scan every block goes
// through the inverse DCT, chroma is upsampled to the frame and converted
// to RGB (JFIF, or none under an Adobe RGB marker), then stored as BGR.
// Huffman codes are looked up in a 2^16-entry table indexed by the next 16
// bits of the scan, which gives each symbol in one step.
#include "image_jpeg.h"

#include <cmath>
#include <cstdint>
#include <cstring>

namespace gbrt_img {
namespace {

struct HuffTable {
  std::vector<uint16_t> lut;  // next 16 bits -> length << 8 | value; 0: no code
  bool ready = false;
  bool build(const uint8_t counts[16], const uint8_t* vals, int nvals) {
    lut.assign(1u << 16, 0);
    uint32_t code = 0;
    int k = 0;
    for (int len = 1; len <= 16; ++len) {
      for (int i = 0; i < counts[len - 1]; ++i) {
        if (k >= nvals) return false;
        if (code >= (1u << len)) return false;  // over-subscribed
        const uint32_t lo = code << (16 - len), hi = (code + 1) << (16 - len);
        for (uint32_t f = lo; f < hi; ++f) lut[f] = uint16_t(len << 8 | vals[k]);
        ++code;
        ++k;
      }
      code <<= 1;
    }
    ready = true;
    return true;
  }
};

struct Component {
  int id = 0, h = 1, v = 1, tq = 0;
  int bw = 0, bh = 0;            // blocks per row / column in the coefficient plane (padded to MCUs)
  std::vector<int32_t> coef;     // bw x bh blocks of 64 dequantised coefficients, natural order
  int pred = 0;                  // DC predictor
  int td = 0, ta = 0;            // tables of the current scan
};

// Entropy-coded segment reader: MSB first, 0xFF00 -> 0xFF, a marker ends the
// data (zeros are supplied after it).
struct ScanBits {
  const uint8_t* p;
  size_t n, pos;
  uint32_t acc = 0;
  int cnt = 0;
  bool marker = false;  // a marker was reached
  size_t zeros = 0;     // zero bytes supplied after it
  ScanBits(const uint8_t* d, size_t size, size_t start) : p(d), n(size), pos(start) {}
  void fill() {
    while (cnt <= 24) {
      uint32_t b = 0;
      if (!marker && pos < n) {
        b = p[pos];
        if (b == 0xFF) {
          const uint8_t nx = pos + 1 < n ? p[pos + 1] : 0xD9;
          if (nx == 0x00) {
            pos += 2;
          } else {
            marker = true;  // leave pos at the marker
            b = 0;
            ++zeros;
          }
        } else {
          ++pos;
        }
      } else {
        ++zeros;
      }
      acc |= b << (24 - cnt);
      cnt += 8;
    }
  }
  uint32_t peek16() {
    if (cnt < 16) fill();
    return acc >> 16;
  }
  void drop(int k) {
    acc <<= k;
    cnt -= k;
  }
  int get(int k) {  // k <= 16
    if (k == 0) return 0;
    if (cnt < k) fill();
    const int v = int(acc >> (32 - k));
    drop(k);
    return v;
  }
  bool overrun() const { return zeros > 4; }
  // Skips to the marker after the bits, consumes an RSTn there.
  bool restart() {
    acc = 0;
    cnt = 0;
    marker = false;
    zeros = 0;
    while (pos + 1 < n && !(p[pos] == 0xFF && p[pos + 1] >= 0xD0 && p[pos + 1] <= 0xD7)) ++pos;
    if (pos + 1 >= n) return false;
    pos += 2;
    return true;
  }
};

// receive_extend of T.81 F.2.2.1: s bits as a signed value.
inline int extend(int v, int s) { return v < (1 << (s - 1)) ? v - (1 << s) + 1 : v; }

int decode_symbol(ScanBits& b, const HuffTable& t) {
  const uint16_t e = t.lut[b.peek16()];
  if (!e) return -1;
  b.drop(e >> 8);
  return e & 0xFF;
}

// Natural index of each zigzag position: anti-diagonals, alternating direction.
struct Zigzag {
  int nat[64];
  Zigzag() {
    int k = 0;
    for (int s = 0; s < 15; ++s) {
      if (s & 1) {
        for (int r = s < 8 ? 0 : s - 7; r <= (s < 8 ? s : 7); ++r) nat[k++] = r * 8 + (s - r);
      } else {
        for (int r = s < 8 ? s : 7; r >= (s < 8 ? 0 : s - 7); --r) nat[k++] = r * 8 + (s - r);
      }
    }
  }
};
const Zigzag kZigzag;

// Inverse DCT of one block (T.81 A.3.3), exact in double: samples 0..255.
struct Idct {
  double c[8][8];  // c[x][u] = C(u) cos((2x + 1) u pi / 16) / 2
  Idct() {
    for (int x = 0; x < 8; ++x)
      for (int u = 0; u < 8; ++u)
        c[x][u] = (u == 0 ? std::sqrt(0.5) : 1.0) * std::cos((2 * x + 1) * u * M_PI / 16.0) / 2.0;
  }
  void run(const int32_t* f, uint8_t* out, int stride) const {
    double tmp[64];
    for (int v = 0; v < 8; ++v)  // rows of coefficients: along u
      for (int x = 0; x < 8; ++x) {
        double s = 0;
        for (int u = 0; u < 8; ++u) s += c[x][u] * f[v * 8 + u];
        tmp[v * 8 + x] = s;
      }
    for (int x = 0; x < 8; ++x)
      for (int y = 0; y < 8; ++y) {
        double s = 0;
        for (int v = 0; v < 8; ++v) s += c[y][v] * tmp[v * 8 + x];
        const double q = std::floor(s + 128.0 + 0.5);
        out[y * stride + x] = uint8_t(q < 0 ? 0 : (q > 255 ? 255 : q));
      }
  }
};

uint16_t be16(const uint8_t* p) { return uint16_t(p[0] << 8 | p[1]); }

}  // namespace

bool is_jpeg(const std::string& data) {
  return data.size() >= 3 && uint8_t(data[0]) == 0xFF && uint8_t(data[1]) == 0xD8 && uint8_t(data[2]) == 0xFF;
}

bool decode_jpeg(const std::string& data, std::vector<float>& bgr, int& W, int& H, std::string& why) {
  if (!is_jpeg(data)) { why = "not a JPEG file"; return false; }
  const uint8_t* p = reinterpret_cast<const uint8_t*>(data.data());
  const size_t n = data.size();
  uint16_t qt[4][64];
  bool qready[4] = {false, false, false, false};
  HuffTable dc[4], ac[4];
  std::vector<Component> comp;
  int X = 0, Y = 0, hmax = 1, vmax = 1, restart = 0, adobe = -1;
  bool frame = false, anyScan = false, eoi = false;
  size_t pos = 2;
  while (pos < n && !eoi) {
    if (p[pos] != 0xFF) { why = "JPEG marker expected"; return false; }
    while (pos < n && p[pos] == 0xFF) ++pos;  // fill bytes
    if (pos >= n) break;
    const uint8_t m = p[pos++];
    if (m == 0xD9) { eoi = true; break; }
    if (m == 0x01 || (m >= 0xD0 && m <= 0xD7)) continue;  // no length
    if (pos + 2 > n) { why = "truncated JPEG segment"; return false; }
    const size_t len = be16(p + pos);
    if (len < 2 || pos + len > n) { why = "truncated JPEG segment"; return false; }
    const uint8_t* seg = p + pos + 2;
    const size_t sl = len - 2;
    pos += len;
    if (m == 0xC0 || m == 0xC1) {
      if (frame) { why = "JPEG with two frames"; return false; }
      if (sl < 6 || seg[0] != 8) { why = "JPEG sample precision other than 8 bits"; return false; }
      Y = be16(seg + 1);
      X = be16(seg + 3);
      const int nf = seg[5];
      if (sl < size_t(6 + 3 * nf) || (nf != 1 && nf != 3)) {
        why = nf == 4 ? "four-component (CMYK) JPEG not supported" : "bad JPEG frame header";
        return false;
      }
      if (X <= 0 || Y <= 0 || X > 65535 || Y > 65535 || int64_t(X) * Y > (int64_t(1) << 28)) {
        why = "unsupported JPEG size (zero height needs a DNL marker)";
        return false;
      }
      comp.resize(size_t(nf));
      for (int i = 0; i < nf; ++i) {
        Component& c = comp[size_t(i)];
        c.id = seg[6 + 3 * i];
        c.h = seg[7 + 3 * i] >> 4;
        c.v = seg[7 + 3 * i] & 15;
        c.tq = seg[8 + 3 * i];
        if (c.h < 1 || c.h > 4 || c.v < 1 || c.v > 4 || c.tq > 3) { why = "bad JPEG sampling factors"; return false; }
        hmax = c.h > hmax ? c.h : hmax;
        vmax = c.v > vmax ? c.v : vmax;
      }
      const int mcux = (X + 8 * hmax - 1) / (8 * hmax), mcuy = (Y + 8 * vmax - 1) / (8 * vmax);
      for (Component& c : comp) {
        c.bw = mcux * c.h;
        c.bh = mcuy * c.v;
        c.coef.assign(size_t(c.bw) * c.bh * 64, 0);
      }
      frame = true;
    } else if (m >= 0xC2 && m <= 0xCF && m != 0xC4 && m != 0xC8 && m != 0xCC) {
      why = "progressive, lossless, hierarchical or arithmetic-coded JPEG not supported";
      return false;
    } else if (m == 0xDB) {
      size_t k = 0;
      while (k < sl) {
        const int pq = seg[k] >> 4, tq = seg[k] & 15;
        if (tq > 3 || pq > 1 || k + 1 + 64 * (pq + 1) > sl) { why = "bad JPEG quantisation table"; return false; }
        for (int i = 0; i < 64; ++i) qt[tq][i] = pq ? be16(seg + k + 1 + 2 * i) : seg[k + 1 + i];
        qready[tq] = true;
        k += 1 + 64 * (pq + 1);
      }
    } else if (m == 0xC4) {
      size_t k = 0;
      while (k < sl) {
        if (k + 17 > sl) { why = "bad JPEG Huffman table"; return false; }
        const int tc = seg[k] >> 4, th = seg[k] & 15;
        uint8_t counts[16];
        int total = 0;
        for (int i = 0; i < 16; ++i) total += counts[i] = seg[k + 1 + i];
        if (tc > 1 || th > 3 || total > 256 || k + 17 + size_t(total) > sl) { why = "bad JPEG Huffman table"; return false; }
        if (!(tc ? ac[th] : dc[th]).build(counts, seg + k + 17, total)) { why = "bad JPEG Huffman code"; return false; }
        k += 17 + size_t(total);
      }
    } else if (m == 0xDD) {
      if (sl < 2) { why = "bad JPEG restart interval"; return false; }
      restart = be16(seg);
    } else if (m == 0xEE) {
      if (sl >= 12 && std::memcmp(seg, "Adobe", 5) == 0) adobe = seg[11];
    } else if (m == 0xDA) {
      if (!frame || sl < 1) { why = "JPEG scan before its frame"; return false; }
      const int ns = seg[0];
      if (ns < 1 || ns > 4 || sl < size_t(4 + 2 * ns)) { why = "bad JPEG scan header"; return false; }
      std::vector<Component*> sc;
      for (int i = 0; i < ns; ++i) {
        Component* c = nullptr;
        for (Component& x : comp)
          if (x.id == seg[1 + 2 * i]) c = &x;
        if (!c) { why = "JPEG scan of an unknown component"; return false; }
        c->td = seg[2 + 2 * i] >> 4;
        c->ta = seg[2 + 2 * i] & 15;
        if (c->td > 3 || c->ta > 3 || !dc[c->td].ready || !ac[c->ta].ready || !qready[c->tq]) {
          why = "JPEG scan without its tables";
          return false;
        }
        c->pred = 0;
        sc.push_back(c);
      }
      const size_t t0 = 1 + 2 * size_t(ns);
      if (seg[t0] != 0 || seg[t0 + 1] != 63 || seg[t0 + 2] != 0) { why = "JPEG scan is not sequential"; return false; }
      // MCUs of the scan: interleaved (every component's h x v blocks), or
      // one block of a single component over its own extent.
      int mx, my;
      if (ns == 1) {
        const Component& c = *sc[0];
        const int cw = (X * c.h + hmax - 1) / hmax, ch = (Y * c.v + vmax - 1) / vmax;
        mx = (cw + 7) / 8;
        my = (ch + 7) / 8;
      } else {
        mx = (X + 8 * hmax - 1) / (8 * hmax);
        my = (Y + 8 * vmax - 1) / (8 * vmax);
      }
      ScanBits bits(p, n, pos);
      const int nmcu = mx * my;
      for (int mcu = 0; mcu < nmcu; ++mcu) {
        if (restart && mcu > 0 && mcu % restart == 0) {
          if (!bits.restart()) { why = "JPEG restart marker missing"; return false; }
          for (Component* c : sc) c->pred = 0;
        }
        const int ux = mcu % mx, uy = mcu / mx;
        for (Component* c : sc) {
          const int bh = ns == 1 ? 1 : c->h, bv = ns == 1 ? 1 : c->v;
          for (int by = 0; by < bv; ++by)
            for (int bx = 0; bx < bh; ++bx) {
              const int col = ux * bh + bx, row = uy * bv + by;
              int32_t* f = c->coef.data() + (size_t(row) * c->bw + col) * 64;
              const uint16_t* q = qt[c->tq];
              const int t = decode_symbol(bits, dc[c->td]);
              if (t < 0 || t > 11) { why = "bad JPEG DC code"; return false; }
              c->pred += t ? extend(bits.get(t), t) : 0;
              f[0] = c->pred * int32_t(q[0]);
              for (int k = 1; k < 64;) {
                const int rs = decode_symbol(bits, ac[c->ta]);
                if (rs < 0) { why = "bad JPEG AC code"; return false; }
                const int r = rs >> 4, s = rs & 15;
                if (s == 0) {
                  if (r != 15) break;  // end of block
                  k += 16;
                  continue;
                }
                k += r;
                if (k > 63) { why = "JPEG coefficient run past the block"; return false; }
                f[kZigzag.nat[k]] = extend(bits.get(s), s) * int32_t(q[k]);
                ++k;
              }
              if (bits.overrun()) { why = "truncated JPEG scan"; return false; }
            }
        }
      }
      // continue at the marker after the scan's data
      pos = bits.pos;
      while (pos + 1 < n && !(p[pos] == 0xFF && p[pos + 1] != 0x00 && !(p[pos + 1] >= 0xD0 && p[pos + 1] <= 0xD7)))
        ++pos;
      anyScan = true;
    }
    // APPn, COM and other segments: skipped
  }
  if (!frame || !anyScan) { why = "JPEG without a frame or a scan"; return false; }

  // Inverse DCT of every block into each component's sample plane.
  static const Idct idct;
  std::vector<std::vector<uint8_t>> plane(comp.size());
  for (size_t ci = 0; ci < comp.size(); ++ci) {
    const Component& c = comp[ci];
    const int pw = c.bw * 8;
    plane[ci].assign(size_t(pw) * c.bh * 8, 0);
    for (int by = 0; by < c.bh; ++by)
      for (int bx = 0; bx < c.bw; ++bx)
        idct.run(c.coef.data() + (size_t(by) * c.bw + bx) * 64, plane[ci].data() + size_t(by) * 8 * pw + bx * 8, pw);
  }
  // A component's sample at frame pixel (x, y).
  auto sample = [&](size_t ci, int x, int y) -> double {
    const Component& c = comp[ci];
    const int pw = c.bw * 8;
    const std::vector<uint8_t>& pl = plane[ci];
    const int fx = hmax / c.h, fy = vmax / c.v;
    const int cw = (X * c.h + hmax - 1) / hmax, ch = (Y * c.v + vmax - 1) / vmax;
    auto at = [&](int i, int j) {
      i = i < 0 ? 0 : (i >= cw ? cw - 1 : i);
      j = j < 0 ? 0 : (j >= ch ? ch - 1 : j);
      return double(pl[size_t(j) * pw + i]);
    };
    if (fx == 1 && fy == 1 && c.h == hmax && c.v == vmax) return at(x, y);
    if (fx <= 2 && fy <= 2 && fx * c.h == hmax && fy * c.v == vmax) {
      // triangle filter: 3/4 of the nearer input sample, 1/4 of the farther
      auto hpass = [&](int j) -> double {
        if (fx == 1) return at(x, j);
        const int i0 = x >> 1, side = (x & 1) ? 1 : -1;
        return 0.75 * at(i0, j) + 0.25 * at(i0 + side, j);
      };
      if (fy == 1) return hpass(y);
      const int j0 = y >> 1, side = (y & 1) ? 1 : -1;
      return 0.75 * hpass(j0) + 0.25 * hpass(j0 + side);
    }
    return at(int(int64_t(x) * c.h / hmax), int(int64_t(y) * c.v / vmax));  // replication
  };
  W = X;
  H = Y;
  bgr.assign(size_t(X) * Y * 3, 0.f);
  auto clamp8 = [](double v) { v = std::floor(v + 0.5); return float(v < 0 ? 0 : (v > 255 ? 255 : v)); };
  for (int y = 0; y < Y; ++y)
    for (int x = 0; x < X; ++x) {
      float* o = bgr.data() + (size_t(y) * X + x) * 3;
      if (comp.size() == 1) {
        const float g = clamp8(sample(0, x, y));
        o[0] = o[1] = o[2] = g;
      } else if (adobe == 0) {  // Adobe: components are R, G, B
        o[2] = clamp8(sample(0, x, y));
        o[1] = clamp8(sample(1, x, y));
        o[0] = clamp8(sample(2, x, y));
      } else {  // JFIF YCbCr
        const double Yv = sample(0, x, y), cb = sample(1, x, y) - 128.0, cr = sample(2, x, y) - 128.0;
        o[2] = clamp8(Yv + 1.402 * cr);
        o[1] = clamp8(Yv - 0.344136 * cb - 0.714136 * cr);
        o[0] = clamp8(Yv + 1.772 * cb);
      }
    }
  return true;
}

}  // namespace gbrt_img
