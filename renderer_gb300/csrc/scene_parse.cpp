// scene_parse.cpp — the renderer's scene language, its OBJ/MTL reader and its
// environment-image loading, as pure host code behind the C ABI
// (gbrt_parse_scene_file / _string, gbrt_parsed_scene_desc, gbrt_read_hdr).
//
// Follows, in three passes like the renderer:
//   parse       SceneGrammar (src/sceneparser.cpp:36-156; skipper
//               src/sceneparser.h:44-50): a recursive-descent parser over
//               `name = value;` statements, with // and /* */ comments.
//   resolve     resolveVars (src/sceneast.cpp:730-747): OBJ files are loaded
//               (src/objreader.cpp:142-366) and their MTL materials become
//               variables defined before every statement; relative OBJ paths
//               are taken from the scene file's directory (src/sceneast.cpp:811-815).
//   build       buildScene / scene_builder (src/sceneast.cpp:321-728): the
//               variables camera, lights and intersectable form the scene.
// Differences, for the GPU layout: an instance of a subtree of at least 1,024
// triangles (obj / t / lists of them) under an affine transform becomes an
// instance of a shared mesh (two-level BVH; the mesh keeps no texture
// coordinates); other instances are flattened by transforming their
// primitives (a sphere needs a similarity transform); a pre-built
// b(left, right, box) node contributes its children (the BVH is rebuilt);
// box(min, max, m) and isect / union / diff / xor trees of spheres and boxes
// become CSG objects (a box under an instance must stay axis-aligned).
// Texture images are read from PNG (image_png.cpp), JPEG (image_jpeg.cpp),
// PPM (P6/P3), PFM and Radiance files, all decoded here, and scaled by 1/255
// like the renderer's cv::imread + convertTo; an unreadable image gives
// DarkMatter.
// Each primitive's position in the scene's root list (lights, then the
// intersectables in file order) is kept as gbrt_scene_desc.list_rank, for the
// list's tie rule under GBRT_SCENE_LIST_ORDER.
// An environment map that fails to load becomes a BlackLight, as in the renderer
// (src/sceneast.cpp:598-610). As an extension, environmentmap("f", c,
// "latlong") selects an equirectangular image.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/gbrt.h"
#include "image_jpeg.h"
#include "image_png.h"

namespace {

struct ParseError : std::runtime_error {
  gbrt_status st;
  ParseError(gbrt_status s, const std::string& m) : std::runtime_error(m), st(s) {}
};

// --------------------------------------------------------------- lexer ----
enum TokKind { TK_END, TK_IDENT, TK_NUM, TK_STR, TK_PUNCT };
struct Tok {
  TokKind kind;
  std::string text;
  double num = 0;
  int line = 0;
};

std::vector<Tok> lex(const std::string& s) {
  std::vector<Tok> out;
  size_t i = 0, n = s.size();
  int line = 1;
  while (i < n) {
    char c = s[i];
    if (c == '\n') { ++line; ++i; continue; }
    if (std::isspace((unsigned char)c)) { ++i; continue; }
    if (c == '/' && i + 1 < n && s[i + 1] == '/') {
      while (i < n && s[i] != '\n') ++i;
      continue;
    }
    if (c == '/' && i + 1 < n && s[i + 1] == '*') {
      size_t e = s.find("*/", i + 2);
      if (e == std::string::npos) throw ParseError(GBRT_ERR_PARSE, "unterminated comment at line " + std::to_string(line));
      for (size_t k = i; k < e; ++k) if (s[k] == '\n') ++line;
      i = e + 2;
      continue;
    }
    Tok t;
    t.line = line;
    if (std::isalpha((unsigned char)c) || c == '_') {
      size_t j = i;
      while (j < n && (std::isalnum((unsigned char)s[j]) || s[j] == '_')) ++j;
      t.kind = TK_IDENT;
      t.text = s.substr(i, j - i);
      if (t.text == "inf" || t.text == "infinity" || t.text == "nan") {
        t.kind = TK_NUM;
        t.num = t.text == "nan" ? NAN : INFINITY;
      }
      i = j;
    } else if (std::isdigit((unsigned char)c) || c == '.' ||
               ((c == '-' || c == '+') && i + 1 < n &&
                (std::isdigit((unsigned char)s[i + 1]) || s[i + 1] == '.' || std::isalpha((unsigned char)s[i + 1])))) {
      size_t j = i;
      if (s[j] == '-' || s[j] == '+') ++j;
      if (std::isalpha((unsigned char)s[j])) {  // +inf / -inf / nan
        size_t k = j;
        while (k < n && std::isalpha((unsigned char)s[k])) ++k;
        std::string w = s.substr(j, k - j);
        if (w != "inf" && w != "infinity" && w != "nan") throw ParseError(GBRT_ERR_PARSE, "bad number at line " + std::to_string(line));
        t.kind = TK_NUM;
        t.num = (w == "nan") ? NAN : (s[i] == '-' ? -INFINITY : INFINITY);
        i = k;
      } else {
        while (j < n && std::isdigit((unsigned char)s[j])) ++j;
        if (j < n && s[j] == '.') { ++j; while (j < n && std::isdigit((unsigned char)s[j])) ++j; }
        if (j < n && (s[j] == 'e' || s[j] == 'E')) {
          size_t k = j + 1;
          if (k < n && (s[k] == '+' || s[k] == '-')) ++k;
          if (k < n && std::isdigit((unsigned char)s[k])) {
            while (k < n && std::isdigit((unsigned char)s[k])) ++k;
            j = k;
          }
        }
        t.kind = TK_NUM;
        t.text = s.substr(i, j - i);
        t.num = std::strtod(t.text.c_str(), nullptr);
        i = j;
      }
    } else if (c == '"') {
      size_t e = s.find('"', i + 1);
      if (e == std::string::npos) throw ParseError(GBRT_ERR_PARSE, "unterminated string at line " + std::to_string(line));
      t.kind = TK_STR;
      t.text = s.substr(i + 1, e - i - 1);
      i = e + 1;
    } else if (std::strchr("=;{}()[],*", c)) {
      t.kind = TK_PUNCT;
      t.text = std::string(1, c);
      ++i;
    } else {
      throw ParseError(GBRT_ERR_PARSE, std::string("unexpected character '") + c + "' at line " + std::to_string(line));
    }
    out.push_back(t);
  }
  Tok e;
  e.kind = TK_END;
  e.line = line;
  out.push_back(e);
  return out;
}

// ----------------------------------------------------------------- AST ----
struct V3 { float x = 0, y = 0, z = 0; };
struct V4 { float x = 0, y = 0, z = 0, w = 0; };

struct Mat4 {  // row-major m[r][c]
  float m[4][4];
  Mat4() { for (int r = 0; r < 4; ++r) for (int c = 0; c < 4; ++c) m[r][c] = r == c ? 1.f : 0.f; }
  Mat4 operator*(const Mat4& o) const {
    Mat4 R;
    for (int r = 0; r < 4; ++r)
      for (int c = 0; c < 4; ++c) {
        float s = 0;
        for (int k = 0; k < 4; ++k) s += m[r][k] * o.m[k][c];
        R.m[r][c] = s;
      }
    return R;
  }
  V3 point(V3 p) const {
    float v[4] = {p.x, p.y, p.z, 1.f}, o[4];
    for (int r = 0; r < 4; ++r) o[r] = m[r][0] * v[0] + m[r][1] * v[1] + m[r][2] * v[2] + m[r][3] * v[3];
    if (o[3] != 1.f && o[3] != 0.f) return {o[0] / o[3], o[1] / o[3], o[2] / o[3]};
    return {o[0], o[1], o[2]};
  }
  V3 dir(V3 d) const {
    return {m[0][0] * d.x + m[0][1] * d.y + m[0][2] * d.z, m[1][0] * d.x + m[1][1] * d.y + m[1][2] * d.z,
            m[2][0] * d.x + m[2][1] * d.y + m[2][2] * d.z};
  }
};

struct MatNode {
  int kind = -1;   // gbrt_material_type, or -1 for an identifier, -2 for a texture
  V3 kd, ks;
  float exponent = 0, ior = 1, coef = 1;
  std::string ident;
};

struct Node;
using NodeP = std::shared_ptr<Node>;
struct Node {
  enum Kind { LIST, QUAD, PLANE, OBJ, TRI, INSTANCE, BVH, SPHERE, BOX, CSG } kind;
  std::vector<NodeP> children;
  V3 p[4];
  V3 n[3];
  float uv[6] = {0, 0, 0, 0, 0, 0};
  V4 plane;
  float radius = 0;
  std::string file, op;
  MatNode mat;
  Mat4 xf;
};

struct LightNode {
  int kind;  // 0 point, 1 area, 2 cone, 3 env
  V3 a, b, c, I;
  float angle = 0;
  std::string file, mapping;
};

struct CameraNode {
  V3 eye, at, up;
  float fov = 0, xres = 0, yres = 0;
};

struct Value {
  enum Kind { INTERSECTABLE, LIGHTS, CAMERA, MATERIAL, IDENT } kind;
  NodeP node;
  std::vector<LightNode> lights;
  CameraNode cam;
  MatNode mat;
  std::string ident;
};

struct Assignment {
  std::string name;
  Value value;
};

// -------------------------------------------------------------- parser ----
struct Parser {
  std::vector<Tok> t;
  size_t i = 0;
  explicit Parser(std::vector<Tok> toks) : t(std::move(toks)) {}

  [[noreturn]] void err(const std::string& what) {
    const Tok& k = t[i];
    std::string got = k.kind == TK_END ? "end of input" : ("'" + (k.kind == TK_NUM && k.text.empty() ? std::string("number") : k.text) + "'");
    throw ParseError(GBRT_ERR_PARSE, "line " + std::to_string(k.line) + ": expected " + what + ", got " + got);
  }
  bool isP(const char* p) const { return t[i].kind == TK_PUNCT && t[i].text == p; }
  void expect(const char* p) { if (!isP(p)) err(std::string("'") + p + "'"); ++i; }
  bool peekCall(const char* kw) const {
    return t[i].kind == TK_IDENT && t[i].text == kw && t[i + 1].kind == TK_PUNCT &&
           (t[i + 1].text == "(" || t[i + 1].text == "{");
  }
  float num() {
    if (t[i].kind != TK_NUM) err("a number");
    return float(t[i++].num);
  }
  std::string str() {
    if (t[i].kind != TK_STR) err("a string");
    return t[i++].text;
  }
  std::string ident() {
    if (t[i].kind != TK_IDENT) err("an identifier");
    return t[i++].text;
  }
  V3 v3() { expect("["); V3 v; v.x = num(); v.y = num(); v.z = num(); expect("]"); return v; }
  V4 v4() { expect("["); V4 v; v.x = num(); v.y = num(); v.z = num(); v.w = num(); expect("]"); return v; }
  void v2(float* o) { expect("["); o[0] = num(); o[1] = num(); expect("]"); }

  std::vector<Assignment> file() {
    std::vector<Assignment> out;
    while (t[i].kind != TK_END) {
      Assignment a;
      a.name = ident();
      expect("=");
      a.value = value();
      expect(";");
      out.push_back(std::move(a));
    }
    return out;
  }

  static bool isMaterialKw(const std::string& s) {
    return s == "diffuse" || s == "phong" || s == "blinn" || s == "mirror" || s == "texture" || s == "refractive";
  }
  static bool isIntersectableKw(const std::string& s) {
    return s == "intersectables" || s == "quad" || s == "plane" || s == "obj" || s == "t" || s == "instance" ||
           s == "b" || s == "sphere" || s == "box" || s == "isect" || s == "union" || s == "diff" || s == "xor";
  }

  Value value() {
    Value v;
    if (t[i].kind == TK_IDENT && t[i + 1].kind == TK_PUNCT && (t[i + 1].text == "(" || t[i + 1].text == "{")) {
      const std::string& w = t[i].text;
      if (isIntersectableKw(w)) { v.kind = Value::INTERSECTABLE; v.node = intersectable(); return v; }
      if (w == "lights") { v.kind = Value::LIGHTS; v.lights = lightList(); return v; }
      if (w == "camera") { v.kind = Value::CAMERA; v.cam = camera(); return v; }
      if (isMaterialKw(w)) { v.kind = Value::MATERIAL; v.mat = material(); return v; }
      err("an intersectable, lights, camera or material");
    }
    v.kind = Value::IDENT;
    v.ident = ident();
    return v;
  }

  MatNode material() {
    MatNode m;
    if (t[i].kind == TK_IDENT && !(t[i + 1].kind == TK_PUNCT && t[i + 1].text == "(" && isMaterialKw(t[i].text))) {
      m.kind = -1;
      m.ident = ident();
      return m;
    }
    std::string w = ident();
    expect("(");
    if (w == "diffuse") { m.kind = GBRT_MAT_DIFFUSE; m.kd = v3(); }
    else if (w == "phong") { m.kind = GBRT_MAT_PHONG; m.kd = v3(); expect(","); m.ks = v3(); expect(","); m.exponent = num(); }
    else if (w == "blinn") { m.kind = GBRT_MAT_BLINN; m.kd = v3(); expect(","); m.ks = v3(); expect(","); m.exponent = num(); }
    else if (w == "mirror") { m.kind = GBRT_MAT_MIRROR; m.coef = num(); }
    else if (w == "texture") { m.kind = -2; m.ident = str(); expect(","); m.kd = v3(); expect(","); m.exponent = num(); }
    else if (w == "refractive") { m.kind = GBRT_MAT_TRANSPARENT; m.ior = num(); }
    else err("a material");
    expect(")");
    return m;
  }

  Mat4 basicMatrix() {
    Mat4 M;
    if (isP("[")) {
      expect("[");
      for (int r = 0; r < 4; ++r) { V4 row = v4(); M.m[r][0] = row.x; M.m[r][1] = row.y; M.m[r][2] = row.z; M.m[r][3] = row.w; }
      expect("]");
      return M;
    }
    std::string w = ident();
    expect("(");
    if (w == "translate") {
      V3 v = v3();
      M.m[0][3] = v.x; M.m[1][3] = v.y; M.m[2][3] = v.z;
    } else if (w == "rotate") {
      // QMatrix4x4::rotate(angle in degrees, axis).
      float ang = num(); expect(",");
      V3 a = v3();
      double len = std::sqrt(double(a.x) * a.x + double(a.y) * a.y + double(a.z) * a.z);
      if (len > 0) {
        double x = a.x / len, y = a.y / len, z = a.z / len;
        double rad = double(ang) * M_PI / 180.0, c = std::cos(rad), s = std::sin(rad), ic = 1 - c;
        double R[3][3] = {{x * x * ic + c, x * y * ic - z * s, x * z * ic + y * s},
                          {y * x * ic + z * s, y * y * ic + c, y * z * ic - x * s},
                          {z * x * ic - y * s, z * y * ic + x * s, z * z * ic + c}};
        for (int r = 0; r < 3; ++r) for (int c2 = 0; c2 < 3; ++c2) M.m[r][c2] = float(R[r][c2]);
      }
    } else if (w == "scale") {
      if (isP("[")) { V3 v = v3(); M.m[0][0] = v.x; M.m[1][1] = v.y; M.m[2][2] = v.z; }
      else { float f = num(); M.m[0][0] = M.m[1][1] = M.m[2][2] = f; }
    } else {
      err("a matrix");
    }
    expect(")");
    return M;
  }
  Mat4 matrix() {
    Mat4 M = basicMatrix();
    while (isP("*")) { ++i; M = M * basicMatrix(); }
    return M;
  }

  NodeP intersectable() {
    auto nd = std::make_shared<Node>();
    if (t[i].kind != TK_IDENT) err("an intersectable");
    std::string w = t[i].text;
    if (w == "intersectables") {
      ++i;
      expect("{");
      nd->kind = Node::LIST;
      while (!isP("}")) nd->children.push_back(intersectable());
      expect("}");
      return nd;
    }
    ++i;
    expect("(");
    if (w == "quad") {
      nd->kind = Node::QUAD;
      for (int k = 0; k < 4; ++k) { nd->p[k] = v3(); expect(","); }
      nd->mat = material();
    } else if (w == "plane") {
      nd->kind = Node::PLANE; nd->plane = v4(); expect(","); nd->mat = material();
    } else if (w == "obj") {
      nd->kind = Node::OBJ; nd->file = str(); expect(","); nd->mat = material();
    } else if (w == "t") {
      nd->kind = Node::TRI;
      for (int k = 0; k < 3; ++k) { nd->p[k] = v3(); expect(","); }
      for (int k = 0; k < 3; ++k) { nd->n[k] = v3(); expect(","); }
      for (int k = 0; k < 3; ++k) { v2(nd->uv + 2 * k); expect(","); }
      nd->mat = material();
    } else if (w == "instance") {
      nd->kind = Node::INSTANCE; nd->xf = matrix(); expect(","); nd->children.push_back(intersectable());
    } else if (w == "b") {
      nd->kind = Node::BVH;
      nd->children.push_back(intersectable()); expect(",");
      nd->children.push_back(intersectable()); expect(",");
      NodeP box = intersectable();  // box(min, max, material): the node's bounds, unused
      if (box->kind != Node::BOX) err("a box");
    } else if (w == "sphere") {
      nd->kind = Node::SPHERE; nd->p[0] = v3(); expect(","); nd->radius = num(); expect(","); nd->mat = material();
    } else if (w == "box") {
      nd->kind = Node::BOX; nd->p[0] = v3(); expect(","); nd->p[1] = v3(); expect(","); nd->mat = material();
    } else if (w == "isect" || w == "union" || w == "diff" || w == "xor") {
      nd->kind = Node::CSG; nd->op = w;
      nd->children.push_back(intersectable()); expect(",");
      nd->children.push_back(intersectable());
    } else {
      --i;
      err("an intersectable");
    }
    expect(")");
    return nd;
  }

  std::vector<LightNode> lightList() {
    ident();  // lights
    expect("{");
    std::vector<LightNode> out;
    while (!isP("}")) {
      LightNode L;
      std::string w = ident();
      expect("(");
      if (w == "pointlight") { L.kind = 0; L.a = v3(); expect(","); L.I = v3(); }
      else if (w == "arealight") { L.kind = 1; L.a = v3(); expect(","); L.b = v3(); expect(","); L.c = v3(); expect(","); L.I = v3(); }
      else if (w == "conelight") { L.kind = 2; L.a = v3(); expect(","); L.b = v3(); expect(","); L.angle = num(); expect(","); L.I = v3(); }
      else if (w == "environmentmap") {
        L.kind = 3; L.file = str(); expect(","); L.I = v3();
        if (isP(",")) { ++i; L.mapping = str(); }
      } else { --i; err("a light"); }
      expect(")");
      out.push_back(L);
    }
    expect("}");
    return out;
  }

  CameraNode camera() {
    ident();
    expect("(");
    CameraNode c;
    c.eye = v3(); expect(","); c.at = v3(); expect(","); c.up = v3(); expect(",");
    c.fov = num(); expect(","); c.xres = num(); expect(","); c.yres = num();
    expect(")");
    return c;
  }
};

// ----------------------------------------------------------- file helpers --
std::string dirOf(const std::string& path) {
  size_t s = path.find_last_of('/');
  return s == std::string::npos ? std::string() : path.substr(0, s);
}
std::string joinPath(const std::string& dir, const std::string& f) {
  if (f.empty() || f[0] == '/' || dir.empty()) return f;
  return dir + "/" + f;
}
bool readFile(const std::string& p, std::string& out) {
  std::ifstream in(p, std::ios::binary);
  if (!in) return false;
  std::ostringstream ss;
  ss << in.rdbuf();
  out = ss.str();
  return true;
}

// Radiance RGBE (.hdr): new-style run-length rows and flat rows.
bool readHDR(const std::string& path, std::vector<float>& bgr, int& W, int& H, std::string& why) {
  std::string data;
  if (!readFile(path, data)) { why = "cannot open " + path; return false; }
  size_t pos = 0;
  auto line = [&]() {
    size_t e = data.find('\n', pos);
    if (e == std::string::npos) e = data.size();
    std::string l = data.substr(pos, e - pos);
    pos = std::min(data.size(), e + 1);
    return l;
  };
  std::string first = line();
  if (first.rfind("#?", 0) != 0) { why = "not a Radiance file"; return false; }
  bool rgbe = false;
  for (;;) {
    if (pos >= data.size()) { why = "truncated header"; return false; }
    std::string l = line();
    if (l.empty()) break;
    if (l == "FORMAT=32-bit_rle_rgbe") rgbe = true;
    if (l.rfind("FORMAT=", 0) == 0 && !rgbe) { why = "unsupported format " + l; return false; }
  }
  std::string res = line();
  char ya[4] = {0}, xa[4] = {0};
  if (std::sscanf(res.c_str(), "%2s %d %2s %d", ya, &H, xa, &W) != 4 || std::string(ya) != "-Y" ||
      std::string(xa) != "+X" || W <= 0 || H <= 0) {
    why = "unsupported orientation '" + res + "'";
    return false;
  }
  bgr.assign(size_t(W) * H * 3, 0.f);
  std::vector<unsigned char> scan(size_t(W) * 4);
  const unsigned char* d = reinterpret_cast<const unsigned char*>(data.data());
  size_t n = data.size();
  for (int y = 0; y < H; ++y) {
    if (pos + 4 <= n && W >= 8 && W < 32768 && d[pos] == 2 && d[pos + 1] == 2 && ((d[pos + 2] << 8) | d[pos + 3]) == W) {
      pos += 4;
      for (int c = 0; c < 4; ++c) {
        int x = 0;
        while (x < W) {
          if (pos >= n) { why = "truncated data"; return false; }
          int cnt = d[pos++];
          if (cnt > 128) {
            cnt -= 128;
            if (pos >= n || x + cnt > W) { why = "bad run"; return false; }
            unsigned char v = d[pos++];
            for (int k = 0; k < cnt; ++k) scan[size_t(x++) * 4 + c] = v;
          } else {
            if (cnt == 0 || x + cnt > W || pos + cnt > n) { why = "bad literal run"; return false; }
            for (int k = 0; k < cnt; ++k) scan[size_t(x++) * 4 + c] = d[pos++];
          }
        }
      }
    } else {
      if (pos + size_t(W) * 4 > n) { why = "truncated flat data"; return false; }
      std::memcpy(scan.data(), d + pos, size_t(W) * 4);
      pos += size_t(W) * 4;
    }
    for (int x = 0; x < W; ++x) {
      const unsigned char* p = &scan[size_t(x) * 4];
      // mantissa * 2^(exponent - 136), zero exponent = black (the decoding
      // OpenCV's Radiance reader applies).
      float f = p[3] ? std::ldexp(1.0f, int(p[3]) - (128 + 8)) : 0.f;
      float* o = &bgr[(size_t(y) * W + x) * 3];
      o[0] = p[2] * f;  // B
      o[1] = p[1] * f;  // G
      o[2] = p[0] * f;  // R
    }
  }
  return true;
}

// Portable float map (.pfm, colour "PF"), rows stored bottom-up.
bool readPFM(const std::string& path, std::vector<float>& bgr, int& W, int& H, std::string& why) {
  std::string data;
  if (!readFile(path, data)) { why = "cannot open " + path; return false; }
  std::istringstream in(data);
  std::string magic;
  double scale;
  in >> magic >> W >> H >> scale;
  if (magic != "PF" || W <= 0 || H <= 0) { why = "not a colour PFM"; return false; }
  in.get();
  size_t off = size_t(in.tellg());
  if (off + size_t(W) * H * 12 > data.size()) { why = "truncated PFM"; return false; }
  bool little = scale < 0;
  bgr.assign(size_t(W) * H * 3, 0.f);
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x)
      for (int c = 0; c < 3; ++c) {
        uint32_t u;
        std::memcpy(&u, data.data() + off + ((size_t(H - 1 - y) * W + x) * 3 + c) * 4, 4);
        if (!little) u = __builtin_bswap32(u);
        float f;
        std::memcpy(&f, &u, 4);
        bgr[(size_t(y) * W + x) * 3 + (2 - c)] = f;
      }
  return true;
}

// Netpbm colour images (P6 binary, P3 ASCII) with at most 8 bits per sample:
// samples 0..maxval, returned as they are (the caller scales them).
bool readPPM(const std::string& path, std::vector<float>& bgr, int& W, int& H, std::string& why) {
  std::string data;
  if (!readFile(path, data)) { why = "cannot read " + path; return false; }
  size_t pos = 0;
  auto token = [&]() -> std::string {
    while (pos < data.size()) {
      if (data[pos] == '#') { while (pos < data.size() && data[pos] != '\n') ++pos; }
      else if (std::isspace((unsigned char)data[pos])) ++pos;
      else break;
    }
    size_t b = pos;
    while (pos < data.size() && !std::isspace((unsigned char)data[pos]) && data[pos] != '#') ++pos;
    return data.substr(b, pos - b);
  };
  std::string magic = token();
  if (magic != "P6" && magic != "P3") { why = path + ": not a P6/P3 image"; return false; }
  long w = std::atol(token().c_str()), h = std::atol(token().c_str()), mx = std::atol(token().c_str());
  if (w <= 0 || h <= 0 || mx <= 0 || mx > 255 || w > 65536 || h > 65536) {
    why = path + ": unsupported size or sample depth";
    return false;
  }
  W = int(w);
  H = int(h);
  bgr.assign(size_t(W) * H * 3, 0.f);
  if (magic == "P6") {
    ++pos;  // the single whitespace after maxval
    if (data.size() < pos + size_t(W) * H * 3) { why = path + ": truncated"; return false; }
    for (size_t i = 0; i < size_t(W) * H; ++i)
      for (int c = 0; c < 3; ++c) bgr[i * 3 + (2 - c)] = float((unsigned char)data[pos + i * 3 + c]);
  } else {
    for (size_t i = 0; i < size_t(W) * H; ++i)
      for (int c = 0; c < 3; ++c) {
        std::string t = token();
        if (t.empty()) { why = path + ": truncated"; return false; }
        bgr[i * 3 + (2 - c)] = float(std::atol(t.c_str()));
      }
  }
  return true;
}

bool readImage(const std::string& path, std::vector<float>& bgr, int& W, int& H, std::string& why) {
  {
    // PNG and JPEG are recognised by their signatures, as cv::imread
    // recognises formats.
    std::ifstream in(path, std::ios::binary);
    char sig[8] = {0};
    if (in && in.read(sig, 8)) {
      const std::string head(sig, 8);
      const bool png = gbrt_img::is_png(head), jpeg = gbrt_img::is_jpeg(head);
      if (png || jpeg) {
        std::string data;
        if (!readFile(path, data)) { why = "cannot read " + path; return false; }
        const bool ok = png ? gbrt_img::decode_png(data, bgr, W, H, why) : gbrt_img::decode_jpeg(data, bgr, W, H, why);
        if (!ok) { why = path + ": " + why; return false; }
        return true;
      }
    }
  }
  std::string lower = path;
  std::transform(lower.begin(), lower.end(), lower.begin(), ::tolower);
  if (lower.size() >= 4 && lower.substr(lower.size() - 4) == ".pfm") return readPFM(path, bgr, W, H, why);
  if (lower.size() >= 4 && (lower.substr(lower.size() - 4) == ".ppm" || lower.substr(lower.size() - 4) == ".pnm"))
    return readPPM(path, bgr, W, H, why);
  return readHDR(path, bgr, W, H, why);
}

// ------------------------------------------------------------ OBJ / MTL ----
struct ObjTri {
  V3 p[3], n[3];
  float uv[6];
  bool hasN;
  std::string mtl;  // empty: the obj statement's material
};

void sanitizeName(std::string& s) {
  for (char& c : s) if (!(std::isalnum((unsigned char)c) || c == '_')) c = '_';
  if (!s.empty() && std::isdigit((unsigned char)s[0])) s[0] = '_';
}

// ObjReader::getMaterials + createMaterial, src/objreader.cpp:271-366.
void readMTL(const std::string& path, std::map<std::string, MatNode>& out) {
  std::ifstream in(path);
  if (!in) return;
  struct M { V3 kd, ks; float ns = 0, ni = 0; int illum = 0; std::string tex; } cur;
  std::string name;
  auto flush = [&]() {
    MatNode m;
    if (cur.illum <= 2) {
      if (!cur.tex.empty()) {
        // relative to the MTL file, with Windows separators turned around
        std::string tex = cur.tex;
        std::replace(tex.begin(), tex.end(), '\\', '/');
        m.kind = -2;
        m.ident = joinPath(dirOf(path), tex);
        m.kd = (cur.kd.x != 0 || cur.kd.y != 0 || cur.kd.z != 0) ? cur.kd : V3{1, 1, 1};
        m.exponent = 1;
      } else if ((cur.ks.x == 0 && cur.ks.y == 0 && cur.ks.z == 0) || cur.ns == 0) {
        m.kind = GBRT_MAT_DIFFUSE; m.kd = cur.kd;
      } else {
        m.kind = GBRT_MAT_BLINN; m.kd = cur.kd; m.ks = cur.ks; m.exponent = cur.ns;
      }
    } else if (cur.illum == 11) {
      m.kind = GBRT_MAT_MIRROR;
    } else {
      m.kind = GBRT_MAT_TRANSPARENT; m.ior = cur.ni;
    }
    out[name] = m;
  };
  std::string line;
  while (std::getline(in, line)) {
    std::istringstream ss(line);
    std::string tok;
    ss >> tok;
    if (tok == "newmtl") {
      if (!name.empty()) { flush(); cur = M(); }
      ss >> name;
      sanitizeName(name);
    } else if (tok == "illum") ss >> cur.illum;
    else if (tok == "Kd") ss >> cur.kd.x >> cur.kd.y >> cur.kd.z;
    else if (tok == "map_Kd") ss >> cur.tex;
    else if (tok == "Ks") ss >> cur.ks.x >> cur.ks.y >> cur.ks.z;
    else if (tok == "Ns") ss >> cur.ns;
    else if (tok == "Ni") ss >> cur.ni;
  }
  flush();
}

// ObjReader::load, src/objreader.cpp:142-269: v/vt/vn/f with fan
// triangulation and negative (relative) indices, usemtl, mtllib.
bool readOBJ(const std::string& path, std::vector<ObjTri>& tris, std::map<std::string, MatNode>& mats) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  std::vector<V3> P, N;
  std::vector<std::pair<float, float>> T;
  std::string cur;
  std::string dir = dirOf(path);
  char buf[4096];
  std::string line;
  auto readIdx = [](const char*& s, int& pi, int& ti, int& ni, int np, int nt, int nn) -> bool {
    while (*s == ' ' || *s == '\t') ++s;
    char* e;
    long v = std::strtol(s, &e, 10);
    if (e == s) return false;
    s = e;
    pi = int(v < 0 ? v + np + 1 : v);
    ti = ni = 0;
    if (*s == '/') {
      ++s;
      if (*s != '/') {
        v = std::strtol(s, &e, 10);
        if (e == s) return false;
        s = e;
        ti = int(v < 0 ? v + nt + 1 : v);
      }
      if (*s == '/') {
        ++s;
        v = std::strtol(s, &e, 10);
        if (e == s) return false;
        s = e;
        ni = int(v < 0 ? v + nn + 1 : v);
      }
    }
    return true;
  };
  while (std::fgets(buf, sizeof buf, f)) {
    line.assign(buf);
    while (line.size() == sizeof(buf) - 1 && line.back() != '\n' && std::fgets(buf, sizeof buf, f)) line += buf;
    const char* s = line.c_str();
    while (*s == ' ' || *s == '\t') ++s;
    if (s[0] == 'v' && (s[1] == ' ' || s[1] == '\t')) {
      V3 p; float w = 0;
      int k = std::sscanf(s + 1, "%f %f %f %f", &p.x, &p.y, &p.z, &w);
      if (k == 4 && w != 0) { p.x /= w; p.y /= w; p.z /= w; }
      P.push_back(p);
    } else if (s[0] == 'v' && s[1] == 'n') {
      V3 n;
      std::sscanf(s + 2, "%f %f %f", &n.x, &n.y, &n.z);
      N.push_back(n);
    } else if (s[0] == 'v' && s[1] == 't') {
      float u = 0, v = 0;
      std::sscanf(s + 2, "%f %f", &u, &v);
      T.push_back({u, v});
    } else if (s[0] == 'f' && (s[1] == ' ' || s[1] == '\t')) {
      const char* q = s + 1;
      int idx[3][3];
      int np = int(P.size()), nt = int(T.size()), nn = int(N.size());
      if (!readIdx(q, idx[0][0], idx[0][1], idx[0][2], np, nt, nn)) continue;
      if (!readIdx(q, idx[2][0], idx[2][1], idx[2][2], np, nt, nn)) continue;
      for (;;) {
        idx[1][0] = idx[2][0]; idx[1][1] = idx[2][1]; idx[1][2] = idx[2][2];
        if (!readIdx(q, idx[2][0], idx[2][1], idx[2][2], np, nt, nn)) break;
        ObjTri tr{};
        bool okP = idx[0][0] > 0 && idx[1][0] > 0 && idx[2][0] > 0 && idx[0][0] <= np && idx[1][0] <= np && idx[2][0] <= np;
        if (!okP) continue;
        for (int k = 0; k < 3; ++k) tr.p[k] = P[idx[k][0] - 1];
        tr.hasN = idx[0][2] > 0 && idx[1][2] > 0 && idx[2][2] > 0 && idx[0][2] <= nn && idx[1][2] <= nn && idx[2][2] <= nn;
        if (tr.hasN) for (int k = 0; k < 3; ++k) tr.n[k] = N[idx[k][2] - 1];
        bool hasT = idx[0][1] > 0 && idx[1][1] > 0 && idx[2][1] > 0 && idx[0][1] <= nt && idx[1][1] <= nt && idx[2][1] <= nt;
        for (int k = 0; k < 3; ++k) {
          tr.uv[2 * k] = hasT ? T[idx[k][1] - 1].first : 0.f;
          tr.uv[2 * k + 1] = hasT ? T[idx[k][1] - 1].second : 0.f;
        }
        tr.mtl = cur;
        tris.push_back(tr);
      }
    } else if (std::strncmp(s, "usemtl", 6) == 0) {
      char name[1024] = {0};
      std::sscanf(s + 6, "%1023s", name);
      cur = name;
      sanitizeName(cur);
    } else if (std::strncmp(s, "mtllib", 6) == 0) {
      char name[1024] = {0};
      std::sscanf(s + 6, "%1023s", name);
      readMTL(joinPath(dir, name), mats);
    }
  }
  std::fclose(f);
  return true;
}

}  // namespace

// -------------------------------------------------------- parsed scene ----
struct gbrt_parsed_scene {
  std::vector<gbrt_material> materials;
  std::vector<float> tri_pos, tri_nrm, tri_uv;
  std::vector<std::vector<float>> texels;  // per texture
  std::vector<gbrt_texture> textures;
  std::map<std::string, int> texture_ids;  // path -> texture
  std::vector<gbrt_csg_node> csg_nodes;
  std::vector<int32_t> csg_roots;
  std::vector<int32_t> tri_mat;
  std::vector<gbrt_quad> quads;
  std::vector<gbrt_sphere> spheres;
  std::vector<gbrt_plane> planes;
  std::vector<gbrt_light> lights;
  std::vector<float> env_texels;
  gbrt_env_map env{};
  bool has_env = false;
  gbrt_camera camera{};
  bool has_camera = false;
  bool any_smooth = false;
  // instanced meshes (triangles in the mesh's own space) and their instances
  struct MeshData {
    std::vector<float> pos, nrm;
    std::vector<int32_t> mat;
    bool smooth = false;
  };
  std::vector<MeshData> meshes;
  std::vector<gbrt_mesh> mesh_descs;
  std::vector<gbrt_instance> instances;
  // The scene's intersectables in the order the scene file lists them
  // (kind, index within its kind), and the list ranks built from it.
  enum Kind { kTri, kQuad, kSphere, kPlane, kCsg, kInstance };
  std::vector<std::pair<int, int64_t>> listed;
  std::vector<int32_t> list_rank;
};

namespace {

struct Builder {
  gbrt_parsed_scene& ps;
  std::string baseDir;
  std::map<std::string, int> matVars;                       // material variables
  std::map<std::string, MatNode> objMats;                   // from MTL files
  std::map<std::string, NodeP> isectVars;
  std::map<std::string, std::vector<LightNode>> lightVars;
  std::map<std::string, CameraNode> camVars;
  std::map<std::string, std::pair<std::vector<ObjTri>, std::map<std::string, MatNode>>> objCache;
  int inMesh = 0;  // > 0 while a mesh instance's triangles are being emitted

  Builder(gbrt_parsed_scene& p, std::string dir) : ps(p), baseDir(std::move(dir)) {}

  // The texture of an image file, loaded once (TextureMaterial::load,
  // src/texturematerial.cpp:48-60: cv::imread converted with scale 1/255);
  // -1 when it cannot be read.
  int loadTexture(const std::string& file) {
    std::string path = joinPath(baseDir, file);
    auto it = ps.texture_ids.find(path);
    if (it != ps.texture_ids.end()) return it->second;
    std::vector<float> bgr;
    int W = 0, H = 0;
    std::string why;
    int id = -1;
    if (readImage(path, bgr, W, H, why)) {
      for (float& x : bgr) x *= 1.f / 255.f;
      ps.texels.push_back(std::move(bgr));
      ps.textures.push_back(gbrt_texture{W, H, nullptr});
      id = int(ps.textures.size()) - 1;
    }
    ps.texture_ids[path] = id;
    return id;
  }

  int addMat(const MatNode& m) {
    gbrt_material g{};
    g.texture = -1;
    if (m.kind == -2) {
      // TextureMaterial(coefficient, gamma); an image that cannot be read
      // gives DarkMatter (src/sceneast.cpp:345-365).
      int tex = loadTexture(m.ident);
      if (tex >= 0) {
        g.type = GBRT_MAT_TEXTURE;
        g.texture = tex;
        g.kd[0] = m.kd.z; g.kd[1] = m.kd.y; g.kd[2] = m.kd.x;
        g.exponent = m.exponent;
      } else {
        g.type = GBRT_MAT_DARK;
      }
    } else {
      g.type = m.kind;
      // asSpectrum: RGB -> BGR (src/sceneast.cpp:410-414)
      g.kd[0] = m.kd.z; g.kd[1] = m.kd.y; g.kd[2] = m.kd.x;
      g.ks[0] = m.ks.z; g.ks[1] = m.ks.y; g.ks[2] = m.ks.x;
      g.exponent = m.exponent;
      g.ior = m.ior;
      g.coefficient = m.coef;
    }
    ps.materials.push_back(g);
    return int(ps.materials.size()) - 1;
  }

  // material_builder (src/sceneast.cpp:321-404): a missing variable is DarkMatter.
  int resolveMat(const MatNode& m) {
    if (m.kind == -1) {
      auto it = matVars.find(m.ident);
      if (it != matVars.end()) return it->second;
      auto jt = objMats.find(m.ident);
      if (jt != objMats.end()) {
        int id = addMat(jt->second);
        matVars[m.ident] = id;
        return id;
      }
      return -1;
    }
    return addMat(m);
  }

  void addTri(V3 a, V3 b, V3 c, const V3* n, const float* uv, int mat, const Mat4* xf) {
    static const float kDefaultUV[6] = {0, 0, 0, 1, 1, 0};
    const float* t = uv ? uv : kDefaultUV;
    ps.tri_uv.insert(ps.tri_uv.end(), t, t + 6);
    V3 p[3] = {a, b, c};
    for (int k = 0; k < 3; ++k) {
      V3 q = xf ? xf->point(p[k]) : p[k];
      ps.tri_pos.push_back(q.x); ps.tri_pos.push_back(q.y); ps.tri_pos.push_back(q.z);
    }
    for (int k = 0; k < 3; ++k) {
      V3 m = n ? n[k] : V3{};
      if (n && xf) {
        Mat4 inv = inverse(*xf);
        m = {inv.m[0][0] * n[k].x + inv.m[1][0] * n[k].y + inv.m[2][0] * n[k].z,
             inv.m[0][1] * n[k].x + inv.m[1][1] * n[k].y + inv.m[2][1] * n[k].z,
             inv.m[0][2] * n[k].x + inv.m[1][2] * n[k].y + inv.m[2][2] * n[k].z};
      }
      ps.tri_nrm.push_back(m.x); ps.tri_nrm.push_back(m.y); ps.tri_nrm.push_back(m.z);
    }
    if (n) ps.any_smooth = true;
    if (!inMesh) ps.listed.emplace_back(gbrt_parsed_scene::kTri, int64_t(ps.tri_mat.size()));
    ps.tri_mat.push_back(mat);
  }

  static Mat4 inverse(const Mat4& a) {
    double m[16], inv[16];
    for (int r = 0; r < 4; ++r) for (int c = 0; c < 4; ++c) m[r * 4 + c] = a.m[r][c];
    inv[0] = m[5] * m[10] * m[15] - m[5] * m[11] * m[14] - m[9] * m[6] * m[15] + m[9] * m[7] * m[14] + m[13] * m[6] * m[11] - m[13] * m[7] * m[10];
    inv[4] = -m[4] * m[10] * m[15] + m[4] * m[11] * m[14] + m[8] * m[6] * m[15] - m[8] * m[7] * m[14] - m[12] * m[6] * m[11] + m[12] * m[7] * m[10];
    inv[8] = m[4] * m[9] * m[15] - m[4] * m[11] * m[13] - m[8] * m[5] * m[15] + m[8] * m[7] * m[13] + m[12] * m[5] * m[11] - m[12] * m[7] * m[9];
    inv[12] = -m[4] * m[9] * m[14] + m[4] * m[10] * m[13] + m[8] * m[5] * m[14] - m[8] * m[6] * m[13] - m[12] * m[5] * m[10] + m[12] * m[6] * m[9];
    inv[1] = -m[1] * m[10] * m[15] + m[1] * m[11] * m[14] + m[9] * m[2] * m[15] - m[9] * m[3] * m[14] - m[13] * m[2] * m[11] + m[13] * m[3] * m[10];
    inv[5] = m[0] * m[10] * m[15] - m[0] * m[11] * m[14] - m[8] * m[2] * m[15] + m[8] * m[3] * m[14] + m[12] * m[2] * m[11] - m[12] * m[3] * m[10];
    inv[9] = -m[0] * m[9] * m[15] + m[0] * m[11] * m[13] + m[8] * m[1] * m[15] - m[8] * m[3] * m[13] - m[12] * m[1] * m[11] + m[12] * m[3] * m[9];
    inv[13] = m[0] * m[9] * m[14] - m[0] * m[10] * m[13] - m[8] * m[1] * m[14] + m[8] * m[2] * m[13] + m[12] * m[1] * m[10] - m[12] * m[2] * m[9];
    inv[2] = m[1] * m[6] * m[15] - m[1] * m[7] * m[14] - m[5] * m[2] * m[15] + m[5] * m[3] * m[14] + m[13] * m[2] * m[7] - m[13] * m[3] * m[6];
    inv[6] = -m[0] * m[6] * m[15] + m[0] * m[7] * m[14] + m[4] * m[2] * m[15] - m[4] * m[3] * m[14] - m[12] * m[2] * m[7] + m[12] * m[3] * m[6];
    inv[10] = m[0] * m[5] * m[15] - m[0] * m[7] * m[13] - m[4] * m[1] * m[15] + m[4] * m[3] * m[13] + m[12] * m[1] * m[7] - m[12] * m[3] * m[5];
    inv[14] = -m[0] * m[5] * m[14] + m[0] * m[6] * m[13] + m[4] * m[1] * m[14] - m[4] * m[2] * m[13] - m[12] * m[1] * m[6] + m[12] * m[2] * m[5];
    inv[3] = -m[1] * m[6] * m[11] + m[1] * m[7] * m[10] + m[5] * m[2] * m[11] - m[5] * m[3] * m[10] - m[9] * m[2] * m[7] + m[9] * m[3] * m[6];
    inv[7] = m[0] * m[6] * m[11] - m[0] * m[7] * m[10] - m[4] * m[2] * m[11] + m[4] * m[3] * m[10] + m[8] * m[2] * m[7] - m[8] * m[3] * m[6];
    inv[11] = -m[0] * m[5] * m[11] + m[0] * m[7] * m[9] + m[4] * m[1] * m[11] - m[4] * m[3] * m[9] - m[8] * m[1] * m[7] + m[8] * m[3] * m[5];
    inv[15] = m[0] * m[5] * m[10] - m[0] * m[6] * m[9] - m[4] * m[1] * m[10] + m[4] * m[2] * m[9] + m[8] * m[1] * m[6] - m[8] * m[2] * m[5];
    double det = m[0] * inv[0] + m[1] * inv[4] + m[2] * inv[8] + m[3] * inv[12];
    Mat4 out;
    if (det == 0) throw ParseError(GBRT_ERR_UNSUPPORTED, "singular instance transform");
    for (int i = 0; i < 16; ++i) out.m[i / 4][i % 4] = float(inv[i] / det);
    return out;
  }

  void addQuad(const V3* p, int mat, const Mat4* xf) {
    gbrt_quad q{};
    for (int k = 0; k < 4; ++k) {
      V3 v = xf ? xf->point(p[k]) : p[k];
      q.p[k][0] = v.x; q.p[k][1] = v.y; q.p[k][2] = v.z;
    }
    q.material = mat;
    ps.listed.emplace_back(gbrt_parsed_scene::kQuad, int64_t(ps.quads.size()));
    ps.quads.push_back(q);
  }

  void emit(const NodeP& n, const Mat4* xf) {
    switch (n->kind) {
      case Node::LIST:
      case Node::BVH:
        for (auto& c : n->children) emit(c, xf);
        break;
      case Node::QUAD:
        addQuad(n->p, resolveMat(n->mat), xf);
        break;
      case Node::TRI: {
        bool smooth = !(isNull(n->n[0]) || isNull(n->n[1]) || isNull(n->n[2]));
        addTri(n->p[0], n->p[1], n->p[2], smooth ? n->n : nullptr, n->uv, resolveMat(n->mat), xf);
        break;
      }
      case Node::PLANE: {
        gbrt_plane p{};
        V4 P = n->plane;
        if (xf) {  // a plane transforms by the inverse transpose
          Mat4 inv = inverse(*xf);
          float v[4] = {P.x, P.y, P.z, P.w}, o[4];
          for (int c = 0; c < 4; ++c) o[c] = inv.m[0][c] * v[0] + inv.m[1][c] * v[1] + inv.m[2][c] * v[2] + inv.m[3][c] * v[3];
          P = {o[0], o[1], o[2], o[3]};
        }
        p.plane[0] = P.x; p.plane[1] = P.y; p.plane[2] = P.z; p.plane[3] = P.w;
        p.material = resolveMat(n->mat);
        ps.listed.emplace_back(gbrt_parsed_scene::kPlane, int64_t(ps.planes.size()));
        ps.planes.push_back(p);
        break;
      }
      case Node::SPHERE: {
        gbrt_sphere s{};
        V3 c = n->p[0];
        float r = n->radius;
        sphereXf(c, r, xf);
        s.center[0] = c.x; s.center[1] = c.y; s.center[2] = c.z;
        s.radius = r;
        s.material = resolveMat(n->mat);
        ps.listed.emplace_back(gbrt_parsed_scene::kSphere, int64_t(ps.spheres.size()));
        ps.spheres.push_back(s);
        break;
      }
      case Node::BOX:  // an AxisAlignedBox is a CSG object of its own
      case Node::CSG: {
        int leaves = 0;
        ps.listed.emplace_back(gbrt_parsed_scene::kCsg, int64_t(ps.csg_roots.size()));
        ps.csg_roots.push_back(csgNode(n, xf, leaves));
        if (leaves > GBRT_CSG_MAX_LEAVES)
          throw ParseError(GBRT_ERR_UNSUPPORTED, "CSG object with more than 8 spheres and boxes");
        break;
      }
      case Node::INSTANCE: {
        Mat4 M = xf ? (*xf) * n->xf : n->xf;
        const bool affine = M.m[3][0] == 0.f && M.m[3][1] == 0.f && M.m[3][2] == 0.f && M.m[3][3] == 1.f;
        int64_t tris = 0;
        if (affine && meshOnly(n->children[0], tris) && tris >= kInstanceMinTriangles) {
          gbrt_instance in{};
          for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 4; ++c) in.transform[4 * r + c] = M.m[r][c];
          in.mesh = meshFor(n->children[0]);
          ps.listed.emplace_back(gbrt_parsed_scene::kInstance, int64_t(ps.instances.size()));
          ps.instances.push_back(in);
        } else {
          emit(n->children[0], &M);
        }
        break;
      }
      case Node::OBJ: {
        const auto& obj = loadObj(n);
        for (auto& kv : obj.second) objMats.emplace(kv.first, kv.second);
        int deflt = resolveMat(n->mat);
        std::map<std::string, int> local;
        for (const ObjTri& t : obj.first) {
          int m = deflt;
          if (!t.mtl.empty()) {
            auto lt = local.find(t.mtl);
            if (lt == local.end()) {
              MatNode ref;
              ref.kind = -1;
              ref.ident = t.mtl;
              lt = local.emplace(t.mtl, resolveMat(ref)).first;
            }
            m = lt->second;
          }
          addTri(t.p[0], t.p[1], t.p[2], t.hasN ? t.n : nullptr, t.uv, m, xf);
        }
        break;
      }
    }
  }

  // An OBJ file's triangles and MTL materials, read once per path.
  const std::pair<std::vector<ObjTri>, std::map<std::string, MatNode>>& loadObj(const NodeP& n) {
    std::string path = joinPath(baseDir, n->file);
    auto it = objCache.find(path);
    if (it == objCache.end()) {
      std::vector<ObjTri> tris;
      std::map<std::string, MatNode> mats;
      if (!readOBJ(path, tris, mats)) throw ParseError(GBRT_ERR_IO, "cannot open OBJ file " + path);
      it = objCache.emplace(path, std::make_pair(std::move(tris), std::move(mats))).first;
    }
    return it->second;
  }

  // Smallest subtree an instance keeps as a shared mesh (smaller ones are
  // cheaper flattened into the scene's own tree).
  static constexpr int64_t kInstanceMinTriangles = 1024;

  // Whether a subtree holds only triangles (obj files, t(...), lists of
  // them), and how many.
  bool meshOnly(const NodeP& n, int64_t& count) {
    switch (n->kind) {
      case Node::TRI: ++count; return true;
      case Node::OBJ: count += int64_t(loadObj(n).first.size()); return true;
      case Node::LIST:
      case Node::BVH:
        for (auto& c : n->children)
          if (!meshOnly(c, count)) return false;
        return true;
      default: return false;
    }
  }

  // The shared mesh of a subtree (its triangles in its own space), built once
  // per subtree; obj(...) subtrees with the same file and material share one
  // (the grammar has no references to intersectables, so every instance of
  // a file writes its own obj(...)).
  std::map<std::string, int> meshIds;
  int meshFor(const NodeP& n) {
    char ptr[32];
    std::snprintf(ptr, sizeof ptr, "node:%p", static_cast<const void*>(n.get()));
    const std::string key =
        n->kind == Node::OBJ ? "obj:" + joinPath(baseDir, n->file) + ":" + std::to_string(resolveMat(n->mat)) : ptr;
    auto it = meshIds.find(key);
    if (it != meshIds.end()) return it->second;
    std::vector<float> pos, nrm, uv;
    std::vector<int32_t> mat;
    bool smooth = false;
    ps.tri_pos.swap(pos); ps.tri_nrm.swap(nrm); ps.tri_uv.swap(uv); ps.tri_mat.swap(mat);
    std::swap(ps.any_smooth, smooth);
    ++inMesh;  // the subtree's triangles belong to the mesh, not to the root list
    emit(n, nullptr);
    --inMesh;
    ps.tri_pos.swap(pos); ps.tri_nrm.swap(nrm); ps.tri_uv.swap(uv); ps.tri_mat.swap(mat);
    std::swap(ps.any_smooth, smooth);
    gbrt_parsed_scene::MeshData md;
    md.pos = std::move(pos);
    md.nrm = std::move(nrm);
    md.mat = std::move(mat);
    md.smooth = smooth;
    ps.meshes.push_back(std::move(md));
    const int id = int(ps.meshes.size()) - 1;
    meshIds[key] = id;
    return id;
  }

  // Instances move a sphere by a similarity transform (centre, radius).
  static void sphereXf(V3& c, float& r, const Mat4* xf) {
    if (!xf) return;
    V3 cx = xf->point(c);
    V3 ax = xf->dir({1, 0, 0}), ay = xf->dir({0, 1, 0}), az = xf->dir({0, 0, 1});
    auto L = [](V3 v) { return std::sqrt(double(v.x) * v.x + double(v.y) * v.y + double(v.z) * v.z); };
    double sx = L(ax), sy = L(ay), sz = L(az);
    if (std::fabs(sx - sy) > 1e-5 * sx || std::fabs(sx - sz) > 1e-5 * sx)
      throw ParseError(GBRT_ERR_UNSUPPORTED, "instance of a sphere with a non-uniform scale");
    c = cx;
    r = float(r * sx);
  }

  // A CSG tree into gbrt_csg_node entries; returns the root's index.
  int32_t csgNode(const NodeP& n, const Mat4* xf, int& leaves) {
    gbrt_csg_node g{};
    g.left = g.right = -1;
    if (n->kind == Node::SPHERE) {
      V3 c = n->p[0];
      float r = n->radius;
      sphereXf(c, r, xf);
      g.op = GBRT_CSG_SPHERE;
      g.a[0] = c.x; g.a[1] = c.y; g.a[2] = c.z;
      g.b[0] = r;
      g.material = resolveMat(n->mat);
      ++leaves;
    } else if (n->kind == Node::BOX) {
      V3 lo = n->p[0], hi = n->p[1];
      if (xf) {
        // axis-aligned only: no rotation or shear
        for (int r = 0; r < 3; ++r)
          for (int c = 0; c < 3; ++c)
            if (r != c && xf->m[r][c] != 0.f)
              throw ParseError(GBRT_ERR_UNSUPPORTED, "instance of a box that is not axis-aligned");
        V3 a = xf->point(lo), b = xf->point(hi);
        lo = {std::min(a.x, b.x), std::min(a.y, b.y), std::min(a.z, b.z)};
        hi = {std::max(a.x, b.x), std::max(a.y, b.y), std::max(a.z, b.z)};
      }
      g.op = GBRT_CSG_BOX;
      g.a[0] = lo.x; g.a[1] = lo.y; g.a[2] = lo.z;
      g.b[0] = hi.x; g.b[1] = hi.y; g.b[2] = hi.z;
      g.material = resolveMat(n->mat);
      ++leaves;
    } else if (n->kind == Node::CSG) {
      g.op = n->op == "isect" ? GBRT_CSG_ISECT : n->op == "union" ? GBRT_CSG_UNION
           : n->op == "diff" ? GBRT_CSG_DIFF : GBRT_CSG_XOR;
      g.left = csgNode(n->children[0], xf, leaves);
      g.right = csgNode(n->children[1], xf, leaves);
      g.material = -1;
    } else if (n->kind == Node::INSTANCE) {
      Mat4 M = xf ? (*xf) * n->xf : n->xf;
      return csgNode(n->children[0], &M, leaves);
    } else {
      throw ParseError(GBRT_ERR_PARSE, "a CSG operand must be a sphere, a box or a CSG operation");
    }
    ps.csg_nodes.push_back(g);
    return int32_t(ps.csg_nodes.size()) - 1;
  }
  static bool isNull(V3 v) { return v.x == 0 && v.y == 0 && v.z == 0; }

  void run(const std::vector<Assignment>& as) {
    // resolveVars: OBJ materials first (src/sceneast.cpp:730-747).
    std::vector<NodeP> stack;
    for (auto& a : as)
      if (a.value.kind == Value::INTERSECTABLE) stack.push_back(a.value.node);
    while (!stack.empty()) {
      NodeP n = stack.back();
      stack.pop_back();
      for (auto& c : n->children) stack.push_back(c);
      if (n->kind == Node::OBJ) {
        std::string path = joinPath(baseDir, n->file);
        if (!objCache.count(path)) {
          std::vector<ObjTri> tris;
          std::map<std::string, MatNode> mats;
          if (!readOBJ(path, tris, mats)) throw ParseError(GBRT_ERR_IO, "cannot open OBJ file " + path);
          objCache.emplace(path, std::make_pair(std::move(tris), std::move(mats)));
        }
        for (auto& kv : objCache[path].second) objMats.emplace(kv.first, kv.second);
      }
    }
    // scene_builder::addAssignment in order.
    std::map<std::string, NodeP> isect;
    for (auto& a : as) {
      const std::string& nm = a.name;
      auto eraseAll = [&]() { isect.erase(nm); lightVars.erase(nm); camVars.erase(nm); matVars.erase(nm); };
      switch (a.value.kind) {
        case Value::INTERSECTABLE: eraseAll(); isect[nm] = a.value.node; matSnapshot[nm] = matVars; break;
        case Value::LIGHTS: eraseAll(); lightVars[nm] = a.value.lights; break;
        case Value::CAMERA: eraseAll(); camVars[nm] = a.value.cam; break;
        case Value::MATERIAL: {
          MatNode m = a.value.mat;
          int id = resolveMat(m);
          eraseAll();
          matVars[nm] = id;
          break;
        }
        case Value::IDENT: {
          const std::string& src = a.value.ident;
          if (camVars.count(src)) { auto c = camVars[src]; eraseAll(); camVars[nm] = c; }
          else if (isect.count(src)) { auto n = isect[src]; auto snap = matSnapshot[src]; eraseAll(); isect[nm] = n; matSnapshot[nm] = snap; }
          else if (lightVars.count(src)) { auto l = lightVars[src]; eraseAll(); lightVars[nm] = l; }
          else if (matVars.count(src)) { int m = matVars[src]; eraseAll(); matVars[nm] = m; }
          break;  // the renderer prints "no such variable" and keeps going
        }
      }
    }
    // getScene: lights first, then the intersectable (src/sceneast.cpp:673-695).
    for (const LightNode& L : lightVars["lights"]) {
      gbrt_light g{};
      if (L.kind == 0) {
        g.type = GBRT_LIGHT_POINT;
        g.origin[0] = L.a.x; g.origin[1] = L.a.y; g.origin[2] = L.a.z;
      } else if (L.kind == 1) {
        g.type = GBRT_LIGHT_AREA;
        g.origin[0] = L.a.x; g.origin[1] = L.a.y; g.origin[2] = L.a.z;
        g.u[0] = L.b.x; g.u[1] = L.b.y; g.u[2] = L.b.z;
        g.v[0] = L.c.x; g.v[1] = L.c.y; g.v[2] = L.c.z;
      } else if (L.kind == 2) {
        g.type = GBRT_LIGHT_CONE;
        g.origin[0] = L.a.x; g.origin[1] = L.a.y; g.origin[2] = L.a.z;
        g.u[0] = L.b.x; g.u[1] = L.b.y; g.u[2] = L.b.z;
        g.v[0] = L.angle;
      } else {
        std::vector<float> tex;
        int W = 0, H = 0;
        std::string why;
        bool ok = !ps.has_env && (readImage(L.file, tex, W, H, why) || readImage(joinPath(baseDir, L.file), tex, W, H, why));
        if (ok) {
          g.type = GBRT_LIGHT_ENV;
          ps.env_texels.swap(tex);
          ps.env.width = W;
          ps.env.height = H;
          ps.env.mapping = (L.mapping == "latlong") ? GBRT_ENV_LATLONG : GBRT_ENV_ANGULAR;
          ps.has_env = true;
        } else {
          g.type = GBRT_LIGHT_BLACK;  // failed map, src/sceneast.cpp:598-610
        }
      }
      g.intensity[0] = L.I.z; g.intensity[1] = L.I.y; g.intensity[2] = L.I.x;
      ps.lights.push_back(g);
    }
    if (camVars.count("camera")) {
      const CameraNode& c = camVars["camera"];
      gbrt_camera& g = ps.camera;
      g.eye[0] = c.eye.x; g.eye[1] = c.eye.y; g.eye[2] = c.eye.z;
      g.look_at[0] = c.at.x; g.look_at[1] = c.at.y; g.look_at[2] = c.at.z;
      g.up[0] = c.up.x; g.up[1] = c.up.y; g.up[2] = c.up.z;
      g.fov = c.fov;
      g.width = int(c.xres);
      g.height = int(c.yres);
      ps.has_camera = true;
    }
    if (isect.count("intersectable")) {
      // Materials named inside the intersectable resolve against the
      // variables defined before its assignment.
      matVars = matSnapshot["intersectable"];
      emit(isect["intersectable"], nullptr);
    }
    if (ps.env.width) ps.env.texels = ps.env_texels.data();
  }
  std::map<std::string, std::map<std::string, int>> matSnapshot;
};

gbrt_status parseText(const std::string& text, const std::string& baseDir, gbrt_parsed_scene** out, char* err,
                      int32_t err_len) {
  auto setErr = [&](const std::string& m) {
    if (err && err_len > 0) {
      std::strncpy(err, m.c_str(), size_t(err_len) - 1);
      err[err_len - 1] = 0;
    }
  };
  try {
    Parser p(lex(text));
    std::vector<Assignment> as = p.file();
    std::unique_ptr<gbrt_parsed_scene> ps(new gbrt_parsed_scene());
    Builder b(*ps, baseDir);
    b.run(as);
    *out = ps.release();
    setErr("");
    return GBRT_OK;
  } catch (const ParseError& e) {
    setErr(e.what());
    return e.st;
  } catch (const std::bad_alloc&) {
    setErr("out of host memory");
    return GBRT_ERR_OOM;
  } catch (const std::exception& e) {
    setErr(e.what());
    return GBRT_ERR_PARSE;
  }
}

}  // namespace

extern "C" {

gbrt_status gbrt_parse_scene_string(const char* text, const char* base_dir, gbrt_parsed_scene** out, char* err,
                                    int32_t err_len) {
  if (!text || !out) return GBRT_ERR_INVALID_ARG;
  *out = nullptr;
  return parseText(text, base_dir ? base_dir : "", out, err, err_len);
}

gbrt_status gbrt_parse_scene_file(const char* path, gbrt_parsed_scene** out, char* err, int32_t err_len) {
  if (!path || !out) return GBRT_ERR_INVALID_ARG;
  *out = nullptr;
  std::string text;
  if (!readFile(path, text)) {
    if (err && err_len > 0) {
      std::snprintf(err, size_t(err_len), "Failed to open file %s", path);
    }
    return GBRT_ERR_IO;
  }
  return parseText(text, dirOf(path), out, err, err_len);
}

gbrt_status gbrt_parsed_scene_desc(const gbrt_parsed_scene* ps, gbrt_scene_desc* d, gbrt_camera* cam,
                                   int32_t* has_camera) {
  if (!ps || !d) return GBRT_ERR_INVALID_ARG;
  std::memset(d, 0, sizeof *d);
  d->materials = ps->materials.empty() ? nullptr : ps->materials.data();
  d->n_materials = int32_t(ps->materials.size());
  d->n_tri = int64_t(ps->tri_mat.size());
  d->tri_pos = d->n_tri ? ps->tri_pos.data() : nullptr;
  d->tri_nrm = (d->n_tri && ps->any_smooth) ? ps->tri_nrm.data() : nullptr;
  d->tri_mat = d->n_tri ? ps->tri_mat.data() : nullptr;
  d->tri_uv = d->n_tri ? ps->tri_uv.data() : nullptr;
  d->quads = ps->quads.empty() ? nullptr : ps->quads.data();
  d->n_quads = int32_t(ps->quads.size());
  d->spheres = ps->spheres.empty() ? nullptr : ps->spheres.data();
  d->n_spheres = int32_t(ps->spheres.size());
  d->planes = ps->planes.empty() ? nullptr : ps->planes.data();
  d->n_planes = int32_t(ps->planes.size());
  d->lights = ps->lights.empty() ? nullptr : ps->lights.data();
  d->n_lights = int32_t(ps->lights.size());
  d->env = ps->has_env ? &ps->env : nullptr;
  auto* mps = const_cast<gbrt_parsed_scene*>(ps);
  for (size_t i = 0; i < mps->textures.size(); ++i) mps->textures[i].texels = mps->texels[i].data();
  d->textures = ps->textures.empty() ? nullptr : ps->textures.data();
  d->n_textures = int32_t(ps->textures.size());
  d->csg_nodes = ps->csg_nodes.empty() ? nullptr : ps->csg_nodes.data();
  d->n_csg_nodes = int32_t(ps->csg_nodes.size());
  d->csg_roots = ps->csg_roots.empty() ? nullptr : ps->csg_roots.data();
  d->n_csg = int32_t(ps->csg_roots.size());
  // List ranks by primitive id: the lights first (the root list's head,
  // src/sceneast.cpp:676-678), then the intersectables as listed.
  {
    // first primitive id of each kind, in gbrt_parsed_scene::Kind order
    const int64_t nL = d->n_lights;
    int64_t first[6];
    first[gbrt_parsed_scene::kTri] = nL;
    first[gbrt_parsed_scene::kQuad] = first[gbrt_parsed_scene::kTri] + d->n_tri;
    first[gbrt_parsed_scene::kSphere] = first[gbrt_parsed_scene::kQuad] + d->n_quads;
    first[gbrt_parsed_scene::kPlane] = first[gbrt_parsed_scene::kSphere] + d->n_spheres;
    first[gbrt_parsed_scene::kCsg] = first[gbrt_parsed_scene::kPlane] + d->n_planes;
    first[gbrt_parsed_scene::kInstance] = first[gbrt_parsed_scene::kCsg] + d->n_csg;
    const int64_t n = first[gbrt_parsed_scene::kInstance] + int64_t(ps->instances.size());
    mps->list_rank.resize(size_t(n));
    for (int64_t i = 0; i < n; ++i) mps->list_rank[size_t(i)] = int32_t(i);
    if (int64_t(ps->listed.size()) == n - nL) {
      int64_t r = nL;
      for (const auto& e : ps->listed) mps->list_rank[size_t(first[e.first] + e.second)] = int32_t(r++);
    }
    d->list_rank = n ? mps->list_rank.data() : nullptr;
  }
  mps->mesh_descs.resize(ps->meshes.size());
  for (size_t i = 0; i < ps->meshes.size(); ++i) {
    const auto& m = ps->meshes[i];
    gbrt_mesh& g = mps->mesh_descs[i];
    g.tri_pos = m.pos.data();
    g.tri_nrm = m.smooth ? m.nrm.data() : nullptr;
    g.tri_mat = m.mat.data();
    g.n_tri = int64_t(m.mat.size());
  }
  d->meshes = ps->mesh_descs.empty() ? nullptr : ps->mesh_descs.data();
  d->n_meshes = int32_t(ps->mesh_descs.size());
  d->instances = ps->instances.empty() ? nullptr : ps->instances.data();
  d->n_instances = int32_t(ps->instances.size());
  if (cam) *cam = ps->camera;
  if (has_camera) *has_camera = ps->has_camera ? 1 : 0;
  return GBRT_OK;
}

void gbrt_parsed_scene_free(gbrt_parsed_scene* ps) { delete ps; }

gbrt_status gbrt_read_hdr(const char* path, float** texels, int32_t* width, int32_t* height) {
  if (!path || !texels || !width || !height) return GBRT_ERR_INVALID_ARG;
  std::vector<float> v;
  int W = 0, H = 0;
  std::string why;
  if (!readImage(path, v, W, H, why)) return GBRT_ERR_IO;
  float* p = static_cast<float*>(std::malloc(v.size() * sizeof(float)));
  if (!p) return GBRT_ERR_OOM;
  std::memcpy(p, v.data(), v.size() * sizeof(float));
  *texels = p;
  *width = W;
  *height = H;
  return GBRT_OK;
}

}  // extern "C"
