// Scene-folder loader: scene.json, scene.obj, scene.mtl, HDRI/<name>.hdr and
// the BMP textures the .mtl names -- the reference's loadScene
// (SceneLoader.hpp:7-143, ObjLoader.hpp:20-206, Texture.hpp:41-68,
// HDRI.hpp:42-60), reading the same files into an er_scene_desc.
//
// Reference behaviours kept, so a folder renders the same:
//  - OBJ objects start at lines beginning with 'o'; lines before the first
//    'o' are not parsed; z of v / vn is negated (ObjLoader.hpp:85,91);
//    normals are normalised; the last `usemtl` of an object names its
//    material, matched against .mtl names (last match wins, else 0).
//  - Faces: the first three vertices of an `f` line, v/vt/vn indices.
//  - MTL: Kd -> albedo, Ks.x -> specular, Ke -> emission, Ni -> eta;
//    map_Kd (sRGB), map_Ns (roughness), refl (metallic), map_Bump (normal)
//    map names matched anywhere in a line, textures assigned in the key
//    order map_Bump, map_Kd, map_Ns, refl and shared between materials by
//    path.  Numbers in Kd/Ks/Ke lines are read by the reference's
//    digit/'.'/'-' scanner (Vector.hpp:15-62).
//  - scene.json: hdri.yOffset is written into the x offset
//    (SceneLoader.hpp:64-65).
//  - LDR textures decode through fastPow(b/255, 2.2) for map_Kd and
//    fastPow(b/255, 1.0) otherwise, rows flipped; the HDR environment is
//    RGBE-decoded and not flipped.
// Extension (ignored by the reference's parser): MTL keys Pr, Pm, Pc, Ps
// set roughness, metallic, clearcoat and sheen, which the reference's .mtl
// reader cannot express.
// Texture paths are tried as written (the reference resolves them against
// the working directory) and then relative to the scene folder.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "internal.h"

namespace er {
namespace {

// ------------------------------------------------------------------- I/O

bool read_file(const std::string& path, std::string* out) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  std::ostringstream ss;
  ss << f.rdbuf();
  *out = ss.str();
  return true;
}

bool file_exists(const std::string& p) {
  std::ifstream f(p);
  return (bool)f;
}

// ------------------------------------------------------------------ JSON

struct JVal {
  enum Kind { NUL, BOOL, NUM, STR, ARR, OBJ } kind = NUL;
  std::string text;  // number text / string value
  bool b = false;
  std::vector<JVal> arr;
  std::vector<std::pair<std::string, JVal>> obj;
  const JVal* get(const char* k) const {
    if (kind != OBJ) return nullptr;
    for (auto& kv : obj)
      if (kv.first == k) return &kv.second;
    return nullptr;
  }
};

struct JParser {
  const std::string& s;
  size_t i = 0;
  std::string err;
  explicit JParser(const std::string& src) : s(src) {}
  void ws() {
    while (i < s.size() && (s[i] == ' ' || s[i] == '\t' || s[i] == '\n' || s[i] == '\r')) i++;
  }
  bool lit(const char* w) {
    size_t n = std::strlen(w);
    if (s.compare(i, n, w) == 0) {
      i += n;
      return true;
    }
    return false;
  }
  bool str(std::string* out) {
    if (i >= s.size() || s[i] != '"') return false;
    i++;
    out->clear();
    while (i < s.size() && s[i] != '"') {
      if (s[i] == '\\' && i + 1 < s.size()) {
        char c = s[i + 1];
        out->push_back(c == 'n' ? '\n' : c == 't' ? '\t' : c);
        i += 2;
      } else {
        out->push_back(s[i++]);
      }
    }
    if (i >= s.size()) return false;
    i++;
    return true;
  }
  bool val(JVal* v, int depth = 0) {
    if (depth > 64) return false;
    ws();
    if (i >= s.size()) return false;
    char c = s[i];
    if (c == '{') {
      i++;
      v->kind = JVal::OBJ;
      ws();
      if (i < s.size() && s[i] == '}') { i++; return true; }
      while (true) {
        ws();
        std::string k;
        if (!str(&k)) return false;
        ws();
        if (i >= s.size() || s[i] != ':') return false;
        i++;
        JVal x;
        if (!val(&x, depth + 1)) return false;
        v->obj.emplace_back(k, std::move(x));
        ws();
        if (i < s.size() && s[i] == ',') { i++; continue; }
        if (i < s.size() && s[i] == '}') { i++; return true; }
        return false;
      }
    }
    if (c == '[') {
      i++;
      v->kind = JVal::ARR;
      ws();
      if (i < s.size() && s[i] == ']') { i++; return true; }
      while (true) {
        JVal x;
        if (!val(&x, depth + 1)) return false;
        v->arr.push_back(std::move(x));
        ws();
        if (i < s.size() && s[i] == ',') { i++; continue; }
        if (i < s.size() && s[i] == ']') { i++; return true; }
        return false;
      }
    }
    if (c == '"') {
      v->kind = JVal::STR;
      return str(&v->text);
    }
    if (lit("true")) { v->kind = JVal::BOOL; v->b = true; return true; }
    if (lit("false")) { v->kind = JVal::BOOL; v->b = false; return true; }
    if (lit("null")) { v->kind = JVal::NUL; return true; }
    size_t j = i;
    while (j < s.size() && (std::isdigit((unsigned char)s[j]) || s[j] == '-' || s[j] == '+' || s[j] == '.' ||
                            s[j] == 'e' || s[j] == 'E'))
      j++;
    if (j == i) return false;
    v->kind = JVal::NUM;
    v->text = s.substr(i, j - i);
    i = j;
    return true;
  }
};

// RSJresource::as<double>: atof of the (unquoted) text
bool jnum(const JVal* v, double* out) {
  if (!v) return false;
  if (v->kind == JVal::NUM || v->kind == JVal::STR) {
    *out = std::atof(v->text.c_str());
    return true;
  }
  if (v->kind == JVal::BOOL) {
    *out = v->b ? 1.0 : 0.0;
    return true;
  }
  return false;
}

// RSJresource::as<bool>: "true"/"TRUE"/"True" or a nonzero integer
bool jbool(const JVal* v) {
  if (!v) return false;
  if (v->kind == JVal::BOOL) return v->b;
  const std::string& t = v->text;
  return t == "true" || t == "TRUE" || t == "True" || std::atoi(t.c_str()) != 0;
}

// RSJparser.hpp:773-785: {x,y,z} or {r,g,b}
bool jvec3(const JVal* v, float out[3]) {
  if (!v) return false;
  const char* k[2][3] = {{"x", "y", "z"}, {"r", "g", "b"}};
  for (int s = 0; s < 2; s++) {
    if (v->get(k[s][0])) {
      for (int a = 0; a < 3; a++) {
        double d = 0;
        jnum(v->get(k[s][a]), &d);
        out[a] = (float)d;
      }
      return true;
    }
  }
  return false;
}

// ------------------------------------------------------------ text parsing

// Vector.hpp:15-62: characters 0-9 . - accumulate into x, y, z in turn; any
// other character after the first number switches component; std::stof.
bool ref_vec3(const std::string& str, float out[3]) {
  std::string c[3];
  int k = 0;
  bool start = false;
  for (char ch : str) {
    if (std::isdigit((unsigned char)ch) || ch == '.' || ch == '-') {
      if (k < 3) c[k].push_back(ch);
      start = true;
    } else if (start && k < 3) {
      k++;
    }
  }
  for (int a = 0; a < 3; a++) {
    if (c[a].empty()) c[a] = "0";
    char* end = nullptr;
    out[a] = std::strtof(c[a].c_str(), &end);
    if (end == c[a].c_str()) return false;  // std::stof would throw
  }
  return true;
}

// ObjLoader.hpp:22-25
std::string second_word(const std::string& s) {
  size_t p = s.find_first_of(' ');
  return p == std::string::npos ? s : s.substr(p + 1);
}

std::string rstrip(std::string s) {
  while (!s.empty() && (s.back() == '\r' || s.back() == '\n' || s.back() == ' ' || s.back() == '\t')) s.pop_back();
  return s;
}

std::vector<std::string> lines_of(const std::string& text) {
  std::vector<std::string> out;
  size_t i = 0;
  while (i <= text.size()) {
    size_t j = text.find('\n', i);
    if (j == std::string::npos) {
      if (i < text.size()) out.push_back(rstrip(text.substr(i)));
      break;
    }
    out.push_back(rstrip(text.substr(i, j - i)));
    i = j + 1;
  }
  return out;
}

// ---------------------------------------------------------------- images

// stb_image.h:127-135 / Texture.hpp:41-68: 8-bit channel -> float through
// Ankerl's approximate pow (martin.ankerl.com, 2012).
float ldr_to_float(uint8_t b, float gamma) {
  double a = (double)((float)b / 255.0f);
  int64_t bits;
  std::memcpy(&bits, &a, 8);
  int32_t hi = (int32_t)(bits >> 32);
  hi = (int32_t)((double)gamma * (double)(hi - 1072632447) + 1072632447);
  bits = (int64_t)((uint64_t)(uint32_t)hi << 32);
  double r;
  std::memcpy(&r, &bits, 8);
  return (float)(r * (double)1.0f);
}

uint32_t le16(const uint8_t* p) { return p[0] | (p[1] << 8); }
uint32_t le32u(const uint8_t* p) { return p[0] | (p[1] << 8) | (p[2] << 16) | ((uint32_t)p[3] << 24); }

// Uncompressed BMP (8-bit paletted, 24-bit, 32-bit) -> RGB bytes, row 0 =
// bottom row of the picture (stbi_set_flip_vertically_on_load(true)).
er_status decode_bmp(const std::string& data, const std::string& path, int* w, int* h, std::vector<uint8_t>* rgb) {
  const uint8_t* d = (const uint8_t*)data.data();
  size_t n = data.size();
  if (n < 54 || d[0] != 'B' || d[1] != 'M') return fail(ER_ERR_PARSE, path + ": not a BMP file");
  uint32_t off = le32u(d + 10), hsz = le32u(d + 14);
  int32_t W = (int32_t)le32u(d + 18), H = (int32_t)le32u(d + 22);
  uint32_t bpp = le16(d + 28), comp = le32u(d + 30);
  if (hsz < 40 || W <= 0 || H == 0 || W > (1 << 16) || std::abs(H) > (1 << 16))
    return fail(ER_ERR_PARSE, path + ": bad BMP header");
  if (comp != 0 && !(comp == 3 && bpp == 32)) return fail(ER_ERR_UNSUPPORTED, path + ": compressed BMP");
  if (bpp != 8 && bpp != 24 && bpp != 32) return fail(ER_ERR_UNSUPPORTED, path + ": BMP bit depth " + std::to_string(bpp));
  bool bottom_up = H > 0;
  int32_t AH = std::abs(H);
  size_t stride = (((size_t)W * bpp / 8) + 3) & ~(size_t)3;
  if ((size_t)off + stride * AH > n) return fail(ER_ERR_PARSE, path + ": truncated BMP");
  const uint8_t* pal = d + 14 + hsz;
  uint32_t ncol = bpp == 8 ? (le32u(d + 46) ? le32u(d + 46) : 256u) : 0u;
  if (bpp == 8 && (size_t)(pal - d) + 4 * (size_t)ncol > off) return fail(ER_ERR_PARSE, path + ": bad BMP palette");
  rgb->assign((size_t)W * AH * 3, 0);
  for (int32_t r = 0; r < AH; r++) {
    // file row r; picture row from the top: bottom-up files store the bottom first
    int32_t top = bottom_up ? AH - 1 - r : r;
    int32_t dst_row = AH - 1 - top;  // flipped: row 0 = bottom of the picture
    const uint8_t* src = d + off + stride * r;
    uint8_t* dst = rgb->data() + (size_t)dst_row * W * 3;
    for (int32_t x = 0; x < W; x++) {
      if (bpp == 8) {
        uint32_t ci = src[x];
        if (ci >= ncol) return fail(ER_ERR_PARSE, path + ": BMP palette index out of range");
        const uint8_t* c = pal + 4 * ci;
        dst[3 * x] = c[2]; dst[3 * x + 1] = c[1]; dst[3 * x + 2] = c[0];
      } else {
        const uint8_t* c = src + (size_t)x * (bpp / 8);
        dst[3 * x] = c[2]; dst[3 * x + 1] = c[1]; dst[3 * x + 2] = c[0];
      }
    }
  }
  *w = W;
  *h = AH;
  return ER_OK;
}

// Radiance RGBE (.hdr), flat or new-style RLE scanlines; decode as stb:
// c * ldexp(1, e - 136), e == 0 -> 0.  Row 0 = first scanline in the file.
er_status decode_hdr(const std::string& data, const std::string& path, int* w, int* h, std::vector<float>* out) {
  const uint8_t* d = (const uint8_t*)data.data();
  size_t n = data.size(), i = 0;
  auto line = [&](std::string* l) {
    l->clear();
    while (i < n && d[i] != '\n') l->push_back((char)d[i++]);
    if (i < n) i++;
    return i <= n;
  };
  std::string l;
  line(&l);
  if (l.rfind("#?RADIANCE", 0) != 0 && l.rfind("#?RGBE", 0) != 0) return fail(ER_ERR_PARSE, path + ": not a Radiance HDR");
  bool fmt_ok = false;
  while (i < n) {
    line(&l);
    if (l.empty()) break;
    if (l == "FORMAT=32-bit_rle_rgbe") fmt_ok = true;
  }
  if (!fmt_ok) return fail(ER_ERR_UNSUPPORTED, path + ": HDR format is not 32-bit_rle_rgbe");
  line(&l);
  int H = 0, W = 0;
  if (std::sscanf(l.c_str(), "-Y %d +X %d", &H, &W) != 2 || W <= 0 || H <= 0 || W > (1 << 16) || H > (1 << 16))
    return fail(ER_ERR_UNSUPPORTED, path + ": HDR orientation must be -Y h +X w");
  // Each scanline takes at least its run-length minimum (a 4-byte header,
  // then per channel one 2-byte run per 127 pixels) or its flat size: a
  // header the remaining bytes cannot hold is rejected before anything is
  // allocated for it.
  const size_t flat = (size_t)W * 4;
  const size_t rle = (W >= 8 && W < 32768) ? 4 + 8 * (((size_t)W + 126) / 127) : flat;
  if ((n - i) / std::min(flat, rle) < (size_t)H) return fail(ER_ERR_PARSE, path + ": truncated HDR");
  out->assign((size_t)W * H * 3, 0.0f);
  std::vector<uint8_t> scan((size_t)W * 4);
  for (int y = 0; y < H; y++) {
    if (W >= 8 && W < 32768 && i + 4 <= n && d[i] == 2 && d[i + 1] == 2 && !(d[i + 2] & 0x80)) {
      if ((int)((d[i + 2] << 8) | d[i + 3]) != W) return fail(ER_ERR_PARSE, path + ": bad RLE scanline width");
      i += 4;
      for (int c = 0; c < 4; c++) {
        int x = 0;
        while (x < W) {
          if (i >= n) return fail(ER_ERR_PARSE, path + ": truncated HDR");
          int cnt = d[i++];
          if (cnt > 128) {
            cnt -= 128;
            if (i >= n || x + cnt > W) return fail(ER_ERR_PARSE, path + ": bad HDR run");
            uint8_t v = d[i++];
            for (int k = 0; k < cnt; k++) scan[4 * (x++) + c] = v;
          } else {
            if (cnt == 0 || i + cnt > n || x + cnt > W) return fail(ER_ERR_PARSE, path + ": bad HDR run");
            for (int k = 0; k < cnt; k++) scan[4 * (x++) + c] = d[i++];
          }
        }
      }
    } else {
      if (i + (size_t)W * 4 > n) return fail(ER_ERR_PARSE, path + ": truncated HDR");
      std::memcpy(scan.data(), d + i, (size_t)W * 4);
      i += (size_t)W * 4;
    }
    for (int x = 0; x < W; x++) {
      const uint8_t* p = &scan[4 * x];
      float* o = &(*out)[3 * ((size_t)y * W + x)];
      if (p[3]) {
        float f = std::ldexp(1.0f, (int)p[3] - (128 + 8));
        o[0] = p[0] * f; o[1] = p[1] * f; o[2] = p[2] * f;
      }
    }
  }
  *w = W;
  *h = H;
  return ER_OK;
}

// --------------------------------------------------------------- scene

struct Mtl {
  std::string name;
  er_material m;
  std::map<std::string, std::string> maps;  // ordered like std::map in the reference
};

void default_material(er_material* m) {  // Material.hpp:21-36
  std::memset(m, 0, sizeof *m);
  m->albedo_tex = m->emission_tex = m->roughness_tex = m->metallic_tex = m->normal_tex = -1;
  m->albedo[0] = m->albedo[1] = m->albedo[2] = 0.5f;
  m->roughness = 1.0f;
  m->specular = 0.5f;
}

// ObjLoader.hpp:33-69 + 193-206
er_status parse_mtl(const std::string& text, std::vector<Mtl>* out) {
  std::vector<std::string> L = lines_of(text);
  for (size_t i = 0; i < L.size(); i++) {
    if (L[i].find("newmtl") == std::string::npos) continue;
    Mtl mt;
    mt.name = second_word(L[i]);
    default_material(&mt.m);
    for (size_t j = i + 1; j < L.size() && L[j].find("newmtl") == std::string::npos; j++) {
      const std::string& l = L[j];
      float v[3];
      if (l.size() >= 2 && l[0] == 'K' && l[1] == 'd') {
        if (!ref_vec3(l.substr(2), v)) return fail(ER_ERR_PARSE, "scene.mtl: bad Kd: " + l);
        std::memcpy(mt.m.albedo, v, sizeof v);
      }
      if (l.size() >= 2 && l[0] == 'K' && l[1] == 's') {
        if (!ref_vec3(l.substr(2), v)) return fail(ER_ERR_PARSE, "scene.mtl: bad Ks: " + l);
        mt.m.specular = v[0];
      }
      if (l.size() >= 2 && l[0] == 'K' && l[1] == 'e') {
        if (!ref_vec3(l.substr(2), v)) return fail(ER_ERR_PARSE, "scene.mtl: bad Ke: " + l);
        std::memcpy(mt.m.emission, v, sizeof v);
      }
      if (l.size() >= 2 && l[0] == 'N' && l[1] == 'i') mt.m.eta = std::strtof(second_word(l).c_str(), nullptr);
      if (l.size() >= 3 && l[0] == 'P' && l[2] == ' ') {  // PBR extension keys
        float x = std::strtof(second_word(l).c_str(), nullptr);
        if (l[1] == 'r') mt.m.roughness = x;
        if (l[1] == 'm') mt.m.metallic = x;
        if (l[1] == 'c') mt.m.clearcoat = x;
        if (l[1] == 's') mt.m.sheen = x;
      }
      static const char* names[] = {"map_Kd", "map_Ns", "map_Bump", "refl"};
      for (const char* nm : names)
        if (l.find(nm) != std::string::npos) mt.maps[nm] = second_word(l);
    }
    out->push_back(std::move(mt));
  }
  return ER_OK;
}

struct Obj {
  std::string mat;
  std::vector<float> pos, nrm, uv;  // per triangle vertex
};

int parse_index(const std::string& s, int n, int* out) {
  if (s.empty()) return 0;
  long v = std::strtol(s.c_str(), nullptr, 10);
  if (v < 1 || v > n) return -1;
  *out = (int)v - 1;
  return 1;
}

// ObjLoader.hpp:71-189
er_status parse_obj(const std::string& text, std::vector<Obj>* objs) {
  std::vector<std::string> L = lines_of(text);
  std::vector<float> V, T, N;  // global lists (OBJ indices are global)
  Obj* cur = nullptr;
  for (const std::string& l : L) {
    if (!l.empty() && l[0] == 'o') {
      objs->emplace_back();
      cur = &objs->back();
      continue;
    }
    if (!cur) continue;  // lines before the first object are not parsed
    if (l.find("usemtl") != std::string::npos) cur->mat = second_word(l);
    float v[3];
    if (l.size() >= 2 && l[0] == 'v' && l[1] == ' ') {
      if (!ref_vec3(l.substr(2), v)) return fail(ER_ERR_PARSE, "scene.obj: bad vertex: " + l);
      V.push_back(v[0]); V.push_back(v[1]); V.push_back(v[2] * -1.0f);
    }
    if (l.size() >= 2 && l[0] == 'v' && l[1] == 't') {
      if (!ref_vec3(l.substr(2), v)) return fail(ER_ERR_PARSE, "scene.obj: bad vt: " + l);
      T.push_back(v[0]); T.push_back(v[1]);
    }
    if (l.size() >= 2 && l[0] == 'v' && l[1] == 'n') {
      if (!ref_vec3(l.substr(2), v)) return fail(ER_ERR_PARSE, "scene.obj: bad vn: " + l);
      N.push_back(v[0]); N.push_back(v[1]); N.push_back(v[2] * -1.0f);
    }
    if (!l.empty() && l[0] == 'f') {
      // ObjLoader.hpp:92-118: digits and '/' go to vertex slot idx; every
      // other character after the first digit advances idx (so "1  2"
      // leaves slot 1 empty); slots beyond the third are dropped.
      std::string f[3];
      int idx = -1;
      for (char ch : l) {
        if (std::isdigit((unsigned char)ch) || ch == '/') {
          if (idx == -1) idx = 0;
          if (idx < 3) f[idx].push_back(ch);
        } else if (idx > -1) {
          idx++;
        }
      }
      for (int k = 0; k < 3; k++) {
        std::string part[3];
        int pi = 0;
        for (char ch : f[k]) {
          if (ch == '/') { if (++pi > 2) break; }
          else part[pi].push_back(ch);
        }
        int vi = 0, ti = 0, ni = 0;
        int rv = parse_index(part[0], (int)V.size() / 3, &vi);
        int rt = parse_index(part[1], (int)T.size() / 2, &ti);
        int rn = parse_index(part[2], (int)N.size() / 3, &ni);
        if (rv < 0 || rt < 0 || rn < 0) return fail(ER_ERR_PARSE, "scene.obj: index out of range: " + l);
        for (int a = 0; a < 3; a++) cur->pos.push_back(rv ? V[3 * vi + a] : 0.0f);
        for (int a = 0; a < 2; a++) cur->uv.push_back(rt ? T[2 * ti + a] : 0.0f);
        float nx = 0, ny = 0, nz = 0;
        if (rn) {  // Vector3::normalized
          nx = N[3 * ni]; ny = N[3 * ni + 1]; nz = N[3 * ni + 2];
          float len = std::sqrt(nx * nx + ny * ny + nz * nz);
          if (len != 0.0f) { nx /= len; ny /= len; nz /= len; }
        }
        cur->nrm.push_back(nx); cur->nrm.push_back(ny); cur->nrm.push_back(nz);
      }
    }
  }
  return ER_OK;
}

std::string join(const std::string& dir, const std::string& f) {
  if (dir.empty() || dir.back() == '/') return dir + f;
  return dir + "/" + f;
}

}  // namespace
}  // namespace er

// A parsed scene folder: the description and the arrays it points into.
struct er_folder {
  er_scene_desc d{};
  std::vector<float> env_data, pos, nrm, uv, tan, tsign;
  std::vector<std::vector<float>> tex_data;
  std::vector<er_texture> texs;
  std::vector<er_material> mats;
  std::vector<int32_t> tri_obj, obj_mat;
  std::vector<er_point_light> lights;
};

namespace er {
namespace {

// The reference's loadScene (SceneLoader.hpp:7-143) into an er_folder.
er_status read_folder(const std::string& dir, er_folder* F) {
  std::string text;
  if (!read_file(join(dir, "scene.json"), &text)) return fail(ER_ERR_IO, "cannot read " + join(dir, "scene.json"));
  JVal root;
  JParser jp(text);
  if (!jp.val(&root) || root.kind != JVal::OBJ) return fail(ER_ERR_PARSE, "scene.json: malformed JSON");

  er_scene_desc& d = F->d;
  d = er_scene_desc{};
  // camera (SceneLoader.hpp:25-46; Camera(xRes, yRes), Camera.hpp:29-37)
  const JVal* cam = root.get("camera");
  if (!cam) return fail(ER_ERR_PARSE, "scene.json: no camera");
  double xr = 0, yr = 0, fl = 0, fd = 0, ap = 0;
  if (!jnum(cam->get("xRes"), &xr) || !jnum(cam->get("yRes"), &yr))
    return fail(ER_ERR_PARSE, "scene.json: camera needs xRes and yRes");
  d.camera.x_res = (int32_t)xr;
  d.camera.y_res = (int32_t)yr;
  d.camera.sensor_width = (float)(35 * 0.001);
  d.camera.sensor_height = d.camera.sensor_width * ((float)d.camera.y_res / (float)d.camera.x_res);
  // a missing field reads as 0, as RSJresource::as<double>() returns its
  // default argument, which overwrites Camera's own defaults
  d.camera.focal_length = jnum(cam->get("focalLength"), &fl) ? (float)fl : 0.0f;
  d.camera.focus_distance = jnum(cam->get("focusDistance"), &fd) ? (float)fd : 0.0f;
  d.camera.aperture = jnum(cam->get("aperture"), &ap) ? (float)ap : 0.0f;
  d.camera.bokeh = jbool(cam->get("bokeh")) ? 1 : 0;
  if (!jvec3(cam->get("position"), d.camera.position)) std::memset(d.camera.position, 0, sizeof d.camera.position);
  if (!jvec3(cam->get("rotation"), d.camera.rotation)) std::memset(d.camera.rotation, 0, sizeof d.camera.rotation);

  // environment (SceneLoader.hpp:51-65, HDRI.hpp:22-60)
  const JVal* hd = root.get("hdri");
  if (!hd) return fail(ER_ERR_PARSE, "scene.json: no hdri");
  int ew = 0, eh = 0;
  if (const JVal* nm = hd->get("name")) {
    std::string hp = join(join(dir, "HDRI"), nm->text + ".hdr");
    std::string bytes;
    if (!read_file(hp, &bytes)) return fail(ER_ERR_IO, "cannot read " + hp);
    er_status st = decode_hdr(bytes, hp, &ew, &eh, &F->env_data);
    if (st != ER_OK) return st;
  } else if (const JVal* col = hd->get("color")) {
    float c[3];
    if (!jvec3(col, c)) return fail(ER_ERR_PARSE, "scene.json: hdri.color needs r, g, b");
    ew = eh = 1024;
    F->env_data.resize((size_t)ew * eh * 3);
    for (size_t i = 0; i < (size_t)ew * eh; i++) {
      F->env_data[3 * i] = c[0];
      F->env_data[3 * i + 1] = c[1];
      F->env_data[3 * i + 2] = c[2];
    }
  } else {
    return fail(ER_ERR_PARSE, "scene.json: hdri needs name or color");
  }
  d.env.width = ew;
  d.env.height = eh;
  d.env.data = F->env_data.data();
  d.env.x_tile = d.env.y_tile = 1.0f;
  double off = 0;
  if (jnum(hd->get("xOffset"), &off)) d.env.x_offset = (float)off;
  if (jnum(hd->get("yOffset"), &off)) d.env.x_offset = (float)off;  // SceneLoader.hpp:64-65

  // materials and textures (SceneLoader.hpp:67-107)
  std::vector<Mtl> mtls;
  if (read_file(join(dir, "scene.mtl"), &text)) {
    er_status st = parse_mtl(text, &mtls);
    if (st != ER_OK) return st;
  }
  std::vector<std::string> tex_paths;
  for (Mtl& mt : mtls) {
    for (auto& kv : mt.maps) {
      const std::string& key = kv.first;
      const std::string& mp = kv.second;
      int id = (int)tex_paths.size();
      bool dup = false;
      for (size_t j = 0; j < tex_paths.size(); j++)
        if (tex_paths[j] == mp) { id = (int)j; dup = true; }
      float gamma = 1.0f;
      if (key == "map_Kd") { mt.m.albedo_tex = id; gamma = 2.2f; }
      if (key == "map_Ns") mt.m.roughness_tex = id;
      if (key == "refl") mt.m.metallic_tex = id;
      if (key == "map_Bump") mt.m.normal_tex = id;
      if (dup) continue;
      std::string p = file_exists(mp) ? mp : join(dir, mp);
      std::string bytes;
      if (!read_file(p, &bytes)) return fail(ER_ERR_IO, "cannot read texture " + mp);
      int w = 0, h = 0;
      std::vector<uint8_t> rgb;
      er_status st = decode_bmp(bytes, p, &w, &h, &rgb);
      if (st != ER_OK) return st;
      std::vector<float> f(rgb.size());
      for (size_t i = 0; i < rgb.size(); i++) f[i] = ldr_to_float(rgb[i], gamma);
      tex_paths.push_back(mp);
      F->tex_data.push_back(std::move(f));
      er_texture t{};
      t.width = w;
      t.height = h;
      t.x_tile = t.y_tile = 1.0f;
      F->texs.push_back(t);
    }
  }
  for (size_t i = 0; i < F->texs.size(); i++) F->texs[i].data = F->tex_data[i].data();
  for (const Mtl& mt : mtls) F->mats.push_back(mt.m);
  if (F->mats.empty()) {  // no .mtl: one default material
    er_material m;
    default_material(&m);
    F->mats.push_back(m);
  }

  // geometry (SceneLoader.hpp:109-123)
  if (!read_file(join(dir, "scene.obj"), &text)) return fail(ER_ERR_IO, "cannot read " + join(dir, "scene.obj"));
  std::vector<Obj> objs;
  er_status st = parse_obj(text, &objs);
  if (st != ER_OK) return st;
  for (size_t o = 0; o < objs.size(); o++) {
    int mid = 0;
    for (size_t j = 0; j < mtls.size(); j++)
      if (mtls[j].name == objs[o].mat) mid = (int)j;
    F->obj_mat.push_back(mid);
    size_t nt = objs[o].pos.size() / 9;
    F->pos.insert(F->pos.end(), objs[o].pos.begin(), objs[o].pos.end());
    F->nrm.insert(F->nrm.end(), objs[o].nrm.begin(), objs[o].nrm.end());
    F->uv.insert(F->uv.end(), objs[o].uv.begin(), objs[o].uv.end());
    F->tri_obj.insert(F->tri_obj.end(), nt, (int32_t)o);
  }
  d.tri_count = (int64_t)(F->pos.size() / 9);
  // tangents per object, as the reference's loader does (ObjLoader.hpp:167-168)
  F->tan.resize(F->pos.size());
  F->tsign.resize((size_t)d.tri_count);
  for (int64_t b = 0, o = 0; b < d.tri_count; o++) {
    int64_t e = b;
    while (e < d.tri_count && F->tri_obj[(size_t)e] == o) e++;
    compute_tangents(e - b, F->pos.data() + 9 * b, F->nrm.data() + 9 * b, F->uv.data() + 6 * b,
                     F->tan.data() + 9 * b, F->tsign.data() + b);
    b = e;
  }

  // point lights (SceneLoader.hpp:125-141)
  if (const JVal* pl = root.get("pointLights")) {
    for (const JVal& l : pl->arr) {
      er_point_light p{};
      if (!jvec3(l.get("position"), p.position) || !jvec3(l.get("radiance"), p.radiance))
        return fail(ER_ERR_PARSE, "scene.json: point light needs position and radiance");
      F->lights.push_back(p);
    }
  }
  d.positions = F->pos.data();
  d.normals = F->nrm.data();
  d.uvs = F->uv.data();
  d.tangents = F->tan.data();
  d.tangent_sign = F->tsign.data();
  d.tri_object = F->tri_obj.data();
  d.object_count = (int32_t)F->obj_mat.size();
  d.object_material = F->obj_mat.data();
  d.material_count = (int32_t)F->mats.size();
  d.materials = F->mats.data();
  d.texture_count = (int32_t)F->texs.size();
  d.textures = F->texs.data();
  d.light_count = (int32_t)F->lights.size();
  d.lights = F->lights.data();
  return ER_OK;
}

}  // namespace
}  // namespace er

using namespace er;

extern "C" er_status er_scene_folder_read(const char* dir, er_folder** out) {
  return guarded("er_scene_folder_read", [&]() -> er_status {
    if (out) *out = nullptr;
    if (!dir || !out) return fail(ER_ERR_INVALID_ARG, "NULL argument");
    std::unique_ptr<er_folder> F(new er_folder());
    er_status st = read_folder(dir, F.get());
    if (st != ER_OK) return st;
    *out = F.release();
    return ER_OK;
  });
}

extern "C" er_status er_folder_desc(const er_folder* f, er_scene_desc* out) {
  if (!f || !out) return fail(ER_ERR_INVALID_ARG, "NULL argument");
  *out = f->d;
  return ER_OK;
}

extern "C" er_status er_folder_free(er_folder* f) {
  delete f;
  return ER_OK;
}

extern "C" er_status er_scene_load(const char* dir_c, const er_scene_opts* opts, er_scene** out) {
  return guarded("er_scene_load", [&]() -> er_status {
    if (out) *out = nullptr;
    if (!dir_c || !out) return fail(ER_ERR_INVALID_ARG, "NULL argument");
    er_folder F;
    er_status st = read_folder(dir_c, &F);
    if (st != ER_OK) return st;
    return er_scene_create(&F.d, opts, out);
  });
}
