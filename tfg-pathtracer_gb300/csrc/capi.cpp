// Status reporting and the image output step of the C-ABI.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "internal.h"

namespace er {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

er_status fail(er_status s, const std::string& msg) {
  g_last_error = msg;
  return s;
}

er_status cuda_fail(cudaError_t e, const char* what) {
  g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
  cudaGetLastError();
  return e == cudaErrorMemoryAllocation ? ER_ERR_OOM : ER_ERR_CUDA;
}

namespace {

// Ankerl's approximate pow on the high 32 bits of a double (published at
// martin.ankerl.com, 2012), as the reference's output step applies it
// (stb_image.h:127-135, main.cpp:157).  Little-endian word order.
double fast_pow(double a, double b) {
  int64_t bits;
  std::memcpy(&bits, &a, 8);
  int32_t hi = (int32_t)(bits >> 32);
  hi = (int32_t)(b * (double)(hi - 1072632447) + 1072632447);
  bits = (int64_t)((uint64_t)(uint32_t)hi << 32);
  double r;
  std::memcpy(&r, &bits, 8);
  return r;
}

struct CrcTable {
  uint32_t v[256];
  CrcTable() {
    for (uint32_t i = 0; i < 256; i++) {
      uint32_t x = i;
      for (int k = 0; k < 8; k++) x = (x & 1) ? 0xEDB88320u ^ (x >> 1) : x >> 1;
      v[i] = x;
    }
  }
};

uint32_t crc32(const uint8_t* p, size_t n, uint32_t c = 0xFFFFFFFFu) {
  static const CrcTable table;  // initialised once, thread-safe
  for (size_t i = 0; i < n; i++) c = table.v[(c ^ p[i]) & 0xFFu] ^ (c >> 8);
  return c;
}

void be32(std::vector<uint8_t>& v, uint32_t x) {
  v.push_back((uint8_t)(x >> 24)); v.push_back((uint8_t)(x >> 16));
  v.push_back((uint8_t)(x >> 8)); v.push_back((uint8_t)x);
}

void chunk(std::vector<uint8_t>& out, const char* type, const std::vector<uint8_t>& data) {
  be32(out, (uint32_t)data.size());
  size_t start = out.size();
  out.insert(out.end(), type, type + 4);
  out.insert(out.end(), data.begin(), data.end());
  be32(out, crc32(out.data() + start, out.size() - start) ^ 0xFFFFFFFFu);
}

// PNG, 8-bit RGBA, filter 0, zlib stream of stored deflate blocks.
std::vector<uint8_t> encode_png(const uint8_t* rgba, int32_t w, int32_t h) {
  std::vector<uint8_t> raw;
  raw.reserve((size_t)h * (4 * (size_t)w + 1));
  for (int32_t y = 0; y < h; y++) {
    raw.push_back(0);
    raw.insert(raw.end(), rgba + (size_t)y * w * 4, rgba + (size_t)(y + 1) * w * 4);
  }
  std::vector<uint8_t> z = {0x78, 0x01};
  size_t pos = 0;
  do {
    size_t len = std::min<size_t>(65535, raw.size() - pos);
    bool last = pos + len == raw.size();
    z.push_back(last ? 1 : 0);
    z.push_back((uint8_t)len); z.push_back((uint8_t)(len >> 8));
    z.push_back((uint8_t)~len); z.push_back((uint8_t)(~len >> 8));
    z.insert(z.end(), raw.begin() + pos, raw.begin() + pos + len);
    pos += len;
  } while (pos < raw.size());
  uint32_t a = 1, b = 0;
  for (uint8_t c : raw) { a = (a + c) % 65521u; b = (b + a) % 65521u; }
  be32(z, (b << 16) | a);
  std::vector<uint8_t> out = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
  std::vector<uint8_t> ihdr;
  be32(ihdr, (uint32_t)w); be32(ihdr, (uint32_t)h);
  ihdr.push_back(8); ihdr.push_back(6); ihdr.push_back(0); ihdr.push_back(0); ihdr.push_back(0);
  chunk(out, "IHDR", ihdr);
  // a chunk length is 31 bits: the zlib stream goes into consecutive IDAT
  // chunks of at most 1 GiB
  const size_t kChunk = (size_t)1 << 30;
  for (size_t p = 0; p < z.size(); p += kChunk)
    chunk(out, "IDAT", std::vector<uint8_t>(z.begin() + p, z.begin() + std::min(z.size(), p + kChunk)));
  chunk(out, "IEND", {});
  return out;
}

void le32(std::vector<uint8_t>& v, uint32_t x) {
  v.push_back((uint8_t)x); v.push_back((uint8_t)(x >> 8));
  v.push_back((uint8_t)(x >> 16)); v.push_back((uint8_t)(x >> 24));
}

// 24-bit BI_RGB, bottom-up rows padded to 4 bytes.  The input row 0 is the
// top of the image.
std::vector<uint8_t> encode_bmp(const uint8_t* rgba, int32_t w, int32_t h) {
  size_t stride = ((size_t)w * 3 + 3) & ~(size_t)3;
  std::vector<uint8_t> out;
  out.reserve(54 + stride * h);
  out.push_back('B'); out.push_back('M');
  le32(out, (uint32_t)(54 + stride * h)); le32(out, 0); le32(out, 54);
  le32(out, 40); le32(out, (uint32_t)w); le32(out, (uint32_t)h);
  out.push_back(1); out.push_back(0); out.push_back(24); out.push_back(0);
  le32(out, 0); le32(out, (uint32_t)(stride * h)); le32(out, 2835); le32(out, 2835); le32(out, 0); le32(out, 0);
  for (int32_t y = h - 1; y >= 0; y--) {
    size_t row = out.size();
    for (int32_t x = 0; x < w; x++) {
      const uint8_t* p = rgba + ((size_t)y * w + x) * 4;
      out.push_back(p[2]); out.push_back(p[1]); out.push_back(p[0]);
    }
    while (out.size() - row < stride) out.push_back(0);
  }
  return out;
}

}  // namespace
}  // namespace er

using namespace er;

extern "C" const char* er_status_string(er_status s) {
  switch (s) {
    case ER_OK: return "ok";
    case ER_ERR_INVALID_ARG: return "invalid argument";
    case ER_ERR_IO: return "file not found or unreadable";
    case ER_ERR_PARSE: return "malformed input file";
    case ER_ERR_CUDA: return "CUDA runtime error";
    case ER_ERR_OOM: return "out of memory";
    case ER_ERR_DEVICE_CHECK: return "device bounds check failed";
    case ER_ERR_TIMEOUT: return "device wait timed out";
    case ER_ERR_UNSUPPORTED: return "unsupported";
    case ER_ERR_NO_DEVICE: return "no CUDA device";
    default: return "unknown status";
  }
}

extern "C" const char* er_last_error(void) { return g_last_error.c_str(); }

extern "C" int32_t er_abi_version(void) { return ER_ABI_VERSION; }

// main.cpp:99 (clampPixels, PostProcessing.cpp:30-33) then main.cpp:156-158
extern "C" er_status er_encode_ldr(const float* rgba, int32_t width, int32_t height, uint8_t* out) {
  return guarded("er_encode_ldr", [&]() -> er_status {
    if (!rgba || !out || width <= 0 || height <= 0) return fail(ER_ERR_INVALID_ARG, "bad image arguments");
    size_t n = (size_t)width * height * 4;
    for (size_t i = 0; i < n; i++) {
      float v = rgba[i];
      v = v < 0.0f ? 0.0f : v > 1.0f ? 1.0f : v;  // Math.hpp:30-32 clamp, NaN kept
      double e = fast_pow((double)v, 1.0 / 2.2) * 255.0;
      if (!(e >= 0.0 && e < 256.0)) e = 0.0;  // NaN input: defined as 0
      out[i] = (uint8_t)(int32_t)e;
    }
    return ER_OK;
  });
}

extern "C" er_status er_write_image(const char* path, const uint8_t* rgba, int32_t width, int32_t height,
                                    int32_t as_bmp) {
  return guarded("er_write_image", [&]() -> er_status {
    if (!path || !rgba || width <= 0 || height <= 0) return fail(ER_ERR_INVALID_ARG, "bad image arguments");
    if (as_bmp && 54 + (((uint64_t)width * 3 + 3) & ~(uint64_t)3) * (uint64_t)height > 0xFFFFFFFFull)
      return fail(ER_ERR_INVALID_ARG, "image too large for a BMP file (32-bit sizes)");
    std::vector<uint8_t> bytes = as_bmp ? encode_bmp(rgba, width, height) : encode_png(rgba, width, height);
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(ER_ERR_IO, std::string("cannot open ") + path);
    size_t wr = std::fwrite(bytes.data(), 1, bytes.size(), f);
    int rc = std::fclose(f);
    if (wr != bytes.size() || rc != 0) return fail(ER_ERR_IO, std::string("write failed: ") + path);
    return ER_OK;
  });
}
