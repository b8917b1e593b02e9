// st_rawio.cpp -- raw HDR frame I/O (save_raw / load_raw, src/rawio.jl:18-42):
// a linear, unclamped 32-bit float RGB TIFF in display orientation plus a
// TOML sidecar <path>.toml recording how the frame was traced.
//
// Display orientation is the reference's rotr90 of the (width, height) frame:
// TIFF pixel (row r, column c) holds frame pixel (width - 1 - c, r).
//
// The TIFF is baseline, little-endian, uncompressed, one chunky strip:
// ImageWidth, ImageLength, BitsPerSample 32/32/32, Compression 1,
// PhotometricInterpretation 2 (RGB), StripOffsets, SamplesPerPixel 3,
// RowsPerStrip, StripByteCounts, PlanarConfiguration 1, SampleFormat 3/3/3
// (IEEE float).  The reader accepts any uncompressed chunky 3-sample float32
// TIFF with strips, in either byte order.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

#include "../../include/spacetime_gb300.h"

namespace {

void put16(std::vector<uint8_t>& b, uint16_t v) { b.push_back(v & 0xff); b.push_back(v >> 8); }
void put32(std::vector<uint8_t>& b, uint32_t v) {
  for (int k = 0; k < 4; ++k) b.push_back((v >> (8 * k)) & 0xff);
}

struct Reader {
  const std::vector<uint8_t>& d;
  bool le;
  bool ok = true;
  uint16_t u16(size_t o) {
    if (o + 2 > d.size()) { ok = false; return 0; }
    return le ? (uint16_t)(d[o] | d[o + 1] << 8) : (uint16_t)(d[o] << 8 | d[o + 1]);
  }
  uint32_t u32(size_t o) {
    if (o + 4 > d.size()) { ok = false; return 0; }
    return le ? (uint32_t)d[o] | (uint32_t)d[o + 1] << 8 | (uint32_t)d[o + 2] << 16 | (uint32_t)d[o + 3] << 24
              : (uint32_t)d[o] << 24 | (uint32_t)d[o + 1] << 16 | (uint32_t)d[o + 2] << 8 | (uint32_t)d[o + 3];
  }
};

struct TiffInfo {
  uint32_t width = 0, height = 0, rows_per_strip = 0;
  uint32_t bits = 0, samples = 0, compression = 1, planar = 1, format = 1;
  std::vector<uint32_t> offsets, counts;
};

bool read_file(const char* path, std::vector<uint8_t>* out) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  std::fseek(f, 0, SEEK_END);
  const long n = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  if (n <= 0) { std::fclose(f); return false; }
  out->resize((size_t)n);
  const size_t got = std::fread(out->data(), 1, (size_t)n, f);
  std::fclose(f);
  return got == (size_t)n;
}

// Tag value(s): SHORT or LONG, inline when they fit in 4 bytes.
std::vector<uint32_t> tag_values(Reader& R, size_t entry) {
  const uint16_t type = R.u16(entry + 2);
  const uint32_t count = R.u32(entry + 4);
  const size_t sz = type == 3 ? 2 : (type == 4 ? 4 : 0);
  std::vector<uint32_t> v;
  if (!sz || count > (1u << 24)) { R.ok = false; return v; }
  const size_t base = count * sz <= 4 ? entry + 8 : R.u32(entry + 8);
  for (uint32_t k = 0; k < count && R.ok; ++k) v.push_back(sz == 2 ? R.u16(base + 2 * k) : R.u32(base + 4 * k));
  return v;
}

int parse(const std::vector<uint8_t>& d, TiffInfo* t) {
  if (d.size() < 8) return ST_EINVAL;
  const bool le = d[0] == 'I' && d[1] == 'I';
  if (!le && !(d[0] == 'M' && d[1] == 'M')) return ST_EINVAL;
  Reader R{d, le};
  if (R.u16(2) != 42) return ST_EINVAL;
  const size_t ifd = R.u32(4);
  const uint16_t n = R.u16(ifd);
  for (uint16_t e = 0; e < n && R.ok; ++e) {
    const size_t entry = ifd + 2 + 12 * (size_t)e;
    const uint16_t tag = R.u16(entry);
    const std::vector<uint32_t> v = tag_values(R, entry);
    if (!R.ok || v.empty()) break;
    switch (tag) {
      case 256: t->width = v[0]; break;
      case 257: t->height = v[0]; break;
      case 258: t->bits = v[0]; for (uint32_t b : v) if (b != v[0]) return ST_EUNSUPPORTED; break;
      case 259: t->compression = v[0]; break;
      case 273: t->offsets = v; break;
      case 277: t->samples = v[0]; break;
      case 278: t->rows_per_strip = v[0]; break;
      case 279: t->counts = v; break;
      case 284: t->planar = v[0]; break;
      case 339: t->format = v[0]; break;
      default: break;
    }
  }
  if (!R.ok || !t->width || !t->height) return ST_EINVAL;
  if (t->bits != 32 || t->samples != 3 || t->compression != 1 || t->planar != 1 || t->format != 3 ||
      t->offsets.empty() || t->offsets.size() != t->counts.size())
    return ST_EUNSUPPORTED;
  if (!t->rows_per_strip) t->rows_per_strip = t->height;
  return ST_OK;
}

}  // namespace

extern "C" {

int st_save_raw(const char* path, const float* rgb, int width, int height, const char* metadata_toml) {
  if (!path || !rgb || width <= 0 || height <= 0 || (long long)width * height > (1ll << 28)) return ST_EINVAL;
  const uint32_t W = (uint32_t)width, H = (uint32_t)height;
  const uint32_t nbytes = W * H * 12u;
  std::vector<uint8_t> b;
  b.reserve(nbytes + 512);
  // header; IFD right after it, then the BitsPerSample / SampleFormat arrays, then the pixels
  b.push_back('I'); b.push_back('I'); put16(b, 42); put32(b, 8);
  const uint16_t ntags = 11;
  const uint32_t ifd_end = 8 + 2 + 12 * ntags + 4;
  const uint32_t bps_off = ifd_end, fmt_off = ifd_end + 6, data_off = ifd_end + 12 + 4;  // 16-aligned-ish
  put16(b, ntags);
  auto tag = [&](uint16_t t, uint16_t type, uint32_t count, uint32_t value) {
    put16(b, t); put16(b, type); put32(b, count);
    if (type == 3 && count == 1) { put16(b, (uint16_t)value); put16(b, 0); }
    else put32(b, value);
  };
  tag(256, 4, 1, W);
  tag(257, 4, 1, H);
  tag(258, 3, 3, bps_off);
  tag(259, 3, 1, 1);
  tag(262, 3, 1, 2);
  tag(273, 4, 1, data_off);
  tag(277, 3, 1, 3);
  tag(278, 4, 1, H);
  tag(279, 4, 1, nbytes);
  tag(284, 3, 1, 1);
  tag(339, 3, 3, fmt_off);
  put32(b, 0);  // no next IFD
  put16(b, 32); put16(b, 32); put16(b, 32);
  put16(b, 3); put16(b, 3); put16(b, 3);
  while (b.size() < data_off) b.push_back(0);
  b.resize(data_off + (size_t)nbytes);
  uint8_t* px = b.data() + data_off;
  for (uint32_t r = 0; r < H; ++r)
    for (uint32_t c = 0; c < W; ++c) {
      const float* s = rgb + 3 * ((size_t)(W - 1 - c) + (size_t)W * r);
      for (int k = 0; k < 3; ++k) {
        uint32_t u;
        std::memcpy(&u, s + k, 4);
        uint8_t* o = px + 12 * ((size_t)r * W + c) + 4 * k;
        o[0] = u & 0xff; o[1] = (u >> 8) & 0xff; o[2] = (u >> 16) & 0xff; o[3] = u >> 24;
      }
    }
  FILE* f = std::fopen(path, "wb");
  if (!f) return ST_EINVAL;
  const bool ok = std::fwrite(b.data(), 1, b.size(), f) == b.size();
  if (std::fclose(f) != 0 || !ok) return ST_EINVAL;
  // sidecar: the caller's metadata, then the format and the save time
  const std::string side = std::string(path) + ".toml";
  FILE* g = std::fopen(side.c_str(), "w");
  if (!g) return ST_EINVAL;
  char stamp[32];
  const std::time_t now = std::time(nullptr);
  std::tm tmv{};
  localtime_r(&now, &tmv);
  std::strftime(stamp, sizeof stamp, "%Y-%m-%dT%H:%M:%S", &tmv);
  if (metadata_toml && *metadata_toml) {
    std::fputs(metadata_toml, g);
    const size_t L = std::strlen(metadata_toml);
    if (metadata_toml[L - 1] != '\n') std::fputc('\n', g);
  }
  std::fprintf(g, "format = \"SpaceTime raw v1: linear Float32 RGB, display orientation\"\n");
  std::fprintf(g, "saved_at = \"%s\"\n", stamp);
  return std::fclose(g) == 0 ? ST_OK : ST_EINVAL;
}

int st_load_raw_size(const char* path, int* width, int* height) {
  if (!path || !width || !height) return ST_EINVAL;
  std::vector<uint8_t> d;
  if (!read_file(path, &d)) return ST_EINVAL;
  TiffInfo t;
  const int rc = parse(d, &t);
  if (rc != ST_OK) return rc;
  // the frame is the TIFF turned back (rotl90): width = TIFF columns
  *width = (int)t.width;
  *height = (int)t.height;
  return ST_OK;
}

int st_load_raw(const char* path, float* rgb, int width, int height) {
  if (!path || !rgb || width <= 0 || height <= 0) return ST_EINVAL;
  std::vector<uint8_t> d;
  if (!read_file(path, &d)) return ST_EINVAL;
  TiffInfo t;
  int rc = parse(d, &t);
  if (rc != ST_OK) return rc;
  if ((int)t.width != width || (int)t.height != height) return ST_EINVAL;
  const bool le = d[0] == 'I';
  const size_t row_bytes = (size_t)t.width * 12;
  for (uint32_t r = 0; r < t.height; ++r) {
    const uint32_t s = r / t.rows_per_strip, rin = r % t.rows_per_strip;
    if (s >= t.offsets.size()) return ST_EINVAL;
    const size_t o = (size_t)t.offsets[s] + rin * row_bytes;
    if (o + row_bytes > d.size() || (size_t)(rin + 1) * row_bytes > t.counts[s]) return ST_EINVAL;
    for (uint32_t c = 0; c < t.width; ++c)
      for (int k = 0; k < 3; ++k) {
        const uint8_t* q = d.data() + o + 12 * (size_t)c + 4 * k;
        const uint32_t u = le ? (uint32_t)q[0] | (uint32_t)q[1] << 8 | (uint32_t)q[2] << 16 | (uint32_t)q[3] << 24
                              : (uint32_t)q[0] << 24 | (uint32_t)q[1] << 16 | (uint32_t)q[2] << 8 | (uint32_t)q[3];
        float v;
        std::memcpy(&v, &u, 4);
        rgb[3 * ((size_t)(t.width - 1 - c) + (size_t)t.width * r) + k] = v;
      }
  }
  return ST_OK;
}

}  // extern "C"
