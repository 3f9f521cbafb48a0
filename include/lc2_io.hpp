// lc2_io.hpp -- file outputs of a finished registration, as the reference
// writes them:
//   * NRRD volumes (text header, raw little-endian float32 body)
//     -- Interpolator3D::WriteOut (src/Interpolator/interpolator.cu:681-849);
//   * the moving->fixed matrix as comma-terminated rows, MovingToFixed.mat
//     -- interpolator.cu:839-848;
//   * 8-bit grey PNG of a registered 2D image -- Interpolator2D::WriteOut
//     (interpolator.cu:1500-1530; the reference uses stb_image_write).
// The PNG encoder is written from the PNG and zlib specifications (RFC 2083,
// RFC 1950/1951): stored (uncompressed) deflate blocks, filter type 0,
// CRC-32 and Adler-32 checksums.
#pragma once

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace lc2io {

// "/name" of a path without its extension, as the reference takes it
// (path from the last '/' up to the last '.'); "/<fallback>" when empty.
inline std::string stem_with_slash(const std::string& path, const std::string& fallback) {
  if (path.empty()) return "/" + fallback;
  const size_t slash = path.find_last_of('/');
  const size_t start = (slash == std::string::npos) ? 0 : slash;
  size_t dot = path.find_last_of('.');
  if (dot == std::string::npos || dot < start) dot = path.size();
  std::string s = path.substr(start, dot - start);
  if (s.empty() || s[0] != '/') s = "/" + s;
  return s;
}

struct NrrdHeader {
  int sizes[3];
  float directions[3][3];  // space directions, one vector per axis
  float origin[3];
};

// Header in the reference's layout, then the raw float32 body.
inline void write_nrrd(const std::string& path, const NrrdHeader& h, const float* data) {
  std::ofstream f(path, std::ios::out | std::ios::binary);
  if (!f) throw std::runtime_error("cannot write " + path);
  std::ostringstream o;
  o << "NRRD0004\n"
    << "type: float\n"
    << "dimension: 3\n"
    << "space: scanner-xyz\n"
    << "sizes: " << h.sizes[0] << " " << h.sizes[1] << " " << h.sizes[2] << "\n"
    << "space directions:";
  for (int a = 0; a < 3; ++a)
    o << " (" << h.directions[a][0] << "," << h.directions[a][1] << "," << h.directions[a][2]
      << ")";
  o << "\n"
    << "kinds: domain domain domain\n"
    << "endian: little\n"
    << "encoding: raw\n"
    << "space origin: (" << h.origin[0] << "," << h.origin[1] << "," << h.origin[2] << ")\n\n";
  const std::string head = o.str();
  f.write(head.data(), (std::streamsize)head.size());
  const size_t n = (size_t)h.sizes[0] * h.sizes[1] * h.sizes[2];
  f.write(reinterpret_cast<const char*>(data), (std::streamsize)(n * sizeof(float)));
}

// rows x cols matrix, each value followed by ',' and each row by a newline.
inline void write_matrix(const std::string& path, const float* m, int rows, int cols) {
  std::ofstream f(path);
  if (!f) throw std::runtime_error("cannot write " + path);
  for (int r = 0; r < rows; ++r) {
    for (int c = 0; c < cols; ++c) f << m[r * cols + c] << ",";
    f << "\n";
  }
}

namespace detail {
inline uint32_t crc32(const uint8_t* p, size_t n, uint32_t crc = 0) {
  static uint32_t table[256];
  static bool init = false;
  if (!init) {
    for (uint32_t i = 0; i < 256; ++i) {
      uint32_t c = i;
      for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
      table[i] = c;
    }
    init = true;
  }
  crc = ~crc;
  for (size_t i = 0; i < n; ++i) crc = table[(crc ^ p[i]) & 0xffu] ^ (crc >> 8);
  return ~crc;
}
inline void put32(std::vector<uint8_t>& v, uint32_t x) {
  v.push_back((uint8_t)(x >> 24));
  v.push_back((uint8_t)(x >> 16));
  v.push_back((uint8_t)(x >> 8));
  v.push_back((uint8_t)x);
}
inline void chunk(std::vector<uint8_t>& out, const char* type, const std::vector<uint8_t>& data) {
  put32(out, (uint32_t)data.size());
  std::vector<uint8_t> td(type, type + 4);
  td.insert(td.end(), data.begin(), data.end());
  out.insert(out.end(), td.begin(), td.end());
  put32(out, crc32(td.data(), td.size()));
}
}  // namespace detail

// 8-bit greyscale PNG, rows top to bottom.
inline void write_png_gray8(const std::string& path, int width, int height, const uint8_t* px) {
  using namespace detail;
  std::vector<uint8_t> raw;
  raw.reserve((size_t)(width + 1) * height);
  for (int y = 0; y < height; ++y) {
    raw.push_back(0);  // filter: none
    raw.insert(raw.end(), px + (size_t)y * width, px + (size_t)(y + 1) * width);
  }
  // zlib stream of stored deflate blocks
  std::vector<uint8_t> z{0x78, 0x01};
  size_t pos = 0;
  do {
    const size_t len = std::min<size_t>(65535, raw.size() - pos);
    const bool last = pos + len == raw.size();
    z.push_back(last ? 1 : 0);
    z.push_back((uint8_t)(len & 0xff));
    z.push_back((uint8_t)(len >> 8));
    z.push_back((uint8_t)(~len & 0xff));
    z.push_back((uint8_t)((~len >> 8) & 0xff));
    z.insert(z.end(), raw.begin() + pos, raw.begin() + pos + len);
    pos += len;
  } while (pos < raw.size());
  uint32_t a = 1, b = 0;  // Adler-32
  for (uint8_t c : raw) {
    a = (a + c) % 65521u;
    b = (b + a) % 65521u;
  }
  put32(z, (b << 16) | a);
  std::vector<uint8_t> out{0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};
  std::vector<uint8_t> ihdr;
  put32(ihdr, (uint32_t)width);
  put32(ihdr, (uint32_t)height);
  ihdr.insert(ihdr.end(), {8, 0, 0, 0, 0});  // 8 bit, grey, deflate, filter 0, no interlace
  chunk(out, "IHDR", ihdr);
  chunk(out, "IDAT", z);
  chunk(out, "IEND", {});
  std::ofstream f(path, std::ios::out | std::ios::binary);
  if (!f) throw std::runtime_error("cannot write " + path);
  f.write(reinterpret_cast<const char*>(out.data()), (std::streamsize)out.size());
}

}  // namespace lc2io
