// Minimal PNG writer for the path tracer's 8-bit frames (the reference writes its
// frames with lodepng::encode, src/pathtracer.cpp:660-677): RGBA, 8 bits per channel,
// the zlib stream made of stored (uncompressed) deflate blocks, so no compressor is
// needed. CRC-32 (ISO 3309 / PNG) and Adler-32 (RFC 1950) are computed here.
#pragma once

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

namespace pbf_host {

inline uint32_t png_crc(const uint8_t* p, size_t n, uint32_t c = 0xffffffffu) {
  for (size_t i = 0; i < n; ++i) {
    c ^= p[i];
    for (int k = 0; k < 8; ++k) c = (c >> 1) ^ (0xedb88320u & (0u - (c & 1u)));
  }
  return c;
}

// rgba: width * height * 4 bytes, top row first. Returns false on an I/O error.
inline bool write_png(const std::string& path, const uint8_t* rgba, uint32_t width, uint32_t height) {
  std::vector<uint8_t> raw;
  raw.reserve(static_cast<size_t>(height) * (1 + 4 * static_cast<size_t>(width)));
  for (uint32_t y = 0; y < height; ++y) {
    raw.push_back(0);  // filter: none
    raw.insert(raw.end(), rgba + static_cast<size_t>(y) * 4 * width, rgba + static_cast<size_t>(y + 1) * 4 * width);
  }
  std::vector<uint8_t> z = {0x78, 0x01};
  uint32_t a = 1, b = 0;
  for (uint8_t v : raw) {
    a = (a + v) % 65521u;
    b = (b + a) % 65521u;
  }
  size_t off = 0;
  do {
    const size_t len = std::min<size_t>(65535, raw.size() - off);
    const bool last = off + len == raw.size();
    z.push_back(last ? 1 : 0);
    z.push_back(static_cast<uint8_t>(len & 0xff));
    z.push_back(static_cast<uint8_t>(len >> 8));
    z.push_back(static_cast<uint8_t>(~len & 0xff));
    z.push_back(static_cast<uint8_t>((~len >> 8) & 0xff));
    z.insert(z.end(), raw.begin() + off, raw.begin() + off + len);
    off += len;
  } while (off < raw.size());
  const uint32_t adler = (b << 16) | a;
  for (int s = 24; s >= 0; s -= 8) z.push_back(static_cast<uint8_t>(adler >> s));

  std::FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) return false;
  auto be32 = [](std::vector<uint8_t>& o, uint32_t v) {
    for (int s = 24; s >= 0; s -= 8) o.push_back(static_cast<uint8_t>(v >> s));
  };
  auto chunk = [&](const char* type, const std::vector<uint8_t>& body) {
    std::vector<uint8_t> c;
    be32(c, static_cast<uint32_t>(body.size()));
    c.insert(c.end(), type, type + 4);
    c.insert(c.end(), body.begin(), body.end());
    const uint32_t crc = png_crc(c.data() + 4, c.size() - 4) ^ 0xffffffffu;
    be32(c, crc);
    return std::fwrite(c.data(), 1, c.size(), f) == c.size();
  };
  static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};
  bool ok = std::fwrite(sig, 1, 8, f) == 8;
  std::vector<uint8_t> ihdr;
  be32(ihdr, width);
  be32(ihdr, height);
  ihdr.insert(ihdr.end(), {8, 6, 0, 0, 0});  // 8-bit RGBA, deflate, no filter method, no interlace
  ok = ok && chunk("IHDR", ihdr) && chunk("IDAT", z) && chunk("IEND", {});
  return std::fclose(f) == 0 && ok;
}

}  // namespace pbf_host
