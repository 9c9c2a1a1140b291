// Host-side decoders for ROOT's "L4" compression blocks (step tables written with the LZ4 setting): the LZ4 block
// format (token = literal-length and match-length nibbles, 255-continued lengths, 16-bit little-endian match
// offsets, overlapping copies) and the XXH64 checksum ROOT stores in front of each block.  Both are restated from
// their published specifications (LZ4 Block Format; xxHash XXH64).  Every read and write is bounds-checked: a
// malformed block returns a negative status, never touches memory outside the two buffers.
#include <cstdint>
#include <cstring>

#include "crvgpu.h"

namespace {

constexpr uint64_t P1 = 0x9E3779B185EBCA87ull;
constexpr uint64_t P2 = 0xC2B2AE3D27D4EB4Full;
constexpr uint64_t P3 = 0x165667B19E3779F9ull;
constexpr uint64_t P4 = 0x85EBCA77C2B2AE63ull;
constexpr uint64_t P5 = 0x27D4EB2F165667C5ull;

inline uint64_t rotl(uint64_t x, int r) { return (x << r) | (x >> (64 - r)); }

inline uint64_t le64(const uint8_t* p) {
  uint64_t v = 0;
  for (int i = 7; i >= 0; --i) v = (v << 8) | p[i];
  return v;
}

inline uint32_t le32(const uint8_t* p) {
  return uint32_t(p[0]) | (uint32_t(p[1]) << 8) | (uint32_t(p[2]) << 16) | (uint32_t(p[3]) << 24);
}

inline uint64_t round1(uint64_t acc, uint64_t in) {
  acc += in * P2;
  acc = rotl(acc, 31);
  return acc * P1;
}

inline uint64_t merge(uint64_t acc, uint64_t v) {
  acc ^= round1(0, v);
  return acc * P1 + P4;
}

}  // namespace

extern "C" uint64_t crv_xxh64(const uint8_t* data, int64_t n, uint64_t seed) {
  const uint8_t* p = data;
  const uint8_t* end = data + (n > 0 ? n : 0);
  uint64_t h;
  if (n >= 32) {
    uint64_t v1 = seed + P1 + P2, v2 = seed + P2, v3 = seed, v4 = seed - P1;
    const uint8_t* limit = end - 32;
    do {
      v1 = round1(v1, le64(p));
      v2 = round1(v2, le64(p + 8));
      v3 = round1(v3, le64(p + 16));
      v4 = round1(v4, le64(p + 24));
      p += 32;
    } while (p <= limit);
    h = rotl(v1, 1) + rotl(v2, 7) + rotl(v3, 12) + rotl(v4, 18);
    h = merge(h, v1);
    h = merge(h, v2);
    h = merge(h, v3);
    h = merge(h, v4);
  } else {
    h = seed + P5;
  }
  h += uint64_t(n > 0 ? n : 0);
  while (end - p >= 8) {
    h ^= round1(0, le64(p));
    h = rotl(h, 27) * P1 + P4;
    p += 8;
  }
  if (end - p >= 4) {
    h ^= uint64_t(le32(p)) * P1;
    h = rotl(h, 23) * P2 + P3;
    p += 4;
  }
  while (p < end) {
    h ^= uint64_t(*p) * P5;
    h = rotl(h, 11) * P1;
    ++p;
  }
  h ^= h >> 33;
  h *= P2;
  h ^= h >> 29;
  h *= P3;
  h ^= h >> 32;
  return h;
}

extern "C" int64_t crv_lz4_block_decompress(const uint8_t* src, int64_t n, uint8_t* dst, int64_t cap) {
  if (!src || !dst || n < 0 || cap < 0) return -1;
  int64_t i = 0, o = 0;
  while (i < n) {
    const uint8_t token = src[i++];
    int64_t lit = token >> 4;
    if (lit == 15) {
      uint8_t b;
      do {
        if (i >= n) return -2;
        b = src[i++];
        lit += b;
      } while (b == 255);
    }
    if (lit > n - i || lit > cap - o) return -3;
    std::memcpy(dst + o, src + i, size_t(lit));
    i += lit;
    o += lit;
    if (i == n) break;                       // the last sequence carries literals only
    if (n - i < 2) return -4;
    const int64_t off = int64_t(src[i]) | (int64_t(src[i + 1]) << 8);
    i += 2;
    if (off == 0 || off > o) return -5;
    int64_t len = (token & 15) + 4;
    if ((token & 15) == 15) {
      uint8_t b;
      do {
        if (i >= n) return -6;
        b = src[i++];
        len += b;
      } while (b == 255);
    }
    if (len > cap - o) return -7;
    const uint8_t* m = dst + o - off;
    for (int64_t k = 0; k < len; ++k) dst[o + k] = m[k];   // overlapping copies repeat the pattern
    o += len;
  }
  return o;
}
