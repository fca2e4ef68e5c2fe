// ORACLE — test infrastructure only (see field.h).
// BLAKE2s-256 restated from RFC 7693 (the algorithm of the `blake2 = 0.10.6` crate the
// reference pins, Cargo.lock:183-185), plus the raw compression of
// crates/prover/src/core/vcs/blake2s_ref.rs:168-217 used by Blake2sChannel::mix_u64 and grind.
// Merkle node hashing follows crates/prover/src/core/vcs/blake2_merkle.rs:14-30.
#pragma once
#include <cstdint>
#include <cstring>
#include <array>
#include <vector>
#include <string>

namespace oracle {

inline constexpr uint32_t B2S_IV[8] = {0x6A09E667, 0xBB67AE85, 0x3C6EF372, 0xA54FF53A,
                                       0x510E527F, 0x9B05688C, 0x1F83D9AB, 0x5BE0CD19};
inline constexpr uint8_t B2S_SIGMA[10][16] = {
    {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15},
    {14, 10, 4, 8, 9, 15, 13, 6, 1, 12, 0, 2, 11, 7, 5, 3},
    {11, 8, 12, 0, 5, 2, 15, 13, 10, 14, 3, 6, 7, 1, 9, 4},
    {7, 9, 3, 1, 13, 12, 11, 14, 2, 6, 5, 10, 4, 0, 15, 8},
    {9, 0, 5, 7, 2, 4, 10, 15, 14, 1, 11, 12, 6, 8, 3, 13},
    {2, 12, 6, 10, 0, 11, 8, 3, 4, 13, 7, 5, 15, 14, 1, 9},
    {12, 5, 1, 15, 14, 13, 4, 10, 0, 7, 6, 3, 9, 2, 8, 11},
    {13, 11, 7, 14, 12, 1, 3, 9, 5, 0, 15, 4, 8, 6, 2, 10},
    {6, 15, 14, 9, 11, 3, 0, 8, 12, 2, 13, 7, 1, 4, 10, 5},
    {10, 2, 8, 4, 7, 6, 1, 5, 15, 11, 9, 14, 3, 12, 13, 0},
};

inline uint32_t rotr32(uint32_t x, int n) { return (x >> n) | (x << (32 - n)); }

// RFC 7693 section 3.2 compression F; t = (t0, t1), f = (f0, f1).
inline std::array<uint32_t, 8> b2s_compress(const uint32_t h[8], const uint32_t m[16], uint32_t t0,
                                            uint32_t t1, uint32_t f0, uint32_t f1) {
  uint32_t v[16];
  for (int i = 0; i < 8; i++) {
    v[i] = h[i];
    v[i + 8] = B2S_IV[i];
  }
  v[12] ^= t0;
  v[13] ^= t1;
  v[14] ^= f0;
  v[15] ^= f1;
  auto G = [&](int a, int b, int c, int d, uint32_t x, uint32_t y) {
    v[a] = v[a] + v[b] + x;
    v[d] = rotr32(v[d] ^ v[a], 16);
    v[c] = v[c] + v[d];
    v[b] = rotr32(v[b] ^ v[c], 12);
    v[a] = v[a] + v[b] + y;
    v[d] = rotr32(v[d] ^ v[a], 8);
    v[c] = v[c] + v[d];
    v[b] = rotr32(v[b] ^ v[c], 7);
  };
  for (int r = 0; r < 10; r++) {
    const uint8_t* s = B2S_SIGMA[r];
    G(0, 4, 8, 12, m[s[0]], m[s[1]]);
    G(1, 5, 9, 13, m[s[2]], m[s[3]]);
    G(2, 6, 10, 14, m[s[4]], m[s[5]]);
    G(3, 7, 11, 15, m[s[6]], m[s[7]]);
    G(0, 5, 10, 15, m[s[8]], m[s[9]]);
    G(1, 6, 11, 12, m[s[10]], m[s[11]]);
    G(2, 7, 8, 13, m[s[12]], m[s[13]]);
    G(3, 4, 9, 14, m[s[14]], m[s[15]]);
  }
  std::array<uint32_t, 8> out;
  for (int i = 0; i < 8; i++) out[i] = h[i] ^ v[i] ^ v[i + 8];
  return out;
}

struct Hash32 {
  uint8_t b[32] = {0};
  bool operator==(const Hash32& o) const { return std::memcmp(b, o.b, 32) == 0; }
  bool operator!=(const Hash32& o) const { return !(*this == o); }
  std::string hex() const {
    static const char* d = "0123456789abcdef";
    std::string s;
    for (int i = 0; i < 32; i++) {
      s += d[b[i] >> 4];
      s += d[b[i] & 15];
    }
    return s;
  }
  void words(uint32_t w[8]) const { std::memcpy(w, b, 32); }
  static Hash32 from_words(const uint32_t w[8]) {
    Hash32 h;
    std::memcpy(h.b, w, 32);
    return h;
  }
};

// Incremental unkeyed BLAKE2s-256 (RFC 7693 section 3.3).
struct Blake2s {
  uint32_t h[8];
  uint8_t buf[64];
  size_t buflen = 0;
  uint64_t t = 0;
  Blake2s() {
    for (int i = 0; i < 8; i++) h[i] = B2S_IV[i];
    h[0] ^= 0x01010000u ^ 32u;
  }
  void compress_block(const uint8_t* blk, bool last) {
    uint32_t m[16];
    std::memcpy(m, blk, 64);
    auto r = b2s_compress(h, m, (uint32_t)t, (uint32_t)(t >> 32), last ? 0xffffffffu : 0, 0);
    for (int i = 0; i < 8; i++) h[i] = r[i];
  }
  void update(const void* data, size_t len) {
    const uint8_t* p = (const uint8_t*)data;
    while (len) {
      if (buflen == 64) {
        t += 64;
        compress_block(buf, false);
        buflen = 0;
      }
      size_t take = 64 - buflen < len ? 64 - buflen : len;
      std::memcpy(buf + buflen, p, take);
      buflen += take;
      p += take;
      len -= take;
    }
  }
  Hash32 finalize() {
    t += buflen;
    std::memset(buf + buflen, 0, 64 - buflen);
    compress_block(buf, true);
    return Hash32::from_words(h);
  }
  static Hash32 hash(const void* data, size_t len) {
    Blake2s s;
    s.update(data, len);
    return s.finalize();
  }
};

// blake2_merkle.rs:14-30
inline Hash32 hash_node(const Hash32* left, const Hash32* right, const uint32_t* vals, size_t n) {
  Blake2s s;
  if (left) {
    s.update(left->b, 32);
    s.update(right->b, 32);
  }
  for (size_t i = 0; i < n; i++) s.update(&vals[i], 4);  // little-endian u32
  return s.finalize();
}

}  // namespace oracle
