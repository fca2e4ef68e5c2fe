// Host-side Fiat-Shamir transcript of the prover: BLAKE2s-256 (RFC 7693) and the Blake2s channel.
// The transcript is O(#commitments + #samples) hashing of 32-byte digests; it stays on the host
// as in the reference (crates/prover/src/core/channel/blake2s.rs:15-110).
#pragma once
#include <array>
#include <cstdint>
#include <cstring>
#include <vector>
#include "common.cuh"

namespace stwo {

struct Digest {
  uint8_t b[32] = {0};
  void words(uint32_t w[8]) const { std::memcpy(w, b, 32); }
  static Digest from_words(const uint32_t w[8]) {
    Digest d;
    std::memcpy(d.b, w, 32);
    return d;
  }
  bool operator==(const Digest& o) const { return std::memcmp(b, o.b, 32) == 0; }
};

inline uint32_t h_rotr(uint32_t x, int n) { return (x >> n) | (x << (32 - n)); }

// RFC 7693 compression F(h, m, t, f).
inline void h_b2s_compress(uint32_t h[8], const uint32_t m[16], uint64_t t, bool last, bool raw_iv = true) {
  static const uint32_t IV[8] = {0x6A09E667u, 0xBB67AE85u, 0x3C6EF372u, 0xA54FF53Au,
                                 0x510E527Fu, 0x9B05688Cu, 0x1F83D9ABu, 0x5BE0CD19u};
  static const uint8_t S[10][16] = {
      {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15}, {14, 10, 4, 8, 9, 15, 13, 6, 1, 12, 0, 2, 11, 7, 5, 3},
      {11, 8, 12, 0, 5, 2, 15, 13, 10, 14, 3, 6, 7, 1, 9, 4}, {7, 9, 3, 1, 13, 12, 11, 14, 2, 6, 5, 10, 4, 0, 15, 8},
      {9, 0, 5, 7, 2, 4, 10, 15, 14, 1, 11, 12, 6, 8, 3, 13}, {2, 12, 6, 10, 0, 11, 8, 3, 4, 13, 7, 5, 15, 14, 1, 9},
      {12, 5, 1, 15, 14, 13, 4, 10, 0, 7, 6, 3, 9, 2, 8, 11}, {13, 11, 7, 14, 12, 1, 3, 9, 5, 0, 15, 4, 8, 6, 2, 10},
      {6, 15, 14, 9, 11, 3, 0, 8, 12, 2, 13, 7, 1, 4, 10, 5}, {10, 2, 8, 4, 7, 6, 1, 5, 15, 11, 9, 14, 3, 12, 13, 0}};
  (void)raw_iv;
  uint32_t v[16];
  for (int i = 0; i < 8; i++) {
    v[i] = h[i];
    v[i + 8] = IV[i];
  }
  v[12] ^= (uint32_t)t;
  v[13] ^= (uint32_t)(t >> 32);
  if (last) v[14] = ~v[14];
  auto G = [&](int a, int b, int c, int d, uint32_t x, uint32_t y) {
    v[a] = v[a] + v[b] + x;
    v[d] = h_rotr(v[d] ^ v[a], 16);
    v[c] = v[c] + v[d];
    v[b] = h_rotr(v[b] ^ v[c], 12);
    v[a] = v[a] + v[b] + y;
    v[d] = h_rotr(v[d] ^ v[a], 8);
    v[c] = v[c] + v[d];
    v[b] = h_rotr(v[b] ^ v[c], 7);
  };
  for (int r = 0; r < 10; r++) {
    const uint8_t* s = S[r];
    G(0, 4, 8, 12, m[s[0]], m[s[1]]);
    G(1, 5, 9, 13, m[s[2]], m[s[3]]);
    G(2, 6, 10, 14, m[s[4]], m[s[5]]);
    G(3, 7, 11, 15, m[s[6]], m[s[7]]);
    G(0, 5, 10, 15, m[s[8]], m[s[9]]);
    G(1, 6, 11, 12, m[s[10]], m[s[11]]);
    G(2, 7, 8, 13, m[s[12]], m[s[13]]);
    G(3, 4, 9, 14, m[s[14]], m[s[15]]);
  }
  for (int i = 0; i < 8; i++) h[i] ^= v[i] ^ v[i + 8];
}

struct HostBlake2s {
  uint32_t h[8];
  uint8_t buf[64];
  size_t len = 0;
  uint64_t t = 0;
  HostBlake2s() {
    static const uint32_t IV[8] = {0x6A09E667u, 0xBB67AE85u, 0x3C6EF372u, 0xA54FF53Au,
                                   0x510E527Fu, 0x9B05688Cu, 0x1F83D9ABu, 0x5BE0CD19u};
    for (int i = 0; i < 8; i++) h[i] = IV[i];
    h[0] ^= 0x01010020u;
  }
  void update(const void* data, size_t n) {
    const uint8_t* p = (const uint8_t*)data;
    while (n) {
      if (len == 64) {
        t += 64;
        uint32_t m[16];
        std::memcpy(m, buf, 64);
        h_b2s_compress(h, m, t, false);
        len = 0;
      }
      size_t k = std::min(n, 64 - len);
      std::memcpy(buf + len, p, k);
      len += k;
      p += k;
      n -= k;
    }
  }
  Digest finalize() {
    t += len;
    std::memset(buf + len, 0, 64 - len);
    uint32_t m[16];
    std::memcpy(m, buf, 64);
    h_b2s_compress(h, m, t, true);
    return Digest::from_words(h);
  }
};

// Blake2sChannel (channel/blake2s.rs:15-110) with the Merkle root mixing of
// vcs/blake2_merkle.rs:36-45.
struct HostChannel {
  Digest digest;
  uint64_t n_sent = 0;

  void update(const Digest& d) {
    digest = d;
    n_sent = 0;
  }
  void mix_root(const Digest& root) {
    HostBlake2s s;
    s.update(digest.b, 32);
    s.update(root.b, 32);
    update(s.finalize());
  }
  void mix_felts(const std::vector<hq>& felts) {
    HostBlake2s s;
    s.update(digest.b, 32);
    for (const hq& f : felts) s.update(f.v, 16);
    update(s.finalize());
  }
  void mix_u64(uint64_t v) {
    uint32_t h[8], m[16] = {0};
    digest.words(h);
    m[0] = (uint32_t)v;
    m[1] = (uint32_t)(v >> 32);
    h_b2s_compress(h, m, 0, false);
    update(Digest::from_words(h));
  }
  Digest draw_random_bytes() {
    uint8_t in[64] = {0};
    std::memcpy(in, digest.b, 32);
    std::memcpy(in + 32, &n_sent, 8);
    n_sent++;
    HostBlake2s s;
    s.update(in, 64);
    return s.finalize();
  }
  std::array<uint32_t, 8> draw_base_felts() {
    while (true) {
      Digest d = draw_random_bytes();
      uint32_t w[8];
      d.words(w);
      bool ok = true;
      for (int i = 0; i < 8; i++) ok = ok && w[i] < 2 * P;
      if (ok) {
        std::array<uint32_t, 8> r;
        for (int i = 0; i < 8; i++) r[i] = w[i] >= P ? w[i] - P : w[i];
        return r;
      }
    }
  }
  hq draw_felt() {
    auto f = draw_base_felts();
    return hq_make(f[0], f[1], f[2], f[3]);
  }
  uint32_t trailing_zeros() const {
    for (int i = 0; i < 16; i++)
      if (digest.b[i]) return 8 * i + (uint32_t)__builtin_ctz(digest.b[i]);
    return 128;
  }
};

}  // namespace stwo
