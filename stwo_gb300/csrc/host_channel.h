// Host-side Fiat-Shamir transcript of the prover: BLAKE2s-256 (RFC 7693) and the Blake2s channel.
// The transcript is O(#commitments + #samples) hashing of 32-byte digests; it stays on the host
// as in the reference (crates/prover/src/core/channel/blake2s.rs:15-110).
#pragma once
#include <array>
#include <cstdint>
#include <cstring>
#include <vector>
#include "common.cuh"
#include "blake2s_rounds.cuh"

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
  (void)raw_iv;
  uint32_t v[16];
  for (int i = 0; i < 8; i++) {
    v[i] = h[i];
    v[i + 8] = IV[i];
  }
  v[12] ^= (uint32_t)t;
  v[13] ^= (uint32_t)(t >> 32);
  if (last) v[14] = ~v[14];
  // The ten rounds unrolled with the schedule of blake2s_rounds.cuh (constant message indices).
#define H_B2S_G(a, b, c, d, x, y) \
  do {                            \
    a = a + b + (x);              \
    d = h_rotr(d ^ a, 16);        \
    c = c + d;                    \
    b = h_rotr(b ^ c, 12);        \
    a = a + b + (y);              \
    d = h_rotr(d ^ a, 8);         \
    c = c + d;                    \
    b = h_rotr(b ^ c, 7);         \
  } while (0)
#pragma push_macro("B2S_G")
#undef B2S_G
#define B2S_G(a, b, c, d, x, y) H_B2S_G(a, b, c, d, x, y)
  B2S_ROUNDS(v, m)
#pragma pop_macro("B2S_G")
#undef H_B2S_G
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
