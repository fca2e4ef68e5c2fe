// ORACLE — test infrastructure only (see field.h).
// Poseidon252 Merkle hasher and channel, restated from the reference:
//   Poseidon252MerkleHasher  crates/prover/src/core/vcs/poseidon252_merkle.rs:11-58
//   Poseidon252Channel       crates/prover/src/core/channel/poseidon252.rs:15-126
//   GrindOps<Poseidon252Channel> crates/prover/src/core/backend/simd/grind.rs:65-79
// The hash functions come from the third-party crate starknet-crypto 0.6.2 (over starknet-ff
// 0.3.7's FieldElement), absent from the reference tree. Their published algorithm is restated:
//   field      p = 2^251 + 17 * 2^192 + 1 (the STARK field)
//   Hades      state width 3, 8 full rounds (4 before, 4 after) and 83 partial rounds; each round
//              adds its 3 round constants, applies x^3 to every word (full) or to the last word
//              (partial), then the MDS matrix [[3, 1, 1], [1, -1, 1], [1, 1, -2]]
//   constants  round constant k (k = 3 * round + word) = SHA-256("Hades" || decimal k) read as a
//              big-endian integer, mod p
//   hash(x, y) = Hades([x, y, 2])[0]
//   hash_many  a sponge of rate 2 from [0, 0, 0]: pairs are added to words 0 and 1, each followed
//              by the permutation; a last single value is added to word 0; then 1 is added to
//              word (number of values left over) and a final permutation gives word 0
// Pinned by the reference's own vectors (poseidon252_merkle.rs:72-91, `test_vector`).
#pragma once
#include "field.h"
#include <array>
#include <cstring>
#include <string>
#include <vector>

namespace oracle {

// ---------------------------------------------------------------- SHA-256 (FIPS 180-4)
inline std::array<uint8_t, 32> sha256(const uint8_t* data, size_t len) {
  static const uint32_t K[64] = {
      0x428a2f98, 0x71374491, 0xb5c0fbcf, 0xe9b5dba5, 0x3956c25b, 0x59f111f1, 0x923f82a4, 0xab1c5ed5,
      0xd807aa98, 0x12835b01, 0x243185be, 0x550c7dc3, 0x72be5d74, 0x80deb1fe, 0x9bdc06a7, 0xc19bf174,
      0xe49b69c1, 0xefbe4786, 0x0fc19dc6, 0x240ca1cc, 0x2de92c6f, 0x4a7484aa, 0x5cb0a9dc, 0x76f988da,
      0x983e5152, 0xa831c66d, 0xb00327c8, 0xbf597fc7, 0xc6e00bf3, 0xd5a79147, 0x06ca6351, 0x14292967,
      0x27b70a85, 0x2e1b2138, 0x4d2c6dfc, 0x53380d13, 0x650a7354, 0x766a0abb, 0x81c2c92e, 0x92722c85,
      0xa2bfe8a1, 0xa81a664b, 0xc24b8b70, 0xc76c51a3, 0xd192e819, 0xd6990624, 0xf40e3585, 0x106aa070,
      0x19a4c116, 0x1e376c08, 0x2748774c, 0x34b0bcb5, 0x391c0cb3, 0x4ed8aa4a, 0x5b9cca4f, 0x682e6ff3,
      0x748f82ee, 0x78a5636f, 0x84c87814, 0x8cc70208, 0x90befffa, 0xa4506ceb, 0xbef9a3f7, 0xc67178f2};
  uint32_t h[8] = {0x6a09e667, 0xbb67ae85, 0x3c6ef372, 0xa54ff53a, 0x510e527f, 0x9b05688c, 0x1f83d9ab, 0x5be0cd19};
  std::vector<uint8_t> m(data, data + len);
  m.push_back(0x80);
  while (m.size() % 64 != 56) m.push_back(0);
  const uint64_t bits = (uint64_t)len * 8;
  for (int i = 7; i >= 0; i--) m.push_back((uint8_t)(bits >> (8 * i)));
  auto rotr = [](uint32_t x, int n) { return (x >> n) | (x << (32 - n)); };
  for (size_t off = 0; off < m.size(); off += 64) {
    uint32_t w[64];
    for (int i = 0; i < 16; i++)
      w[i] = (uint32_t)m[off + 4 * i] << 24 | (uint32_t)m[off + 4 * i + 1] << 16 | (uint32_t)m[off + 4 * i + 2] << 8 |
             m[off + 4 * i + 3];
    for (int i = 16; i < 64; i++) {
      uint32_t s0 = rotr(w[i - 15], 7) ^ rotr(w[i - 15], 18) ^ (w[i - 15] >> 3);
      uint32_t s1 = rotr(w[i - 2], 17) ^ rotr(w[i - 2], 19) ^ (w[i - 2] >> 10);
      w[i] = w[i - 16] + s0 + w[i - 7] + s1;
    }
    uint32_t a = h[0], b = h[1], c = h[2], d = h[3], e = h[4], f = h[5], g = h[6], hh = h[7];
    for (int i = 0; i < 64; i++) {
      uint32_t t1 = hh + (rotr(e, 6) ^ rotr(e, 11) ^ rotr(e, 25)) + ((e & f) ^ (~e & g)) + K[i] + w[i];
      uint32_t t2 = (rotr(a, 2) ^ rotr(a, 13) ^ rotr(a, 22)) + ((a & b) ^ (a & c) ^ (b & c));
      hh = g; g = f; f = e; e = d + t1; d = c; c = b; b = a; a = t1 + t2;
    }
    h[0] += a; h[1] += b; h[2] += c; h[3] += d; h[4] += e; h[5] += f; h[6] += g; h[7] += hh;
  }
  std::array<uint8_t, 32> out;
  for (int i = 0; i < 8; i++)
    for (int j = 0; j < 4; j++) out[4 * i + j] = (uint8_t)(h[i] >> (24 - 8 * j));
  return out;
}

// ---------------------------------------------------------------- the STARK field
// Integers as 4 little-endian 64-bit limbs. F252 holds a value in Montgomery form (x * 2^256 mod p).
using U256 = std::array<uint64_t, 4>;
constexpr U256 P252 = {1ull, 0ull, 0ull, 0x0800000000000011ull};

inline bool u256_geq(const U256& a, const U256& b) {
  for (int i = 3; i >= 0; i--)
    if (a[i] != b[i]) return a[i] > b[i];
  return true;
}
inline U256 u256_sub(const U256& a, const U256& b) {
  U256 r;
  unsigned __int128 borrow = 0;
  for (int i = 0; i < 4; i++) {
    unsigned __int128 d = (unsigned __int128)a[i] - b[i] - borrow;
    r[i] = (uint64_t)d;
    borrow = (d >> 64) ? 1 : 0;
  }
  return r;
}
inline U256 u256_add(const U256& a, const U256& b, bool& carry) {
  U256 r;
  unsigned __int128 c = 0;
  for (int i = 0; i < 4; i++) {
    c += (unsigned __int128)a[i] + b[i];
    r[i] = (uint64_t)c;
    c >>= 64;
  }
  carry = c != 0;
  return r;
}

struct F252 {
  U256 m{};  // Montgomery form, canonical (< p)
};

// Montgomery product (CIOS) with R = 2^256; -p^-1 mod 2^64 = 2^64 - 1 because p = 1 mod 2^64.
inline U256 mont_mul(const U256& a, const U256& b) {
  uint64_t t[6] = {0, 0, 0, 0, 0, 0};
  for (int i = 0; i < 4; i++) {
    unsigned __int128 c = 0;
    for (int j = 0; j < 4; j++) {
      c += (unsigned __int128)a[j] * b[i] + t[j];
      t[j] = (uint64_t)c;
      c >>= 64;
    }
    c += t[4];
    t[4] = (uint64_t)c;
    t[5] = (uint64_t)(c >> 64);
    const uint64_t m = t[0] * 0xFFFFFFFFFFFFFFFFull;
    c = (unsigned __int128)m * P252[0] + t[0];
    c >>= 64;
    for (int j = 1; j < 4; j++) {
      c += (unsigned __int128)m * P252[j] + t[j];
      t[j - 1] = (uint64_t)c;
      c >>= 64;
    }
    c += t[4];
    t[3] = (uint64_t)c;
    t[4] = t[5] + (uint64_t)(c >> 64);
  }
  U256 r = {t[0], t[1], t[2], t[3]};
  if (t[4] || u256_geq(r, P252)) r = u256_sub(r, P252);
  return r;
}

inline const U256& r2_mod_p() {
  static const U256 r2 = [] {
    U256 x = {1, 0, 0, 0};
    for (int i = 0; i < 512; i++) {  // 2^512 mod p by doubling
      bool carry;
      x = u256_add(x, x, carry);
      if (carry || u256_geq(x, P252)) x = u256_sub(x, P252);
    }
    return x;
  }();
  return r2;
}
// Any integer below 2^256 (reduced mod p on the way in).
inline F252 f252_from_int(const U256& x) { return F252{mont_mul(x, r2_mod_p())}; }
inline F252 f252_from_u64(uint64_t v) { return f252_from_int(U256{v, 0, 0, 0}); }
inline U256 f252_to_int(const F252& a) { return mont_mul(a.m, U256{1, 0, 0, 0}); }
inline F252 operator+(const F252& a, const F252& b) {
  bool carry;
  U256 r = u256_add(a.m, b.m, carry);
  if (carry || u256_geq(r, P252)) r = u256_sub(r, P252);
  return F252{r};
}
inline F252 operator-(const F252& a, const F252& b) {
  if (u256_geq(a.m, b.m)) return F252{u256_sub(a.m, b.m)};
  bool carry;
  return F252{u256_add(u256_sub(a.m, b.m), P252, carry)};  // wraps back into [0, p)
}
inline F252 operator*(const F252& a, const F252& b) { return F252{mont_mul(a.m, b.m)}; }
inline bool operator==(const F252& a, const F252& b) { return a.m == b.m; }

// 8 little-endian u32 limbs of the canonical integer (the ABI's hash words).
inline void f252_to_words(const F252& a, uint32_t w[8]) {
  U256 x = f252_to_int(a);
  for (int i = 0; i < 4; i++) {
    w[2 * i] = (uint32_t)x[i];
    w[2 * i + 1] = (uint32_t)(x[i] >> 32);
  }
}
inline F252 f252_from_words(const uint32_t w[8]) {
  U256 x;
  for (int i = 0; i < 4; i++) x[i] = (uint64_t)w[2 * i] | ((uint64_t)w[2 * i + 1] << 32);
  return f252_from_int(x);
}

// ---------------------------------------------------------------- Hades / Poseidon
constexpr int HADES_FULL = 8, HADES_PARTIAL = 83;

inline const std::vector<F252>& hades_constants() {
  static const std::vector<F252> ark = [] {
    std::vector<F252> v;
    for (int k = 0; k < 3 * (HADES_FULL + HADES_PARTIAL); k++) {
      std::string s = "Hades" + std::to_string(k);
      auto d = sha256(reinterpret_cast<const uint8_t*>(s.data()), s.size());
      U256 x;
      for (int i = 0; i < 4; i++) {
        uint64_t limb = 0;
        for (int j = 0; j < 8; j++) limb = (limb << 8) | d[8 * (3 - i) + j];
        x[i] = limb;
      }
      v.push_back(f252_from_int(x));
    }
    return v;
  }();
  return ark;
}

inline void hades_permutation(F252 s[3]) {
  const auto& ark = hades_constants();
  for (int r = 0; r < HADES_FULL + HADES_PARTIAL; r++) {
    for (int i = 0; i < 3; i++) s[i] = s[i] + ark[3 * r + i];
    const bool full = r < HADES_FULL / 2 || r >= HADES_FULL / 2 + HADES_PARTIAL;
    for (int i = full ? 0 : 2; i < 3; i++) s[i] = s[i] * s[i] * s[i];
    const F252 a = s[0], b = s[1], c = s[2];
    s[0] = a + a + a + b + c;
    s[1] = a - b + c;
    s[2] = a + b - c - c;
  }
}

inline F252 poseidon_hash(const F252& x, const F252& y) {
  F252 s[3] = {x, y, f252_from_u64(2)};
  hades_permutation(s);
  return s[0];
}

inline F252 poseidon_hash_many(const std::vector<F252>& v) {
  F252 s[3] = {F252{}, F252{}, F252{}};
  size_t i = 0;
  for (; i + 2 <= v.size(); i += 2) {
    s[0] = s[0] + v[i];
    s[1] = s[1] + v[i + 1];
    hades_permutation(s);
  }
  const size_t rem = v.size() - i;
  if (rem == 1) s[0] = s[0] + v[i];
  s[rem] = s[rem] + f252_from_u64(1);
  hades_permutation(s);
  return s[0];
}

// Poseidon252MerkleHasher::hash_node (poseidon252_merkle.rs:17-45): children, then the column
// values packed 8 per felt (value k of a block times 2^(31 (7 - k))), zero-padded.
inline F252 p252_hash_node(const F252* left, const F252* right, const uint32_t* vals, size_t n) {
  std::vector<F252> v;
  if (left) {
    v.push_back(*left);
    v.push_back(*right);
  }
  const F252 shift = f252_from_u64(1ull << 31);
  for (size_t b = 0; b < (n + 7) / 8; b++) {
    F252 w{};
    for (size_t k = 0; k < 8; k++) {
      const size_t idx = 8 * b + k;
      w = w * shift + f252_from_u64(idx < n ? vals[idx] : 0u);
    }
    v.push_back(w);
  }
  return poseidon_hash_many(v);
}

// ---------------------------------------------------------------- channel
struct Poseidon252Channel {
  F252 digest{};
  uint64_t n_sent = 0, n_challenges = 0;
  void update_digest(const F252& d) {
    digest = d;
    n_challenges++;
    n_sent = 0;
  }
  void mix_root(const F252& root) { update_digest(poseidon_hash(digest, root)); }  // Poseidon252MerkleChannel
  void mix_u64(uint64_t v) { update_digest(poseidon_hash(digest, f252_from_u64(v))); }
  void mix_felts(const std::vector<QM31>& felts) {
    const F252 shift = f252_from_u64(1ull << 31);
    std::vector<F252> res = {digest};
    for (size_t i = 0; i < felts.size(); i += 2) {
      F252 cur{};
      for (size_t k = i; k < i + 2 && k < felts.size(); k++) {
        const M31 w[4] = {felts[k].a.a, felts[k].a.b, felts[k].b.a, felts[k].b.b};
        for (auto x : w) cur = cur * shift + f252_from_u64(x.v);
      }
      res.push_back(cur);
    }
    update_digest(poseidon_hash_many(res));
  }
  F252 draw_felt252() {
    F252 r = poseidon_hash(digest, f252_from_u64(n_sent));
    n_sent++;
    return r;
  }
  // Eight 31-bit digits of the drawn felt, lowest first, each reduced mod P.
  std::array<M31, 8> draw_base_felts() {
    U256 cur = f252_to_int(draw_felt252());
    std::array<M31, 8> out;
    for (int k = 0; k < 8; k++) {
      out[k] = M31::reduce(cur[0] & 0x7fffffffull);
      for (int i = 0; i < 4; i++) cur[i] = (cur[i] >> 31) | (i < 3 ? cur[i + 1] << 33 : 0);
    }
    return out;
  }
  QM31 draw_felt() {
    auto f = draw_base_felts();
    return QM31::from_m31(f[0], f[1], f[2], f[3]);
  }
  std::vector<QM31> draw_felts(size_t n) {
    std::vector<QM31> out;
    while (out.size() < n) {
      auto f = draw_base_felts();
      out.push_back(QM31::from_m31(f[0], f[1], f[2], f[3]));
      if (out.size() < n) out.push_back(QM31::from_m31(f[4], f[5], f[6], f[7]));
    }
    return out;
  }
  // poseidon252.rs:59-62: the first 16 bytes of the big-endian encoding read as a little-endian u128.
  uint32_t trailing_zeros() const {
    U256 x = f252_to_int(digest);
    uint8_t be[32];
    for (int i = 0; i < 32; i++) be[i] = (uint8_t)(x[3 - i / 8] >> (56 - 8 * (i % 8)));
    for (int i = 0; i < 16; i++)
      if (be[i]) return 8 * i + (uint32_t)__builtin_ctz(be[i]);
    return 128;
  }
};

// GrindOps<Poseidon252Channel>::grind: the smallest nonce whose mix_u64 leaves >= pow_bits
// trailing zeros.
inline uint64_t p252_grind(const Poseidon252Channel& ch, uint32_t pow_bits) {
  for (uint64_t nonce = 0;; nonce++) {
    Poseidon252Channel c = ch;
    c.mix_u64(nonce);
    if (c.trailing_zeros() >= pow_bits) return nonce;
  }
}

}  // namespace oracle
