// Blake2sChannel on the device (crates/prover/src/core/channel/blake2s.rs:15-110), for transcript
// steps that would otherwise stop the stream for a host round trip: mixing a Merkle root
// (vcs/blake2_merkle.rs:36-45) or felts, and drawing felts by rejection sampling. One thread runs
// the channel; the byte layouts are those of the host channel, so the host can hand its state to
// the device and take it back at any point.
#pragma once
#include "blake2s.cuh"
#include "field.cuh"

namespace stwo {

struct DevChannel {
  uint32_t digest[8];
  uint32_t n_sent_lo, n_sent_hi;
  uint32_t error;  // non-zero: a draw exhausted its retry bound
  uint32_t pad;
};

// Message schedule of RFC 7693 section 2.7.
__constant__ uint8_t D_B2S_SIGMA[10][16] = {
    {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15}, {14, 10, 4, 8, 9, 15, 13, 6, 1, 12, 0, 2, 11, 7, 5, 3},
    {11, 8, 12, 0, 5, 2, 15, 13, 10, 14, 3, 6, 7, 1, 9, 4}, {7, 9, 3, 1, 13, 12, 11, 14, 2, 6, 5, 10, 4, 0, 15, 8},
    {9, 0, 5, 7, 2, 4, 10, 15, 14, 1, 11, 12, 6, 8, 3, 13}, {2, 12, 6, 10, 0, 11, 8, 3, 4, 13, 7, 5, 15, 14, 1, 9},
    {12, 5, 1, 15, 14, 13, 4, 10, 0, 7, 6, 3, 9, 2, 8, 11}, {13, 11, 7, 14, 12, 1, 3, 9, 5, 0, 15, 4, 8, 6, 2, 10},
    {6, 15, 14, 9, 11, 3, 0, 8, 12, 2, 13, 7, 1, 4, 10, 5}, {10, 2, 8, 4, 7, 6, 1, 5, 15, 11, 9, 14, 3, 12, 13, 0}};

// BLAKE2s compression with the ten rounds as a loop (the unrolled form of blake2s.cuh is for the
// many-hash kernels; on the one channel thread a small instruction footprint matters more).
static __device__ __noinline__ void d_compress_rolled(uint32_t h[8], const uint32_t m[16], uint32_t t0, bool last) {
  uint32_t v[16];
  for (int i = 0; i < 8; i++) v[i] = h[i];
  v[8] = 0x6A09E667u;
  v[9] = 0xBB67AE85u;
  v[10] = 0x3C6EF372u;
  v[11] = 0xA54FF53Au;
  v[12] = 0x510E527Fu ^ t0;
  v[13] = 0x9B05688Cu;
  v[14] = last ? ~0x1F83D9ABu : 0x1F83D9ABu;
  v[15] = 0x5BE0CD19u;
#pragma unroll 1
  for (int r = 0; r < 10; r++) {
    const uint8_t* s = D_B2S_SIGMA[r];
    B2S_G(v[0], v[4], v[8], v[12], m[s[0]], m[s[1]]);
    B2S_G(v[1], v[5], v[9], v[13], m[s[2]], m[s[3]]);
    B2S_G(v[2], v[6], v[10], v[14], m[s[4]], m[s[5]]);
    B2S_G(v[3], v[7], v[11], v[15], m[s[6]], m[s[7]]);
    B2S_G(v[0], v[5], v[10], v[15], m[s[8]], m[s[9]]);
    B2S_G(v[1], v[6], v[11], v[12], m[s[10]], m[s[11]]);
    B2S_G(v[2], v[7], v[8], v[13], m[s[12]], m[s[13]]);
    B2S_G(v[3], v[4], v[9], v[14], m[s[14]], m[s[15]]);
  }
  for (int i = 0; i < 8; i++) h[i] ^= v[i] ^ v[i + 8];
}

// Blake2s-256 of `n` little-endian words (4n bytes), out of line.
static __device__ __noinline__ void d_hash_words(const uint32_t* w, uint32_t n, uint32_t out[8]) {
  uint32_t h[8];
  b2s_init(h);
  uint32_t m[16];
  uint32_t done = 0;
  do {
    const uint32_t take = min(16u, n - done);
    for (int i = 0; i < 16; i++) m[i] = (uint32_t)i < take ? w[done + i] : 0u;
    done += take;
    d_compress_rolled(h, m, done * 4, done == n);
  } while (done < n);
#pragma unroll
  for (int i = 0; i < 8; i++) out[i] = h[i];
}

__device__ inline void d_ch_update(DevChannel* c, const uint32_t d[8]) {
#pragma unroll
  for (int i = 0; i < 8; i++) c->digest[i] = d[i];
  c->n_sent_lo = c->n_sent_hi = 0;
}

// digest <- H(digest || root).
__device__ inline void d_ch_mix_root(DevChannel* c, const uint32_t* root) {
  uint32_t w[16], d[8];
#pragma unroll
  for (int i = 0; i < 8; i++) {
    w[i] = c->digest[i];
    w[8 + i] = root[i];
  }
  d_hash_words(w, 16, d);
  d_ch_update(c, d);
}

// digest <- H(digest || felts), at most 16 felts.
__device__ inline void d_ch_mix_felts(DevChannel* c, const qm31* f, uint32_t n) {
  uint32_t w[8 + 4 * 16], d[8];
  for (int i = 0; i < 8; i++) w[i] = c->digest[i];
  for (uint32_t k = 0; k < n; k++) {
    w[8 + 4 * k] = f[k].a.a;
    w[9 + 4 * k] = f[k].a.b;
    w[10 + 4 * k] = f[k].b.a;
    w[11 + 4 * k] = f[k].b.b;
  }
  d_hash_words(w, 8 + 4 * n, d);
  d_ch_update(c, d);
}

// draw_base_felts: H(digest || n_sent as u64 || zeros) until all eight words are < 2P, each
// reduced mod P. Gives up after 64 draws (probability ~2^-1500), setting c->error.
__device__ inline bool d_ch_draw_base8(DevChannel* c, uint32_t out[8]) {
  for (int attempt = 0; attempt < 64; attempt++) {
    uint32_t w[16];
#pragma unroll
    for (int i = 0; i < 8; i++) w[i] = c->digest[i];
    w[8] = c->n_sent_lo;
    w[9] = c->n_sent_hi;
#pragma unroll
    for (int i = 10; i < 16; i++) w[i] = 0u;
    if (++c->n_sent_lo == 0) c->n_sent_hi++;
    uint32_t h[8];
    d_hash_words(w, 16, h);
    bool ok = true;
#pragma unroll
    for (int i = 0; i < 8; i++) ok = ok && h[i] < 2u * P;
    if (ok) {
#pragma unroll
      for (int i = 0; i < 8; i++) out[i] = h[i] >= P ? h[i] - P : h[i];
      return true;
    }
  }
  c->error = 1u;
  return false;
}

__device__ inline qm31 d_ch_draw_felt(DevChannel* c) {
  uint32_t f[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  d_ch_draw_base8(c, f);
  return qm31_from_u32(f[0], f[1], f[2], f[3]);
}

}  // namespace stwo
