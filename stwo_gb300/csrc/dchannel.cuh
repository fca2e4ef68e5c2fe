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

// One BLAKE2s compression, out of line: the channel thread executes a single copy of the
// unrolled rounds, with the additions split onto the FMA pipe (b2s_compress_lat).
static __device__ __noinline__ void d_compress(uint32_t h[8], const uint32_t m[16], uint32_t t0, bool last) {
  uint32_t hh[8], mm[16];
#pragma unroll
  for (int i = 0; i < 8; i++) hh[i] = h[i];
#pragma unroll
  for (int i = 0; i < 16; i++) mm[i] = m[i];
  b2s_compress_lat(hh, mm, t0, last);
#pragma unroll
  for (int i = 0; i < 8; i++) h[i] = hh[i];
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
    d_compress(h, m, done * 4, done == n);
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
