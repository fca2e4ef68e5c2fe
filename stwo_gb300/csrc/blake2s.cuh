// BLAKE2s compression on the INT pipes: one hash per thread, message words and state in
// registers, rotations as funnel shifts. Algorithm: RFC 7693 (the `blake2 = 0.10.6` crate used
// by crates/prover/src/core/vcs/blake2_merkle.rs:14-30 and the raw compression of
// crates/prover/src/core/vcs/blake2s_ref.rs:168-217).
#pragma once
#include <cstdint>

namespace stwo {

__device__ __forceinline__ uint32_t rotr32(uint32_t x, uint32_t n) { return __funnelshift_r(x, x, n); }

#define B2S_G(a, b, c, d, x, y)   \
  do {                            \
    a = a + b + (x);              \
    d = rotr32(d ^ a, 16);        \
    c = c + d;                    \
    b = rotr32(b ^ c, 12);        \
    a = a + b + (y);              \
    d = rotr32(d ^ a, 8);         \
    c = c + d;                    \
    b = rotr32(b ^ c, 7);         \
  } while (0)

#include "blake2s_rounds.cuh"


// h <- F(h, m, t, f): t = byte counter (low word only; messages here are < 4 GiB), f = final flag.
__device__ __forceinline__ void b2s_compress(uint32_t h[8], const uint32_t m[16], uint32_t t0, bool last) {
  uint32_t v[16];
#pragma unroll
  for (int i = 0; i < 8; i++) v[i] = h[i];
  v[8] = 0x6A09E667u;
  v[9] = 0xBB67AE85u;
  v[10] = 0x3C6EF372u;
  v[11] = 0xA54FF53Au;
  v[12] = 0x510E527Fu ^ t0;
  v[13] = 0x9B05688Cu;
  v[14] = last ? ~0x1F83D9ABu : 0x1F83D9ABu;
  v[15] = 0x5BE0CD19u;
  B2S_ROUNDS(v, m)
#pragma unroll
  for (int i = 0; i < 8; i++) h[i] ^= v[i] ^ v[i + 8];
}

// c + d issued as an integer multiply-add (c = d * one + c, with one == 1 supplied at run time so
// that the compiler cannot fold it): it executes on the FMA pipe, which BLAKE2s otherwise leaves
// idle, and takes load off the integer ALU pipe that bounds the many-hash kernels.
__device__ __forceinline__ uint32_t add_on_fma(uint32_t c, uint32_t d, uint32_t one) {
  uint32_t r;
  asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(d), "r"(one), "r"(c));
  return r;
}

#define B2S_G_FMA(a, b, c, d, x, y) \
  do {                              \
    a = a + b + (x);                \
    d = rotr32(d ^ a, 16);          \
    c = add_on_fma(c, d, one);      \
    b = rotr32(b ^ c, 12);          \
    a = a + b + (y);                \
    d = rotr32(d ^ a, 8);           \
    c = add_on_fma(c, d, one);      \
    b = rotr32(b ^ c, 7);           \
  } while (0)

// b2s_compress with the G additions c + d moved to the FMA pipe (`one` must be 1).
__device__ __forceinline__ void b2s_compress_fma(uint32_t h[8], const uint32_t m[16], uint32_t t0, bool last,
                                                 uint32_t one) {
  uint32_t v[16];
#pragma unroll
  for (int i = 0; i < 8; i++) v[i] = h[i];
  v[8] = 0x6A09E667u;
  v[9] = 0xBB67AE85u;
  v[10] = 0x3C6EF372u;
  v[11] = 0xA54FF53Au;
  v[12] = 0x510E527Fu ^ t0;
  v[13] = 0x9B05688Cu;
  v[14] = last ? ~0x1F83D9ABu : 0x1F83D9ABu;
  v[15] = 0x5BE0CD19u;
#pragma push_macro("B2S_G")
#undef B2S_G
#define B2S_G(a, b, c, d, x, y) B2S_G_FMA(a, b, c, d, x, y)
  B2S_ROUNDS(v, m)
#pragma pop_macro("B2S_G")
#pragma unroll
  for (int i = 0; i < 8; i++) h[i] ^= v[i] ^ v[i + 8];
}

// Every G addition on the FMA pipe (a + b + x as two multiply-adds), for code where one thread or
// one warp hashes alone (tree tops, the transcript): a single warp issues at most one ALU
// instruction every other cycle, so splitting the work between the ALU and FMA pipes shortens a
// compression that no other warp overlaps.
#define B2S_G_LAT(a, b, c, d, x, y)                        \
  do {                                                     \
    a = add_on_fma(add_on_fma(a, b, one), (x), one);       \
    d = rotr32(d ^ a, 16);                                 \
    c = add_on_fma(c, d, one);                             \
    b = rotr32(b ^ c, 12);                                 \
    a = add_on_fma(add_on_fma(a, b, one), (y), one);       \
    d = rotr32(d ^ a, 8);                                  \
    c = add_on_fma(c, d, one);                             \
    b = rotr32(b ^ c, 7);                                  \
  } while (0)

// A run-time 1 for the FMA-pipe additions (a literal would be folded back into plain adds).
static __device__ uint32_t g_b2s_one = 1u;

__device__ __forceinline__ void b2s_compress_lat(uint32_t h[8], const uint32_t m[16], uint32_t t0, bool last) {
  const uint32_t one = g_b2s_one;
  uint32_t v[16];
#pragma unroll
  for (int i = 0; i < 8; i++) v[i] = h[i];
  v[8] = 0x6A09E667u;
  v[9] = 0xBB67AE85u;
  v[10] = 0x3C6EF372u;
  v[11] = 0xA54FF53Au;
  v[12] = 0x510E527Fu ^ t0;
  v[13] = 0x9B05688Cu;
  v[14] = last ? ~0x1F83D9ABu : 0x1F83D9ABu;
  v[15] = 0x5BE0CD19u;
#pragma push_macro("B2S_G")
#undef B2S_G
#define B2S_G(a, b, c, d, x, y) B2S_G_LAT(a, b, c, d, x, y)
  B2S_ROUNDS(v, m)
#pragma pop_macro("B2S_G")
#pragma unroll
  for (int i = 0; i < 8; i++) h[i] ^= v[i] ^ v[i + 8];
}

// Initial chaining value of unkeyed BLAKE2s-256: IV[0] ^ 0x01010020.
__device__ __forceinline__ void b2s_init(uint32_t h[8]) {
  h[0] = 0x6A09E667u ^ 0x01010020u;
  h[1] = 0xBB67AE85u;
  h[2] = 0x3C6EF372u;
  h[3] = 0xA54FF53Au;
  h[4] = 0x510E527Fu;
  h[5] = 0x9B05688Cu;
  h[6] = 0x1F83D9ABu;
  h[7] = 0x5BE0CD19u;
}

}  // namespace stwo
