// Device arithmetic for M31 / CM31 / QM31, always canonical in [0, P).
//
// Semantics follow crates/prover/src/core/fields/{m31,cm31,qm31}.rs of the reference
// (p = 2^31 - 1; CM31 = M31[i]/(i^2 + 1); QM31 = CM31[u]/(u^2 - 2 - i)). Values that feed
// a hash are raw u32 words (backend/simd/blake2s.rs:124-138), so every routine here returns
// the canonical representative: 0 is never stored as P.
#pragma once
#ifndef __CUDACC_RTC__
#include <cstdint>
#endif

namespace stwo {

constexpr uint32_t P = 0x7fffffffu;

__device__ __forceinline__ uint32_t m31_add(uint32_t a, uint32_t b) {
  uint32_t s = a + b;   // [0, 2P-2]
  return min(s, s - P); // s - P wraps above s when s < P
}
__device__ __forceinline__ uint32_t m31_sub(uint32_t a, uint32_t b) {
  uint32_t d = a - b;
  return min(d, d + P);
}
__device__ __forceinline__ uint32_t m31_neg(uint32_t a) { return m31_sub(0u, a); }
__device__ __forceinline__ uint32_t m31_mul(uint32_t a, uint32_t b) {
  uint64_t p = (uint64_t)a * b;                 // < 2^62
  uint32_t lo = (uint32_t)p & P;                // p mod 2^31, in [0, P]
  uint32_t hi = (uint32_t)(p >> 31);            // < P - 2
  uint32_t s = lo + hi;                         // <= 2P - 3
  return min(s, s - P);
}
__device__ __forceinline__ uint32_t m31_sqr(uint32_t a) { return m31_mul(a, a); }
__device__ __forceinline__ uint32_t m31_pow(uint32_t b, uint32_t e) {
  uint32_t r = 1;
  while (e) {
    if (e & 1) r = m31_mul(r, b);
    b = m31_mul(b, b);
    e >>= 1;
  }
  return r;
}
__device__ __forceinline__ uint32_t m31_sqn(uint32_t x, int n) {
#pragma unroll 1
  for (int i = 0; i < n; i++) x = m31_sqr(x);
  return x;
}
// Fermat inverse a^(P-2) with P - 2 = 4 (2^29 - 1) + 1, through the powers a^(2^k - 1) for
// k = 1, 2, 3, 6, 12, 24, 27, 29: 30 squarings and 8 products instead of 30 and 29. The caller
// guarantees a != 0.
__device__ __forceinline__ uint32_t m31_inv(uint32_t a) {
  const uint32_t e1 = a;
  const uint32_t e2 = m31_mul(m31_sqr(e1), e1);
  const uint32_t e3 = m31_mul(m31_sqr(e2), e1);
  const uint32_t e6 = m31_mul(m31_sqn(e3, 3), e3);
  const uint32_t e12 = m31_mul(m31_sqn(e6, 6), e6);
  const uint32_t e24 = m31_mul(m31_sqn(e12, 12), e12);
  const uint32_t e27 = m31_mul(m31_sqn(e24, 3), e3);
  const uint32_t e29 = m31_mul(m31_sqn(e27, 2), e2);
  return m31_mul(m31_sqn(e29, 2), a);
}

struct cm31 { uint32_t a, b; };
struct qm31 { cm31 a, b; };

__device__ __forceinline__ cm31 cm31_add(cm31 x, cm31 y) { return {m31_add(x.a, y.a), m31_add(x.b, y.b)}; }
__device__ __forceinline__ cm31 cm31_sub(cm31 x, cm31 y) { return {m31_sub(x.a, y.a), m31_sub(x.b, y.b)}; }
__device__ __forceinline__ cm31 cm31_mul(cm31 x, cm31 y) {
  return {m31_sub(m31_mul(x.a, y.a), m31_mul(x.b, y.b)), m31_add(m31_mul(x.a, y.b), m31_mul(x.b, y.a))};
}
__device__ __forceinline__ cm31 cm31_mul_m31(cm31 x, uint32_t y) { return {m31_mul(x.a, y), m31_mul(x.b, y)}; }
__device__ __forceinline__ cm31 cm31_inv(cm31 x) {
  uint32_t d = m31_inv(m31_add(m31_sqr(x.a), m31_sqr(x.b)));
  return {m31_mul(x.a, d), m31_mul(m31_neg(x.b), d)};
}
// (2 + i) * x
__device__ __forceinline__ cm31 cm31_mul_r(cm31 x) {
  return {m31_sub(m31_add(x.a, x.a), x.b), m31_add(x.a, m31_add(x.b, x.b))};
}

__device__ __forceinline__ qm31 qm31_add(qm31 x, qm31 y) { return {cm31_add(x.a, y.a), cm31_add(x.b, y.b)}; }
__device__ __forceinline__ qm31 qm31_sub(qm31 x, qm31 y) { return {cm31_sub(x.a, y.a), cm31_sub(x.b, y.b)}; }
// Reductions of 64-bit sums of M31 products. fold: x < 2^64 -> < 2^34, same residue.
__host__ __device__ __forceinline__ unsigned long long m31_fold64(unsigned long long x) { return (x & P) + (x >> 31); }
// x < 2^64 -> the canonical residue.
__host__ __device__ __forceinline__ uint32_t m31_reduce64(unsigned long long x) {
  x = m31_fold64(m31_fold64(x));  // < 2^31 + 2^3
  const uint32_t r = (uint32_t)x;
  return r >= P ? r - P : r;
}

__device__ __forceinline__ qm31 qm31_mul(qm31 x, qm31 y) {
  // (a + bu)(c + du) = (ac + (2+i) bd) + (ad + bc) u
  cm31 ac = cm31_mul(x.a, y.a), bd = cm31_mul(x.b, y.b);
  cm31 ad_bc = cm31_add(cm31_mul(x.a, y.b), cm31_mul(x.b, y.a));
  return {cm31_add(ac, cm31_mul_r(bd)), ad_bc};
}
__device__ __forceinline__ qm31 qm31_mul_m31(qm31 x, uint32_t y) { return {cm31_mul_m31(x.a, y), cm31_mul_m31(x.b, y)}; }
__device__ __forceinline__ qm31 qm31_mul_cm31(qm31 x, cm31 y) { return {cm31_mul(x.a, y), cm31_mul(x.b, y)}; }
__device__ __forceinline__ qm31 qm31_from_u32(uint32_t a, uint32_t b, uint32_t c, uint32_t d) { return {{a, b}, {c, d}}; }
__device__ __forceinline__ qm31 qm31_zero() { return {{0u, 0u}, {0u, 0u}}; }
// x^-1 = cof / norm with norm in M31: cof = (a - bu) * conj(a^2 - (2+i) b^2) and norm = |a^2 -
// (2+i) b^2|^2, so x * cof = norm. Callers with several inverses to take share one M31 inversion
// of the norms' product.
__device__ __forceinline__ void qm31_inv_parts(qm31 x, qm31& cof, uint32_t& norm) {
  const cm31 b2 = cm31_mul(x.b, x.b);
  const cm31 den = cm31_sub(cm31_mul(x.a, x.a), cm31_mul_r(b2));
  const cm31 cd = {den.a, m31_neg(den.b)};
  norm = m31_add(m31_sqr(den.a), m31_sqr(den.b));
  cof = {cm31_mul(x.a, cd), cm31_mul(cm31_sub({0u, 0u}, x.b), cd)};
}
__device__ __forceinline__ qm31 qm31_inv(qm31 x) {
  // (a + bu)^-1 = (a - bu) / (a^2 - (2+i) b^2)  (fields/qm31.rs:121-129)
  cm31 b2 = cm31_mul(x.b, x.b);
  cm31 denom = cm31_sub(cm31_mul(x.a, x.a), cm31_mul_r(b2));
  cm31 di = cm31_inv(denom);
  return {cm31_mul(x.a, di), cm31_mul(cm31_sub({0u, 0u}, x.b), di)};
}

// Circle point over M31.
struct cpoint { uint32_t x, y; };
__device__ __forceinline__ cpoint cpoint_add(cpoint p, cpoint q) {
  return {m31_sub(m31_mul(p.x, q.x), m31_mul(p.y, q.y)), m31_add(m31_mul(p.x, q.y), m31_mul(p.y, q.x))};
}

// Radix-2 butterflies of crates/prover/src/core/fft.rs:5-21.
__device__ __forceinline__ void bfly(uint32_t& v0, uint32_t& v1, uint32_t t) {
  uint32_t tmp = m31_mul(v1, t);
  v1 = m31_sub(v0, tmp);
  v0 = m31_add(v0, tmp);
}
__device__ __forceinline__ void ibfly(uint32_t& v0, uint32_t& v1, uint32_t it) {
  uint32_t tmp = v0;
  v0 = m31_add(tmp, v1);
  v1 = m31_mul(m31_sub(tmp, v1), it);
}

}  // namespace stwo

namespace stwo {
// i * M31_CIRCLE_GEN (crates/prover/src/core/circle.rs:203-206, CirclePointIndex::to_point),
// by double-and-add over the 31 index bits.
__device__ __forceinline__ cpoint index_to_point(uint32_t idx) {
  cpoint r = {1u, 0u};
  cpoint g = {2u, 1268011823u};
  idx &= 0x7fffffffu;
#pragma unroll 1
  while (idx) {
    if (idx & 1) r = cpoint_add(r, g);
    g = cpoint_add(g, g);
    idx >>= 1;
  }
  return r;
}
__device__ __forceinline__ uint32_t brev(uint32_t i, uint32_t log) { return log ? (__brev(i) >> (32 - log)) : 0u; }
}  // namespace stwo
