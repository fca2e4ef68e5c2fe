// Runtime of the generated constraint kernels: their launch arguments and the row helpers they
// use. The library compiles each generated kernel at run time with NVRTC and hands it this header
// and field.cuh by name, so nothing here may include a host header.
//
// A generated kernel evaluates one component's constraints at every row of its evaluation domain
// and adds row_res * denom_inv to the accumulation column, as the reference's
// ComponentProver::evaluate_constraint_quotients_on_domain does (crates/prover/src/
// constraint_framework/component.rs:278-416, with SimdDomainEvaluator simd_domain.rs:24-114).
#pragma once
#ifdef __CUDACC_RTC__
typedef unsigned int uint32_t;
typedef int int32_t;
typedef unsigned long long uint64_t;
#endif
#include "field.cuh"

namespace stwo {

// Launch arguments of a generated constraint kernel (passed by value).
struct GenArgs {
  const uint32_t* const* cols;  // column table: interaction 0, then 1, then 2 (device pointers)
  const uint32_t* params;       // 4 words per parameter (a base parameter uses word 0)
  const uint32_t* powers;       // 4 words per constraint: constraint i's random-coefficient power
  const uint32_t* dinv;         // 2^(eval_log - trace_log) bit-reversed vanishing inverses
  uint32_t* acc0;
  uint32_t* acc1;
  uint32_t* acc2;
  uint32_t* acc3;
  uint32_t trace_log, eval_log;
};

// offset_bit_reversed_circle_domain_index (crates/prover/src/core/utils.rs:74-90): the row that
// holds the value `offset` trace steps away from row i of a bit-reversed circle evaluation of
// size 2^eval_log. The step offset * 2^(eval_log - trace_log - 1) is taken modulo half (a power
// of two), so wrapping 32-bit arithmetic gives rem_euclid.
__device__ __forceinline__ uint32_t gen_offset_row(uint32_t i, uint32_t trace_log, uint32_t eval_log, int offset) {
  uint32_t prev = brev(i, eval_log);
  const uint32_t half = 1u << (eval_log - 1);
  const uint32_t mask = half - 1;
  const uint32_t step = (uint32_t)offset << (eval_log - trace_log - 1);
  if (prev < half) prev = (prev + step) & mask;
  else prev = ((prev - step) & mask) + half;
  return brev(prev, eval_log);
}

// x * 2^k mod P for canonical x and 0 <= k < 31: a rotation of the 31-bit word (2^31 = 1 mod P).
// The result is canonical: only x = P would rotate to P, and canonical x is below P.
__device__ __forceinline__ uint32_t gen_mul_pow2(uint32_t x, int k) {
  return k ? (((x << k) | (x >> (31 - k))) & P) : x;
}
__device__ __forceinline__ qm31 gen_param_q(const uint32_t* p, int k) {
  return qm31_from_u32(__ldg(p + 4 * k), __ldg(p + 4 * k + 1), __ldg(p + 4 * k + 2), __ldg(p + 4 * k + 3));
}
__device__ __forceinline__ qm31 gen_q_add_m31(qm31 x, uint32_t a) { x.a.a = m31_add(x.a.a, a); return x; }
__device__ __forceinline__ qm31 gen_q_sub_m31(qm31 x, uint32_t a) { x.a.a = m31_sub(x.a.a, a); return x; }
__device__ __forceinline__ qm31 gen_m31_sub_q(uint32_t a, qm31 x) {
  return {{m31_sub(a, x.a.a), m31_neg(x.a.b)}, {m31_neg(x.b.a), m31_neg(x.b.b)}};
}
__device__ __forceinline__ qm31 gen_q_neg(qm31 x) {
  return {{m31_neg(x.a.a), m31_neg(x.a.b)}, {m31_neg(x.b.a), m31_neg(x.b.b)}};
}
// acc += p * c for a base-field constraint value c, one 64-bit lane per coordinate (each
// product < 2^62; the caller folds every third product).
__device__ __forceinline__ void gen_acc_base(uint64_t acc[4], const uint4& p, uint32_t c) {
  acc[0] += (uint64_t)p.x * c;
  acc[1] += (uint64_t)p.y * c;
  acc[2] += (uint64_t)p.z * c;
  acc[3] += (uint64_t)p.w * c;
}
__device__ __forceinline__ void gen_fold(uint64_t acc[4]) {
#pragma unroll
  for (int j = 0; j < 4; j++) acc[j] = m31_fold64(acc[j]);
}
__device__ __forceinline__ qm31 gen_q_of_u4(const uint4& p) { return qm31_from_u32(p.x, p.y, p.z, p.w); }
// A relation entry sum_i alpha_i v_i - z over n base values, the alpha powers being parameters
// k0 .. k0 + n - 1 and z parameter kz: four 64-bit coordinate sums folded every third product, in
// a loop kept rolled so that a wide entry (96 values) is a few instructions of code, not 96
// inlined QM31 products.
__device__ __forceinline__ qm31 gen_combine(const uint32_t* p, int k0, const uint32_t* v, int n, int kz) {
  uint64_t acc[4] = {0ull, 0ull, 0ull, 0ull};
#pragma unroll 1
  for (int i = 0; i < n; i++) {
    const uint32_t* al = p + 4 * (k0 + i);
    gen_acc_base(acc, make_uint4(__ldg(al), __ldg(al + 1), __ldg(al + 2), __ldg(al + 3)), v[i]);
    if (i % 3 == 2) gen_fold(acc);
  }
  gen_fold(acc);
  const qm31 s = qm31_from_u32(m31_reduce64(acc[0]), m31_reduce64(acc[1]), m31_reduce64(acc[2]),
                               m31_reduce64(acc[3]));
  return qm31_sub(s, gen_param_q(p, kz));
}

}  // namespace stwo
