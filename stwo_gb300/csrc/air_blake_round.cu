// Blake2s round AIR on the device: the reference's BlakeRoundComponent
// (crates/prover/src/examples/blake/round/{constraints,gen}.rs) proved on its own, with the
// statement mixing of the Blake example (blake/air.rs:83-183): the log size before the trace
// commitment, the round's claimed LogUp sum before the interaction commitment. Relation elements
// are drawn in AllElements order without the scheduler's: RoundElements (96 values), then the
// five 3-value XOR relations (blake/mod.rs:55-121).
//
// Kernels (one thread per row):
//   k_br_trace        the 384 trace columns of one BLAKE2s round (gen.rs:75-204)
//   k_br_interaction_rows / _warps
//                     64 cumulative columns of paired XOR lookups and one of the Round relation
//                     (gen.rs:237-280), one thread per row or one warp per G-function; the row's
//                     round is recomputed from its inputs, so no lookup columns are stored
//   k_br_composition  the 64 carry constraints and 65 LogUp constraints (constraints.rs:22-206,
//                     finalize_logup_in_pairs) with random-coefficient accumulation, times 1/Z
#include "common.cuh"
#include "prover.cuh"

namespace stwo {

constexpr int BR_ST = 16;
constexpr int BR_COLS = 384;            // 2 * (16 + 16) + 8 G-functions * 40
constexpr int BR_ROUND_FELTS = 96;      // (input state, output state, message) as (low, high) halves
constexpr int BR_XOR_PAIRS = 64;        // 128 xor lookups per row, in pairs
constexpr int BR_INTER_SECURE = BR_XOR_PAIRS + 1;
constexpr int BR_N_CONSTRAINTS = 64 + BR_INTER_SECURE;  // 129

// Relation elements: z and alpha powers per relation (XOR widths 12, 9, 8, 7, 4, then Round).
struct BrElements {
  uint32_t xz[5][4];
  uint32_t xa[5][3][4];
  uint32_t rz[4];
  uint32_t ra[BR_ROUND_FELTS][4];
};

__device__ __forceinline__ int br_xor_index(uint32_t w) { return w == 12 ? 0 : w == 9 ? 1 : w == 8 ? 2 : w == 7 ? 3 : 4; }
// Four words of the relation elements (a block's shared-memory copy; plain loads, valid for any
// address space).
__device__ __forceinline__ qm31 br_q(const uint32_t* v) { return qm31_from_u32(v[0], v[1], v[2], v[3]); }

// The block's copy of the relation elements (1,856 bytes), read by every row's combines.
__device__ __forceinline__ void br_stage_elements(const BrElements* __restrict__ e, BrElements* s) {
  const uint32_t* src = reinterpret_cast<const uint32_t*>(e);
  uint32_t* dst = reinterpret_cast<uint32_t*>(s);
  for (uint32_t i = threadIdx.x; i < sizeof(BrElements) / 4; i += blockDim.x) dst[i] = __ldg(src + i);
}

// LookupElements::combine for one XOR lookup: a + alpha b + alpha^2 c - z (logup.rs:95-113).
// The elements reach the kernels through device memory, staged into shared memory per block: a
// kernel parameter of this size, addressed by index, would be copied to each thread's stack.
__device__ __forceinline__ qm31 br_xor_combine(const BrElements* e, uint32_t w, uint32_t a, uint32_t b, uint32_t c) {
  const int k = br_xor_index(w);
  qm31 acc = qm31_add(qm31_add(qm31_mul_m31(br_q(e->xa[k][0]), a), qm31_mul_m31(br_q(e->xa[k][1]), b)),
                      qm31_mul_m31(br_q(e->xa[k][2]), c));
  return qm31_sub(acc, br_q(e->xz[k]));
}

// Word i of row r's round inputs: the 16 state words then the 16 message words, or the
// reference test's inputs (v_i = i, m_i = i + 1) when `in` is NULL.
__device__ __forceinline__ uint32_t br_input(const uint32_t* in, uint32_t r, uint32_t i) {
  return in ? __ldg(in + (size_t)r * 32 + i) : (i < BR_ST ? i : i - BR_ST + 1);
}

// The state is kept as four rows of four words (v[0..3] the a's, v[4..7] the b's, v[8..11] the
// c's, v[12..15] the d's), and every G works on column 0: after each G all rows rotate left by
// one, and between the column and the diagonal half the rows are diagonalised (row k rotated
// left by k). The eight G-functions then run as one loop body with fixed register operands; the
// order of G calls, and so of trace columns and lookups, is the reference's
// (round/constraints.rs:25-64).
template <class T>
__device__ __forceinline__ void br_rotate_rows(T v[BR_ST]) {
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const T t = v[4 * k];
    v[4 * k] = v[4 * k + 1];
    v[4 * k + 1] = v[4 * k + 2];
    v[4 * k + 2] = v[4 * k + 3];
    v[4 * k + 3] = t;
  }
}
template <class T>
__device__ __forceinline__ void br_rotate_row(T v[BR_ST], int k, int by) {
  T t[4];
#pragma unroll
  for (int j = 0; j < 4; j++) t[j] = v[4 * k + ((j + by) & 3)];
#pragma unroll
  for (int j = 0; j < 4; j++) v[4 * k + j] = t[j];
}
template <class T>
__device__ __forceinline__ void br_diagonalize(T v[BR_ST]) {
  br_rotate_row(v, 1, 1);
  br_rotate_row(v, 2, 2);
  br_rotate_row(v, 3, 3);
}
template <class T>
__device__ __forceinline__ void br_undiagonalize(T v[BR_ST]) {
  br_rotate_row(v, 1, 3);
  br_rotate_row(v, 2, 2);
  br_rotate_row(v, 3, 1);
}

// ------------------------------------------------------------------------------------------ trace
// One row of TraceGeneratorRow::generate from the G-functions on: the visitor gets every trace
// felt in column order and every XOR lookup (w, a, b, a ^ b) in lookup order; msg(i) is message
// word i.
template <class V, class M>
__device__ __forceinline__ void br_round(uint32_t v[BR_ST], M msg, V& vis) {
  auto u32 = [&](uint32_t x) {
    vis.felt(x & 0xffffu);
    vis.felt(x >> 16);
  };
  auto split = [&](uint32_t a, uint32_t rr, uint32_t& l, uint32_t& h) {
    h = a >> rr;
    l = a & ((1u << rr) - 1);
    vis.felt(h);
  };
  auto xor1 = [&](uint32_t w, uint32_t a, uint32_t b) {
    const uint32_t c = a ^ b;
    vis.felt(c);
    vis.lookup(w, a, b, c);
  };
  // xor_rotr_u32 (rr < 16) and xor_rotr16_u32 (both halves split at 8, all four lookups of width 8).
  auto xor_rotr = [&](uint32_t a, uint32_t b, uint32_t rr) {
    const uint32_t c = a ^ b;
    const uint32_t sp = rr == 16 ? 8 : rr;
    uint32_t all, alh, ahl, ahh, bll, blh, bhl, bhh;
    split(a & 0xffffu, sp, all, alh);
    split(a >> 16, sp, ahl, ahh);
    split(b & 0xffffu, sp, bll, blh);
    split(b >> 16, sp, bhl, bhh);
    xor1(sp, all, bll);
    xor1(sp, ahl, bhl);
    xor1(16 - sp, alh, blh);
    xor1(16 - sp, ahh, bhh);
    return (c >> rr) | (c << (32 - rr));
  };
#pragma unroll 1
  for (int it = 0; it < 8; it++) {
    if (it == 4) br_diagonalize(v);
    uint32_t a = v[0], b = v[4], c = v[8], d = v[12];
    a = a + b + msg(2 * it);
    u32(a);
    d = xor_rotr(a, d, 16);
    c = c + d;
    u32(c);
    b = xor_rotr(b, c, 12);
    a = a + b + msg(2 * it + 1);
    u32(a);
    d = xor_rotr(a, d, 8);
    c = c + d;
    u32(c);
    b = xor_rotr(b, c, 7);
    v[0] = a;
    v[4] = b;
    v[8] = c;
    v[12] = d;
    br_rotate_rows(v);
  }
  br_undiagonalize(v);
}

struct BrTraceWriter {
  uint32_t* trace;
  size_t n;
  uint32_t r;
  uint32_t col = 0;
  __device__ void felt(uint32_t x) { trace[(size_t)col++ * n + r] = x; }
  __device__ void lookup(uint32_t, uint32_t, uint32_t, uint32_t) {}
};

// inputs: per row 16 state words then 16 message words, or NULL for the reference test's inputs.
__global__ void __launch_bounds__(128) k_br_trace(uint32_t n_rows, const uint32_t* __restrict__ inputs,
                                                  uint32_t* __restrict__ trace) {
  pdl_enter();
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_rows) return;
  uint32_t v[BR_ST];
  BrTraceWriter w{trace, n_rows, r};
#pragma unroll
  for (int i = 0; i < BR_ST; i++) {
    v[i] = br_input(inputs, r, i);
    w.felt(v[i] & 0xffffu);
    w.felt(v[i] >> 16);
  }
#pragma unroll
  for (int i = 0; i < BR_ST; i++) {
    const uint32_t m = br_input(inputs, r, BR_ST + i);
    w.felt(m & 0xffffu);
    w.felt(m >> 16);
  }
  br_round(v, [&](int i) { return br_input(inputs, r, BR_ST + i); }, w);
}

// ------------------------------------------------------------------------------------ interaction
// Each XOR pair contributes 1/p0 + 1/p1 = (p0 + p1) / (p0 p1) to the next cumulative column; the
// pairs come in the evaluator's lookup order, eight per G-function (two per xor_rotr call), so
// G-function g owns columns 8g .. 8g + 7.
//
// A fraction is taken in cofactor form: g = (p0 + p1) * cof and the M31 norm n of p0 p1, with
// (p0 p1) * cof = n (qm31_inv_parts), so it equals g / n. The four pairs of half a G-function
// share one M31 inversion of their norms' product (Montgomery's batch trick in the base field),
// which removes three of every four M31 inversions, the bulk of the kernel's instructions. The
// denominators are z minus a random combination and nonzero except with negligible probability,
// as the reference's batch inversion of the same columns (constraint_framework/logup.rs:224) also
// assumes.
//
// Two schedules give the same columns. With many rows, one thread per row (k_br_interaction_rows)
// fills the GPU and does the least work. With few rows, each thread's chain of dependent
// inversions would set the kernel's time, and one warp per G-function (k_br_interaction_warps)
// divides that chain by eight.
constexpr uint32_t BI_ROWS = 32;
constexpr uint32_t BI_WARPS_MAX_LOG = 15;  // k_br_interaction_warps up to 2^15 rows

__device__ __forceinline__ void br_pair_parts(const qm31& p0, const qm31& p1, qm31& g, uint32_t& n) {
  qm31 cof;
  qm31_inv_parts(qm31_mul(p0, p1), cof, n);
  g = qm31_mul(qm31_add(p0, p1), cof);
}

// The two pairs of one xor_rotr_u32 (RR < 16) or xor_rotr16_u32 (RR == 16, halves split at 8):
// lookups (ll, hl) and (lh, hh), into slots K and K + 1. Returns the rotated xor.
template <int K, uint32_t RR>
__device__ __forceinline__ uint32_t br_xr_parts(const BrElements* e, uint32_t a, uint32_t b, qm31 g[4], uint32_t n[4]) {
  constexpr uint32_t SP = RR == 16 ? 8 : RR;
  constexpr uint32_t M = (1u << SP) - 1;
  const uint32_t al = a & 0xffffu, ah = a >> 16, bl = b & 0xffffu, bh = b >> 16;
  const uint32_t all = al & M, alh = al >> SP, ahl = ah & M, ahh = ah >> SP;
  const uint32_t bll = bl & M, blh = bl >> SP, bhl = bh & M, bhh = bh >> SP;
  br_pair_parts(br_xor_combine(e, SP, all, bll, all ^ bll), br_xor_combine(e, SP, ahl, bhl, ahl ^ bhl), g[K], n[K]);
  br_pair_parts(br_xor_combine(e, 16 - SP, alh, blh, alh ^ blh), br_xor_combine(e, 16 - SP, ahh, bhh, ahh ^ bhh),
                g[K + 1], n[K + 1]);
  const uint32_t c = a ^ b;
  return (c >> RR) | (c << (32 - RR));
}

// Half a G-function (a += b + m, then the xor_rotr calls with rotations R1 and R2) and its four
// pair fractions, in lookup order.
template <uint32_t R1, uint32_t R2>
__device__ __forceinline__ void br_half_g(const BrElements* e, uint32_t& a, uint32_t& b, uint32_t& c, uint32_t& d,
                                          uint32_t m, qm31 f[4]) {
  qm31 g[4];
  uint32_t n[4];
  a = a + b + m;
  d = br_xr_parts<0, R1>(e, a, d, g, n);
  c = c + d;
  b = br_xr_parts<2, R2>(e, b, c, g, n);
  const uint32_t n01 = m31_mul(n[0], n[1]);
  const uint32_t n012 = m31_mul(n01, n[2]);
  uint32_t inv = m31_inv(m31_mul(n012, n[3]));  // 1 / (n0 n1 n2 n3)
  const uint32_t i3 = m31_mul(inv, n012);
  inv = m31_mul(inv, n[3]);  // 1 / (n0 n1 n2)
  const uint32_t i2 = m31_mul(inv, n01);
  inv = m31_mul(inv, n[2]);  // 1 / (n0 n1)
  f[0] = qm31_mul_m31(g[0], m31_mul(inv, n[1]));
  f[1] = qm31_mul_m31(g[1], m31_mul(inv, n[0]));
  f[2] = qm31_mul_m31(g[2], i2);
  f[3] = qm31_mul_m31(g[3], i3);
}

__device__ __forceinline__ void br_write_q(uint32_t* out, size_t n, uint32_t r, uint32_t col, const qm31& x) {
  out[((size_t)4 * col + 0) * n + r] = x.a.a;
  out[((size_t)4 * col + 1) * n + r] = x.a.b;
  out[((size_t)4 * col + 2) * n + r] = x.b.a;
  out[((size_t)4 * col + 3) * n + r] = x.b.b;
}

// The Round relation's denominator: sum_k alpha^k x_k - z over the (input, output, message)
// halves; `vo` is the state after the round.
__device__ __forceinline__ qm31 br_round_denominator(const BrElements* e, const uint32_t* inputs, uint32_t r,
                                                     const uint32_t vo[BR_ST]) {
  qm31 p = qm31_zero();
#pragma unroll
  for (int i = 0; i < BR_ST; i++) {
    const uint32_t x = br_input(inputs, r, i);
    const uint32_t m = br_input(inputs, r, BR_ST + i);
    p = qm31_add(p, qm31_mul_m31(br_q(e->ra[2 * i]), x & 0xffffu));
    p = qm31_add(p, qm31_mul_m31(br_q(e->ra[2 * i + 1]), x >> 16));
    p = qm31_add(p, qm31_mul_m31(br_q(e->ra[32 + 2 * i]), vo[i] & 0xffffu));
    p = qm31_add(p, qm31_mul_m31(br_q(e->ra[32 + 2 * i + 1]), vo[i] >> 16));
    p = qm31_add(p, qm31_mul_m31(br_q(e->ra[64 + 2 * i]), m & 0xffffu));
    p = qm31_add(p, qm31_mul_m31(br_q(e->ra[64 + 2 * i + 1]), m >> 16));
  }
  return qm31_sub(p, br_q(e->rz));
}

// One thread per row, the G-functions in br_round's rotating-state order.
__global__ void __launch_bounds__(128) k_br_interaction_rows(uint32_t n_rows, const uint32_t* __restrict__ inputs,
                                                             const BrElements* __restrict__ e_dev,
                                                             uint32_t* __restrict__ out) {
  pdl_enter();
  __shared__ BrElements s_e;
  br_stage_elements(e_dev, &s_e);
  __syncthreads();
  const BrElements* e = &s_e;
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_rows) return;
  uint32_t v[BR_ST];
#pragma unroll
  for (int i = 0; i < BR_ST; i++) v[i] = br_input(inputs, r, i);
  qm31 cum = qm31_zero();
  uint32_t col = 0;
#pragma unroll 1
  for (uint32_t it = 0; it < 8; it++) {
    if (it == 4) br_diagonalize(v);
    uint32_t a = v[0], b = v[4], c = v[8], d = v[12];
    qm31 f[4];
    br_half_g<16, 12>(e, a, b, c, d, br_input(inputs, r, BR_ST + 2 * it), f);
#pragma unroll
    for (int k = 0; k < 4; k++) {
      cum = qm31_add(cum, f[k]);
      br_write_q(out, n_rows, r, col++, cum);
    }
    br_half_g<8, 7>(e, a, b, c, d, br_input(inputs, r, BR_ST + 2 * it + 1), f);
#pragma unroll
    for (int k = 0; k < 4; k++) {
      cum = qm31_add(cum, f[k]);
      br_write_q(out, n_rows, r, col++, cum);
    }
    v[0] = a;
    v[4] = b;
    v[8] = c;
    v[12] = d;
    br_rotate_rows(v);
  }
  br_undiagonalize(v);
  // -1 / p of the Round relation, added to the sum of all 64 pairs.
  const qm31 p = br_round_denominator(e, inputs, r, v);
  br_write_q(out, n_rows, r, BR_XOR_PAIRS, qm31_add(cum, qm31_sub(qm31_zero(), qm31_inv(p))));
}

__device__ __forceinline__ uint32_t br_rotr(uint32_t x, uint32_t r) { return (x >> r) | (x << (32 - r)); }

// One warp per G-function: warp g of a block takes 32 consecutive rows, replays the integer state
// of G-functions 0 .. g-1 (cheap next to the fractions), then computes its own eight pair
// fractions. The eight warps' fraction sums meet in shared memory, and each warp writes its
// columns as prefix sums from the sum of the warps before it. Every column store of a warp is one
// 128-byte line.
__global__ void __launch_bounds__(256) k_br_interaction_warps(uint32_t n_rows, const uint32_t* __restrict__ inputs,
                                                              const BrElements* __restrict__ e_dev,
                                                              uint32_t* __restrict__ out) {
  pdl_enter();
  __shared__ BrElements s_e;
  __shared__ qm31 s_tot[8][BI_ROWS];
  br_stage_elements(e_dev, &s_e);
  __syncthreads();
  const BrElements* e = &s_e;
  const uint32_t lane = threadIdx.x & 31, g = threadIdx.x >> 5;
  const uint32_t r = blockIdx.x * BI_ROWS + lane;
  const bool live = r < n_rows;
  const uint32_t rr = live ? r : n_rows - 1;  // lanes past the end replay a real row, write nothing
  uint32_t v[BR_ST];
#pragma unroll
  for (int i = 0; i < BR_ST; i++) v[i] = br_input(inputs, rr, i);
  // The integer state before G-function g, in br_round's rotating-state order.
#pragma unroll 1
  for (uint32_t it = 0; it < g; it++) {
    if (it == 4) br_diagonalize(v);
    uint32_t a = v[0], b = v[4], c = v[8], d = v[12];
    a = a + b + br_input(inputs, rr, BR_ST + 2 * it);
    d = br_rotr(a ^ d, 16);
    c = c + d;
    b = br_rotr(b ^ c, 12);
    a = a + b + br_input(inputs, rr, BR_ST + 2 * it + 1);
    d = br_rotr(a ^ d, 8);
    c = c + d;
    b = br_rotr(b ^ c, 7);
    v[0] = a;
    v[4] = b;
    v[8] = c;
    v[12] = d;
    br_rotate_rows(v);
  }
  if (g == 4) br_diagonalize(v);
  qm31 f[8];
  {
    uint32_t a = v[0], b = v[4], c = v[8], d = v[12];
    br_half_g<16, 12>(e, a, b, c, d, br_input(inputs, rr, BR_ST + 2 * g), f);
    br_half_g<8, 7>(e, a, b, c, d, br_input(inputs, rr, BR_ST + 2 * g + 1), f + 4);
    v[0] = a;
    v[4] = b;
    v[8] = c;
    v[12] = d;
  }
  qm31 tot = f[0];
#pragma unroll
  for (int k = 1; k < 8; k++) tot = qm31_add(tot, f[k]);
  s_tot[g][lane] = tot;
  __syncthreads();
  qm31 cum = qm31_zero();
  for (uint32_t h = 0; h < g; h++) cum = qm31_add(cum, s_tot[h][lane]);
#pragma unroll
  for (int k = 0; k < 8; k++) {
    cum = qm31_add(cum, f[k]);
    if (live) br_write_q(out, n_rows, r, 8 * g + k, cum);
  }
  if (g != 7) return;
  // The Round relation, last column: -1 / p added to the sum of all 64 pairs.
  br_rotate_rows(v);
  br_undiagonalize(v);
  const qm31 p = br_round_denominator(e, inputs, rr, v);
  if (live) br_write_q(out, n_rows, r, BR_XOR_PAIRS, qm31_add(cum, qm31_sub(qm31_zero(), qm31_inv(p))));
}

// ------------------------------------------------------------------------------------ composition
struct BrParams {
  uint32_t trace_log, eval_log;
  uint32_t accumulate;  // add row_res * denom_inv to the output columns instead of writing it
  uint32_t shift[4];  // claimed_sum / 2^trace_log
};

__device__ __forceinline__ uint32_t br_prev_row(uint32_t r, uint32_t trace_log, uint32_t eval_log) {
  // offset_bit_reversed_circle_domain_index(r, trace_log, eval_log, -1) (core/utils.rs:74-90)
  uint32_t prev = brev(r, eval_log);
  const uint32_t half = 1u << (eval_log - 1);
  const uint32_t step = 1u << (eval_log - trace_log - 1);
  if (prev < half) prev = (prev + half - step) & (half - 1);
  else prev = ((prev - half + step) & (half - 1)) + half;
  return brev(prev, eval_log);
}

__device__ __forceinline__ uint32_t br_inv16(uint32_t x) { return m31_mul(x, 1u << 15); }
// A 64-bit sum of M31 products, reduced to [0, P).
__device__ __forceinline__ uint32_t br_fold64(unsigned long long x) {
  x = (x & P) + (x >> 31);
  x = (x & P) + (x >> 31);
  const uint32_t r = (uint32_t)x;
  return r >= P ? r - P : r;
}

struct BrU {
  uint32_t l, h;
};

// The constraint evaluator at one row of the evaluation domain (F = M31). Trace masks are read in
// the evaluator's column order; each XOR pair's LogUp constraint is accumulated as soon as its two
// lookups are known, with its own coefficient (the random-coefficient sum is exact in the field,
// so the order of accumulation does not change it).
struct BrRowEval {
  const uint32_t* trace;
  const uint32_t* inter;
  const BrElements* e;
  const uint32_t* coeffs;  // 4 words per constraint, in constraint order (shared memory)
  uint32_t el, r;
  uint32_t col;
  uint32_t ci = 0;     // carry constraint index
  uint32_t batch = 0;  // LogUp batch index
  unsigned long long a0 = 0, a1 = 0, a2 = 0, a3 = 0;
  uint32_t cnt = 0;
  qm31 logup = qm31_zero();
  qm31 prev_col = qm31_zero();
  qm31 round_p = qm31_zero();

  __device__ __forceinline__ uint32_t load(uint32_t c) const { return __ldg(trace + ((size_t)c << el) + r); }
  __device__ __forceinline__ uint32_t mask() { return load(col++); }
  __device__ __forceinline__ void carry_constraint(uint32_t c) {
    const uint32_t* k = coeffs + 4 * ci++;
    a0 += (unsigned long long)k[0] * c;
    a1 += (unsigned long long)k[1] * c;
    a2 += (unsigned long long)k[2] * c;
    a3 += (unsigned long long)k[3] * c;
    // Products are at most (P - 1)^2 and a folded sum is below 2^33 + 2^31: four products fit
    // between folds without passing 2^64.
    if (++cnt == 4) {
      a0 = (a0 & P) + (a0 >> 31);
      a1 = (a1 & P) + (a1 >> 31);
      a2 = (a2 & P) + (a2 >> 31);
      a3 = (a3 & P) + (a3 >> 31);
      cnt = 0;
    }
  }
  __device__ __forceinline__ void logup_constraint(const qm31& c) {
    const uint32_t* k = coeffs + 4 * (64 + batch++);
    logup = qm31_add(logup, qm31_mul(qm31_from_u32(k[0], k[1], k[2], k[3]), c));
  }
  __device__ __forceinline__ qm31 inter_at(uint32_t b, uint32_t row) const {
    const uint32_t* base = inter + (((size_t)4 * b) << el) + row;
    return qm31_from_u32(__ldg(base), __ldg(base + ((size_t)1 << el)), __ldg(base + ((size_t)2 << el)),
                         __ldg(base + ((size_t)3 << el)));
  }
  // Round relation contribution of one (low, high) pair at position k of the 96 values.
  __device__ __forceinline__ void round_felts(uint32_t k, const BrU& x) {
    round_p = qm31_add(round_p, qm31_mul_m31(br_q(e->ra[k]), x.l));
    round_p = qm31_add(round_p, qm31_mul_m31(br_q(e->ra[k + 1]), x.h));
  }
  // Message word i (columns 32 + 2i, 33 + 2i), used once, by its G.
  __device__ __forceinline__ BrU msg(uint32_t i) {
    BrU x{load(2 * BR_ST + 2 * i), load(2 * BR_ST + 2 * i + 1)};
    round_felts(64 + 2 * i, x);
    return x;
  }
  __device__ __forceinline__ BrU add2(BrU a, BrU b) {
    BrU s{mask(), mask()};
    const uint32_t cl = br_inv16(m31_sub(m31_add(a.l, b.l), s.l));
    carry_constraint(m31_sub(m31_mul(cl, cl), cl));
    const uint32_t ch = br_inv16(m31_sub(m31_add(m31_add(a.h, b.h), cl), s.h));
    carry_constraint(m31_sub(m31_mul(ch, ch), ch));
    return s;
  }
  __device__ __forceinline__ BrU add3(BrU a, BrU b, BrU c) {
    BrU s{mask(), mask()};
    const uint32_t cl = br_inv16(m31_sub(m31_add(m31_add(a.l, b.l), c.l), s.l));
    carry_constraint(m31_mul(m31_mul(cl, m31_sub(cl, 1u)), m31_sub(cl, 2u)));
    const uint32_t ch = br_inv16(m31_sub(m31_add(m31_add(m31_add(a.h, b.h), c.h), cl), s.h));
    carry_constraint(m31_mul(m31_mul(ch, m31_sub(ch, 1u)), m31_sub(ch, 2u)));
    return s;
  }
  // split_unchecked: (a - h 2^rr, h) with h from the trace.
  __device__ __forceinline__ void split(uint32_t a, uint32_t rr, uint32_t& l, uint32_t& h) {
    h = mask();
    l = m31_sub(a, m31_mul(h, 1u << rr));
  }
  // Two XOR lookups (one LogUp batch): constraint (cur - prev) * p0 p1 - (p0 + p1).
  __device__ __forceinline__ void xor2(uint32_t w, uint32_t a0, uint32_t a1, uint32_t b0, uint32_t b1, uint32_t& c0,
                                       uint32_t& c1) {
    c0 = mask();
    c1 = mask();
    const qm31 p0 = br_xor_combine(e, w, a0, b0, c0);
    const qm31 p1 = br_xor_combine(e, w, a1, b1, c1);
    const qm31 cur = inter_at(batch, r);
    const qm31 diff = qm31_sub(cur, prev_col);
    prev_col = cur;
    logup_constraint(qm31_sub(qm31_mul(diff, qm31_mul(p0, p1)), qm31_add(p0, p1)));
  }
  // xor_rotr_u32 (rr < 16) or xor_rotr16_u32 (rr == 16: halves split at 8); rr may be a run-time
  // value, the same for every thread.
  __device__ __forceinline__ BrU xor_rotr(BrU a, BrU b, uint32_t rr) {
    const uint32_t sp = rr == 16 ? 8 : rr;
    uint32_t all, alh, ahl, ahh, bll, blh, bhl, bhh;
    split(a.l, sp, all, alh);
    split(a.h, sp, ahl, ahh);
    split(b.l, sp, bll, blh);
    split(b.h, sp, bhl, bhh);
    uint32_t xll, xhl, xlh, xhh;
    xor2(sp, all, ahl, bll, bhl, xll, xhl);
    xor2(16 - sp, alh, ahh, blh, bhh, xlh, xhh);
    if (rr == 16) return BrU{m31_add(m31_mul(xhh, 1u << 8), xhl), m31_add(m31_mul(xlh, 1u << 8), xll)};
    return BrU{m31_add(m31_mul(xhl, 1u << (16 - rr)), xlh), m31_add(m31_mul(xll, 1u << (16 - rr)), xhh)};
  }
};

__global__ void __launch_bounds__(128, 4) k_br_composition(const uint32_t* __restrict__ trace,
                                                        const uint32_t* __restrict__ inter, uint32_t n_rows,
                                                        BrParams pp, const BrElements* __restrict__ e_dev,
                                                        const uint32_t* __restrict__ coeffs,
                                                        const uint32_t* __restrict__ dinv, uint32_t* o0,
                                                        uint32_t* o1, uint32_t* o2, uint32_t* o3) {
  pdl_enter();
  __shared__ uint32_t s_coeffs[4 * BR_N_CONSTRAINTS];
  __shared__ BrElements s_e;
  for (uint32_t i = threadIdx.x; i < 4 * BR_N_CONSTRAINTS; i += blockDim.x) s_coeffs[i] = coeffs[i];
  br_stage_elements(e_dev, &s_e);
  __syncthreads();
  const BrElements* e = &s_e;
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_rows) return;
  BrRowEval ev{trace, inter, e, s_coeffs, pp.eval_log, r, 0};
  BrU v[BR_ST];
#pragma unroll
  for (int i = 0; i < BR_ST; i++) {
    v[i].l = ev.mask();
    v[i].h = ev.mask();
    ev.round_felts(2 * i, v[i]);
  }
  // The message masks (columns 32..63) are read by their G; the G masks follow them. Each G is
  // two iterations with the same operand roles (a += b + m, d = (a ^ d) >>> r1, c += d,
  // b = (b ^ c) >>> r2), rotations (16, 12) then (8, 7): half the loop body, which keeps the
  // kernel's instruction footprint small.
  ev.col = 4 * BR_ST;
#pragma unroll 1
  for (int it = 0; it < 16; it++) {
    const int half = it & 1;
    if (it == 8) br_diagonalize(v);
    BrU a = v[0], b = v[4], c = v[8], d = v[12];
    a = ev.add3(a, b, ev.msg(it));
    d = ev.xor_rotr(a, d, half ? 8u : 16u);
    c = ev.add2(c, d);
    b = ev.xor_rotr(b, c, half ? 7u : 12u);
    v[0] = a;
    v[4] = b;
    v[8] = c;
    v[12] = d;
    if (half) br_rotate_rows(v);
  }
  br_undiagonalize(v);
#pragma unroll
  for (int i = 0; i < BR_ST; i++) ev.round_felts(32 + 2 * i, v[i]);
  const qm31 round_p = qm31_sub(ev.round_p, br_q(e->rz));
  // Last batch: the Round entry alone (multiplicity -1), against the last cumulative column at
  // the previous and current trace rows plus the cumsum shift.
  {
    const uint32_t rp = br_prev_row(r, pp.trace_log, pp.eval_log);
    const qm31 prev_row = ev.inter_at(BR_XOR_PAIRS, rp);
    const qm31 cur = ev.inter_at(BR_XOR_PAIRS, r);
    const qm31 shift = qm31_from_u32(pp.shift[0], pp.shift[1], pp.shift[2], pp.shift[3]);  // a kernel parameter
    const qm31 fixed = qm31_add(qm31_sub(qm31_sub(cur, prev_row), ev.prev_col), shift);
    // fixed * p - (-1)
    ev.logup_constraint(qm31_add(qm31_mul(fixed, round_p), qm31_from_u32(1, 0, 0, 0)));
  }
  const qm31 res = qm31_add(qm31_from_u32(br_fold64(ev.a0), br_fold64(ev.a1), br_fold64(ev.a2), br_fold64(ev.a3)),
                            ev.logup);
  const uint32_t dv = __ldg(dinv + (r >> pp.trace_log));
  uint32_t v0 = m31_mul(res.a.a, dv), v1 = m31_mul(res.a.b, dv), v2 = m31_mul(res.b.a, dv), v3 = m31_mul(res.b.b, dv);
  if (pp.accumulate) {
    v0 = m31_add(o0[r], v0);
    v1 = m31_add(o1[r], v1);
    v2 = m31_add(o2[r], v2);
    v3 = m31_add(o3[r], v3);
  }
  o0[r] = v0;
  o1[r] = v1;
  o2[r] = v2;
  o3[r] = v3;
}

// ------------------------------------------------------------------------------------ host side
struct HRel {
  hq z;
  std::vector<hq> alpha_pow;
  // LookupElements::draw: draw_felts(2) (logup.rs:80-94).
  void draw(HostChannel& ch, size_t n) {
    auto f = ch.draw_base_felts();
    z = hq_make(f[0], f[1], f[2], f[3]);
    const hq alpha = hq_make(f[4], f[5], f[6], f[7]);
    hq cur = hq_make(1, 0, 0, 0);
    alpha_pow.resize(n);
    for (size_t i = 0; i < n; i++) {
      alpha_pow[i] = cur;
      cur = hq_mul(cur, alpha);
    }
  }
  hq combine(const hq* v, size_t n) const {
    hq acc = hq_make(0, 0, 0, 0);
    for (size_t i = 0; i < n; i++) acc = hq_add(acc, hq_mul(alpha_pow[i], v[i]));
    return hq_sub(acc, z);
  }
};

struct HBrElements {
  HRel round, xr[5];  // XOR widths 12, 9, 8, 7, 4
  static int xi(uint32_t w) { return w == 12 ? 0 : w == 9 ? 1 : w == 8 ? 2 : w == 7 ? 3 : 4; }
  void to_device(BrElements& d) const {
    for (int k = 0; k < 5; k++) {
      for (int i = 0; i < 4; i++) d.xz[k][i] = xr[k].z.v[i];
      for (int j = 0; j < 3; j++)
        for (int i = 0; i < 4; i++) d.xa[k][j][i] = xr[k].alpha_pow[j].v[i];
    }
    for (int i = 0; i < 4; i++) d.rz[i] = round.z.v[i];
    for (int j = 0; j < BR_ROUND_FELTS; j++)
      for (int i = 0; i < 4; i++) d.ra[j][i] = round.alpha_pow[j].v[i];
  }
};

static hq hq_sc(hq x, uint32_t k) {
  for (int i = 0; i < 4; i++) x.v[i] = h_mul(x.v[i], k);
  return x;
}

struct BlakeRoundGpuAir : GpuAir {
  uint32_t log_n;
  HBrElements el;
  hq claimed_sum;
  BlakeRoundGpuAir(uint32_t l, const HBrElements& e, hq cs) : log_n(l), el(e), claimed_sum(cs) {}
  uint32_t log_size() const override { return log_n; }
  uint32_t max_constraint_log_degree_bound() const override { return log_n + 1; }
  size_t n_constraints() const override { return BR_N_CONSTRAINTS; }
  std::vector<std::vector<std::vector<int>>> mask_offsets() const override {
    std::vector<std::vector<std::vector<int>>> m(3);
    m[1].assign(BR_COLS, {0});
    for (int b = 0; b + 1 < BR_INTER_SECURE; b++)
      for (int k = 0; k < 4; k++) m[2].push_back({0});
    for (int k = 0; k < 4; k++) m[2].push_back({-1, 0});
    return m;
  }
  hq shift() const { return hq_sc(claimed_sum, h_inv((uint32_t)((1ull << log_n) % P))); }
  int32_t eval_composition(const std::vector<std::vector<const uint32_t*>>& cols, const uint32_t* coeffs,
                           const uint32_t* dinv, uint32_t* const acc[4], bool accumulate,
                           cudaStream_t s) const override {
    STWO_REQUIRE(cols.size() >= 3 && cols[1].size() == BR_COLS && cols[2].size() == 4 * BR_INTER_SECURE,
                 "trace trees mismatch");
    const uint32_t el_log = log_n + 1;
    for (int c = 0; c < BR_COLS; c++)
      STWO_REQUIRE(cols[1][c] == cols[1][0] + ((size_t)c << el_log), "trace columns are not one contiguous block");
    for (int c = 0; c < 4 * BR_INTER_SECURE; c++)
      STWO_REQUIRE(cols[2][c] == cols[2][0] + ((size_t)c << el_log),
                   "interaction columns are not one contiguous block");
    BrParams pp;
    pp.trace_log = log_n;
    pp.eval_log = el_log;
    pp.accumulate = accumulate ? 1u : 0u;
    const hq sh = shift();
    for (int i = 0; i < 4; i++) pp.shift[i] = sh.v[i];
    BrElements he;
    el.to_device(he);
    BrElements* de = nullptr;
    int32_t st = scratch_alloc((void**)&de, sizeof(BrElements), s);
    if (st) return st;
    cudaError_t e = cudaMemcpyAsync(de, &he, sizeof(BrElements), cudaMemcpyHostToDevice, s);
    const uint32_t n_rows = 1u << el_log;
    if (!e) {
      launch_pdl(k_br_composition, dim3((n_rows + 127) / 128), dim3(128), 0, s, cols[1][0], cols[2][0], n_rows, pp, de,
                 coeffs, dinv, acc[0], acc[1], acc[2], acc[3]);
      note_launch();
      e = cudaGetLastError();
    }
    scratch_free(de, s);
    if (e) {
      set_error("blake round composition: %s", cudaGetErrorString(e));
      return STWO_ERR_CUDA;
    }
    return STWO_OK;
  }
  // The same constraints over QM31 at the OODS point, the PointEvaluator accumulation with the
  // vanishing inverse factored out of the sum.
  hq eval_at_point(const std::vector<std::vector<std::vector<hq>>>& mask, hq rc, hq denom_inv) const override {
    const auto& t = mask[1];
    const auto& it = mask[2];
    size_t mc = 0;
    hq acc = hq_make(0, 0, 0, 0);
    auto add = [&](hq c) { acc = hq_add(hq_mul(acc, rc), c); };
    auto next = [&]() { return t[mc++][0]; };
    const hq one = hq_make(1, 0, 0, 0), two = hq_make(2, 0, 0, 0);
    const uint32_t inv16 = 1u << 15;
    struct U {
      hq l, h;
    };
    std::vector<std::pair<hq, hq>> fr;  // (numerator, denominator) of every relation entry
    auto add2 = [&](U a, U b) {
      U s{next(), next()};
      hq cl = hq_sc(hq_sub(hq_add(a.l, b.l), s.l), inv16);
      add(hq_sub(hq_mul(cl, cl), cl));
      hq ch = hq_sc(hq_sub(hq_add(hq_add(a.h, b.h), cl), s.h), inv16);
      add(hq_sub(hq_mul(ch, ch), ch));
      return s;
    };
    auto add3 = [&](U a, U b, U c) {
      U s{next(), next()};
      hq cl = hq_sc(hq_sub(hq_add(hq_add(a.l, b.l), c.l), s.l), inv16);
      add(hq_mul(hq_mul(cl, hq_sub(cl, one)), hq_sub(cl, two)));
      hq ch = hq_sc(hq_sub(hq_add(hq_add(hq_add(a.h, b.h), c.h), cl), s.h), inv16);
      add(hq_mul(hq_mul(ch, hq_sub(ch, one)), hq_sub(ch, two)));
      return s;
    };
    auto split = [&](hq a, uint32_t rr, hq& l, hq& h) {
      h = next();
      l = hq_sub(a, hq_sc(h, 1u << rr));
    };
    auto xor2 = [&](uint32_t w, hq a0, hq a1, hq b0, hq b1, hq& c0, hq& c1) {
      c0 = next();
      c1 = next();
      const HRel& rel = el.xr[HBrElements::xi(w)];
      hq v0[3] = {a0, b0, c0}, v1[3] = {a1, b1, c1};
      fr.push_back({one, rel.combine(v0, 3)});
      fr.push_back({one, rel.combine(v1, 3)});
    };
    auto xor_rotr = [&](U a, U b, uint32_t rr) {
      hq all, alh, ahl, ahh, bll, blh, bhl, bhh, xll, xhl, xlh, xhh;
      split(a.l, rr, all, alh);
      split(a.h, rr, ahl, ahh);
      split(b.l, rr, bll, blh);
      split(b.h, rr, bhl, bhh);
      xor2(rr, all, ahl, bll, bhl, xll, xhl);
      xor2(16 - rr, alh, ahh, blh, bhh, xlh, xhh);
      return U{hq_add(hq_sc(xhl, 1u << (16 - rr)), xlh), hq_add(hq_sc(xll, 1u << (16 - rr)), xhh)};
    };
    auto xor_rotr16 = [&](U a, U b) {
      hq all, alh, ahl, ahh, bll, blh, bhl, bhh, xll, xhl, xlh, xhh;
      split(a.l, 8, all, alh);
      split(a.h, 8, ahl, ahh);
      split(b.l, 8, bll, blh);
      split(b.h, 8, bhl, bhh);
      xor2(8, all, ahl, bll, bhl, xll, xhl);
      xor2(8, alh, ahh, blh, bhh, xlh, xhh);
      return U{hq_add(hq_sc(xhh, 1u << 8), xhl), hq_add(hq_sc(xlh, 1u << 8), xll)};
    };
    U v[BR_ST], m[BR_ST], in[BR_ST];
    for (int i = 0; i < BR_ST; i++) v[i] = U{next(), next()};
    for (int i = 0; i < BR_ST; i++) in[i] = v[i];
    for (int i = 0; i < BR_ST; i++) m[i] = U{next(), next()};
    auto g = [&](int ia, int ib, int ic, int id, int mi) {
      U a = v[ia], b = v[ib], c = v[ic], d = v[id];
      a = add3(a, b, m[mi]);
      d = xor_rotr16(a, d);
      c = add2(c, d);
      b = xor_rotr(b, c, 12);
      a = add3(a, b, m[mi + 1]);
      d = xor_rotr(a, d, 8);
      c = add2(c, d);
      b = xor_rotr(b, c, 7);
      v[ia] = a;
      v[ib] = b;
      v[ic] = c;
      v[id] = d;
    };
    g(0, 4, 8, 12, 0);
    g(1, 5, 9, 13, 2);
    g(2, 6, 10, 14, 4);
    g(3, 7, 11, 15, 6);
    g(0, 5, 10, 15, 8);
    g(1, 6, 11, 12, 10);
    g(2, 7, 8, 13, 12);
    g(3, 4, 9, 14, 14);
    std::vector<hq> vals;
    for (int i = 0; i < BR_ST; i++) vals.push_back(in[i].l), vals.push_back(in[i].h);
    for (int i = 0; i < BR_ST; i++) vals.push_back(v[i].l), vals.push_back(v[i].h);
    for (int i = 0; i < BR_ST; i++) vals.push_back(m[i].l), vals.push_back(m[i].h);
    fr.push_back({hq_sub(hq_make(0, 0, 0, 0), one), el.round.combine(vals.data(), vals.size())});
    // finalize_logup_in_pairs (constraint_framework/mod.rs:180-243).
    auto comb = [&](size_t col, size_t j) {
      return hq_add(hq_add(it[4 * col][j], hq_mul(it[4 * col + 1][j], hq_make(0, 1, 0, 0))),
                    hq_add(hq_mul(it[4 * col + 2][j], hq_make(0, 0, 1, 0)), hq_mul(it[4 * col + 3][j], hq_make(0, 0, 0, 1))));
    };
    const size_t n_batches = (fr.size() + 1) / 2;
    auto batch = [&](size_t b) {
      std::pair<hq, hq> f = fr[2 * b];
      if (2 * b + 1 < fr.size()) {
        const auto& g2 = fr[2 * b + 1];
        f = {hq_add(hq_mul(g2.second, f.first), hq_mul(f.second, g2.first)), hq_mul(f.second, g2.second)};
      }
      return f;
    };
    hq prev_col = hq_make(0, 0, 0, 0);
    for (size_t b = 0; b + 1 < n_batches; b++) {
      auto f = batch(b);
      const hq cur = comb(b, 0);
      const hq diff = hq_sub(cur, prev_col);
      prev_col = cur;
      add(hq_sub(hq_mul(diff, f.second), f.first));
    }
    auto f = batch(n_batches - 1);
    const hq pr = comb(n_batches - 1, 0), cur = comb(n_batches - 1, 1);
    const hq fixed = hq_add(hq_sub(hq_sub(cur, pr), prev_col), shift());
    add(hq_sub(hq_mul(fixed, f.second), f.first));
    return hq_mul(acc, denom_inv);
  }
};

GpuAir* new_blake_round_air(uint32_t log_n, const hq* z_alpha, const hq& claimed_sum) {
  auto rel = [](HRel& r, hq z, hq alpha, size_t n) {
    r.z = z;
    hq cur = hq_make(1, 0, 0, 0);
    r.alpha_pow.resize(n);
    for (size_t i = 0; i < n; i++) {
      r.alpha_pow[i] = cur;
      cur = hq_mul(cur, alpha);
    }
  };
  HBrElements el;
  rel(el.round, z_alpha[0], z_alpha[1], BR_ROUND_FELTS);
  for (int k = 0; k < 5; k++) rel(el.xr[k], z_alpha[2 + 2 * k], z_alpha[3 + 2 * k], 3);
  return new BlakeRoundGpuAir(log_n, el, claimed_sum);
}

// ------------------------------------------------------------------ the full Blake example's trace
// prove_blake's trace (blake/air.rs:331-400) for 2^L instances, one thread per row:
//   k_bf_scheduler  the scheduler's 384 columns (messages, then the 11 states, as 16-bit limbs;
//                   scheduler/gen.rs:45-118) and the round inputs it hands on: input
//                   p = 10 vec_row + r holds, lane by lane, the state before round r of instance
//                   16 vec_row + lane and its SIGMA[r]-permuted messages, i.e. row 16 p + lane;
//   k_bf_rounds     one round component's 384 columns from those inputs (br_round, as k_br_trace)
//                   and every XOR lookup counted into the tables' multiplicity columns, column
//                   (ah << e) + bh, row (al << limb) + bl (xor_table/mod.rs:60-90).
// Instance 16 vec_row + lane has every state word vec_row + 2 lane and every message word one
// more (air.rs:331-338).
__constant__ uint8_t c_bf_sigma[10][16] = {
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
constexpr uint32_t BF_ROUNDS = 10;
constexpr uint32_t BF_SCHED_COLS = 384;

__device__ __forceinline__ uint32_t bf_rotr(uint32_t x, uint32_t r) { return (x >> r) | (x << (32 - r)); }

__global__ void __launch_bounds__(128) k_bf_scheduler(uint32_t log_n, uint32_t* __restrict__ trace,
                                                      uint32_t* __restrict__ round_inputs) {
  pdl_enter();
  const size_t n = (size_t)1 << log_n;
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const uint32_t vec_row = s >> 4, lane = s & 15;
  uint32_t v[BR_ST], m[BR_ST];
#pragma unroll
  for (int k = 0; k < BR_ST; k++) {
    v[k] = vec_row + 2 * lane;
    m[k] = v[k] + 1;
  }
  uint32_t col = 0;
  auto put = [&](const uint32_t* w) {
#pragma unroll
    for (int k = 0; k < BR_ST; k++) {
      trace[(size_t)col++ * n + s] = w[k] & 0xffffu;
      trace[(size_t)col++ * n + s] = w[k] >> 16;
    }
  };
  put(m);
  put(v);
#pragma unroll 1
  for (uint32_t r = 0; r < BF_ROUNDS; r++) {
    uint32_t* in = round_inputs + ((((size_t)vec_row * BF_ROUNDS + r) << 4) + lane) * 32;
#pragma unroll
    for (int k = 0; k < BR_ST; k++) {
      in[k] = v[k];
      in[BR_ST + k] = m[c_bf_sigma[r][k]];
    }
    auto g = [&](int a, int b, int c, int d, uint32_t x, uint32_t y) {
      v[a] = v[a] + v[b] + x;
      v[d] = bf_rotr(v[d] ^ v[a], 16);
      v[c] = v[c] + v[d];
      v[b] = bf_rotr(v[b] ^ v[c], 12);
      v[a] = v[a] + v[b] + y;
      v[d] = bf_rotr(v[d] ^ v[a], 8);
      v[c] = v[c] + v[d];
      v[b] = bf_rotr(v[b] ^ v[c], 7);
    };
    const uint8_t* sg = c_bf_sigma[r];
    g(0, 4, 8, 12, m[sg[0]], m[sg[1]]);
    g(1, 5, 9, 13, m[sg[2]], m[sg[3]]);
    g(2, 6, 10, 14, m[sg[4]], m[sg[5]]);
    g(3, 7, 11, 15, m[sg[6]], m[sg[7]]);
    g(0, 5, 10, 15, m[sg[8]], m[sg[9]]);
    g(1, 6, 11, 12, m[sg[10]], m[sg[11]]);
    g(2, 7, 8, 13, m[sg[12]], m[sg[13]]);
    g(3, 4, 9, 14, m[sg[14]], m[sg[15]]);
    put(v);
  }
}

// The XOR tables' multiplicity columns, one block per table in the order 12/4, 9/2, 8/2, 7/2,
// 4/0; table t starts at word offset bf_xor_offset(t).
struct BfXorTables {
  uint32_t* base;
  __device__ __forceinline__ void lookup(uint32_t w, uint32_t a, uint32_t b, uint32_t) const {
    uint32_t e, off;
    switch (w) {
      case 12: e = 4, off = 0; break;
      case 9: e = 2, off = 1u << 24; break;
      case 8: e = 2, off = (1u << 24) + (1u << 18); break;
      case 7: e = 2, off = (1u << 24) + (1u << 18) + (1u << 16); break;
      default: e = 0, off = (1u << 24) + (1u << 18) + (1u << 16) + (1u << 14); break;
    }
    const uint32_t lb = w - e, mask = (1u << lb) - 1;
    const uint32_t column = ((a >> lb) << e) + (b >> lb);
    const uint32_t row = ((a & mask) << lb) + (b & mask);
    atomicAdd(base + off + ((size_t)column << (2 * lb)) + row, 1u);
  }
};
constexpr size_t BF_XOR_WORDS = (1u << 24) + (1u << 18) + (1u << 16) + (1u << 14) + (1u << 8);

struct BfRoundWriter {
  uint32_t* trace;
  size_t n;
  uint32_t r;
  BfXorTables xt;
  uint32_t col = 0;
  __device__ void felt(uint32_t x) { trace[(size_t)col++ * n + r] = x; }
  __device__ void lookup(uint32_t w, uint32_t a, uint32_t b, uint32_t c) { xt.lookup(w, a, b, c); }
};

__global__ void __launch_bounds__(128) k_bf_rounds(uint32_t n_rows, const uint32_t* __restrict__ inputs,
                                                   uint32_t* __restrict__ trace, uint32_t* __restrict__ xor_tables) {
  pdl_enter();
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_rows) return;
  uint32_t v[BR_ST];
  BfRoundWriter w{trace, n_rows, r, BfXorTables{xor_tables}};
#pragma unroll
  for (int i = 0; i < BR_ST; i++) {
    v[i] = __ldg(inputs + (size_t)r * 32 + i);
    w.felt(v[i] & 0xffffu);
    w.felt(v[i] >> 16);
  }
#pragma unroll
  for (int i = 0; i < BR_ST; i++) {
    const uint32_t m = __ldg(inputs + (size_t)r * 32 + BR_ST + i);
    w.felt(m & 0xffffu);
    w.felt(m >> 16);
  }
  br_round(v, [&](int i) { return __ldg(inputs + (size_t)r * 32 + BR_ST + i); }, w);
}

}  // namespace stwo

using namespace stwo;

extern "C" stwo_status stwo_gen_blake_example_trace(uint32_t log_n, uint32_t* d_trace, uint32_t* d_scratch,
                                                    void* stream) {
  STWO_REQUIRE(log_n >= 4 && log_n <= 20, "log_n out of [4, 20]");
  STWO_REQUIRE(d_trace && d_scratch, "null buffer");
  cudaStream_t s = as_stream(stream);
  const size_t n = (size_t)1 << log_n;
  uint32_t* sched = d_trace;
  uint32_t* round0 = sched + BF_SCHED_COLS * n;
  uint32_t* round1 = round0 + (size_t)BR_COLS * (8 * n);
  uint32_t* xors = round1 + (size_t)BR_COLS * (2 * n);
  if (cudaMemsetAsync(xors, 0, BF_XOR_WORDS * 4, s) != cudaSuccess) return STWO_ERR_CUDA;
  launch_pdl(k_bf_scheduler, dim3((uint32_t)((n + 127) / 128)), dim3(128), 0, s, log_n, sched, d_scratch);
  launch_pdl(k_bf_rounds, dim3((uint32_t)((8 * n + 127) / 128)), dim3(128), 0, s, (uint32_t)(8 * n),
             (const uint32_t*)d_scratch, round0, xors);
  launch_pdl(k_bf_rounds, dim3((uint32_t)((2 * n + 127) / 128)), dim3(128), 0, s, (uint32_t)(2 * n),
             (const uint32_t*)(d_scratch + 8 * n * 32), round1, xors);
  note_launch();
  note_launch();
  note_launch();
  return cudaGetLastError() == cudaSuccess ? STWO_OK : STWO_ERR_CUDA;
}

extern "C" stwo_status stwo_prove_blake_round(uint32_t log_n_rows, const uint32_t* d_inputs, stwo_pcs_config cfg,
                                              uint8_t* h_proof, size_t capacity, size_t* h_len,
                                              stwo_qm31* h_claimed_sum, void* stream) {
  STWO_REQUIRE(log_n_rows >= 4 && log_n_rows + 1 + cfg.log_blowup_factor <= 28, "bad log_n_rows");
  STWO_REQUIRE(cfg.log_blowup_factor >= 1 && cfg.log_blowup_factor <= 16, "log_blowup_factor out of [1, 16]");
  STWO_REQUIRE(cfg.log_last_layer_degree_bound <= 10, "log_last_layer_degree_bound > 10");
  STWO_REQUIRE(h_len, "null length");
  cudaStream_t s = as_stream(stream);
  std::vector<uint8_t> bytes;
  hq claimed = hq_make(0, 0, 0, 0);
  int32_t st;
  {
    Prover pv(cfg, log_n_rows + 1 + cfg.log_blowup_factor, s);
    if (pv.init_status) return pv.init_status;
    const size_t n = (size_t)1 << log_n_rows;
    st = pv.commit_polys({}, {});
    // BlakeStatement0::mix_into (blake/air.rs:126-128).
    if (!st) pv.ch.mix_u64(log_n_rows);
    uint32_t* trace = nullptr;
    uint32_t* inter = nullptr;
    if (!st) {
      trace = pv.arena.alloc(n * BR_COLS);
      inter = pv.arena.alloc(n * 4 * BR_INTER_SECURE);
      if (!trace || !inter) st = STWO_ERR_OOM;
    }
    if (!st) {
      StageScope stage("Generation", s);
      launch_pdl(k_br_trace, dim3((uint32_t)((n + 127) / 128)), dim3(128), 0, s, (uint32_t)n, d_inputs, trace);
      note_launch();
      if (cudaGetLastError() != cudaSuccess) st = STWO_ERR_CUDA;
    }
    if (!st) {
      std::vector<uint32_t*> cols(BR_COLS);
      for (int c = 0; c < BR_COLS; c++) cols[c] = trace + (size_t)c * n;
      st = pv.commit_evals(cols, log_n_rows);
    }
    HBrElements el;
    if (!st) {
      el.round.draw(pv.ch, BR_ROUND_FELTS);
      for (int k = 0; k < 5; k++) el.xr[k].draw(pv.ch, 3);
      StageScope stage("Interaction", s);
      BrElements he;
      el.to_device(he);
      BrElements* de = reinterpret_cast<BrElements*>(pv.arena.alloc((sizeof(BrElements) + 3) / 4));
      if (!de) st = STWO_ERR_OOM;
      if (!st && cudaMemcpyAsync(de, &he, sizeof(BrElements), cudaMemcpyHostToDevice, s) != cudaSuccess)
        st = STWO_ERR_CUDA;
      if (!st) {
        if (log_n_rows <= BI_WARPS_MAX_LOG)
          launch_pdl(k_br_interaction_warps, dim3((uint32_t)((n + BI_ROWS - 1) / BI_ROWS)), dim3(8 * 32), 0, s,
                     (uint32_t)n, d_inputs, de, inter);
        else
          launch_pdl(k_br_interaction_rows, dim3((uint32_t)((n + 127) / 128)), dim3(128), 0, s, (uint32_t)n, d_inputs, de,
                     inter);
        note_launch();
        if (cudaGetLastError() != cudaSuccess) st = STWO_ERR_CUDA;
      }
    }
    // The claimed sum is mixed before the interaction commitment (BlakeStatement1::mix_into).
    if (!st) st = logup_finalize_last(inter + (size_t)4 * (BR_INTER_SECURE - 1) * n, log_n_rows, pv.arena, s, &claimed);
    if (!st) {
      pv.ch.mix_felts({claimed});
      std::vector<uint32_t*> cols(4 * BR_INTER_SECURE);
      for (int c = 0; c < 4 * BR_INTER_SECURE; c++) cols[c] = inter + (size_t)c * n;
      st = pv.commit_evals(cols, log_n_rows);
    }
    if (!st) {
      BlakeRoundGpuAir air(log_n_rows, el, claimed);
      st = pv.prove(air, bytes);
    }
    cudaStreamSynchronize(s);
  }
  if (st) return st;
  if (h_claimed_sum)
    for (int i = 0; i < 4; i++) h_claimed_sum->v[i] = claimed.v[i];
  *h_len = bytes.size();
  STWO_REQUIRE(bytes.size() <= capacity, "proof buffer too small (%zu bytes needed)", bytes.size());
  if (h_proof) memcpy(h_proof, bytes.data(), bytes.size());
  return STWO_OK;
}
