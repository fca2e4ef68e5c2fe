// GKR and MLE backend operations and the batch GKR prover built on them.
//   GkrOps        crates/prover/src/core/lookups/gkr_prover.rs:22-42
//                 (SIMD crates/prover/src/core/backend/simd/lookups/gkr.rs:20-480)
//   MleOps        crates/prover/src/core/lookups/mle.rs:9-14
//                 (SIMD crates/prover/src/core/backend/simd/lookups/mle.rs:14-91)
//   prove_batch   crates/prover/src/core/lookups/gkr_prover.rs:401-516
//   sum-check     crates/prover/src/core/lookups/sumcheck.rs:62-126
// An Mle column holds a multilinear polynomial's values on the boolean hypercube with the first
// variable as the most significant index bit; a secure column is four coordinate arrays.
//
// GPU shape: every operation is one pass over HBM. A sum-check round reads the current layer,
// folds the previous round's challenge into it on the fly (writing the folded layer), and reduces
// the round's two sums in the same kernel; the last block to finish combines the per-block
// partials and writes the eight result words straight into mapped host memory, so a round costs
// one launch and one stream synchronisation. The Fiat-Shamir transcript stays on the host, as in
// the reference.
#include "common.cuh"
#include "host_channel.h"
#include <atomic>
#include <chrono>

namespace stwo {
namespace {

enum : uint32_t { K_GP = 0, K_GENERIC = 1, K_MULT = 2, K_SINGLES = 3 };

struct Sec { const uint32_t* c[4]; };
struct SecM { uint32_t* c[4]; };
// Columns of one layer: `num` (a grand product's column, secure numerators, or base
// multiplicities in c[0]) and `den`.
struct Cols { Sec num; Sec den; };
struct ColsM { SecM num; SecM den; };

__device__ __forceinline__ qm31 ldq(const Sec& s, size_t i) {
  return qm31_from_u32(s.c[0][i], s.c[1][i], s.c[2][i], s.c[3][i]);
}
__device__ __forceinline__ void stq(const SecM& s, size_t i, qm31 v) {
  s.c[0][i] = v.a.a;
  s.c[1][i] = v.a.b;
  s.c[2][i] = v.b.a;
  s.c[3][i] = v.b.b;
}
__device__ __forceinline__ qm31 q_one() { return qm31_from_u32(1u, 0u, 0u, 0u); }
__device__ __forceinline__ qm31 q_base(uint32_t x) { return qm31_from_u32(x, 0u, 0u, 0u); }
__device__ __forceinline__ qm31 q_dbl(qm31 x) { return qm31_add(x, x); }
// utils.rs:170-176: a * (e1 - e0) + e0.
__device__ __forceinline__ qm31 fold(qm31 a, qm31 e0, qm31 e1) { return qm31_add(qm31_mul(a, qm31_sub(e1, e0)), e0); }
__device__ __forceinline__ qm31 fold_base(qm31 a, uint32_t e0, uint32_t e1) {
  qm31 r = qm31_mul_m31(a, m31_sub(e1, e0));
  r.a.a = m31_add(r.a.a, e0);
  return r;
}

__device__ __forceinline__ qm31 shfl_q(qm31 x, int off) {
  return qm31_from_u32(__shfl_xor_sync(0xffffffffu, x.a.a, off), __shfl_xor_sync(0xffffffffu, x.a.b, off),
                       __shfl_xor_sync(0xffffffffu, x.b.a, off), __shfl_xor_sync(0xffffffffu, x.b.b, off));
}

// ------------------------------------------------------------------------------ gen_eq_evals
// eq(x, y) * v = v * prod_j (x_j ? y_j : 1 - y_j) (cpu/lookups/gkr.rs:214-230). The low
// `lo_bits` variables come from a per-block table in shared memory and the high ones from a
// per-row product, so each output costs one QM31 product.
constexpr uint32_t EQ_MAX_Y = 32;
constexpr uint32_t EQ_LO_BITS = 8;
constexpr uint32_t EQ_ROWS = 16;
struct EqParams {
  qm31 y[EQ_MAX_Y];
  qm31 v;
  uint32_t n_y, lo_bits;
};

__global__ void __launch_bounds__(256) k_eq_evals(EqParams p, SecM out) {
  __shared__ qm31 lo[1u << EQ_LO_BITS];
  __shared__ qm31 hi[EQ_ROWS];
  const uint32_t a = p.lo_bits, nh = p.n_y - a, nlo = 1u << a;
  for (uint32_t t = threadIdx.x; t < nlo; t += blockDim.x) {
    qm31 r = q_one();
    for (uint32_t k = 0; k < a; k++) {
      qm31 yk = p.y[nh + k];
      r = qm31_mul(r, ((t >> (a - 1 - k)) & 1u) ? yk : qm31_sub(q_one(), yk));
    }
    lo[t] = r;
  }
  const uint32_t row0 = blockIdx.x * EQ_ROWS;
  const uint32_t nrows = min(EQ_ROWS, (1u << nh) - row0);
  for (uint32_t t = threadIdx.x; t < nrows; t += blockDim.x) {
    uint32_t h = row0 + t;
    qm31 r = p.v;
    for (uint32_t j = 0; j < nh; j++) r = qm31_mul(r, ((h >> (nh - 1 - j)) & 1u) ? p.y[j] : qm31_sub(q_one(), p.y[j]));
    hi[t] = r;
  }
  __syncthreads();
  const size_t base = (size_t)row0 << a;
  const uint32_t total = nrows << a;
  for (uint32_t t = threadIdx.x; t < total; t += blockDim.x) stq(out, base + t, qm31_mul(hi[t >> a], lo[t & (nlo - 1)]));
}

// ------------------------------------------------------------------------------ next_layer
// cpu/lookups/gkr.rs:232-262: pairwise products, or fraction sums n0/d0 + n1/d1 =
// (d1 n0 + d0 n1) / (d0 d1); every LogUp kind yields a generic layer.
template <uint32_t KIND>
__global__ void __launch_bounds__(256) k_next_layer(Cols in, ColsM out, uint32_t n_out) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_out; i += (size_t)gridDim.x * blockDim.x) {
    if (KIND == K_GP) {
      stq(out.num, i, qm31_mul(ldq(in.num, 2 * i), ldq(in.num, 2 * i + 1)));
      continue;
    }
    qm31 d0 = ldq(in.den, 2 * i), d1 = ldq(in.den, 2 * i + 1), n;
    if (KIND == K_SINGLES) n = qm31_add(d1, d0);
    else if (KIND == K_MULT) n = qm31_add(qm31_mul_m31(d1, in.num.c[0][2 * i]), qm31_mul_m31(d0, in.num.c[0][2 * i + 1]));
    else n = qm31_add(qm31_mul(d1, ldq(in.num, 2 * i)), qm31_mul(d0, ldq(in.num, 2 * i + 1)));
    stq(out.num, i, n);
    stq(out.den, i, qm31_mul(d0, d1));
  }
}

// ------------------------------------------------------------------------------ sum-check round
// Gate j of the current layer. Without FIX the current layer is `src`; with FIX it is `src`
// with its first variable fixed to `c` (length `cur`, src twice that), and the folded values are
// written to `dst` (gkr_prover.rs:167-195; a multiplicities layer becomes generic). Each position
// j < cur belongs to exactly one thread, so dst may alias src.
template <uint32_t KIND, bool FIX>
__device__ __forceinline__ void gate(const Cols& src, const ColsM& dst, qm31 c, uint32_t cur, size_t j, qm31& n,
                                     qm31& d) {
  if (!FIX) {
    if (KIND == K_GP) {
      n = ldq(src.num, j);
      return;
    }
    d = ldq(src.den, j);
    if (KIND == K_SINGLES) n = q_one();
    else if (KIND == K_MULT) n = q_base(src.num.c[0][j]);
    else n = ldq(src.num, j);
    return;
  }
  if (KIND == K_GP) {
    n = fold(c, ldq(src.num, j), ldq(src.num, j + cur));
    stq(dst.num, j, n);
    return;
  }
  d = fold(c, ldq(src.den, j), ldq(src.den, j + cur));
  stq(dst.den, j, d);
  if (KIND == K_SINGLES) {
    n = q_one();
    return;
  }
  if (KIND == K_MULT) n = fold_base(c, src.num.c[0][j], src.num.c[0][j + cur]);
  else n = fold(c, ldq(src.num, j), ldq(src.num, j + cur));
  stq(dst.num, j, n);
}

struct RoundOut {
  uint32_t* partials;  // 8 words per block
  unsigned int* ticket;
  uint32_t* result;    // 8 words: f(0), f(2) before the eq correction
  uint32_t* flag;      // optional (mapped host memory): set to `seq` once `result` is written
  uint32_t seq;
};

// Publishes a completion flag to the host polling mapped memory, after every earlier write.
__device__ __forceinline__ void publish_flag(uint32_t* flag, uint32_t seq) {
  __threadfence_system();
  *reinterpret_cast<volatile uint32_t*>(flag) = seq;
}

// Terms i = first, first + stride, ... of one round (cpu/lookups/gkr.rs:38-212), accumulated into
// (e0, e2): with FIX the previous challenge is folded in on the fly (see gate()).
template <uint32_t KIND, bool FIX>
__device__ __forceinline__ void round_terms(const Cols& src, const ColsM& dst, qm31 c, uint32_t cur, const Sec& eq,
                                            qm31 lambda, uint32_t first, uint32_t stride, qm31& e0, qm31& e2) {
  const uint32_t nt = cur / 4;
  for (uint32_t i = first; i < nt; i += stride) {
    qm31 n00, n01, n10, n11, d00, d01, d10, d11;
    gate<KIND, FIX>(src, dst, c, cur, 2 * (size_t)i, n00, d00);
    gate<KIND, FIX>(src, dst, c, cur, 2 * (size_t)i + 1, n01, d01);
    gate<KIND, FIX>(src, dst, c, cur, 2 * ((size_t)nt + i), n10, d10);
    gate<KIND, FIX>(src, dst, c, cur, 2 * ((size_t)nt + i) + 1, n11, d11);
    const qm31 w = ldq(eq, i);
    if (KIND == K_GP) {
      qm31 r2a = qm31_sub(q_dbl(n10), n00), r2b = qm31_sub(q_dbl(n11), n01);
      e0 = qm31_add(e0, qm31_mul(w, qm31_mul(n00, n01)));
      e2 = qm31_add(e2, qm31_mul(w, qm31_mul(r2a, r2b)));
      continue;
    }
    qm31 d20 = qm31_sub(q_dbl(d10), d00), d21 = qm31_sub(q_dbl(d11), d01);
    qm31 num0, num2;
    if (KIND == K_SINGLES) {
      num0 = qm31_add(d00, d01);
      num2 = qm31_add(d20, d21);
    } else {
      qm31 n20 = qm31_sub(q_dbl(n10), n00), n21 = qm31_sub(q_dbl(n11), n01);
      num0 = qm31_add(qm31_mul(d01, n00), qm31_mul(d00, n01));
      num2 = qm31_add(qm31_mul(d21, n20), qm31_mul(d20, n21));
    }
    e0 = qm31_add(e0, qm31_mul(w, qm31_add(num0, qm31_mul(lambda, qm31_mul(d00, d01)))));
    e2 = qm31_add(e2, qm31_mul(w, qm31_add(num2, qm31_mul(lambda, qm31_mul(d20, d21)))));
  }
}

// Block reduction of (e0, e2), then the last block to arrive reduces the per-block partials into
// ro.result (and publishes ro.flag).
__device__ __forceinline__ void block_reduce_and_finish(qm31 e0, qm31 e2, const RoundOut& ro) {
  __shared__ qm31 s0[8], s2[8];
  __shared__ bool last;
  for (int off = 16; off; off >>= 1) {
    e0 = qm31_add(e0, shfl_q(e0, off));
    e2 = qm31_add(e2, shfl_q(e2, off));
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  if (lane == 0) {
    s0[warp] = e0;
    s2[warp] = e2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    qm31 a = s0[0], b = s2[0];
    for (int w = 1; w < nw; w++) {
      a = qm31_add(a, s0[w]);
      b = qm31_add(b, s2[w]);
    }
    uint32_t* p = ro.partials + 8 * (size_t)blockIdx.x;
    p[0] = a.a.a; p[1] = a.a.b; p[2] = a.b.a; p[3] = a.b.b;
    p[4] = b.a.a; p[5] = b.a.b; p[6] = b.b.a; p[7] = b.b.b;
    __threadfence();
    last = atomicAdd(ro.ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  qm31 a = qm31_zero(), b = qm31_zero();
  for (uint32_t k = threadIdx.x; k < gridDim.x; k += blockDim.x) {
    const uint32_t* p = ro.partials + 8 * (size_t)k;
    a = qm31_add(a, qm31_from_u32(__ldcg(p), __ldcg(p + 1), __ldcg(p + 2), __ldcg(p + 3)));
    b = qm31_add(b, qm31_from_u32(__ldcg(p + 4), __ldcg(p + 5), __ldcg(p + 6), __ldcg(p + 7)));
  }
  for (int off = 16; off; off >>= 1) {
    a = qm31_add(a, shfl_q(a, off));
    b = qm31_add(b, shfl_q(b, off));
  }
  __syncthreads();
  if (lane == 0) {
    s0[warp] = a;
    s2[warp] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < nw; w++) {
      s0[0] = qm31_add(s0[0], s0[w]);
      s2[0] = qm31_add(s2[0], s2[w]);
    }
    uint32_t* r = ro.result;
    r[0] = s0[0].a.a; r[1] = s0[0].a.b; r[2] = s0[0].b.a; r[3] = s0[0].b.b;
    r[4] = s2[0].a.a; r[5] = s2[0].a.b; r[6] = s2[0].b.a; r[7] = s2[0].b.b;
    *ro.ticket = 0u;
    if (ro.flag) publish_flag(ro.flag, ro.seq);
    else __threadfence_system();
  }
}

// (f(0), f(2)) of sum_x eq((0, x), y) P(t, x) over the current layer (cpu/lookups/gkr.rs:38-212).
template <uint32_t KIND, bool FIX>
__global__ void __launch_bounds__(256) k_gkr_round(Cols src, ColsM dst, qm31 c, uint32_t cur, Sec eq, qm31 lambda,
                                                   RoundOut ro) {
  qm31 e0 = qm31_zero(), e2 = qm31_zero();
  round_terms<KIND, FIX>(src, dst, c, cur, eq, lambda, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x,
                         e0, e2);
  block_reduce_and_finish(e0, e2, ro);
}


// The gates at positions 0..cur-1 (cur <= 2) into `out`: numerators at words 4j, denominators at
// 8 + 4j. Used for output layer values and for the masks of constant oracles.
template <uint32_t KIND, bool FIX>
__global__ void k_gkr_gates(Cols src, ColsM dst, qm31 c, uint32_t cur, uint32_t* out, uint32_t* flag, uint32_t seq) {
  const uint32_t j = threadIdx.x;
  if (j < cur) {
    qm31 n, d = qm31_zero();
    gate<KIND, FIX>(src, dst, c, cur, j, n, d);
    uint32_t* o = out + 4 * j;
    o[0] = n.a.a; o[1] = n.a.b; o[2] = n.b.a; o[3] = n.b.b;
    o[8] = d.a.a; o[9] = d.a.b; o[10] = d.b.a; o[11] = d.b.b;
    __threadfence_system();
  }
  __syncthreads();
  if (j == 0 && flag) publish_flag(flag, seq);
}

// ------------------------------------------------------------------------------ small-layer tail
// The last rounds of a GKR layer, once every layer left has at most TAIL_MAX_GATES gates, run in
// one single-block kernel that stays resident and trades each round with the host through mapped
// memory: it publishes the round's sums, waits for the challenge the host draws (the transcript
// stays on the host, as in the reference), folds it in and goes on. A round then costs two
// mapped-memory hand-offs instead of a kernel launch plus a host wait. The wait is bounded: with
// no challenge after about two seconds the kernel records an error and returns.
constexpr uint32_t TAIL_MAXI = 8;
constexpr uint32_t TAIL_MAX_GATES = 4096;
constexpr uint32_t TAIL_THREADS = 512;
constexpr long long TAIL_WAIT_CYCLES = 4000000000ll;
constexpr uint32_t TAIL_ABORT = 0xFFFFFFFFu;

struct TailInst {
  uint32_t kind, vars, cur, pending;
  Cols src;
  ColsM work;
  uint32_t* out;  // mapped: 24 words (round sums, then mask gates)
};
struct TailParams {
  uint32_t n_inst, sc_vars, r0;
  TailInst inst[TAIL_MAXI];
  Sec eq;
  qm31 lambda, chal0;
  uint32_t* to_host;          // mapped: [seq, error]
  const uint32_t* from_host;  // mapped: [seq, challenge (4 words)]
  uint32_t seq0;
};

template <uint32_t KIND>
__device__ void tail_sums(const TailInst& t, qm31 c, const Sec& eq, qm31 lambda, uint32_t* out) {
  __shared__ qm31 r0[TAIL_THREADS / 32], r2[TAIL_THREADS / 32];
  qm31 e0 = qm31_zero(), e2 = qm31_zero();
  if (t.pending) round_terms<KIND, true>(t.src, t.work, c, t.cur, eq, lambda, threadIdx.x, blockDim.x, e0, e2);
  else round_terms<KIND, false>(t.src, t.work, c, t.cur, eq, lambda, threadIdx.x, blockDim.x, e0, e2);
  for (int off = 16; off; off >>= 1) {
    e0 = qm31_add(e0, shfl_q(e0, off));
    e2 = qm31_add(e2, shfl_q(e2, off));
  }
  if ((threadIdx.x & 31) == 0) {
    r0[threadIdx.x >> 5] = e0;
    r2[threadIdx.x >> 5] = e2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    qm31 a = r0[0], b = r2[0];
    for (uint32_t w = 1; w < blockDim.x / 32; w++) {
      a = qm31_add(a, r0[w]);
      b = qm31_add(b, r2[w]);
    }
    out[0] = a.a.a; out[1] = a.a.b; out[2] = a.b.a; out[3] = a.b.b;
    out[4] = b.a.a; out[5] = b.a.b; out[6] = b.b.a; out[7] = b.b.b;
  }
  __syncthreads();
}

template <uint32_t KIND>
__device__ void tail_gates(const TailInst& t, qm31 c, uint32_t* out) {
  const uint32_t j = threadIdx.x;
  if (j < 2) {
    qm31 n, d = qm31_zero();
    if (t.pending) gate<KIND, true>(t.src, t.work, c, 2, j, n, d);
    else gate<KIND, false>(t.src, t.work, c, 2, j, n, d);
    uint32_t* o = out + 4 * j;
    o[0] = n.a.a; o[1] = n.a.b; o[2] = n.b.a; o[3] = n.b.b;
    o[8] = d.a.a; o[9] = d.a.b; o[10] = d.b.a; o[11] = d.b.b;
  }
}

__global__ void __launch_bounds__(TAIL_THREADS) k_gkr_tail(TailParams p) {
  __shared__ TailInst st[TAIL_MAXI];
  __shared__ qm31 s_chal;
  __shared__ uint32_t s_abort;
  if (threadIdx.x < p.n_inst) st[threadIdx.x] = p.inst[threadIdx.x];
  if (threadIdx.x == 0) {
    s_chal = p.chal0;
    s_abort = 0;
  }
  __syncthreads();
  uint32_t seq = p.seq0;
  for (uint32_t r = p.r0; r < p.sc_vars; r++) {
    const uint32_t rem = p.sc_vars - r;
    const qm31 c = s_chal;
    for (uint32_t i = 0; i < p.n_inst; i++) {
      if (st[i].vars != rem) continue;
      switch (st[i].kind) {
        case K_GP: tail_sums<K_GP>(st[i], c, p.eq, p.lambda, st[i].out); break;
        case K_GENERIC: tail_sums<K_GENERIC>(st[i], c, p.eq, p.lambda, st[i].out); break;
        case K_MULT: tail_sums<K_MULT>(st[i], c, p.eq, p.lambda, st[i].out); break;
        default: tail_sums<K_SINGLES>(st[i], c, p.eq, p.lambda, st[i].out); break;
      }
    }
    if (threadIdx.x == 0) {
      // The live layers now hold their folded values in `work`; their first variable is next.
      for (uint32_t i = 0; i < p.n_inst; i++) {
        if (st[i].vars != rem) continue;
        if (st[i].pending) {
          for (int k = 0; k < 4; k++) {
            st[i].src.num.c[k] = st[i].work.num.c[k];
            st[i].src.den.c[k] = st[i].work.den.c[k];
          }
          if (st[i].kind == K_MULT) st[i].kind = K_GENERIC;
        }
        st[i].pending = 1;
        st[i].cur >>= 1;
        st[i].vars--;
      }
      ++seq;
      publish_flag(p.to_host, seq);
      const volatile uint32_t* fh = p.from_host;
      const long long t0 = clock64();
      bool ok = false;
      while (clock64() - t0 < TAIL_WAIT_CYCLES) {
        const uint32_t v = fh[0];
        if (v == seq) {
          ok = true;
          break;
        }
        if (v == TAIL_ABORT) break;  // the host gave up on this proof
        __nanosleep(128);
      }
      if (ok) {
        __threadfence_system();
        s_chal = qm31_from_u32(fh[1], fh[2], fh[3], fh[4]);
      } else {
        s_abort = 1;
        reinterpret_cast<volatile uint32_t*>(p.to_host)[1] = 1u;
      }
    }
    __syncthreads();
    if (s_abort) return;
  }
  // Masks of the constant oracles, folded with the last challenge.
  const qm31 c = s_chal;
  for (uint32_t i = 0; i < p.n_inst; i++) {
    switch (st[i].kind) {
      case K_GP: tail_gates<K_GP>(st[i], c, st[i].out); break;
      case K_GENERIC: tail_gates<K_GENERIC>(st[i], c, st[i].out); break;
      case K_MULT: tail_gates<K_MULT>(st[i], c, st[i].out); break;
      default: tail_gates<K_SINGLES>(st[i], c, st[i].out); break;
    }
  }
  __threadfence_system();
  __syncthreads();
  if (threadIdx.x == 0) publish_flag(p.to_host, seq + 1);
}

// ------------------------------------------------------------------------------ MleOps
// cpu/lookups/mle.rs:11-40: out[i] = fold(a, in[i], in[i + h]); out may alias a secure input.
__global__ void __launch_bounds__(256) k_mle_fix_secure(Sec in, SecM out, qm31 a, uint32_t h) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < h; i += (size_t)gridDim.x * blockDim.x)
    stq(out, i, fold(a, ldq(in, i), ldq(in, i + h)));
}
__global__ void __launch_bounds__(256) k_mle_fix_base(const uint32_t* in, SecM out, qm31 a, uint32_t h) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < h; i += (size_t)gridDim.x * blockDim.x)
    stq(out, i, fold_base(a, in[i], in[i + h]));
}

// ------------------------------------------------------------------------------ host helpers
qm31 to_q(stwo_qm31 a) { return {{a.v[0], a.v[1]}, {a.v[2], a.v[3]}}; }
qm31 to_q(hq a) { return {{a.v[0], a.v[1]}, {a.v[2], a.v[3]}}; }
hq hq_of_words(const uint32_t* w) { return hq_make(w[0], w[1], w[2], w[3]); }
bool hq_is_zero(hq a) { return !(a.v[0] | a.v[1] | a.v[2] | a.v[3]); }
bool hq_eq(hq a, hq b) { return !std::memcmp(a.v, b.v, 16); }
const hq HQ_ONE = hq_make(1, 0, 0, 0);
const hq HQ_ZERO = hq_make(0, 0, 0, 0);
const qm31 QZ = {{0u, 0u}, {0u, 0u}};

uint32_t grid_for(size_t n, uint32_t threads, uint32_t cap) {
  size_t g = (n + threads - 1) / threads;
  return (uint32_t)std::max<size_t>(1, std::min<size_t>(g, cap));
}
uint32_t round_grid(uint32_t nt) { return grid_for(nt, 256, 4u * (uint32_t)sm_count()); }
constexpr uint32_t MAX_ROUND_BLOCKS = 4096;

Sec sec_of(const uint32_t* const p[4]) { return Sec{{p[0], p[1], p[2], p[3]}}; }
SecM secm_of(uint32_t* const p[4]) { return SecM{{p[0], p[1], p[2], p[3]}}; }
Sec as_const(const SecM& s) { return Sec{{s.c[0], s.c[1], s.c[2], s.c[3]}}; }
Cols as_const(const ColsM& s) { return Cols{as_const(s.num), as_const(s.den)}; }

// eq(x, y) over equal-length slices (utils.rs:160-167).
hq h_eq(const hq* x, const hq* y, size_t n) {
  hq r = HQ_ONE;
  for (size_t i = 0; i < n; i++)
    r = hq_mul(r, hq_add(hq_mul(x[i], y[i]), hq_mul(hq_sub(HQ_ONE, x[i]), hq_sub(HQ_ONE, y[i]))));
  return r;
}

// UnivariatePoly with the reference's length semantics (utils.rs:12-150): constructors and
// products drop leading zeros, sums keep the longer length.
using HPoly = std::vector<hq>;
void hp_trunc(HPoly& p) {
  while (!p.empty() && hq_is_zero(p.back())) p.pop_back();
}
hq hp_eval(const HPoly& p, hq x) {
  hq acc = HQ_ZERO;
  for (size_t i = p.size(); i-- > 0;) acc = hq_add(hq_mul(acc, x), p[i]);
  return acc;
}
HPoly hp_add(const HPoly& a, const HPoly& b) {
  HPoly r(std::max(a.size(), b.size()));
  for (size_t i = 0; i < r.size(); i++) {
    if (i < a.size() && i < b.size()) r[i] = hq_add(a[i], b[i]);
    else r[i] = i < a.size() ? a[i] : b[i];
  }
  return r;
}
HPoly hp_scale(HPoly a, hq s) {
  for (auto& c : a) c = hq_mul(c, s);
  return a;
}
HPoly hp_new(HPoly p) {
  hp_trunc(p);
  return p;
}
// gkr_prover.rs:527-566. The round polynomial interpolates (0, r0), (1, r1), (2, r2), (b, 0); the
// interpolant is unique, so the Lagrange basis on {0, 1, 2, b} expanded in closed form gives the
// reference's coefficients (leading zeros dropped) with two batched inversions.
int32_t correct_sum(hq f0, hq f2, hq claim, const std::vector<hq>& y, size_t k, HPoly& out) {
  const size_t n = y.size();
  STWO_REQUIRE(k != 0 && k <= n, "sum_as_poly: %zu variables with %zu eq coordinates", k, n);
  hq prod = HQ_ONE;  // eq(0^(n-k+1), y[..n-k+1])
  for (size_t j = 0; j <= n - k; j++) prod = hq_mul(prod, hq_sub(HQ_ONE, y[j]));
  const hq yk = y[n - k];
  const hq omy = hq_sub(HQ_ONE, yk);
  const hq bden = hq_sub(HQ_ONE, hq_add(yk, yk));
  const hq t = hq_mul(prod, bden);
  if (hq_is_zero(t)) {
    set_error("sum_as_poly: zero has no inverse");
    return STWO_ERR_INVALID_ARG;
  }
  const hq ti = hq_inv(t);
  const hq a = hq_mul(ti, bden);
  const hq b = hq_mul(omy, hq_mul(ti, prod));
  const hq two = hq_make(2, 0, 0, 0), three = hq_make(3, 0, 0, 0);
  const hq r0 = hq_mul(hq_mul(f0, omy), a);
  const hq r1 = hq_sub(claim, r0);
  const hq r2 = hq_mul(hq_mul(f2, hq_sub(hq_mul(three, yk), HQ_ONE)), a);  // eq([2], [yk]) = 3 yk - 1
  const hq bm1 = hq_sub(b, HQ_ONE), tmb = hq_sub(two, b);
  const hq p1 = hq_mul(b, bm1), p2 = hq_mul(p1, tmb);
  if (hq_is_zero(p2)) {
    set_error("sum_as_poly: zero has no inverse");
    return STWO_ERR_INVALID_ARG;
  }
  const hq ip2 = hq_inv(p2), ip1 = hq_mul(ip2, tmb);
  const hq inv_b = hq_mul(ip1, bm1), inv_bm1 = hq_mul(ip1, b), inv_tmb = hq_mul(ip2, p1);
  const hq half = hq_make((P + 1) / 2, 0, 0, 0);
  const hq A = hq_sub(HQ_ZERO, hq_mul(hq_mul(r0, inv_b), half));  // r0 / (-2b)
  const hq B = hq_mul(r1, inv_bm1);                              // r1 / (b - 1)
  const hq Cc = hq_mul(hq_mul(r2, inv_tmb), half);               // r2 / (2 (2 - b))
  const hq b2 = hq_add(b, b), b3 = hq_add(b2, b);
  out.assign(4, HQ_ZERO);
  out[3] = hq_add(hq_add(A, B), Cc);
  out[2] = hq_sub(HQ_ZERO, hq_add(hq_add(hq_mul(hq_add(three, b), A), hq_mul(hq_add(two, b), B)),
                                  hq_mul(hq_add(HQ_ONE, b), Cc)));
  out[1] = hq_add(hq_add(hq_mul(hq_add(two, b3), A), hq_mul(b2, B)), hq_mul(b, Cc));
  out[0] = r0;
  hp_trunc(out);
  return STWO_OK;
}

int32_t launch_next_layer(uint32_t kind, const Cols& in, const ColsM& out, uint32_t n_out, cudaStream_t s) {
  uint32_t g = grid_for(n_out, 256, 16u * (uint32_t)sm_count());
  switch (kind) {
    case K_GP: k_next_layer<K_GP><<<g, 256, 0, s>>>(in, out, n_out); break;
    case K_GENERIC: k_next_layer<K_GENERIC><<<g, 256, 0, s>>>(in, out, n_out); break;
    case K_MULT: k_next_layer<K_MULT><<<g, 256, 0, s>>>(in, out, n_out); break;
    default: k_next_layer<K_SINGLES><<<g, 256, 0, s>>>(in, out, n_out); break;
  }
  note_launch();
  STWO_LAUNCH_CHECK();
  return STWO_OK;
}

template <bool FIX>
void round_dispatch(uint32_t kind, const Cols& src, const ColsM& dst, qm31 c, uint32_t cur, const Sec& eq, qm31 lam,
                    const RoundOut& ro, cudaStream_t s) {
  uint32_t g = round_grid(cur / 4);
  switch (kind) {
    case K_GP: k_gkr_round<K_GP, FIX><<<g, 256, 0, s>>>(src, dst, c, cur, eq, lam, ro); break;
    case K_GENERIC: k_gkr_round<K_GENERIC, FIX><<<g, 256, 0, s>>>(src, dst, c, cur, eq, lam, ro); break;
    case K_MULT: k_gkr_round<K_MULT, FIX><<<g, 256, 0, s>>>(src, dst, c, cur, eq, lam, ro); break;
    default: k_gkr_round<K_SINGLES, FIX><<<g, 256, 0, s>>>(src, dst, c, cur, eq, lam, ro); break;
  }
  note_launch();
}

template <bool FIX>
void gates_dispatch(uint32_t kind, const Cols& src, const ColsM& dst, qm31 c, uint32_t cur, uint32_t* out,
                    cudaStream_t s, uint32_t* flag = nullptr, uint32_t seq = 0) {
  switch (kind) {
    case K_GP: k_gkr_gates<K_GP, FIX><<<1, 32, 0, s>>>(src, dst, c, cur, out, flag, seq); break;
    case K_GENERIC: k_gkr_gates<K_GENERIC, FIX><<<1, 32, 0, s>>>(src, dst, c, cur, out, flag, seq); break;
    case K_MULT: k_gkr_gates<K_MULT, FIX><<<1, 32, 0, s>>>(src, dst, c, cur, out, flag, seq); break;
    default: k_gkr_gates<K_SINGLES, FIX><<<1, 32, 0, s>>>(src, dst, c, cur, out, flag, seq); break;
  }
  note_launch();
}

// Waits until a kernel publishes `seq` in the mapped word `flag`: a host spin of about a
// microsecond per round instead of a stream synchronisation. Bounded: a stream error, or no flag
// after 30 s, ends the wait with an error.
int32_t wait_flag(const uint32_t* flag, uint32_t seq, cudaStream_t s) {
  const volatile uint32_t* f = flag;
  const auto t0 = std::chrono::steady_clock::now();
  for (uint64_t it = 1;; it++) {
    if (*f == seq) {
      std::atomic_thread_fence(std::memory_order_acquire);
      return STWO_OK;
    }
    if ((it & 4095) == 0) {
      cudaError_t e = cudaStreamQuery(s);
      if (e != cudaSuccess && e != cudaErrorNotReady) {
        set_error("GKR round: %s", cudaGetErrorString(e));
        return STWO_ERR_CUDA;
      }
      if (e == cudaSuccess && *f != seq) {
        set_error("GKR round: stream finished without publishing its result");
        return STWO_ERR_CUDA;
      }
      if (std::chrono::steady_clock::now() - t0 > std::chrono::seconds(30)) {
        set_error("GKR round: no result after 30 s");
        return STWO_ERR_TIMEOUT;
      }
    }
  }
}

int32_t launch_eq_evals(const std::vector<hq>& y, hq v, const SecM& out, cudaStream_t s) {
  STWO_REQUIRE(y.size() <= 30, "gen_eq_evals: %zu coordinates (at most 30)", y.size());
  EqParams p{};
  for (size_t i = 0; i < y.size(); i++) p.y[i] = to_q(y[i]);
  p.v = to_q(v);
  p.n_y = (uint32_t)y.size();
  p.lo_bits = std::min<uint32_t>(p.n_y, EQ_LO_BITS);
  uint32_t rows = 1u << (p.n_y - p.lo_bits);
  k_eq_evals<<<(rows + EQ_ROWS - 1) / EQ_ROWS, 256, 0, s>>>(p, out);
  note_launch();
  STWO_LAUNCH_CHECK();
  return STWO_OK;
}

bool valid_kind(uint32_t k) { return k <= K_SINGLES; }

// ------------------------------------------------------------------------------ prove_batch
struct Layer {
  uint32_t kind;
  Cols cols;
};

struct Instance {
  uint32_t n_vars = 0;
  std::vector<Layer> layers;  // layers[v]: the circuit layer with v variables (2^v gates)
  SecM work_num{}, work_den{};
  // Sum-check oracle state.
  Cols src{};
  uint32_t kind = 0, cur = 0, oracle_vars = 0;
  bool fix_pending = false;
  hq pending{}, correction{}, claim{};
  bool active = false;
  std::vector<hq> claims_to_verify;
  std::vector<hq> output_claims;
  std::vector<std::vector<hq>> masks;  // flattened per layer
};

struct Writer {
  std::vector<uint8_t>& b;
  void u64(uint64_t v) {
    for (int i = 0; i < 8; i++) b.push_back((uint8_t)(v >> (8 * i)));
  }
  void q(const hq& x) {
    for (int k = 0; k < 4; k++)
      for (int i = 0; i < 4; i++) b.push_back((uint8_t)(x.v[k] >> (8 * i)));
  }
  void qs(const std::vector<hq>& v) {
    u64(v.size());
    for (auto& x : v) q(x);
  }
};

int32_t prove_batch(uint32_t n_inst, const uint32_t* kinds, const uint32_t* logs, const uint32_t* const* num,
                    const uint32_t* const* den, const uint8_t* digest_in, std::vector<uint8_t>& bytes,
                    uint8_t* digest_out, cudaStream_t s) {
  STWO_REQUIRE(n_inst >= 1 && kinds && logs, "prove_batch: no instances");
  for (uint32_t i = 0; i < n_inst; i++) {
    STWO_REQUIRE(kinds[i] == K_SINGLES || num, "prove_batch: null numerator table");
    STWO_REQUIRE(kinds[i] == K_GP || den, "prove_batch: null denominator table");
  }
  std::vector<Instance> inst(n_inst);
  uint32_t n_layers = 0;
  size_t arena_words = 0;
  for (uint32_t i = 0; i < n_inst; i++) {
    STWO_REQUIRE(valid_kind(kinds[i]), "prove_batch: instance %u has unknown layer kind %u", i, kinds[i]);
    STWO_REQUIRE(logs[i] >= 1 && logs[i] <= 28, "prove_batch: instance %u has %u variables (1..28)", i, logs[i]);
    // try_into_mask has no multiplicities case (gkr_prover.rs:336-337).
    STWO_REQUIRE(!(kinds[i] == K_MULT && logs[i] == 1), "prove_batch: a one-variable multiplicities layer has no mask");
    inst[i].n_vars = logs[i];
    n_layers = std::max(n_layers, logs[i]);
    size_t w = kinds[i] == K_GP ? 4 : 8;
    arena_words += w * ((size_t)1 << logs[i]);        // generated layers: 2^n - 1 gates, padded
    arena_words += w * ((size_t)1 << (logs[i] - 1));  // sum-check work buffer
  }
  const size_t eq_words = 4 * ((size_t)1 << (n_layers > 1 ? n_layers - 1 : 0));
  const size_t scratch_words = 8 * (size_t)MAX_ROUND_BLOCKS + 64;
  uint32_t* arena = nullptr;
  int32_t st = scratch_alloc((void**)&arena, (arena_words + eq_words + scratch_words) * 4, s);
  if (st) return st;
  struct Free {
    uint32_t* p;
    cudaStream_t s;
    ~Free() { scratch_free(p, s); }
  } guard{arena, s};
  uint32_t* cursor = arena;
  auto take = [&](size_t words) {
    uint32_t* p = cursor;
    cursor += words;
    return p;
  };
  auto take_sec = [&](size_t n) {
    SecM m;
    for (int c = 0; c < 4; c++) m.c[c] = take(n);
    return m;
  };
  SecM eq = take_sec(eq_words / 4);
  RoundOut ro{take(8 * (size_t)MAX_ROUND_BLOCKS), nullptr, nullptr};
  ro.ticket = reinterpret_cast<unsigned int*>(take(64));
  STWO_CHECK_CUDA(cudaMemsetAsync(ro.ticket, 0, 4, s));

  Mapped mp;
  st = mapped_words((size_t)n_inst * 24 + 8, mp);
  if (st) return st;
  // Completion flag (and error word) of the round and mask kernels, polled by the host
  // (wait_flag), and the host-to-device challenge mailbox of the tail kernel.
  uint32_t* const flag_dev = mp.dev + (size_t)n_inst * 24;
  const uint32_t* const flag_host = mp.host + (size_t)n_inst * 24;
  uint32_t* const mailbox_host = mp.host + (size_t)n_inst * 24 + 2;
  const uint32_t* const mailbox_dev = mp.dev + (size_t)n_inst * 24 + 2;
  for (int k = 0; k < 8; k++) mp.host[(size_t)n_inst * 24 + k] = 0;
  uint32_t seq = 0;

  // Circuit layers (gen_layers, gkr_prover.rs:508-516): layers[n] is the caller's input.
  for (uint32_t i = 0; i < n_inst; i++) {
    Instance& I = inst[i];
    I.layers.resize(I.n_vars + 1);
    Layer in{kinds[i], {}};
    const bool has_num = kinds[i] != K_SINGLES;
    for (int c = 0; c < 4; c++) {
      in.cols.num.c[c] = has_num ? num[4 * (size_t)i + (kinds[i] == K_MULT ? 0 : c)] : nullptr;
      in.cols.den.c[c] = kinds[i] == K_GP ? nullptr : den[4 * (size_t)i + c];
    }
    STWO_REQUIRE(!has_num || in.cols.num.c[0], "prove_batch: instance %u has no numerator column", i);
    STWO_REQUIRE(kinds[i] == K_GP || in.cols.den.c[0], "prove_batch: instance %u has no denominator column", i);
    if (has_num && kinds[i] != K_MULT)
      for (int c = 1; c < 4; c++) STWO_REQUIRE(in.cols.num.c[c], "prove_batch: instance %u numerator coordinate", i);
    if (kinds[i] != K_GP)
      for (int c = 1; c < 4; c++) STWO_REQUIRE(in.cols.den.c[c], "prove_batch: instance %u denominator coordinate", i);
    I.layers[I.n_vars] = in;
    const uint32_t next_kind = kinds[i] == K_GP ? K_GP : K_GENERIC;
    for (uint32_t v = I.n_vars; v-- > 0;) {
      ColsM out{take_sec((size_t)1 << v), {}};
      if (next_kind != K_GP) out.den = take_sec((size_t)1 << v);
      st = launch_next_layer(I.layers[v + 1].kind, I.layers[v + 1].cols, out, 1u << v, s);
      if (st) return st;
      I.layers[v] = Layer{next_kind, as_const(out)};
    }
    const size_t half = (size_t)1 << (I.n_vars - 1);
    I.work_num = take_sec(half);
    if (next_kind != K_GP) I.work_den = take_sec(half);
    // Output layer values (gkr_prover.rs:137-164).
    gates_dispatch<false>(I.layers[0].kind, I.layers[0].cols, ColsM{}, QZ, 1, mp.dev + 24 * i, s);
  }
  STWO_LAUNCH_CHECK();
  STWO_CHECK_CUDA(cudaStreamSynchronize(s));
  for (uint32_t i = 0; i < n_inst; i++) {
    const uint32_t* o = mp.host + 24 * i;
    if (inst[i].layers[0].kind == K_GP) inst[i].output_claims = {hq_of_words(o)};
    else inst[i].output_claims = {hq_of_words(o), hq_of_words(o + 8)};
  }

  HostChannel ch;
  if (digest_in) std::memcpy(ch.digest.b, digest_in, 32);
  std::vector<hq> ood;
  const hq half_inv = hq_make(h_inv(2), 0, 0, 0);
  std::vector<HPoly> proofs_round;  // flattened: per GKR layer, the rounds' polynomials
  std::vector<size_t> rounds_per_layer;

  for (uint32_t L = 0; L < n_layers; L++) {
    const uint32_t remaining = n_layers - L;
    for (auto& I : inst)
      if (I.n_vars == remaining) {
        I.claims_to_verify = I.output_claims;
        I.active = true;
      }
    for (auto& I : inst)
      if (I.active) ch.mix_felts(I.claims_to_verify);
    // EqEvals::generate (gkr_prover.rs:58-69).
    const std::vector<hq> y = ood;
    // With no coordinates every oracle is already constant and the evaluations go unused.
    if (!y.empty()) {
      std::vector<hq> rest(y.begin() + 1, y.end());
      hq zero = HQ_ZERO;
      st = launch_eq_evals(rest, h_eq(&zero, &y[0], 1), eq, s);
      if (st) return st;
    }
    const hq alpha = ch.draw_felt();
    const hq lambda = ch.draw_felt();
    std::vector<uint32_t> act;
    for (uint32_t i = 0; i < n_inst; i++)
      if (inst[i].active) act.push_back(i);
    // Sum-check over the active oracles (sumcheck.rs:62-126).
    uint32_t sc_vars = 0;
    for (uint32_t i : act) {
      Instance& I = inst[i];
      const uint32_t lv = I.n_vars - remaining + 1;  // variables of the layer this oracle reads
      const Layer& lay = I.layers[lv];
      I.src = lay.cols;
      I.kind = lay.kind;
      I.cur = 1u << lv;
      I.oracle_vars = lv - 1;
      I.fix_pending = false;
      I.correction = HQ_ONE;
      hq c = HQ_ZERO;
      for (size_t k = I.claims_to_verify.size(); k-- > 0;) c = hq_add(hq_mul(c, lambda), I.claims_to_verify[k]);
      I.claim = c;
      sc_vars = std::max(sc_vars, I.oracle_vars);
    }
    for (uint32_t i : act) {
      Instance& I = inst[i];
      I.claim = hq_mul(I.claim, hq_make((uint32_t)((1ull << (sc_vars - I.oracle_vars)) % P), 0, 0, 0));
    }
    std::vector<hq> assignment;
    bool tail_on = false;
    // On a failure while the tail kernel waits for a challenge, release it and let it end.
    auto abort_tail = [&](int32_t code) {
      if (tail_on) {
        *reinterpret_cast<volatile uint32_t*>(mailbox_host) = TAIL_ABORT;
        cudaStreamSynchronize(s);
      }
      return code;
    };
    for (uint32_t r = 0; r < sc_vars; r++) {
      const uint32_t rem = sc_vars - r;
      size_t last_live = act.size();
      for (size_t a = 0; a < act.size(); a++)
        if (inst[act[a]].oracle_vars == rem) last_live = a;
      const bool any = last_live < act.size();
      if (!tail_on && act.size() <= TAIL_MAXI && sc_vars - r >= 2) {
        uint32_t biggest = 0;
        for (uint32_t i : act) biggest = std::max(biggest, inst[i].cur);
        if (biggest <= TAIL_MAX_GATES) {
          // The remaining rounds and the masks of this layer run in the resident tail kernel.
          TailParams tp{};
          tp.n_inst = (uint32_t)act.size();
          tp.sc_vars = sc_vars;
          tp.r0 = r;
          for (size_t a = 0; a < act.size(); a++) {
            const Instance& I = inst[act[a]];
            tp.inst[a] = TailInst{I.kind, I.oracle_vars, I.cur, I.fix_pending ? 1u : 0u, I.src,
                                  ColsM{I.work_num, I.work_den}, mp.dev + 24 * act[a]};
            if (I.fix_pending) tp.chal0 = to_q(I.pending);
          }
          tp.eq = as_const(eq);
          tp.lambda = to_q(lambda);
          tp.to_host = flag_dev;
          tp.from_host = mailbox_dev;
          tp.seq0 = seq;
          mailbox_host[0] = 0;
          std::atomic_thread_fence(std::memory_order_release);
          k_gkr_tail<<<1, TAIL_THREADS, 0, s>>>(tp);
          note_launch();
          STWO_LAUNCH_CHECK();
          tail_on = true;
        }
      }
      if (any) seq++;
      for (size_t a = 0; a < act.size() && tail_on; a++) {
        // Mirror of the tail kernel's bookkeeping: a live pending layer is folded this round.
        Instance& I = inst[act[a]];
        if (I.oracle_vars != rem || !I.fix_pending) continue;
        if (I.kind == K_MULT) I.kind = K_GENERIC;
        I.fix_pending = false;
      }
      for (size_t a = 0; a < act.size() && !tail_on; a++) {
        Instance& I = inst[act[a]];
        if (I.oracle_vars != rem) continue;
        RoundOut o = ro;
        o.result = mp.dev + 24 * act[a];
        if (a == last_live) {
          o.flag = flag_dev;
          o.seq = seq;
        }
        ColsM dst{I.work_num, I.work_den};
        if (I.fix_pending) {
          round_dispatch<true>(I.kind, I.src, dst, to_q(I.pending), I.cur, as_const(eq), to_q(lambda), o, s);
          I.src = as_const(dst);
          if (I.kind == K_MULT) I.kind = K_GENERIC;
          I.fix_pending = false;
        } else {
          round_dispatch<false>(I.kind, I.src, dst, QZ, I.cur, as_const(eq), to_q(lambda), o, s);
        }
      }
      if (any) {
        STWO_LAUNCH_CHECK();
        st = wait_flag(flag_host, seq, s);
        if (st) return abort_tail(st);
      }
      std::vector<HPoly> polys;
      for (size_t a = 0; a < act.size(); a++) {
        Instance& I = inst[act[a]];
        HPoly p;
        if (I.oracle_vars == rem) {
          const uint32_t* w = mp.host + 24 * act[a];
          hq f0 = hq_mul(hq_of_words(w), I.correction), f2 = hq_mul(hq_of_words(w + 4), I.correction);
          st = correct_sum(f0, f2, I.claim, y, I.oracle_vars, p);
          if (st) return abort_tail(st);
        } else {
          p = hp_new({hq_mul(I.claim, half_inv)});
        }
        if (!hq_eq(hq_add(hp_eval(p, HQ_ZERO), hp_eval(p, HQ_ONE)), I.claim) || p.size() > 4) {
          set_error("prove_batch: round polynomial inconsistent with its claim (instance %u, round %u)", act[a], r);
          return abort_tail(STWO_ERR_CUDA);
        }
        polys.push_back(std::move(p));
      }
      HPoly comb;
      for (size_t k = polys.size(); k-- > 0;) comb = hp_add(hp_scale(comb, alpha), polys[k]);
      ch.mix_felts(comb);
      const hq chal = ch.draw_felt();
      if (tail_on) {
        for (int k = 0; k < 4; k++) mailbox_host[1 + k] = chal.v[k];
        std::atomic_thread_fence(std::memory_order_release);
        *reinterpret_cast<volatile uint32_t*>(mailbox_host) = seq;
      }
      for (size_t a = 0; a < act.size(); a++) {
        Instance& I = inst[act[a]];
        I.claim = hp_eval(polys[a], chal);
        if (I.oracle_vars == rem) {
          const hq z0 = y[y.size() - I.oracle_vars];
          I.correction = hq_mul(I.correction, h_eq(&chal, &z0, 1));
          I.pending = chal;
          I.fix_pending = true;
          I.cur >>= 1;
          I.oracle_vars--;
        }
      }
      proofs_round.push_back(std::move(comb));
      assignment.push_back(chal);
    }
    rounds_per_layer.push_back(sc_vars);
    // Masks of the now constant oracles (gkr_prover.rs:320-346).
    seq++;
    for (size_t a = 0; a < act.size() && tail_on; a++) {
      Instance& I = inst[act[a]];
      if (I.fix_pending && I.kind == K_MULT) I.kind = K_GENERIC;
    }
    for (size_t a = 0; a < act.size() && !tail_on; a++) {
      Instance& I = inst[act[a]];
      ColsM dst{I.work_num, I.work_den};
      uint32_t* f = a + 1 == act.size() ? flag_dev : nullptr;
      if (I.fix_pending) gates_dispatch<true>(I.kind, I.src, dst, to_q(I.pending), 2, mp.dev + 24 * act[a], s, f, seq);
      else gates_dispatch<false>(I.kind, I.src, dst, QZ, 2, mp.dev + 24 * act[a], s, f, seq);
      if (I.fix_pending && I.kind == K_MULT) I.kind = K_GENERIC;
    }
    STWO_LAUNCH_CHECK();
    st = wait_flag(flag_host, seq, s);
    if (st) return abort_tail(st);
    for (size_t a = 0; a < act.size(); a++) {
      Instance& I = inst[act[a]];
      const uint32_t* w = mp.host + 24 * act[a];
      std::vector<hq> flat;
      if (I.kind == K_GP) {
        flat = {hq_of_words(w), hq_of_words(w + 4)};
      } else {
        hq n0 = hq_of_words(w), n1 = hq_of_words(w + 4);
        if (I.kind == K_SINGLES) n0 = n1 = HQ_ONE;
        flat = {n0, n1, hq_of_words(w + 8), hq_of_words(w + 12)};
      }
      ch.mix_felts(flat);
      I.masks.push_back(flat);
    }
    const hq chal = ch.draw_felt();
    ood = assignment;
    ood.push_back(chal);
    for (size_t a = 0; a < act.size(); a++) {
      Instance& I = inst[act[a]];
      const std::vector<hq>& m = I.masks.back();
      I.claims_to_verify.clear();
      for (size_t c = 0; c + 1 < m.size(); c += 2)
        I.claims_to_verify.push_back(hq_add(hq_mul(chal, hq_sub(m[c + 1], m[c])), m[c]));
    }
  }

  // Canonical bytes: the proof, then the artifact.
  bytes.clear();
  Writer w{bytes};
  w.u64(n_layers);
  size_t pos = 0;
  for (uint32_t L = 0; L < n_layers; L++) {
    w.u64(rounds_per_layer[L]);
    for (size_t r = 0; r < rounds_per_layer[L]; r++) w.qs(proofs_round[pos++]);
  }
  w.u64(n_inst);
  for (auto& I : inst) {
    w.u64(I.masks.size());
    for (auto& m : I.masks) {
      w.u64(m.size() / 2);
      for (auto& x : m) w.q(x);
    }
  }
  w.u64(n_inst);
  for (auto& I : inst) w.qs(I.output_claims);
  w.qs(ood);
  w.u64(n_inst);
  for (auto& I : inst) w.qs(I.claims_to_verify);
  w.u64(n_inst);
  for (auto& I : inst) w.u64(I.n_vars);
  if (digest_out) std::memcpy(digest_out, ch.digest.b, 32);
  return STWO_OK;
}

}  // namespace
}  // namespace stwo

using namespace stwo;

extern "C" {

stwo_status stwo_gkr_gen_eq_evals(const stwo_qm31* h_y, uint32_t n_y, stwo_qm31 v, uint32_t* const d_out[4],
                                  void* stream) {
  STWO_REQUIRE(d_out && d_out[0] && d_out[1] && d_out[2] && d_out[3], "gen_eq_evals: null output");
  STWO_REQUIRE(n_y == 0 || h_y, "gen_eq_evals: null y");
  std::vector<hq> y(n_y);
  for (uint32_t i = 0; i < n_y; i++) y[i] = hq_from(h_y[i]);
  return launch_eq_evals(y, hq_from(v), secm_of(d_out), as_stream(stream));
}

stwo_status stwo_gkr_next_layer(uint32_t kind, uint32_t log_n, const uint32_t* const d_num[4],
                                const uint32_t* const d_den[4], uint32_t* const d_next_num[4],
                                uint32_t* const d_next_den[4], void* stream) {
  STWO_REQUIRE(valid_kind(kind), "next_layer: unknown layer kind %u", kind);
  STWO_REQUIRE(log_n >= 1 && log_n <= 30, "next_layer: log size %u (output layers have no next layer)", log_n);
  STWO_REQUIRE(d_next_num, "next_layer: null output");
  Cols in{};
  ColsM out{secm_of(d_next_num), {}};
  if (kind != K_SINGLES) {
    STWO_REQUIRE(d_num && d_num[0], "next_layer: null numerators");
    in.num = kind == K_MULT ? Sec{{d_num[0], nullptr, nullptr, nullptr}} : sec_of(d_num);
  }
  if (kind != K_GP) {
    STWO_REQUIRE(d_den && d_next_den, "next_layer: null denominators");
    in.den = sec_of(d_den);
    out.den = secm_of(d_next_den);
  }
  return launch_next_layer(kind, in, out, 1u << (log_n - 1), as_stream(stream));
}

stwo_status stwo_gkr_sum_as_poly_in_first_variable(uint32_t kind, uint32_t log_n, const uint32_t* const d_num[4],
                                                   const uint32_t* const d_den[4],
                                                   const uint32_t* const d_eq_evals[4], const stwo_qm31* h_y,
                                                   uint32_t n_y, stwo_qm31 lambda,
                                                   stwo_qm31 eq_fixed_var_correction, stwo_qm31 claim,
                                                   stwo_qm31* h_coeffs, uint32_t* h_n_coeffs, void* stream) {
  STWO_REQUIRE(valid_kind(kind), "sum_as_poly: unknown layer kind %u", kind);
  STWO_REQUIRE(log_n >= 2 && log_n <= 30, "sum_as_poly: layer of %u variables (needs 2..30)", log_n);
  STWO_REQUIRE(log_n - 1 <= n_y && (n_y == 0 || h_y), "sum_as_poly: %u eq coordinates for %u variables", n_y,
               log_n - 1);
  STWO_REQUIRE(d_eq_evals && h_coeffs && h_n_coeffs, "sum_as_poly: null argument");
  cudaStream_t s = as_stream(stream);
  Cols in{};
  if (kind != K_SINGLES) {
    STWO_REQUIRE(d_num && d_num[0], "sum_as_poly: null numerators");
    in.num = kind == K_MULT ? Sec{{d_num[0], nullptr, nullptr, nullptr}} : sec_of(d_num);
  }
  if (kind != K_GP) {
    STWO_REQUIRE(d_den, "sum_as_poly: null denominators");
    in.den = sec_of(d_den);
  }
  uint32_t* buf = nullptr;
  int32_t st = scratch_alloc((void**)&buf, (8 * (size_t)MAX_ROUND_BLOCKS + 64 + 8) * 4, s);
  if (st) return st;
  RoundOut ro{buf, reinterpret_cast<unsigned int*>(buf + 8 * (size_t)MAX_ROUND_BLOCKS),
              buf + 8 * (size_t)MAX_ROUND_BLOCKS + 64};
  uint32_t res[8];
  cudaError_t e = cudaMemsetAsync(ro.ticket, 0, 4, s);
  if (e == cudaSuccess) {
    round_dispatch<false>(kind, in, ColsM{}, QZ, 1u << log_n, sec_of(d_eq_evals), to_q(lambda), ro, s);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(res, ro.result, 32, cudaMemcpyDeviceToHost, s);
  scratch_free(buf, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    set_error("sum_as_poly: %s", cudaGetErrorString(e));
    return STWO_ERR_CUDA;
  }
  std::vector<hq> y(n_y);
  for (uint32_t i = 0; i < n_y; i++) y[i] = hq_from(h_y[i]);
  hq corr = hq_from(eq_fixed_var_correction);
  HPoly p;
  st = correct_sum(hq_mul(hq_of_words(res), corr), hq_mul(hq_of_words(res + 4), corr), hq_from(claim), y, log_n - 1,
                   p);
  if (st) return st;
  for (size_t i = 0; i < p.size(); i++)
    for (int k = 0; k < 4; k++) h_coeffs[i].v[k] = p[i].v[k];
  *h_n_coeffs = (uint32_t)p.size();
  return STWO_OK;
}

stwo_status stwo_mle_fix_first_variable_base(uint32_t log_n, const uint32_t* d_mle, stwo_qm31 assignment,
                                             uint32_t* const d_out[4], void* stream) {
  STWO_REQUIRE(log_n >= 1 && log_n <= 31, "fix_first_variable: log size %u", log_n);
  STWO_REQUIRE(d_mle && d_out, "fix_first_variable: null argument");
  uint32_t h = 1u << (log_n - 1);
  k_mle_fix_base<<<grid_for(h, 256, 16u * (uint32_t)sm_count()), 256, 0, as_stream(stream)>>>(
      d_mle, secm_of(d_out), to_q(assignment), h);
  note_launch();
  STWO_LAUNCH_CHECK();
  return STWO_OK;
}

stwo_status stwo_mle_fix_first_variable_secure(uint32_t log_n, const uint32_t* const d_mle[4], stwo_qm31 assignment,
                                               uint32_t* const d_out[4], void* stream) {
  STWO_REQUIRE(log_n >= 1 && log_n <= 31, "fix_first_variable: log size %u", log_n);
  STWO_REQUIRE(d_mle && d_out, "fix_first_variable: null argument");
  uint32_t h = 1u << (log_n - 1);
  k_mle_fix_secure<<<grid_for(h, 256, 16u * (uint32_t)sm_count()), 256, 0, as_stream(stream)>>>(
      sec_of(d_mle), secm_of(d_out), to_q(assignment), h);
  note_launch();
  STWO_LAUNCH_CHECK();
  return STWO_OK;
}

stwo_status stwo_gkr_prove_batch(uint32_t n_instances, const uint32_t* h_kinds, const uint32_t* h_log_sizes,
                                 const uint32_t* const* h_num, const uint32_t* const* h_den,
                                 const uint8_t* h_digest_in, uint8_t* h_out, size_t capacity, size_t* h_len,
                                 uint8_t* h_digest_out, void* stream) {
  STWO_REQUIRE(h_out && h_len, "prove_batch: null output");
  std::vector<uint8_t> bytes;
  int32_t st = prove_batch(n_instances, h_kinds, h_log_sizes, h_num, h_den, h_digest_in, bytes, h_digest_out,
                           as_stream(stream));
  if (st) return st;
  *h_len = bytes.size();
  STWO_REQUIRE(bytes.size() <= capacity, "prove_batch: proof needs %zu bytes, buffer holds %zu", bytes.size(),
               capacity);
  std::memcpy(h_out, bytes.data(), bytes.size());
  return STWO_OK;
}

}  // extern "C"
