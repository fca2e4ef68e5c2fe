// QuotientOps::accumulate_quotients.
//
// Per row (crates/prover/src/core/backend/cpu/quotients.rs:43-76):
//   acc = sum over batches k, in BTreeMap order:  acc * batch_coeff_k + num_k * den_k^-1
//   num_k = sum_j (c_j * f_j(p) - (a_j * p.y + b_j))      [(a, b, c) of constraints.rs:98-115]
//   den_k = (Re(P.x) - p.x) * Im(P.y) - (Re(P.y) - p.y) * Im(P.x)   (CM31)
// As the reference SIMD backend does (backend/simd/quotients.rs:31-100), rows are computed on
// the sub-domain (the first 2^(n - log_blowup) bit-reversed rows) and the result is extended to
// the full domain through an interpolation and an evaluation; below a sub-domain of 2^6 points
// every row is computed directly (the CPU fallback at simd/quotients.rs:41-58).
//
// GB300 mapping: four consecutive rows per lane with one 16-byte load per column, so a warp
// reads 512 contiguous bytes of each column (one row per lane, 128 bytes, for unaligned
// columns); sum_j c_j * f_j is accumulated in 64-bit lanes (4 products per partial reduction)
// and the linear terms are hoisted per batch (sum_j a_j, sum_j b_j), which leaves ~4 IMAD.WIDE
// per (column, row). The batch tables travel in a small device buffer.
#include "common.cuh"

namespace stwo {

int32_t fft_interpolate_evaluate(const TwiddleTree* tree_src, stwo_coset src_half, uint32_t* const* cols, uint32_t n,
                                 const TwiddleTree* tree_dst, stwo_coset dst_half, uint32_t* const* out,
                                 cudaStream_t s);

struct QBatch {
  uint32_t prx[2], pix[2], pry[2], piy[2];  // CM31 parts of the sample point
  uint32_t sum_a[4], sum_b[4], coeff[4];    // sum of a_j, sum of b_j, random_coeff^(n_j)
  uint32_t e0, e1;                          // entry range
};
struct QEntry {
  uint32_t col;
  uint32_t c[4];
};

constexpr int Q_MAX_COLS = 2048;
struct QCols { const uint32_t* p[Q_MAX_COLS]; };

__device__ __forceinline__ uint32_t red64(unsigned long long x) {
  x = (x & P) + (x >> 31);
  x = (x & P) + (x >> 31);
  uint32_t r = (uint32_t)x;
  return r >= P ? r - P : r;
}
__device__ __forceinline__ unsigned long long fold64(unsigned long long x) { return (x & P) + (x >> 31); }

// Entry staged in shared memory: the column pointer itself and the coefficient c_j.
struct QStage {
  const uint32_t* col;
  uint32_t c[4];
};

// Per-sample input of the line-coefficient kernel: column index and sampled value.
struct QSample {
  uint32_t col;
  uint32_t v[4];
};

__device__ __forceinline__ qm31 q_conj(qm31 x) { return {x.a, cm31_sub({0u, 0u}, x.b)}; }
__device__ __forceinline__ qm31 q_pow(qm31 b, uint32_t e) {
  qm31 r = qm31_from_u32(1u, 0u, 0u, 0u);
  while (e) {
    if (e & 1u) r = qm31_mul(r, b);
    b = qm31_mul(b, b);
    e >>= 1;
  }
  return r;
}

// Line coefficients of one sample batch per block (cpu/quotients.rs:78-125, constraints.rs:98):
// for the batch's j-th column with value v at point p, alpha_j = rc^(j+1), a_j = conj(v) - v,
// c = conj(p.y) - p.y, b_j = v c - a_j p.y; the entry keeps alpha_j c, the batch the sums of
// alpha_j a_j and alpha_j b_j and rc^n. Field sums are exact, so the reduction order is free.
// A batch can hold every column of a group (1,296 for Poseidon2). The powers rc^(j+1) come from
// three tables in shared memory, pw[l][i] = rc^(i * 32^l) for i < 32: two products per entry
// (exponents of 2^15 and above take the square-and-multiply path).
constexpr uint32_t QC_THREADS = 1024;
__global__ void __launch_bounds__(QC_THREADS) k_quotient_coeffs(const QSample* __restrict__ samples, QBatch* batches,
                                                         QEntry* entries, qm31 rc) {
  pdl_enter();
  __shared__ qm31 s_a[QC_THREADS / 32], s_b[QC_THREADS / 32];
  __shared__ qm31 s_pw[3][32];
  QBatch& B = batches[blockIdx.x];
  const uint32_t e0 = B.e0, e1 = B.e1;
  if (threadIdx.x < 96) {
    const uint32_t l = threadIdx.x >> 5, i = threadIdx.x & 31;
    s_pw[l][i] = q_pow(q_pow(rc, 1u << (5 * l)), i);
  }
  __syncthreads();
  const qm31 py = qm31_from_u32(B.pry[0], B.pry[1], B.piy[0], B.piy[1]);
  const qm31 c = qm31_sub(q_conj(py), py);
  qm31 sa = qm31_zero(), sb = qm31_zero();
  for (uint32_t j = threadIdx.x; j < e1 - e0; j += blockDim.x) {
    const QSample sm = samples[e0 + j];
    const qm31 v = qm31_from_u32(sm.v[0], sm.v[1], sm.v[2], sm.v[3]);
    const uint32_t k = j + 1;
    const qm31 alpha =
        k < (1u << 15) ? qm31_mul(qm31_mul(s_pw[0][k & 31], s_pw[1][(k >> 5) & 31]), s_pw[2][k >> 10]) : q_pow(rc, k);
    const qm31 a = qm31_sub(q_conj(v), v);
    const qm31 b = qm31_sub(qm31_mul(v, c), qm31_mul(a, py));
    sa = qm31_add(sa, qm31_mul(alpha, a));
    sb = qm31_add(sb, qm31_mul(alpha, b));
    const qm31 ca = qm31_mul(alpha, c);
    QEntry e;
    e.col = sm.col;
    e.c[0] = ca.a.a; e.c[1] = ca.a.b; e.c[2] = ca.b.a; e.c[3] = ca.b.b;
    entries[e0 + j] = e;
  }
  for (int off = 16; off; off >>= 1) {
    sa = qm31_from_u32(m31_add(sa.a.a, __shfl_xor_sync(~0u, sa.a.a, off)), m31_add(sa.a.b, __shfl_xor_sync(~0u, sa.a.b, off)),
                       m31_add(sa.b.a, __shfl_xor_sync(~0u, sa.b.a, off)), m31_add(sa.b.b, __shfl_xor_sync(~0u, sa.b.b, off)));
    sb = qm31_from_u32(m31_add(sb.a.a, __shfl_xor_sync(~0u, sb.a.a, off)), m31_add(sb.a.b, __shfl_xor_sync(~0u, sb.a.b, off)),
                       m31_add(sb.b.a, __shfl_xor_sync(~0u, sb.b.a, off)), m31_add(sb.b.b, __shfl_xor_sync(~0u, sb.b.b, off)));
  }
  if ((threadIdx.x & 31) == 0) {
    s_a[threadIdx.x >> 5] = sa;
    s_b[threadIdx.x >> 5] = sb;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (uint32_t w = 1; w < blockDim.x / 32; w++) {
      s_a[0] = qm31_add(s_a[0], s_a[w]);
      s_b[0] = qm31_add(s_b[0], s_b[w]);
    }
    const qm31 bc = q_pow(rc, e1 - e0);
    B.sum_a[0] = s_a[0].a.a; B.sum_a[1] = s_a[0].a.b; B.sum_a[2] = s_a[0].b.a; B.sum_a[3] = s_a[0].b.b;
    B.sum_b[0] = s_b[0].a.a; B.sum_b[1] = s_b[0].a.b; B.sum_b[2] = s_b[0].b.a; B.sum_b[3] = s_b[0].b.b;
    B.coeff[0] = bc.a.a; B.coeff[1] = bc.a.b; B.coeff[2] = bc.b.a; B.coeff[3] = bc.b.b;
  }
}

constexpr int Q_ROWS = 32;    // rows per block (one warp-width of consecutive rows)
constexpr int Q_SLICES = 8;   // column slices per row; one warp each
constexpr int Q_STAGE = 512;  // entries staged in shared memory at a time

// One block = 32 consecutive rows x 8 column slices: a warp reads 32 consecutive words of one
// column, the 8 warps stream disjoint columns of the same rows, and the 8 partial sums of a
// batch meet in shared memory. Slice 0 then finishes the batch (line term, denominator).
__global__ void __launch_bounds__(Q_SLICES * 32) k_quotient_rows(uint32_t rows, uint32_t log_n, uint32_t half_init,
                                                       uint32_t half_step, QCols cols,
                                                       const QBatch* __restrict__ batches, uint32_t n_batches,
                                                       const QEntry* __restrict__ entries, uint32_t* o0, uint32_t* o1,
                                                       uint32_t* o2, uint32_t* o3) {
  pdl_enter();
  __shared__ QStage st[Q_STAGE];
  __shared__ uint32_t part[Q_SLICES][Q_ROWS][4];
  const uint32_t lane = threadIdx.x & 31, slice = threadIdx.x >> 5;
  const uint32_t r = blockIdx.x * Q_ROWS + lane;
  const bool live = r < rows;
  cpoint p = {0u, 0u};
  if (slice == 0 && live) {
    // Domain point of bit-reversed row r of the circle domain with half coset (init, step).
    uint32_t k = brev(r, log_n);
    uint32_t half = 1u << (log_n - 1);
    uint32_t idx = k < half ? half_init + half_step * k : (0u - (half_init + half_step * (k - half)));
    p = index_to_point(idx & 0x7fffffffu);
  }
  qm31 acc = qm31_zero();
  for (uint32_t b = 0; b < n_batches; b++) {
    const QBatch& B = batches[b];
    unsigned long long s0 = 0, s1 = 0, s2 = 0, s3 = 0;
    for (uint32_t e0 = B.e0; e0 < B.e1; e0 += Q_STAGE) {
      uint32_t ne = min((uint32_t)Q_STAGE, B.e1 - e0);
      __syncthreads();
      for (uint32_t i = threadIdx.x; i < ne; i += blockDim.x) {
        const QEntry& E = entries[e0 + i];
        st[i].col = cols.p[E.col];
        st[i].c[0] = E.c[0];
        st[i].c[1] = E.c[1];
        st[i].c[2] = E.c[2];
        st[i].c[3] = E.c[3];
      }
      __syncthreads();
      if (live) {
        uint32_t cnt = 0;
        uint32_t i = slice;
        // Sixteen independent column loads in flight per iteration. Products are at most
        // (P - 1)^2 < 2^62 - 2^33 + 4 and a folded sum is below 2^33 + 2^31, so a sum takes four
        // products between folds without passing 2^64.
        for (; i + 15 * Q_SLICES < ne; i += 16 * Q_SLICES) {
          uint32_t v[16];
#pragma unroll
          for (int u = 0; u < 16; u++) v[u] = __ldg(st[i + u * Q_SLICES].col + r);
#pragma unroll
          for (int u = 0; u < 16; u++) {
            const QStage& q = st[i + u * Q_SLICES];
            s0 += (unsigned long long)q.c[0] * v[u];
            s1 += (unsigned long long)q.c[1] * v[u];
            s2 += (unsigned long long)q.c[2] * v[u];
            s3 += (unsigned long long)q.c[3] * v[u];
            if ((u & 3) == 3) {
              s0 = fold64(s0);
              s1 = fold64(s1);
              s2 = fold64(s2);
              s3 = fold64(s3);
            }
          }
        }
        for (; i < ne; i += Q_SLICES) {
          uint32_t v = __ldg(st[i].col + r);
          s0 += (unsigned long long)st[i].c[0] * v;
          s1 += (unsigned long long)st[i].c[1] * v;
          s2 += (unsigned long long)st[i].c[2] * v;
          s3 += (unsigned long long)st[i].c[3] * v;
          if (++cnt == 4) {
            s0 = fold64(s0);
            s1 = fold64(s1);
            s2 = fold64(s2);
            s3 = fold64(s3);
            cnt = 0;
          }
        }
        // The next staged group starts from a folded sum.
        s0 = fold64(s0);
        s1 = fold64(s1);
        s2 = fold64(s2);
        s3 = fold64(s3);
      }
    }
    part[slice][lane][0] = red64(s0);
    part[slice][lane][1] = red64(s1);
    part[slice][lane][2] = red64(s2);
    part[slice][lane][3] = red64(s3);
    __syncthreads();
    if (slice == 0 && live) {
      uint32_t cv[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        uint32_t t = 0;
#pragma unroll
        for (int sl = 0; sl < Q_SLICES; sl++) t = m31_add(t, part[sl][lane][q]);
        cv[q] = t;
      }
      qm31 lin = qm31_add(qm31_mul_m31(qm31_from_u32(B.sum_a[0], B.sum_a[1], B.sum_a[2], B.sum_a[3]), p.y),
                          qm31_from_u32(B.sum_b[0], B.sum_b[1], B.sum_b[2], B.sum_b[3]));
      qm31 num = qm31_sub(qm31_from_u32(cv[0], cv[1], cv[2], cv[3]), lin);
      cm31 px = {p.x, 0u}, py = {p.y, 0u};
      cm31 den = cm31_sub(cm31_mul(cm31_sub({B.prx[0], B.prx[1]}, px), {B.piy[0], B.piy[1]}),
                          cm31_mul(cm31_sub({B.pry[0], B.pry[1]}, py), {B.pix[0], B.pix[1]}));
      acc = qm31_add(qm31_mul(acc, qm31_from_u32(B.coeff[0], B.coeff[1], B.coeff[2], B.coeff[3])),
                     qm31_mul_cm31(num, cm31_inv(den)));
    }
    __syncthreads();  // `part` is rewritten by the next batch
  }
  if (slice == 0 && live) {
    o0[r] = acc.a.a;
    o1[r] = acc.a.b;
    o2[r] = acc.b.a;
    o3[r] = acc.b.b;
  }
}

// The same sums with RPL (4 or 2) consecutive rows per lane: one 16-byte (8-byte) load per column
// gives a warp 512 (256) contiguous bytes of that column, against 128 bytes with a row per lane,
// so the loads keep longer runs within a DRAM page. A block covers 32 RPL rows; two rows per lane
// give small domains twice the blocks (2^16 rows: 1,024 blocks, 6-7 per SM, where 512 blocks left
// the SMs with three blocks idle for a quarter of the launch). Needs 4 RPL-byte aligned columns
// and a multiple of 32 RPL rows. The first RPL warps finish the batches, one row per lane.
template <int RPL>
struct QVec;
template <>
struct QVec<4> {
  using T = uint4;
  static __device__ __forceinline__ void words(const T& v, uint32_t* x) { x[0] = v.x, x[1] = v.y, x[2] = v.z, x[3] = v.w; }
};
template <>
struct QVec<2> {
  using T = uint2;
  static __device__ __forceinline__ void words(const T& v, uint32_t* x) { x[0] = v.x, x[1] = v.y; }
};

template <int RPL>
__global__ void __launch_bounds__(Q_SLICES * 32) k_quotient_rows4(uint32_t rows, uint32_t log_n, uint32_t half_init,
                                                                  uint32_t half_step, QCols cols,
                                                                  const QBatch* __restrict__ batches, uint32_t n_batches,
                                                                  const QEntry* __restrict__ entries, uint32_t* o0,
                                                                  uint32_t* o1, uint32_t* o2, uint32_t* o3) {
  pdl_enter();
  using V = typename QVec<RPL>::T;
  constexpr int BR = 32 * RPL;  // rows per block
  __shared__ QStage st[Q_STAGE];
  __shared__ uint32_t part[Q_SLICES][BR][4];
  const uint32_t lane = threadIdx.x & 31, slice = threadIdx.x >> 5;
  const uint32_t base = blockIdx.x * BR;
  const uint32_t r0 = base + RPL * lane;  // rows r0 .. r0 + RPL - 1 (rows is a multiple of BR)
  const bool fin = slice < RPL;
  const uint32_t rf = base + 32 * slice + lane;  // the row a finishing lane owns
  cpoint p = {0u, 0u};
  if (fin) {
    uint32_t k = brev(rf, log_n);
    uint32_t half = 1u << (log_n - 1);
    uint32_t idx = k < half ? half_init + half_step * k : (0u - (half_init + half_step * (k - half)));
    p = index_to_point(idx & 0x7fffffffu);
  }
  (void)rows;
  qm31 acc = qm31_zero();
  for (uint32_t b = 0; b < n_batches; b++) {
    const QBatch& B = batches[b];
    unsigned long long s[RPL][4];
#pragma unroll
    for (int j = 0; j < RPL; j++)
#pragma unroll
      for (int q = 0; q < 4; q++) s[j][q] = 0;
    auto fold_all = [&]() {
#pragma unroll
      for (int j = 0; j < RPL; j++)
#pragma unroll
        for (int q = 0; q < 4; q++) s[j][q] = fold64(s[j][q]);
    };
    auto add = [&](const QStage& q, const V& v) {
      uint32_t x[RPL];
      QVec<RPL>::words(v, x);
#pragma unroll
      for (int j = 0; j < RPL; j++) {
        s[j][0] += (unsigned long long)q.c[0] * x[j];
        s[j][1] += (unsigned long long)q.c[1] * x[j];
        s[j][2] += (unsigned long long)q.c[2] * x[j];
        s[j][3] += (unsigned long long)q.c[3] * x[j];
      }
    };
    for (uint32_t e0 = B.e0; e0 < B.e1; e0 += Q_STAGE) {
      uint32_t ne = min((uint32_t)Q_STAGE, B.e1 - e0);
      __syncthreads();
      for (uint32_t i = threadIdx.x; i < ne; i += blockDim.x) {
        const QEntry& E = entries[e0 + i];
        st[i].col = cols.p[E.col];
        st[i].c[0] = E.c[0];
        st[i].c[1] = E.c[1];
        st[i].c[2] = E.c[2];
        st[i].c[3] = E.c[3];
      }
      __syncthreads();
      uint32_t i = slice;
      // Eight vector loads in flight per iteration; as in k_quotient_rows, a sum takes four
      // products between folds.
      for (; i + 7 * Q_SLICES < ne; i += 8 * Q_SLICES) {
        V v[8];
#pragma unroll
        for (int u = 0; u < 8; u++) v[u] = __ldg(reinterpret_cast<const V*>(st[i + u * Q_SLICES].col + r0));
#pragma unroll
        for (int u = 0; u < 8; u++) {
          add(st[i + u * Q_SLICES], v[u]);
          if ((u & 3) == 3) fold_all();
        }
      }
      uint32_t cnt = 0;
      for (; i < ne; i += Q_SLICES) {
        add(st[i], __ldg(reinterpret_cast<const V*>(st[i].col + r0)));
        if (++cnt == 4) {
          fold_all();
          cnt = 0;
        }
      }
      fold_all();  // the next staged group starts from a folded sum
    }
#pragma unroll
    for (int j = 0; j < RPL; j++)
#pragma unroll
      for (int q = 0; q < 4; q++) part[slice][RPL * lane + j][q] = red64(s[j][q]);
    __syncthreads();
    if (fin) {
      const uint32_t rl = 32 * slice + lane;
      uint32_t cv[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        uint32_t t = 0;
#pragma unroll
        for (int sl = 0; sl < Q_SLICES; sl++) t = m31_add(t, part[sl][rl][q]);
        cv[q] = t;
      }
      qm31 lin = qm31_add(qm31_mul_m31(qm31_from_u32(B.sum_a[0], B.sum_a[1], B.sum_a[2], B.sum_a[3]), p.y),
                          qm31_from_u32(B.sum_b[0], B.sum_b[1], B.sum_b[2], B.sum_b[3]));
      qm31 num = qm31_sub(qm31_from_u32(cv[0], cv[1], cv[2], cv[3]), lin);
      cm31 px = {p.x, 0u}, py = {p.y, 0u};
      cm31 den = cm31_sub(cm31_mul(cm31_sub({B.prx[0], B.prx[1]}, px), {B.piy[0], B.piy[1]}),
                          cm31_mul(cm31_sub({B.pry[0], B.pry[1]}, py), {B.pix[0], B.pix[1]}));
      acc = qm31_add(qm31_mul(acc, qm31_from_u32(B.coeff[0], B.coeff[1], B.coeff[2], B.coeff[3])),
                     qm31_mul_cm31(num, cm31_inv(den)));
    }
    __syncthreads();  // `part` is rewritten by the next batch
  }
  if (fin) {
    o0[rf] = acc.a.a;
    o1[rf] = acc.a.b;
    o2[rf] = acc.b.a;
    o3[rf] = acc.b.b;
  }
}

// The per-row pass over the columns (with the line coefficients already in d_b / d_e) and, above
// a sub-domain of 2^6 points, the extension of the sub-domain result to the full domain. d_sub
// holds 4 x 2^(log_n - log_blowup) words (unused when the rows are computed directly).
static int32_t quotient_rows_and_extend(uint32_t log_n, const uint32_t* const* cols, uint32_t n_cols, const QBatch* d_b,
                                        uint32_t n_batches, const QEntry* d_e, uint32_t log_blowup, uint32_t* d_sub,
                                        uint32_t* const out[4], cudaStream_t s) {
  stwo_coset dom_half = canonic_half_coset(log_n);
  const uint32_t sub_log = log_n - log_blowup;
  const bool direct = sub_log < 6;
  const uint32_t rows = 1u << (direct ? log_n : sub_log);
  QCols qc;
  for (uint32_t c = 0; c < n_cols; c++) qc.p[c] = cols[c];
  uint32_t* o[4];
  for (int q = 0; q < 4; q++) o[q] = direct ? out[q] : d_sub + (size_t)q * rows;
  // Rows per lane: 4 or 2 (16- or 8-byte column loads; needs that alignment and a multiple of
  // 32 x that many rows), or 1 (the 32-row kernel). Built in: four once the domain gives at least
  // four 128-row blocks per SM, else two.
  auto fits = [&](uint32_t rpl) {
    if (rpl == 1) return true;
    bool ok = rows % (32 * rpl) == 0;
    for (uint32_t c = 0; c < n_cols && ok; c++) ok = (reinterpret_cast<uintptr_t>(cols[c]) & (4 * rpl - 1)) == 0;
    return ok;
  };
  auto launch_rows = [&](uint32_t rpl) -> int32_t {
    if (rpl == 4)
      launch_pdl(k_quotient_rows4<4>, dim3(rows / 128), dim3(Q_SLICES * 32), 0, s, rows, log_n,
                 dom_half.initial_index, dom_half.step_size, qc, d_b, n_batches, d_e, o[0], o[1], o[2], o[3]);
    else if (rpl == 2)
      launch_pdl(k_quotient_rows4<2>, dim3(rows / 64), dim3(Q_SLICES * 32), 0, s, rows, log_n,
                 dom_half.initial_index, dom_half.step_size, qc, d_b, n_batches, d_e, o[0], o[1], o[2], o[3]);
    else
      launch_pdl(k_quotient_rows, dim3((rows + Q_ROWS - 1) / Q_ROWS), dim3(Q_SLICES * 32), 0, s, rows, log_n,
                 dom_half.initial_index, dom_half.step_size, qc, d_b, n_batches, d_e, o[0], o[1], o[2], o[3]);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? STWO_OK : STWO_ERR_CUDA;
  };
  uint32_t rpl = rows >= 4u * 128u * (uint32_t)sm_count() ? 4 : 2;
  if (!fits(rpl)) rpl = fits(2) ? 2 : 1;
  uint32_t cands[3], n_cands = 0;
  for (uint32_t c : {4u, 2u, 1u})
    if (fits(c)) cands[n_cands++] = c;
  int32_t st = STWO_OK;
  if (rows >= 1024) {
    // The row pass recomputes its outputs from the columns, so it can be timed in place.
    const uint64_t key = ((uint64_t)log_n << 40) | ((uint64_t)log_blowup << 32) | n_cols;
    st = tune_choice(TUNE_QUOTIENT_ROWS, key, rpl, cands, n_cands, s, launch_rows, &rpl);
    if (st) return st;
  }
  st = launch_rows(rpl);
  if (st) return st;

  if (!direct) {
    // Interpolate on the sub-domain (its own tree), then evaluate on the full canonic domain.
    stwo_coset sub_half = coset_new(dom_half.initial_index, sub_log - 1);
    TwiddleTree* t_sub = nullptr;
    TwiddleTree* t_dom = nullptr;
    st = get_tree(sub_half, s, &t_sub);
    if (!st) st = get_tree(dom_half, s, &t_dom);
    if (!st) st = fft_interpolate_evaluate(t_sub, sub_half, o, 4, t_dom, dom_half, out, s);
    if (st) return st;
  }
  return STWO_OK;
}

int32_t accumulate_quotients(uint32_t log_n, const uint32_t* const* cols, uint32_t n_cols, stwo_qm31 rc_in,
                             const stwo_sample_batch* batches, uint32_t n_batches, uint32_t log_blowup,
                             uint32_t* const out[4], cudaStream_t s) {
  STWO_REQUIRE(log_n >= 1 && log_n <= 30, "bad domain log size %u", log_n);
  STWO_REQUIRE(log_blowup < log_n, "log_blowup_factor %u >= domain log size %u", log_blowup, log_n);
  STWO_REQUIRE(n_cols <= Q_MAX_COLS, "more than %d columns in one quotient group", Q_MAX_COLS);
  STWO_REQUIRE(n_batches == 0 || batches, "null batches");
  hq rc = hq_from(rc_in);

  // Batch headers on the host (points, entry ranges); the line coefficients on the device.
  std::vector<QBatch> hb(n_batches);
  std::vector<QSample> hs;
  for (uint32_t b = 0; b < n_batches; b++) {
    const stwo_sample_batch& sb = batches[b];
    hq px = hq_from(sb.point.x), py = hq_from(sb.point.y);
    STWO_REQUIRE(!(py.v[2] == 0 && py.v[3] == 0), "Cannot evaluate a line with a single point");
    QBatch& B = hb[b];
    std::memset(&B, 0, sizeof(B));
    B.prx[0] = px.v[0]; B.prx[1] = px.v[1]; B.pix[0] = px.v[2]; B.pix[1] = px.v[3];
    B.pry[0] = py.v[0]; B.pry[1] = py.v[1]; B.piy[0] = py.v[2]; B.piy[1] = py.v[3];
    B.e0 = (uint32_t)hs.size();
    for (uint32_t j = 0; j < sb.n_columns; j++) {
      STWO_REQUIRE(sb.h_column_indices[j] < n_cols, "sample column index out of range");
      QSample q;
      q.col = sb.h_column_indices[j];
      for (int k = 0; k < 4; k++) q.v[k] = sb.h_values[j].v[k];
      hs.push_back(q);
    }
    B.e1 = (uint32_t)hs.size();
  }
  std::vector<QEntry> he(hs.size());
  uint32_t sub_log = log_n - log_blowup;
  bool direct = sub_log < 6;
  uint32_t rows = 1u << (direct ? log_n : sub_log);

  size_t tbl_bytes = hb.size() * sizeof(QBatch) + he.size() * sizeof(QEntry) + hs.size() * sizeof(QSample);
  size_t sub_bytes = direct ? 0 : (size_t)4 * rows * 4;
  char* scratch = nullptr;
  int32_t st = scratch_alloc((void**)&scratch, tbl_bytes + sub_bytes + 256, s);
  if (st) return st;
  QBatch* d_b = reinterpret_cast<QBatch*>(scratch);
  QEntry* d_e = reinterpret_cast<QEntry*>(scratch + hb.size() * sizeof(QBatch));
  QSample* d_s = reinterpret_cast<QSample*>(scratch + hb.size() * sizeof(QBatch) + he.size() * sizeof(QEntry));
  uint32_t* d_sub = reinterpret_cast<uint32_t*>(scratch + ((tbl_bytes + 255) / 256) * 256);
  auto fail = [&](int32_t code) {
    scratch_free(scratch, s);
    return code;
  };
  if (!hb.empty() && cudaMemcpyAsync(d_b, hb.data(), hb.size() * sizeof(QBatch), cudaMemcpyHostToDevice, s) != cudaSuccess)
    return fail(STWO_ERR_CUDA);
  if (!hs.empty() && cudaMemcpyAsync(d_s, hs.data(), hs.size() * sizeof(QSample), cudaMemcpyHostToDevice, s) != cudaSuccess)
    return fail(STWO_ERR_CUDA);
  if (n_batches) {
    launch_pdl(k_quotient_coeffs, dim3(n_batches), dim3(QC_THREADS), 0, s, d_s, d_b, d_e,
               qm31{{rc.v[0], rc.v[1]}, {rc.v[2], rc.v[3]}});
    note_launch();
    if (cudaGetLastError() != cudaSuccess) return fail(STWO_ERR_CUDA);
  }

  st = quotient_rows_and_extend(log_n, cols, n_cols, d_b, n_batches, d_e, log_blowup, d_sub, out, s);
  if (st) return fail(st);
  scratch_free(scratch, s);
  return STWO_OK;
}

// ---------------------------------------------------------------- planned quotients (the prover's)
// The prover knows, before the OODS point is drawn, which columns of a quotient group are sampled
// at which mask offset and which OODS evaluation holds each value; only the points, their order
// (the reference orders batches by point value) and the random coefficient come later. So the
// sample table is uploaded while the device still works on earlier stages, and at run time one
// launch assembles the batch tables from it and from the OODS values left in device memory.
struct QPlanSample {
  uint32_t col, eval;
};
struct QPlanParams {
  uint32_t order[EP_MAX_POINTS];        // point id of batch b
  uint32_t e_first[EP_MAX_POINTS + 1];  // entries of batch b: [e_first[b], e_first[b + 1])
  uint32_t s_first[EP_MAX_POINTS + 1];  // the plan's samples at point id p: [s_first[p], s_first[p + 1])
  uint32_t pt[EP_MAX_POINTS][8];        // point id p: CM31 parts prx, pix, pry, piy
};

// Block b: batch b's header and its samples, in the order k_quotient_coeffs reads them.
__global__ void k_quotient_gather(const QPlanSample* __restrict__ ps, const uint32_t* __restrict__ vals,
                                  QPlanParams pp, QSample* samples, QBatch* batches) {
  pdl_enter();
  const uint32_t b = blockIdx.x, p = pp.order[b];
  const uint32_t s0 = pp.s_first[p], n = pp.s_first[p + 1] - s0, e0 = pp.e_first[b];
  for (uint32_t j = threadIdx.x; j < n; j += blockDim.x) {
    const QPlanSample q = ps[s0 + j];
    QSample o;
    o.col = q.col;
    for (int k = 0; k < 4; k++) o.v[k] = vals[4 * q.eval + k];
    samples[e0 + j] = o;
  }
  if (threadIdx.x == 0) {
    QBatch B = {};
    B.prx[0] = pp.pt[p][0]; B.prx[1] = pp.pt[p][1]; B.pix[0] = pp.pt[p][2]; B.pix[1] = pp.pt[p][3];
    B.pry[0] = pp.pt[p][4]; B.pry[1] = pp.pt[p][5]; B.piy[0] = pp.pt[p][6]; B.piy[1] = pp.pt[p][7];
    B.e0 = e0;
    B.e1 = e0 + n;
    batches[b] = B;
  }
}

int32_t quot_plan_build(uint32_t log_n, const uint32_t* const* cols, uint32_t n_cols, const uint32_t* sample_col,
                        const uint32_t* sample_eval, const uint32_t* sample_point, uint32_t n_samples, uint32_t n_points,
                        uint32_t log_blowup, cudaStream_t s, QuotPlan* plan) {
  STWO_REQUIRE(plan && (n_cols == 0 || cols) && (n_samples == 0 || (sample_col && sample_eval && sample_point)),
               "null argument");
  STWO_REQUIRE(log_n >= 1 && log_n <= 30, "bad domain log size %u", log_n);
  STWO_REQUIRE(log_blowup < log_n, "log_blowup_factor %u >= domain log size %u", log_blowup, log_n);
  STWO_REQUIRE(n_cols <= Q_MAX_COLS, "more than %d columns in one quotient group", Q_MAX_COLS);
  STWO_REQUIRE(n_points >= 1 && n_points <= EP_MAX_POINTS, "%u points (at most %u)", n_points, EP_MAX_POINTS);
  QuotPlan p;
  p.log_n = log_n;
  p.log_blowup = log_blowup;
  p.n_points = n_points;
  p.n_samples = n_samples;
  p.cols.assign(cols, cols + n_cols);
  // Samples bucketed by point id, each bucket in sample order (column, then offset).
  std::vector<uint32_t> count(n_points + 1, 0);
  for (uint32_t j = 0; j < n_samples; j++) {
    STWO_REQUIRE(sample_col[j] < n_cols && sample_point[j] < n_points, "sample %u: index out of range", j);
    count[sample_point[j] + 1]++;
  }
  for (uint32_t q = 0; q < n_points; q++) count[q + 1] += count[q];
  p.s_first.assign(count.begin(), count.end());
  std::vector<QPlanSample> hs(n_samples);
  for (uint32_t j = 0; j < n_samples; j++) hs[count[sample_point[j]]++] = {sample_col[j], sample_eval[j]};
  const uint32_t sub_log = log_n - log_blowup;
  const uint32_t rows = 1u << (sub_log < 6 ? log_n : sub_log);
  auto up256 = [](size_t b) { return (b + 255) / 256 * 256; };
  p.off_samples = up256(n_samples * sizeof(QPlanSample));
  p.off_batches = p.off_samples + up256((size_t)n_samples * sizeof(QSample));
  p.off_entries = p.off_batches + up256((size_t)n_points * sizeof(QBatch));
  p.off_sub = p.off_entries + up256((size_t)n_samples * sizeof(QEntry));
  const size_t bytes = p.off_sub + (size_t)4 * rows * 4;
  int32_t st = scratch_alloc((void**)&p.d, bytes, s);
  if (st) return st;
  if (n_samples) {
    cudaError_t err = cudaMemcpyAsync(p.d, hs.data(), hs.size() * sizeof(QPlanSample), cudaMemcpyHostToDevice, s);
    if (err) {
      scratch_free(p.d, s);
      set_error("quot_plan_build: %s", cudaGetErrorString(err));
      return STWO_ERR_CUDA;
    }
  }
  *plan = std::move(p);
  return STWO_OK;
}

int32_t quot_plan_run(const QuotPlan& p, const uint32_t* d_vals, const stwo_qm31_point* points, const uint32_t* order,
                      uint32_t n_batches, stwo_qm31 rc_in, uint32_t* const out[4], cudaStream_t s) {
  STWO_REQUIRE(p.d && d_vals && points && (n_batches == 0 || order), "null argument");
  STWO_REQUIRE(n_batches <= p.n_points, "%u batches for %u points", n_batches, p.n_points);
  QPlanParams pp{};
  uint32_t e = 0;
  for (uint32_t b = 0; b < n_batches; b++) {
    const uint32_t q = order[b];
    STWO_REQUIRE(q < p.n_points, "batch %u: point id out of range", b);
    pp.order[b] = q;
    pp.e_first[b] = e;
    e += p.s_first[q + 1] - p.s_first[q];
  }
  pp.e_first[n_batches] = e;
  STWO_REQUIRE(e == p.n_samples, "the batch order must take every sampled point once");
  for (uint32_t q = 0; q <= p.n_points; q++) pp.s_first[q] = p.s_first[q];
  for (uint32_t q = 0; q < p.n_points; q++) {
    const stwo_qm31_point& pt = points[q];
    STWO_REQUIRE(!(pt.y.v[2] == 0 && pt.y.v[3] == 0), "Cannot evaluate a line with a single point");
    const uint32_t w[8] = {pt.x.v[0], pt.x.v[1], pt.x.v[2], pt.x.v[3], pt.y.v[0], pt.y.v[1], pt.y.v[2], pt.y.v[3]};
    for (int k = 0; k < 8; k++) pp.pt[q][k] = w[k];
  }
  const hq rc = hq_from(rc_in);
  const QPlanSample* d_ps = reinterpret_cast<const QPlanSample*>(p.d);
  QSample* d_s = reinterpret_cast<QSample*>(p.d + p.off_samples);
  QBatch* d_b = reinterpret_cast<QBatch*>(p.d + p.off_batches);
  QEntry* d_e = reinterpret_cast<QEntry*>(p.d + p.off_entries);
  if (n_batches) {
    launch_pdl(k_quotient_gather, dim3(n_batches), dim3(256), 0, s, d_ps, d_vals, pp, d_s, d_b);
    note_launch();
    if (cudaGetLastError() != cudaSuccess) return STWO_ERR_CUDA;
    launch_pdl(k_quotient_coeffs, dim3(n_batches), dim3(QC_THREADS), 0, s, d_s, d_b, d_e,
               qm31{{rc.v[0], rc.v[1]}, {rc.v[2], rc.v[3]}});
    note_launch();
    if (cudaGetLastError() != cudaSuccess) return STWO_ERR_CUDA;
  }
  return quotient_rows_and_extend(p.log_n, p.cols.data(), (uint32_t)p.cols.size(), d_b, n_batches, d_e,
                                  p.log_blowup, reinterpret_cast<uint32_t*>(p.d + p.off_sub), out, s);
}

void quot_plan_free(QuotPlan& p, cudaStream_t s) {
  if (p.d) scratch_free(p.d, s);
  p.d = nullptr;
}

}  // namespace stwo

using namespace stwo;

extern "C" stwo_status stwo_accumulate_quotients(uint32_t domain_log_size, const uint32_t* const* d_cols,
                                                 uint32_t n_cols, stwo_qm31 random_coeff,
                                                 const stwo_sample_batch* h_batches, uint32_t n_batches,
                                                 uint32_t log_blowup_factor, uint32_t* const d_out[4], void* stream) {
  return accumulate_quotients(domain_log_size, d_cols, n_cols, random_coeff, h_batches, n_batches, log_blowup_factor,
                              d_out, as_stream(stream));
}
