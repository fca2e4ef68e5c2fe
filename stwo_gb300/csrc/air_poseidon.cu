// Poseidon2 AIR on the device (crates/prover/src/examples/poseidon/mod.rs:30-389): 8 width-16
// permutations per row (4 full, 14 partial, 4 full rounds; 1264 trace columns), plus the LogUp
// interaction trace of their initial/final states (constraint_framework/logup.rs:123-260) and
// the composition constraints (1136 round constraints + 8 LogUp constraints, finalize_logup_in_pairs
// of constraint_framework/mod.rs:182-248).
//
// Kernels (one thread per row each):
//   k_poseidon_trace        trace generation; also keeps the lookup states, since committing the
//                           trace replaces it by its coefficients
//   k_poseidon_interaction  8 cumulative LogUp secure columns (QM31 inverses per row)
//   k_coset_scan_*          inclusive prefix sum in coset order of the last column
//                           (backend/simd/prefix_sum.rs:19-139)
//   k_poseidon_composition  all constraints on the 4x evaluation domain, random-coefficient
//                           accumulation in 64-bit lanes, times the vanishing inverse
// Multiplication by 2^k (internal matrix) is a 31-bit rotation, exact modulo 2^31 - 1.
#include "common.cuh"
#include "prover.cuh"

namespace stwo {

constexpr int PS_REPS = 8, PS_ST = 16, PS_PARTIAL = 14, PS_HALF = 4;
constexpr int PS_COLS_PER_REP = PS_ST * (1 + 2 * PS_HALF) + PS_PARTIAL;  // 158
constexpr int PS_COLS = PS_REPS * PS_COLS_PER_REP;                       // 1264
constexpr int PS_INTERACTION_COLS = 4 * PS_REPS;                         // 32
constexpr int PS_N_CONSTRAINTS = PS_REPS * (2 * PS_HALF * PS_ST + PS_PARTIAL) + PS_REPS;  // 1144
constexpr uint32_t PS_RC = 1234;  // round constants of the reference example
constexpr uint32_t PS_LOG_EXPAND = 2;

__device__ __forceinline__ uint32_t m31_mul_pow2(uint32_t x, int k) { return ((x << k) | (x >> (31 - k))) & P; }
__device__ __forceinline__ uint32_t pow5(uint32_t x) {
  uint32_t x2 = m31_sqr(x);
  return m31_mul(m31_sqr(x2), x);
}
// M4 of Poseidon2 section 5.1 (poseidon/mod.rs:72-94).
__device__ __forceinline__ void apply_m4(uint32_t* x) {
  uint32_t t0 = m31_add(x[0], x[1]);
  uint32_t t02 = m31_add(t0, t0);
  uint32_t t1 = m31_add(x[2], x[3]);
  uint32_t t12 = m31_add(t1, t1);
  uint32_t t2 = m31_add(m31_add(x[1], x[1]), t1);
  uint32_t t3 = m31_add(m31_add(x[3], x[3]), t0);
  uint32_t t4 = m31_add(m31_add(t12, t12), t3);
  uint32_t t5 = m31_add(m31_add(t02, t02), t2);
  x[0] = m31_add(t3, t5);
  x[1] = t5;
  x[2] = m31_add(t2, t4);
  x[3] = t4;
}
__device__ __forceinline__ void external_matrix(uint32_t* s) {
#pragma unroll
  for (int i = 0; i < 4; i++) apply_m4(s + 4 * i);
#pragma unroll
  for (int j = 0; j < 4; j++) {
    uint32_t t = m31_add(m31_add(s[j], s[j + 4]), m31_add(s[j + 8], s[j + 12]));
#pragma unroll
    for (int i = 0; i < 4; i++) s[4 * i + j] = m31_add(s[4 * i + j], t);
  }
}
__device__ __forceinline__ void internal_matrix(uint32_t* s) {
  uint32_t sum = s[0];
#pragma unroll
  for (int i = 1; i < 16; i++) sum = m31_add(sum, s[i]);
#pragma unroll
  for (int i = 0; i < 16; i++) s[i] = m31_add(m31_mul_pow2(s[i], i + 1), sum);
}

// ------------------------------------------------------------------------------------------ trace
// init: ((row * 8 + rep) * 16 + i) or NULL for the reference inputs (row + i + rep).
// Warp w of a block computes permutation w of 32 consecutive rows (the layout of
// k_poseidon_composition): its 158 columns are written with coalesced 128-byte stores, and a
// small trace takes the latency of one permutation rather than eight. The block's initial states
// are one contiguous run of 32 x 8 x 16 words: the block reads it with coalesced loads into shared
// memory (word w at w + w / 128, so that the lanes' reads of one state word hit distinct banks).
// `init` may be pinned host memory: the states then cross the host link inside this kernel.
__global__ void __launch_bounds__(32 * PS_REPS) k_poseidon_trace(uint32_t n_rows, const uint32_t* __restrict__ init,
                                                                 uint32_t* __restrict__ trace,
                                                                 uint32_t* __restrict__ lookups) {
  pdl_enter();
  __shared__ uint32_t s_init[32 * PS_REPS * PS_ST + 32];
  const uint32_t lane = threadIdx.x & 31, rep = threadIdx.x >> 5;
  const uint32_t r = blockIdx.x * 32 + lane;
  if (init) {
    const uint32_t valid = min(32u, n_rows - blockIdx.x * 32) * PS_REPS * PS_ST;
    const uint32_t* src = init + (size_t)blockIdx.x * 32 * PS_REPS * PS_ST;
    for (uint32_t w = threadIdx.x; w < valid; w += blockDim.x) s_init[w + (w >> 7)] = src[w];
    __syncthreads();
  }
  if (r >= n_rows) return;
  const size_t n = n_rows;
  uint32_t col = rep * PS_COLS_PER_REP;
  uint32_t s[PS_ST];
#pragma unroll
  for (int i = 0; i < PS_ST; i++) {
    s[i] = init ? s_init[(lane * PS_REPS + rep) * PS_ST + i + lane] : (r + i + rep);
    trace[(size_t)col++ * n + r] = s[i];
    lookups[((size_t)rep * 32 + i) * n + r] = s[i];
  }
  for (int round = 0; round < 2 * PS_HALF + PS_PARTIAL; round++) {
    bool full = round < PS_HALF || round >= PS_HALF + PS_PARTIAL;
    if (full) {
#pragma unroll
      for (int i = 0; i < PS_ST; i++) s[i] = m31_add(s[i], PS_RC);
      external_matrix(s);
#pragma unroll
      for (int i = 0; i < PS_ST; i++) {
        s[i] = pow5(s[i]);
        trace[(size_t)col++ * n + r] = s[i];
      }
    } else {
      s[0] = m31_add(s[0], PS_RC);
      internal_matrix(s);
      s[0] = pow5(s[0]);
      trace[(size_t)col++ * n + r] = s[0];
    }
  }
#pragma unroll
  for (int i = 0; i < PS_ST; i++) lookups[((size_t)rep * 32 + 16 + i) * n + r] = s[i];
}

// ------------------------------------------------------------------------------------ interaction
struct LookupConsts {
  uint32_t z[4];
  uint32_t alpha_pow[PS_ST][4];
};


__device__ __forceinline__ uint32_t fold64_p(unsigned long long x) {
  x = (x & P) + (x >> 31);
  x = (x & P) + (x >> 31);
  uint32_t r = (uint32_t)x;
  return r >= P ? r - P : r;
}

// sum_i alpha^i * v_i - z  (LookupElements::combine, logup.rs:90-105)
__device__ __forceinline__ qm31 combine16(const LookupConsts& lc, const uint32_t* v) {
  unsigned long long a0 = 0, a1 = 0, a2 = 0, a3 = 0;
#pragma unroll
  for (int i = 0; i < PS_ST; i++) {
    a0 += (unsigned long long)lc.alpha_pow[i][0] * v[i];
    a1 += (unsigned long long)lc.alpha_pow[i][1] * v[i];
    a2 += (unsigned long long)lc.alpha_pow[i][2] * v[i];
    a3 += (unsigned long long)lc.alpha_pow[i][3] * v[i];
    if (i % 3 == 2) {
      a0 = (a0 & P) + (a0 >> 31);
      a1 = (a1 & P) + (a1 >> 31);
      a2 = (a2 & P) + (a2 >> 31);
      a3 = (a3 & P) + (a3 >> 31);
    }
  }
  qm31 s = qm31_from_u32(fold64_p(a0), fold64_p(a1), fold64_p(a2), fold64_p(a3));
  return qm31_sub(s, qm31_from_u32(lc.z[0], lc.z[1], lc.z[2], lc.z[3]));
}

__global__ void __launch_bounds__(128) k_poseidon_interaction(uint32_t n_rows, const uint32_t* __restrict__ lookups,
                                                              LookupConsts lc, uint32_t* __restrict__ out) {
  pdl_enter();
  uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_rows) return;
  size_t n = n_rows;
  qm31 cum = qm31_zero();
  for (int rep = 0; rep < PS_REPS; rep++) {
    uint32_t a[PS_ST], b[PS_ST];
#pragma unroll
    for (int i = 0; i < PS_ST; i++) {
      a[i] = __ldg(lookups + ((size_t)rep * 32 + i) * n + r);
      b[i] = __ldg(lookups + ((size_t)rep * 32 + 16 + i) * n + r);
    }
    qm31 d0 = combine16(lc, a), d1 = combine16(lc, b);
    // 1/d0 - 1/d1 = (d1 - d0) / (d0 d1)
    qm31 frac = qm31_mul(qm31_sub(d1, d0), qm31_inv(qm31_mul(d0, d1)));
    cum = qm31_add(cum, frac);
    out[((size_t)4 * rep + 0) * n + r] = cum.a.a;
    out[((size_t)4 * rep + 1) * n + r] = cum.a.b;
    out[((size_t)4 * rep + 2) * n + r] = cum.b.a;
    out[((size_t)4 * rep + 3) * n + r] = cum.b.b;
  }
}

// Per-coordinate column sums into 64-bit accumulators.
__global__ void k_column_sums(const uint32_t* __restrict__ cols, uint32_t n_rows, unsigned long long* acc) {
  pdl_enter();
  uint32_t k = blockIdx.y;
  const uint32_t* c = cols + (size_t)k * n_rows;
  unsigned long long s = 0;
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n_rows; r += gridDim.x * blockDim.x) s += c[r];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(acc + k, s);
}

// Coset order position k <-> bit-reversed circle-domain storage row (utils.rs:96-115):
// coset[2i] = natural[i], coset[2i+1] = natural[n-1-i].
__device__ __forceinline__ uint32_t coset_to_storage(uint32_t k, uint32_t log_n) {
  uint32_t n = 1u << log_n;
  uint32_t nat = (k & 1) ? (n - 1 - (k >> 1)) : (k >> 1);
  return brev(nat, log_n);
}

// tmp[k] = col[storage(k)] - shift  (four coordinate columns, blockIdx.y)
// `sums` holds the column's claimed sum as 64-bit coordinate sums (k_column_sums); the shift
// claimed_sum / 2^log_n is taken on the device, so the host needs no read-back here.
__global__ void k_coset_gather(uint32_t* cols, uint32_t log_n, const unsigned long long* sums, uint32_t inv_n,
                               uint32_t* tmp) {
  pdl_enter();
  uint32_t k = blockIdx.y;
  uint32_t n = 1u << log_n;
  const uint32_t sh = m31_mul(fold64_p(sums[k]), inv_n);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    tmp[(size_t)k * n + i] = m31_sub(cols[(size_t)k * n + coset_to_storage(i, log_n)], sh);
}
__global__ void k_coset_scatter(uint32_t* cols, uint32_t log_n, const uint32_t* tmp) {
  pdl_enter();
  uint32_t k = blockIdx.y;
  uint32_t n = 1u << log_n;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    cols[(size_t)k * n + coset_to_storage(i, log_n)] = tmp[(size_t)k * n + i];
}

// Inclusive M31 scan of `len` words per row (blockIdx.y) in tiles of 4096 (256 threads x 16).
// Tile totals go to `sums` (exclusive offsets are applied by k_scan_add).
__global__ void __launch_bounds__(256) k_scan_tiles(uint32_t* data, uint32_t len, uint32_t* sums, uint32_t n_tiles) {
  pdl_enter();
  __shared__ uint32_t warp_tot[8];
  uint32_t* d = data + (size_t)blockIdx.y * len;
  uint32_t base = blockIdx.x * 4096 + threadIdx.x * 16;
  uint32_t v[16];
  uint32_t run = 0;
#pragma unroll
  for (int i = 0; i < 16; i++) {
    uint32_t x = base + i < len ? d[base + i] : 0;
    run = m31_add(run, x);
    v[i] = run;
  }
  // Exclusive scan of the thread totals within the block.
  uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t incl = run;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= (uint32_t)o) incl = m31_add(incl, y);
  }
  if (lane == 31) warp_tot[w] = incl;
  __syncthreads();
  uint32_t wpre = 0;
  for (uint32_t j = 0; j < w; j++) wpre = m31_add(wpre, warp_tot[j]);
  uint32_t excl = m31_add(wpre, m31_sub(incl, run));
#pragma unroll
  for (int i = 0; i < 16; i++)
    if (base + i < len) d[base + i] = m31_add(v[i], excl);
  if (threadIdx.x == 255) sums[(size_t)blockIdx.y * n_tiles + blockIdx.x] = m31_add(excl, run);
}
__global__ void k_scan_add(uint32_t* data, uint32_t len, const uint32_t* tile_offsets, uint32_t n_tiles) {
  pdl_enter();
  uint32_t* d = data + (size_t)blockIdx.y * len;
  uint32_t t = blockIdx.x;
  if (t == 0) return;
  uint32_t off = tile_offsets[(size_t)blockIdx.y * n_tiles + t - 1];
  for (uint32_t i = threadIdx.x; i < 4096; i += blockDim.x) {
    uint32_t idx = t * 4096 + i;
    if (idx < len) d[idx] = m31_add(d[idx], off);
  }
}

// Inclusive scan of `rows` arrays of `len` words (len <= 4096^2), in place.
// finalize_last for columns of at most 2^FIN_ONE_BLOCK_LOG rows in one launch: block k owns
// coordinate column k. It sums the column (the claimed sum's coordinate, also written to
// sums[k]), then scans the shifted values in coset order: each thread takes a run of consecutive
// coset positions, the run totals are scanned across the block, and a second pass writes the
// prefix sums back. The column stays in L2 between the passes. One block per column is bound by
// the latency of its scattered coset-order accesses, so above 2^14 rows the multi-launch path
// below is faster (2^16 rows: 0.12 ms against 0.045 ms); below it, one launch beats seven.
constexpr uint32_t FIN_ONE_BLOCK_LOG = 14;
constexpr uint32_t FIN_THREADS = 1024;

__global__ void __launch_bounds__(FIN_THREADS) k_logup_finalize_small(uint32_t* cols, uint32_t log_n, uint32_t inv_n,
                                                                      unsigned long long* sums) {
  pdl_enter();
  __shared__ unsigned long long s_sum[FIN_THREADS / 32];
  __shared__ uint32_t s_scan[FIN_THREADS / 32];
  __shared__ uint32_t s_shift;
  const uint32_t k = blockIdx.x, t = threadIdx.x, lane = t & 31, w = t >> 5;
  const uint32_t n = 1u << log_n;
  uint32_t* c = cols + (size_t)k * n;
  unsigned long long sum = 0;
  for (uint32_t r = t; r < n; r += FIN_THREADS) sum += c[r];
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if (lane == 0) s_sum[w] = sum;
  __syncthreads();
  if (t == 0) {
    unsigned long long tot = 0;
    for (uint32_t i = 0; i < FIN_THREADS / 32; i++) tot += s_sum[i];
    sums[k] = tot;
    s_shift = m31_mul(fold64_p(tot), inv_n);
  }
  __syncthreads();
  const uint32_t sh = s_shift;
  // Coset positions [t * run, (t + 1) * run) belong to thread t.
  const uint32_t run = n >= FIN_THREADS ? n / FIN_THREADS : 1u;
  const uint32_t k0 = t * run;
  const bool own = k0 < n;
  uint32_t tot = 0;
  if (own)
    for (uint32_t i = 0; i < run; i++) tot = m31_add(tot, m31_sub(c[coset_to_storage(k0 + i, log_n)], sh));
  // Exclusive scan of the run totals across the block.
  uint32_t inc = tot;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= (uint32_t)o) inc = m31_add(inc, y);
  }
  if (lane == 31) s_scan[w] = inc;
  __syncthreads();
  if (w == 0) {
    uint32_t x = s_scan[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= (uint32_t)o) x = m31_add(x, y);
    }
    s_scan[lane] = x;  // inclusive over warps
  }
  __syncthreads();
  uint32_t acc = m31_sub(inc, tot);  // exclusive within the warp
  if (w > 0) acc = m31_add(acc, s_scan[w - 1]);
  if (own)
    for (uint32_t i = 0; i < run; i++) {
      const uint32_t st = coset_to_storage(k0 + i, log_n);
      acc = m31_add(acc, m31_sub(c[st], sh));
      c[st] = acc;
    }
}

static int32_t scan_rows(uint32_t* data, uint32_t len, uint32_t rows, Arena& arena, cudaStream_t s) {
  uint32_t n_tiles = (len + 4095) / 4096;
  STWO_REQUIRE(n_tiles <= 4096, "scan length too large");
  uint32_t* sums = arena.alloc((size_t)n_tiles * rows);
  if (!sums) return STWO_ERR_OOM;
  launch_pdl(k_scan_tiles, dim3(n_tiles, rows), dim3(256), 0, s, data, len, sums, n_tiles);
  note_launch();
  STWO_LAUNCH_CHECK();
  if (n_tiles > 1) {
    uint32_t* sums2 = arena.alloc(rows);
    if (!sums2) return STWO_ERR_OOM;
    launch_pdl(k_scan_tiles, dim3(1, rows), dim3(256), 0, s, sums, n_tiles, sums2, 1);
    note_launch();
    STWO_LAUNCH_CHECK();
    launch_pdl(k_scan_add, dim3(n_tiles, rows), dim3(256), 0, s, data, len, sums, n_tiles);
    note_launch();
    STWO_LAUNCH_CHECK();
  }
  return STWO_OK;
}

// LogupTraceGenerator::finalize_last (logup.rs:150-190) on the device for the last secure column
// (four contiguous coordinate columns of 2^log_n words): its coordinate sums (the claimed sum),
// the column minus claimed_sum / 2^log_n, and the inclusive prefix sum in coset order. The sums
// land in small_pinned(); with `claimed` set the stream is synchronised and the claimed sum
// returned, otherwise the caller reads small_pinned() after its next synchronisation.
int32_t logup_finalize_last(uint32_t* last, uint32_t log_n, Arena& arena, cudaStream_t s, hq* claimed) {
  const size_t n = (size_t)1 << log_n;
  unsigned long long* d_sums = reinterpret_cast<unsigned long long*>(arena.alloc(8));
  if (!d_sums) return STWO_ERR_OOM;
  if (log_n <= FIN_ONE_BLOCK_LOG) {
    launch_pdl(k_logup_finalize_small, dim3(4), dim3(FIN_THREADS), 0, s, last, log_n, h_inv((uint32_t)(n % P)), d_sums);
    note_launch();
    STWO_LAUNCH_CHECK();
    unsigned long long* hs = small_pinned();
    if (!hs) return STWO_ERR_OOM;
    STWO_CHECK_CUDA(cudaMemcpyAsync(hs, d_sums, 32, cudaMemcpyDeviceToHost, s));
    if (claimed) {
      STWO_CHECK_CUDA(cudaStreamSynchronize(s));
      *claimed = hq_make((uint32_t)(hs[0] % P), (uint32_t)(hs[1] % P), (uint32_t)(hs[2] % P), (uint32_t)(hs[3] % P));
    }
    return STWO_OK;
  }
  uint32_t* tmp = arena.alloc(4 * n);
  if (!tmp) return STWO_ERR_OOM;
  STWO_CHECK_CUDA(cudaMemsetAsync(d_sums, 0, 32, s));
  const uint32_t g = std::min<uint32_t>((uint32_t)((n + 255) / 256), 1024);
  launch_pdl(k_column_sums, dim3(g, 4), dim3(256), 0, s, last, (uint32_t)n, d_sums);
  note_launch();
  STWO_LAUNCH_CHECK();
  unsigned long long* hs = small_pinned();
  if (!hs) return STWO_ERR_OOM;
  STWO_CHECK_CUDA(cudaMemcpyAsync(hs, d_sums, 32, cudaMemcpyDeviceToHost, s));
  launch_pdl(k_coset_gather, dim3(g, 4), dim3(256), 0, s, last, log_n, d_sums, h_inv((uint32_t)(n % P)), tmp);
  note_launch();
  STWO_LAUNCH_CHECK();
  int32_t st = scan_rows(tmp, (uint32_t)n, 4, arena, s);
  if (st) return st;
  launch_pdl(k_coset_scatter, dim3(g, 4), dim3(256), 0, s, last, log_n, tmp);
  note_launch();
  STWO_LAUNCH_CHECK();
  if (claimed) {
    STWO_CHECK_CUDA(cudaStreamSynchronize(s));
    *claimed = hq_make((uint32_t)(hs[0] % P), (uint32_t)(hs[1] % P), (uint32_t)(hs[2] % P), (uint32_t)(hs[3] % P));
  }
  return STWO_OK;
}

// ------------------------------------------------------------------------------------ composition
struct PoseidonParams {
  uint32_t trace_log, eval_log;
  uint32_t accumulate;  // add row_res * denom_inv to the output columns instead of writing it
  uint32_t shift[4];  // claimed_sum / 2^trace_log
  LookupConsts lc;
};

__device__ __forceinline__ uint32_t prev_row_index(uint32_t r, uint32_t trace_log, uint32_t eval_log) {
  // offset_bit_reversed_circle_domain_index(r, trace_log, eval_log, -1) (core/utils.rs:74-90)
  uint32_t prev = brev(r, eval_log);
  uint32_t half = 1u << (eval_log - 1);
  uint32_t step = 1u << (eval_log - trace_log - 1);
  if (prev < half) prev = (prev + half - step) & (half - 1);
  else prev = ((prev - half + step) & (half - 1)) + half;
  return brev(prev, eval_log);
}

// Trace (1264) and interaction (32) columns are contiguous blocks with a stride of 2^eval_log
// words, so a mask value is one load at base + (col << eval_log) + row.
//
// A block takes tiles of 32 rows; warp w evaluates permutation w of every row of the tile (its
// 142 round constraints and LogUp batch w), so each warp reads the columns of one permutation
// with one coalesced 128-byte load per column, and a row's eight partial sums meet in shared
// memory. The random-coefficient sum is exact in the field, so splitting it by permutation gives
// the same words as accumulating the constraints in order. Eight warps per row keep the latency
// of a small evaluation domain at one permutation, and the grid, a few tiles per resident block,
// loads the coefficient table once per block.
constexpr uint32_t PC_ROWS = 32;
constexpr uint32_t PC_THREADS = 32 * PS_REPS;
constexpr uint32_t PC_BLOCKS_PER_SM = 4;  // 64 registers: the rounds still run without spills

__global__ void __launch_bounds__(PC_THREADS, PC_BLOCKS_PER_SM)
    k_poseidon_composition(const uint32_t* __restrict__ trace, const uint32_t* __restrict__ inter, uint32_t n_rows,
                           PoseidonParams pp, const uint32_t* __restrict__ coeffs, const uint32_t* __restrict__ dinv,
                           uint32_t* o0, uint32_t* o1, uint32_t* o2, uint32_t* o3) {
  pdl_enter();
  __shared__ uint32_t s_coeffs[4 * PS_N_CONSTRAINTS];
  __shared__ uint32_t s_part[PS_REPS][4][PC_ROWS];
  extern __shared__ uint32_t s_masks[];  // per warp: 2 slots x 16 columns x 32 rows
  for (uint32_t i = threadIdx.x; i < 4 * PS_N_CONSTRAINTS; i += blockDim.x) s_coeffs[i] = coeffs[i];
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31, rep = threadIdx.x >> 5;
  uint32_t* const mb = s_masks + rep * (2 * PS_ST * PC_ROWS) + lane;
  const uint32_t el = pp.eval_log;
  const uint32_t n_tiles = (n_rows + PC_ROWS - 1) / PC_ROWS;
  auto col = [&](const uint32_t* base, uint32_t c, uint32_t row) { return __ldg(base + ((size_t)c << el) + row); };
  for (uint32_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const uint32_t r_out = tile * PC_ROWS + lane;
    const uint32_t r = min(r_out, n_rows - 1);  // lanes past the end compute a copy and write nothing
    unsigned long long a0 = 0, a1 = 0, a2 = 0, a3 = 0;
    uint32_t cnt = 0;
    int ci = rep * (PS_COLS_PER_REP - PS_ST);  // 142 round constraints per permutation
    auto acc = [&](uint32_t cons) {
      const uint32_t* k = s_coeffs + 4 * ci++;
      a0 += (unsigned long long)k[0] * cons;
      a1 += (unsigned long long)k[1] * cons;
      a2 += (unsigned long long)k[2] * cons;
      a3 += (unsigned long long)k[3] * cons;
      // Products are at most (P - 1)^2 and a folded sum is below 2^33 + 2^31: four products fit
      // between folds without passing 2^64.
      if (++cnt == 4) {
        a0 = (a0 & P) + (a0 >> 31);
        a1 = (a1 & P) + (a1 >> 31);
        a2 = (a2 & P) + (a2 >> 31);
        a3 = (a3 & P) + (a3 >> 31);
        cnt = 0;
      }
    };
    const uint32_t c0 = rep * PS_COLS_PER_REP;
    // First mask column of full round k (four before the partial rounds, four after).
    auto full_col = [&](uint32_t k) {
      return c0 + PS_ST * (1 + k) + (k >= PS_HALF ? PS_PARTIAL : 0u);
    };
    // A full round's 16 mask columns go to this warp's shared-memory slot by cp.async, one round
    // ahead of their use: each lane copies (and later reads) its own row's words, so the copies need
    // no barrier, only the lane's own wait_group.
    auto issue_full = [&](uint32_t slot, uint32_t col0) {
#pragma unroll
      for (int i = 0; i < PS_ST; i++) {
        const uint32_t* g = trace + ((size_t)(col0 + i) << el) + r;
        const uint32_t sa = (uint32_t)__cvta_generic_to_shared(mb + (slot * PS_ST + i) * 32);
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(g) : "memory");
      }
      asm volatile("cp.async.commit_group;\n" ::: "memory");
    };
    issue_full(0, full_col(0));
    uint32_t s[PS_ST];
#pragma unroll
    for (int i = 0; i < PS_ST; i++) s[i] = col(trace, c0 + i, r);
    // The lookup value of the initial state, taken now so that the state need not be kept.
    const qm31 d0 = combine16(pp.lc, s);
    uint32_t mc = c0 + PS_ST * (1 + PS_HALF);  // the first partial round's column
    auto full_round = [&](uint32_t k) {
      if (k + 1 < 2 * PS_HALF) {
        issue_full((k + 1) & 1, full_col(k + 1));
        asm volatile("cp.async.wait_group 1;\n" ::: "memory");
      } else {
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
      }
      const uint32_t* m = mb + (k & 1) * PS_ST * 32;
#pragma unroll
      for (int i = 0; i < PS_ST; i++) s[i] = m31_add(s[i], PS_RC);
      external_matrix(s);
#pragma unroll
      for (int i = 0; i < PS_ST; i++) {
        const uint32_t mi = m[i * 32];
        acc(m31_sub(pow5(s[i]), mi));
        s[i] = mi;
      }
    };
    // The rounds stay loops: fully unrolled, the kernel outgrew the instruction cache and stalled
    // on instruction fetch.
#pragma unroll 1
    for (uint32_t round = 0; round < PS_HALF; round++) full_round(round);
    // A partial round has little arithmetic to hide its one load behind: the mask of the next
    // round is fetched one round ahead.
    uint32_t m_next = col(trace, mc, r);
#pragma unroll 1
    for (int round = 0; round < PS_PARTIAL; round++) {
      const uint32_t m = m_next;
      if (round + 1 < PS_PARTIAL) m_next = col(trace, mc + round + 1, r);
      s[0] = m31_add(s[0], PS_RC);
      internal_matrix(s);
      acc(m31_sub(pow5(s[0]), m));
      s[0] = m;
    }
#pragma unroll 1
    for (uint32_t round = PS_HALF; round < 2 * PS_HALF; round++) full_round(round);
    // LogUp batch `rep`: fraction (1/d0 - 1/d1) = (d1 - d0) / (d0 d1), against the cumulative
    // column of this batch minus that of the previous one (for the last batch: minus its value at
    // the previous trace row and plus claimed_sum / 2^trace_log).
    const qm31 d1 = combine16(pp.lc, s);
    qm31 num = qm31_sub(d1, d0), den = qm31_mul(d0, d1);
    const uint32_t ic = 4 * rep;
    qm31 diff = qm31_from_u32(col(inter, ic, r), col(inter, ic + 1, r), col(inter, ic + 2, r), col(inter, ic + 3, r));
    if (rep > 0)
      diff = qm31_sub(diff, qm31_from_u32(col(inter, ic - 4, r), col(inter, ic - 3, r), col(inter, ic - 2, r),
                                          col(inter, ic - 1, r)));
    if (rep + 1 == PS_REPS) {
      const uint32_t rp = prev_row_index(r, pp.trace_log, pp.eval_log);
      qm31 prev = qm31_from_u32(col(inter, ic, rp), col(inter, ic + 1, rp), col(inter, ic + 2, rp),
                                col(inter, ic + 3, rp));
      diff = qm31_add(qm31_sub(diff, prev), qm31_from_u32(pp.shift[0], pp.shift[1], pp.shift[2], pp.shift[3]));
    }
    qm31 cons = qm31_sub(qm31_mul(diff, den), num);
    const uint32_t* k = s_coeffs + 4 * (PS_N_CONSTRAINTS - PS_REPS + rep);
    qm31 res = qm31_add(qm31_from_u32(fold64_p(a0), fold64_p(a1), fold64_p(a2), fold64_p(a3)),
                        qm31_mul(qm31_from_u32(k[0], k[1], k[2], k[3]), cons));
    s_part[rep][0][lane] = res.a.a;
    s_part[rep][1][lane] = res.a.b;
    s_part[rep][2][lane] = res.b.a;
    s_part[rep][3][lane] = res.b.b;
    __syncthreads();
    // Warps 0..3 each finish one coordinate of the tile's 32 rows.
    if (rep < 4) {
      uint32_t v = s_part[0][rep][lane];
#pragma unroll
      for (int w = 1; w < PS_REPS; w++) v = m31_add(v, s_part[w][rep][lane]);
      if (r_out < n_rows) {
        uint32_t* o = rep == 0 ? o0 : rep == 1 ? o1 : rep == 2 ? o2 : o3;
        v = m31_mul(v, __ldg(dinv + (r_out >> pp.trace_log)));
        if (pp.accumulate) v = m31_add(o[r_out], v);
        o[r_out] = v;
      }
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------------------------ host side
static hq hq_m(hq x, uint32_t m) {
  for (int i = 0; i < 4; i++) x.v[i] = h_mul(x.v[i], m);
  return x;
}

struct HLookup {
  hq z, alpha_pow[PS_ST];
  template <class V>
  hq combine(const V* v) const;
};
template <>
hq HLookup::combine<hq>(const hq* v) const {
  hq acc = hq_make(0, 0, 0, 0);
  for (int i = 0; i < PS_ST; i++) acc = hq_add(acc, hq_mul(alpha_pow[i], v[i]));
  return hq_sub(acc, z);
}

struct PoseidonGpuAir : GpuAir {
  uint32_t log_n;
  HLookup le;
  hq claimed_sum;
  PoseidonGpuAir(uint32_t l, const HLookup& e, hq cs) : log_n(l), le(e), claimed_sum(cs) {}
  uint32_t log_size() const override { return log_n; }
  uint32_t max_constraint_log_degree_bound() const override { return log_n + PS_LOG_EXPAND; }
  size_t n_constraints() const override { return PS_N_CONSTRAINTS; }
  std::vector<std::vector<std::vector<int>>> mask_offsets() const override {
    std::vector<std::vector<std::vector<int>>> m(3);
    m[1].assign(PS_COLS, {0});
    for (int b = 0; b + 1 < PS_REPS; b++)
      for (int k = 0; k < 4; k++) m[2].push_back({0});
    for (int k = 0; k < 4; k++) m[2].push_back({-1, 0});
    return m;
  }
  hq shift() const { return hq_m(claimed_sum, h_inv((uint32_t)((1ull << log_n) % P))); }
  int32_t eval_composition(const std::vector<std::vector<const uint32_t*>>& cols, const uint32_t* coeffs,
                           const uint32_t* dinv, uint32_t* const acc[4], bool accumulate,
                           cudaStream_t s) const override {
    STWO_REQUIRE(cols.size() >= 3 && cols[1].size() == PS_COLS && cols[2].size() == PS_INTERACTION_COLS,
                 "trace trees mismatch");
    // The prover hands each tree's columns on the evaluation domain as one contiguous block.
    const uint32_t el = log_n + PS_LOG_EXPAND;
    for (int c = 0; c < PS_COLS; c++)
      STWO_REQUIRE(cols[1][c] == cols[1][0] + ((size_t)c << el), "trace columns are not one contiguous block");
    for (int c = 0; c < PS_INTERACTION_COLS; c++)
      STWO_REQUIRE(cols[2][c] == cols[2][0] + ((size_t)c << el), "interaction columns are not one contiguous block");
    PoseidonParams pp;
    pp.trace_log = log_n;
    pp.eval_log = log_n + PS_LOG_EXPAND;
    pp.accumulate = accumulate ? 1u : 0u;
    hq sh = shift();
    for (int i = 0; i < 4; i++) pp.shift[i] = sh.v[i];
    for (int i = 0; i < 4; i++) pp.lc.z[i] = le.z.v[i];
    for (int j = 0; j < PS_ST; j++)
      for (int i = 0; i < 4; i++) pp.lc.alpha_pow[j][i] = le.alpha_pow[j].v[i];
    uint32_t n_rows = 1u << pp.eval_log;
    const uint32_t n_tiles = (n_rows + PC_ROWS - 1) / PC_ROWS;
    const uint32_t grid = std::min<uint32_t>(n_tiles, (uint32_t)sm_count() * PC_BLOCKS_PER_SM);
    // 22.4 KB of static shared memory plus the 32 KB of mask slots: above the default 48 KB, so
    // the dynamic part needs the opt-in attribute (once per device, with the carveout).
    constexpr size_t mask_smem = (size_t)PS_REPS * 2 * PS_ST * PC_ROWS * 4;
    {
      static std::mutex mu;
      static bool done[256] = {};
      int dev = 0;
      STWO_CHECK_CUDA(cudaGetDevice(&dev));
      STWO_REQUIRE(dev >= 0 && dev < 256, "device ordinal %d out of range", dev);
      std::lock_guard<std::mutex> g(mu);
      if (!done[dev]) {
        STWO_CHECK_CUDA(cudaFuncSetAttribute(k_poseidon_composition, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)mask_smem));
        // Four blocks of 54.4 KB need the largest shared-memory carveout of the SM.
        STWO_CHECK_CUDA(cudaFuncSetAttribute(k_poseidon_composition, cudaFuncAttributePreferredSharedMemoryCarveout,
                                             (int)cudaSharedmemCarveoutMaxShared));
        done[dev] = true;
      }
    }
    launch_pdl(k_poseidon_composition, dim3(grid), dim3(PC_THREADS), mask_smem, s, cols[1][0], cols[2][0], n_rows, pp,
               coeffs, dinv, acc[0], acc[1], acc[2], acc[3]);
    note_launch();
    cudaError_t e = cudaGetLastError();
    if (e) {
      set_error("poseidon composition: %s", cudaGetErrorString(e));
      return STWO_ERR_CUDA;
    }
    return STWO_OK;
  }
  // The same constraints over QM31 at the OODS point (PointEvaluator).
  hq eval_at_point(const std::vector<std::vector<std::vector<hq>>>& mask, hq rc, hq denom_inv) const override {
    // The PointEvaluator accumulation acc <- acc * rc + denom_inv * c, with denom_inv factored out
    // of the sum (one product per constraint fewer, the same field element).
    hq acc = hq_make(0, 0, 0, 0);
    auto add = [&](hq c) { acc = hq_add(hq_mul(acc, rc), c); };
    auto m4 = [](hq* x) {
      hq t0 = hq_add(x[0], x[1]), t02 = hq_add(t0, t0), t1 = hq_add(x[2], x[3]), t12 = hq_add(t1, t1);
      hq t2 = hq_add(hq_add(x[1], x[1]), t1), t3 = hq_add(hq_add(x[3], x[3]), t0);
      hq t4 = hq_add(hq_add(t12, t12), t3), t5 = hq_add(hq_add(t02, t02), t2);
      x[0] = hq_add(t3, t5);
      x[1] = t5;
      x[2] = hq_add(t2, t4);
      x[3] = t4;
    };
    auto ext = [&](hq* st) {
      for (int i = 0; i < 4; i++) m4(st + 4 * i);
      for (int j = 0; j < 4; j++) {
        hq t = hq_add(hq_add(st[j], st[j + 4]), hq_add(st[j + 8], st[j + 12]));
        for (int i = 0; i < 4; i++) st[4 * i + j] = hq_add(st[4 * i + j], t);
      }
    };
    auto p5 = [](hq x) {
      hq x2 = hq_mul(x, x);
      return hq_mul(hq_mul(x2, x2), x);
    };
    const hq rcq = hq_make(PS_RC, 0, 0, 0);
    const auto& t = mask[1];
    const auto& it = mask[2];
    std::vector<std::pair<hq, hq>> fr;  // (num, den) per batch
    size_t mc = 0;
    for (int rep = 0; rep < PS_REPS; rep++) {
      hq s[PS_ST], init[PS_ST];
      for (int i = 0; i < PS_ST; i++) init[i] = s[i] = t[mc++][0];
      for (int round = 0; round < 2 * PS_HALF + PS_PARTIAL; round++) {
        bool full = round < PS_HALF || round >= PS_HALF + PS_PARTIAL;
        if (full) {
          for (int i = 0; i < PS_ST; i++) s[i] = hq_add(s[i], rcq);
          ext(s);
          for (int i = 0; i < PS_ST; i++) {
            hq m = t[mc++][0];
            add(hq_sub(p5(s[i]), m));
            s[i] = m;
          }
        } else {
          s[0] = hq_add(s[0], rcq);
          hq sum = s[0];
          for (int i = 1; i < 16; i++) sum = hq_add(sum, s[i]);
          for (int i = 0; i < 16; i++) s[i] = hq_add(hq_m(s[i], 1u << (i + 1)), sum);
          hq m = t[mc++][0];
          add(hq_sub(p5(s[0]), m));
          s[0] = m;
        }
      }
      hq d0 = le.combine(init), d1 = le.combine(s);
      fr.push_back({hq_sub(d1, d0), hq_mul(d0, d1)});
    }
    auto comb = [](const std::vector<hq>& c0, const std::vector<hq>& c1, const std::vector<hq>& c2,
                   const std::vector<hq>& c3, size_t j) {
      return hq_add(hq_add(c0[j], hq_mul(c1[j], hq_make(0, 1, 0, 0))),
                    hq_add(hq_mul(c2[j], hq_make(0, 0, 1, 0)), hq_mul(c3[j], hq_make(0, 0, 0, 1))));
    };
    hq prev_col = hq_make(0, 0, 0, 0);
    for (int b = 0; b < PS_REPS; b++) {
      const auto& c0 = it[4 * b];
      const auto& c1 = it[4 * b + 1];
      const auto& c2 = it[4 * b + 2];
      const auto& c3 = it[4 * b + 3];
      hq diff;
      if (b + 1 < PS_REPS) {
        hq cur = comb(c0, c1, c2, c3, 0);
        diff = hq_sub(cur, prev_col);
        prev_col = cur;
      } else {
        hq prev = comb(c0, c1, c2, c3, 0), cur = comb(c0, c1, c2, c3, 1);
        diff = hq_add(hq_sub(hq_sub(cur, prev), prev_col), shift());
      }
      add(hq_sub(hq_mul(diff, fr[b].second), fr[b].first));
    }
    return hq_mul(acc, denom_inv);
  }
};

GpuAir* new_poseidon_air(uint32_t log_n, const hq& z, const hq& alpha, const hq& claimed_sum) {
  HLookup le;
  le.z = z;
  hq cur = hq_make(1, 0, 0, 0);
  for (int i = 0; i < PS_ST; i++) {
    le.alpha_pow[i] = cur;
    cur = hq_mul(cur, alpha);
  }
  return new PoseidonGpuAir(log_n, le, claimed_sum);
}

}  // namespace stwo

using namespace stwo;

extern "C" stwo_status stwo_prove_poseidon(uint32_t log_n_rows, const uint32_t* d_init, stwo_pcs_config cfg,
                                           uint8_t* h_proof, size_t capacity, size_t* h_len,
                                           stwo_qm31* h_claimed_sum, void* stream) {
  STWO_REQUIRE(log_n_rows >= 4 && log_n_rows + PS_LOG_EXPAND + cfg.log_blowup_factor <= 28, "bad log_n_rows");
  STWO_REQUIRE(cfg.log_blowup_factor >= 1 && cfg.log_blowup_factor <= 16, "log_blowup_factor out of [1, 16]");
  STWO_REQUIRE(cfg.log_last_layer_degree_bound <= 10, "log_last_layer_degree_bound > 10");
  STWO_REQUIRE(h_len, "null length");
  cudaStream_t s = as_stream(stream);
  std::vector<uint8_t> bytes;
  hq claimed = hq_make(0, 0, 0, 0);
  int32_t st;
  {
    Prover pv(cfg, log_n_rows + PS_LOG_EXPAND + cfg.log_blowup_factor, s);
    if (pv.init_status) return pv.init_status;
    size_t n = (size_t)1 << log_n_rows;
    st = pv.commit_polys({}, {});
    uint32_t* trace = nullptr;
    uint32_t* lookups = nullptr;
    uint32_t* inter = nullptr;
    if (!st) {
      trace = pv.arena.alloc(n * PS_COLS);
      lookups = pv.arena.alloc(n * 32 * PS_REPS);
      inter = pv.arena.alloc(n * PS_INTERACTION_COLS);
      if (!trace || !lookups || !inter) st = STWO_ERR_OOM;
    }
    if (!st) {
      StageScope stage("Generation", s);
      launch_pdl(k_poseidon_trace, dim3((uint32_t)((n + 31) / 32)), dim3(32 * PS_REPS), 0, s, (uint32_t)n, d_init,
                 trace, lookups);
      note_launch();
      if (cudaGetLastError() != cudaSuccess) st = STWO_ERR_CUDA;
    }
    if (!st) {
      std::vector<uint32_t*> cols(PS_COLS);
      for (int c = 0; c < PS_COLS; c++) cols[c] = trace + (size_t)c * n;
      st = pv.commit_evals(cols, log_n_rows);
    }
    HLookup le;
    if (!st) {
      // PoseidonElements::draw: draw_felts(2) = one draw of 8 base felts (logup.rs:74-88).
      auto f = pv.ch.draw_base_felts();
      le.z = hq_make(f[0], f[1], f[2], f[3]);
      hq alpha = hq_make(f[4], f[5], f[6], f[7]);
      hq cur = hq_make(1, 0, 0, 0);
      for (int i = 0; i < PS_ST; i++) {
        le.alpha_pow[i] = cur;
        cur = hq_mul(cur, alpha);
      }
      StageScope stage("Interaction", s);
      LookupConsts lc;
      for (int i = 0; i < 4; i++) lc.z[i] = le.z.v[i];
      for (int j = 0; j < PS_ST; j++)
        for (int i = 0; i < 4; i++) lc.alpha_pow[j][i] = le.alpha_pow[j].v[i];
      // Two-warp blocks: 2^16 rows make 1,024 blocks, 6-7 per SM (128-thread blocks left some SMs
      // with three of four busy for the last quarter of the launch).
      launch_pdl(k_poseidon_interaction, dim3((uint32_t)((n + 63) / 64)), dim3(64), 0, s, (uint32_t)n, lookups, lc,
                 inter);
      note_launch();
      if (cudaGetLastError() != cudaSuccess) st = STWO_ERR_CUDA;
    }
    if (!st) {
      // Claimed sum of the last column, its shift, and the coset-order prefix sum (logup.rs:155-195).
      // The claimed sum reaches the host with the next synchronisation (the interaction commitment's).
      st = logup_finalize_last(inter + (size_t)(PS_INTERACTION_COLS - 4) * n, log_n_rows, pv.arena, s, nullptr);
    }
    if (!st) {
      std::vector<uint32_t*> cols(PS_INTERACTION_COLS);
      for (int c = 0; c < PS_INTERACTION_COLS; c++) cols[c] = inter + (size_t)c * n;
      st = pv.commit_evals(cols, log_n_rows);
    }
    if (!st) {
      STWO_CHECK_CUDA(cudaStreamSynchronize(s));  // already idle: the commitment read its root
      const unsigned long long* hs = small_pinned();
      claimed = hq_make((uint32_t)(hs[0] % P), (uint32_t)(hs[1] % P), (uint32_t)(hs[2] % P), (uint32_t)(hs[3] % P));
    }
    if (!st) {
      PoseidonGpuAir air(log_n_rows, le, claimed);
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
