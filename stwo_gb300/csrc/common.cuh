// Shared runtime for the sm_103a backend: status codes, error capture, the per-device
// context (twiddle-tree cache, stream-ordered scratch) and launch helpers.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <mutex>
#include <map>
#include <vector>
#include <tuple>
#include <algorithm>
#include <atomic>
#include "../../include/stwo_cuda.h"
#include "field.cuh"

namespace stwo {

// Last error detail, per host thread (the status code is the contract; this is for humans).
void set_error(const char* fmt, ...);

#define STWO_CHECK_CUDA(expr)                                                        \
  do {                                                                               \
    cudaError_t _e = (expr);                                                         \
    if (_e != cudaSuccess) {                                                         \
      ::stwo::set_error("%s:%d %s: %s", __FILE__, __LINE__, #expr, cudaGetErrorString(_e)); \
      return (_e == cudaErrorMemoryAllocation) ? STWO_ERR_OOM : STWO_ERR_CUDA;       \
    }                                                                                \
  } while (0)

#define STWO_REQUIRE(cond, ...)                 \
  do {                                          \
    if (!(cond)) {                              \
      ::stwo::set_error(__VA_ARGS__);           \
      return STWO_ERR_INVALID_ARG;              \
    }                                           \
  } while (0)

#define STWO_LAUNCH_CHECK()                                                          \
  do {                                                                               \
    cudaError_t _e = cudaGetLastError();                                             \
    if (_e != cudaSuccess) {                                                         \
      ::stwo::set_error("%s:%d launch: %s", __FILE__, __LINE__, cudaGetErrorString(_e)); \
      return STWO_ERR_CUDA;                                                          \
    }                                                                                \
  } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Index arithmetic on the circle group (indices mod 2^31), host side.
constexpr uint32_t IDX_MASK = (1u << 31) - 1;
inline uint32_t idx_reduce(uint64_t i) { return (uint32_t)(i & IDX_MASK); }

inline stwo_coset coset_double(stwo_coset c) {
  return {idx_reduce((uint64_t)c.initial_index * 2), idx_reduce((uint64_t)c.step_size * 2),
          c.log_size ? c.log_size - 1 : 0};
}
// Indices compare modulo 2^31 (a log-0 coset's step 2^31 equals a doubled step 0).
inline bool coset_eq(stwo_coset a, stwo_coset b) {
  return idx_reduce(a.initial_index) == idx_reduce(b.initial_index) &&
         idx_reduce(a.step_size) == idx_reduce(b.step_size) && a.log_size == b.log_size;
}
inline bool coset_is_doubling_of(stwo_coset small, stwo_coset big) {
  if (small.log_size > big.log_size) return false;
  stwo_coset c = big;
  for (uint32_t i = small.log_size; i < big.log_size; i++) c = coset_double(c);
  return coset_eq(c, small);
}
inline stwo_coset coset_new(uint32_t initial_index, uint32_t log_size) {
  return {idx_reduce(initial_index), idx_reduce(1ull << (31 - log_size)), log_size};
}
// CanonicCoset(log).half_coset() = Coset::half_odds(log - 1)
inline stwo_coset canonic_half_coset(uint32_t log) {
  return coset_new(1u << (31 - (log - 1 + 2)), log - 1);
}

// Host-side M31 helpers for O(1) setup scalars (never per-element work).
inline uint32_t h_add(uint32_t a, uint32_t b) { uint32_t s = a + b; return s >= P ? s - P : s; }
inline uint32_t h_sub(uint32_t a, uint32_t b) { return a >= b ? a - b : a + P - b; }
inline uint32_t h_mul(uint32_t a, uint32_t b) {
  // (a b) mod P for canonical a, b by folding the 62-bit product at bit 31 twice.
  uint64_t x = (uint64_t)a * b;
  x = (x & P) + (x >> 31);
  uint32_t r = (uint32_t)((x & P) + (x >> 31));
  return r >= P ? r - P : r;
}
inline uint32_t h_pow(uint32_t b, uint64_t e) { uint32_t r = 1; while (e) { if (e & 1) r = h_mul(r, b); b = h_mul(b, b); e >>= 1; } return r; }
inline uint32_t h_inv(uint32_t a) { return h_pow(a, P - 2); }
struct hpoint { uint32_t x, y; };
inline hpoint h_padd(hpoint p, hpoint q) {
  return {h_sub(h_mul(p.x, q.x), h_mul(p.y, q.y)), h_add(h_mul(p.x, q.y), h_mul(p.y, q.x))};
}
hpoint h_index_to_point(uint32_t idx);

// Host QM31 for O(#columns) setup constants (line coefficients, powers, mappings).
struct hq { uint32_t v[4]; };
inline hq hq_make(uint32_t a, uint32_t b, uint32_t c, uint32_t d) { return hq{{a, b, c, d}}; }
inline hq hq_from(const stwo_qm31& x) { return hq{{x.v[0], x.v[1], x.v[2], x.v[3]}}; }
inline hq hq_add(hq x, hq y) { hq r; for (int i = 0; i < 4; i++) r.v[i] = h_add(x.v[i], y.v[i]); return r; }
inline hq hq_sub(hq x, hq y) { hq r; for (int i = 0; i < 4; i++) r.v[i] = h_sub(x.v[i], y.v[i]); return r; }
inline void h_cmul(uint32_t x0, uint32_t x1, uint32_t y0, uint32_t y1, uint32_t* r0, uint32_t* r1) {
  uint32_t a = h_sub(h_mul(x0, y0), h_mul(x1, y1));
  uint32_t b = h_add(h_mul(x0, y1), h_mul(x1, y0));
  *r0 = a;
  *r1 = b;
}
// (a + bu)(c + du) = ac + (2+i) bd + (ad + bc) u over CM31, with a = x0 + x1 i, b = x2 + x3 i,
// c = y0 + y1 i, d = y2 + y3 i. Each product is folded once to below 2^32; the signed
// combinations are offset by a multiple of P and reduced once per coordinate.
inline uint64_t h_fold(uint64_t p) { return (p & P) + (p >> 31); }  // < 2^32, congruent mod P
inline uint32_t h_reduce64(uint64_t x) {
  x = (x & P) + (x >> 31);
  x = (x & P) + (x >> 31);
  uint32_t r = (uint32_t)x;
  return r >= P ? r - P : r;
}
inline hq hq_mul(hq x, hq y) {
  const uint64_t a0 = x.v[0], a1 = x.v[1], b0 = x.v[2], b1 = x.v[3];
  const uint64_t c0 = y.v[0], c1 = y.v[1], d0 = y.v[2], d1 = y.v[3];
  const uint64_t a0c0 = h_fold(a0 * c0), a1c1 = h_fold(a1 * c1), a0c1 = h_fold(a0 * c1), a1c0 = h_fold(a1 * c0);
  const uint64_t b0d0 = h_fold(b0 * d0), b1d1 = h_fold(b1 * d1), b0d1 = h_fold(b0 * d1), b1d0 = h_fold(b1 * d0);
  const uint64_t a0d0 = h_fold(a0 * d0), a1d1 = h_fold(a1 * d1), a0d1 = h_fold(a0 * d1), a1d0 = h_fold(a1 * d0);
  const uint64_t b0c0 = h_fold(b0 * c0), b1c1 = h_fold(b1 * c1), b0c1 = h_fold(b0 * c1), b1c0 = h_fold(b1 * c0);
  // Every folded term is < 2^32 < 3P, so 16P covers the largest negative part (5 terms).
  constexpr uint64_t K = 16ull * P;
  const uint64_t r0 = a0c0 + 2 * b0d0 + K - (a1c1 + 2 * b1d1 + b0d1 + b1d0);
  const uint64_t r1 = a0c1 + a1c0 + b0d0 + 2 * b0d1 + 2 * b1d0 + K - b1d1;
  const uint64_t r2 = a0d0 + b0c0 + K - (a1d1 + b1c1);
  const uint64_t r3 = a0d1 + a1d0 + b0c1 + b1c0;
  return hq{{h_reduce64(r0), h_reduce64(r1), h_reduce64(r2), h_reduce64(r3)}};
}
inline hq hq_conj(hq x) { return hq{{x.v[0], x.v[1], h_sub(0, x.v[2]), h_sub(0, x.v[3])}}; }
inline hq hq_pow(hq b, uint64_t e) { hq r = hq_make(1, 0, 0, 0); while (e) { if (e & 1) r = hq_mul(r, b); b = hq_mul(b, b); e >>= 1; } return r; }
inline hq hq_inv(hq x) {
  // (a + bu)^-1 = (a - bu) / (a^2 - (2+i) b^2), CM31 inverse via the norm (fields/qm31.rs:121-129).
  uint32_t b2r, b2i, a2r, a2i;
  h_cmul(x.v[2], x.v[3], x.v[2], x.v[3], &b2r, &b2i);
  h_cmul(x.v[0], x.v[1], x.v[0], x.v[1], &a2r, &a2i);
  uint32_t rb_r = h_sub(h_add(b2r, b2r), b2i), rb_i = h_add(b2r, h_add(b2i, b2i));
  uint32_t dr = h_sub(a2r, rb_r), di = h_sub(a2i, rb_i);
  uint32_t nrm = h_inv(h_add(h_mul(dr, dr), h_mul(di, di)));
  uint32_t ir = h_mul(dr, nrm), ii = h_mul(h_sub(0, di), nrm);
  uint32_t r0, r1, r2, r3;
  h_cmul(x.v[0], x.v[1], ir, ii, &r0, &r1);
  h_cmul(h_sub(0, x.v[2]), h_sub(0, x.v[3]), ir, ii, &r2, &r3);
  return hq_make(r0, r1, r2, r3);
}

// A twiddle tree resident in HBM: x-coordinates of every coset in the doubling tower of
// `root`, bit-reversed per level, padded with one 1 (cpu/circle.rs:171-188), and inverses.
struct TwiddleTree {
  stwo_coset root;
  uint32_t* d_tw = nullptr;
  uint32_t* d_itw = nullptr;
  // The same twiddles doubled (2t as a 32-bit word) for the FFT butterflies: a product a * 2t
  // splits at bit 32, so its reduction mod P needs one shift fewer (d_itw2 = d_tw2 + size).
  uint32_t* d_tw2 = nullptr;
  uint32_t* d_itw2 = nullptr;
  size_t size = 0;  // 2^root.log_size (>= 1)
};

// Process state: cached twiddle trees keyed by (device, root coset). A tree is complete (its
// build synchronised) before it enters the cache, so any stream may use a cached tree.
struct DeviceContext {
  std::mutex mu;
  std::map<std::tuple<int, uint32_t, uint32_t, uint32_t>, TwiddleTree*> trees;
};
DeviceContext& ctx();

// Builds (or returns the cached) tree for `root` on `stream`.
int32_t get_tree(stwo_coset root, cudaStream_t stream, TwiddleTree** out);
int32_t build_tree(stwo_coset root, cudaStream_t stream, TwiddleTree* t);
// The tree behind a caller-owned handle.
const TwiddleTree* tree_of(stwo_twiddle_tree t);

// Stream-ordered scratch allocation (cudaMallocAsync on the device's default pool).
int32_t scratch_alloc(void** p, size_t bytes, cudaStream_t s);
void scratch_free(void* p, cudaStream_t s);

// Kernel-parameter tables of column pointers. Kernel parameters may be up to 32 KB on
// sm_70+, so batches of this many columns travel in the launch itself and need no copy (two
// tables of 1,536 pointers are 24 KB). 1,536 keeps the 1,264 trace columns of the Poseidon2 AIR
// in one launch per FFT pass: one partial last wave instead of two.
constexpr int MAX_PARAM_COLS = 1536;
struct ColPtrs { uint32_t* p[MAX_PARAM_COLS]; };
struct ConstColPtrs { const uint32_t* p[MAX_PARAM_COLS]; };

// Count of kernel launches issued by this library (diagnostic, read by benchmarks).
void note_launch();

// Optional per-stage device timing of the prover (names follow the reference's tracing spans).
// Disabled by default; when enabled, each scope records a pair of CUDA events on its stream.
void stage_begin(const char* name, cudaStream_t s);
void stage_end(cudaStream_t s);
struct StageScope {
  cudaStream_t s;
  StageScope(const char* name, cudaStream_t st) : s(st) { stage_begin(name, st); }
  ~StageScope() { stage_end(s); }
};

// Number of SMs of the current device (152 on GB300).
int sm_count();

// Register-only throughput probes (diagnostics): a kernel of this signature runs `rounds` rounds of
// one operation per thread on `words` input words per thread (word i of thread g at in[g + i * n],
// n = threads), writes its result the same way to `out`, and has thread 0 of each block call
// probe_record after the loop.
using RateProbeKernel = void (*)(const uint32_t*, uint32_t*, unsigned long long*, uint32_t);
struct RateProbe {
  double ms = 0.0;            // event time of the timed launch
  double sm_cycles = 0.0;     // median over SMs of the SM's busy cycles (first block start to last end)
  double warps_per_sm = 0.0;  // warps that ran on that SM
  double sm_mhz = 0.0;        // SM clock during the loops: block cycles over block nanoseconds
  uint32_t blocks = 0;        // one full wave by the occupancy calculator: blocks per SM x SMs
};
// Launches `kern` twice (warm-up, then timed) with 256-thread blocks.
int32_t run_rate_probe(RateProbeKernel kern, uint32_t words, uint32_t rounds, cudaStream_t s, RateProbe* r);
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Six words per block: SM id, loop start and end (SM cycle counter), start and end (global ns).
__device__ __forceinline__ void probe_record(unsigned long long* span, long long c0, unsigned long long g0) {
  uint32_t smid;
  asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
  unsigned long long* o = span + 6 * blockIdx.x;
  o[0] = smid;
  o[1] = (unsigned long long)c0;
  o[2] = (unsigned long long)clock64();
  o[3] = g0;
  o[4] = global_ns();
  o[5] = 0;
}

// Programmatic dependent launch. A kernel started by launch_pdl may be scheduled while the kernel
// before it on the stream is still running; it calls pdl_wait() before it touches memory (that
// returns once the predecessor has completed and its writes are visible), then pdl_trigger(), which
// lets its own successor be scheduled in the same way. Both are no-ops for a plain launch. What is
// saved is the launch and ramp-up gap between dependent kernels of a proof.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_enter() {
  pdl_wait();
  pdl_trigger();
}
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args&&... args) {
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// A batch of out-of-domain evaluations whose polynomials, and which of a few points each
// evaluation takes, are known before the points are: eval_plan_build lays out and uploads the job
// tables (stream-ordered, while the device still works on earlier stages), eval_plan_run takes the
// points and evaluates, eval_plan_free releases the device block.
// Autotuner. Some launch shapes depend on the sizes in ways a fixed rule only approximates (a
// Merkle leaf layer's kernel variant and block size, how many rows a quotient lane takes). At such
// a site the library asks tune_choice: with tuning off it returns the built-in choice; in "use"
// mode it returns the table's entry for (site, key) when there is one; in "tune" mode a key not yet
// in the table is measured on the caller's own data first — each candidate timed with events on
// the stream — and the choice recorded. Only operations that
// recompute their whole output from their inputs are tuned this way, so the measuring leaves the
// results as they would be. The table is process-wide; the host saves and loads it as entries.
constexpr uint32_t TUNE_MERKLE_LAYER = 1, TUNE_QUOTIENT_ROWS = 2;
struct TuneState {
  std::atomic<int> mode{0};
  std::mutex mu;
  std::map<std::pair<uint32_t, uint64_t>, uint32_t> table;
};
TuneState& tune_state();
int tune_mode();  // 0 off, 1 use the table, 2 tune keys not in it
bool tune_lookup(uint32_t site, uint64_t key, uint32_t* choice);
void tune_record(uint32_t site, uint64_t key, uint32_t choice);
// Candidates are timed as the best of three runs after a warm-up; another shape replaces the
// built-in one only when it is at least 3% faster, so that timing noise does not move the choice.
template <class Launch>
int32_t tune_choice(uint32_t site, uint64_t key, uint32_t builtin, const uint32_t* cands, uint32_t n_cands,
                    cudaStream_t s, Launch&& launch, uint32_t* choice) {
  *choice = builtin;
  const int mode = tune_mode();
  if (mode == 0) return STWO_OK;
  if (tune_lookup(site, key, choice)) return STWO_OK;
  if (mode != 2) return STWO_OK;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  STWO_CHECK_CUDA(cudaEventCreate(&e0));
  STWO_CHECK_CUDA(cudaEventCreate(&e1));
  auto time_of = [&](uint32_t c, float* best_ms) -> int32_t {
    int32_t st = launch(c);  // warm
    *best_ms = 0.f;
    for (int r = 0; r < 3 && !st; r++) {
      float ms = 0.f;
      if (cudaEventRecord(e0, s) != cudaSuccess) return STWO_ERR_CUDA;
      st = launch(c);
      if (st) break;
      if (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
          cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
        return STWO_ERR_CUDA;
      if (r == 0 || ms < *best_ms) *best_ms = ms;
    }
    return st;
  };
  float base = 0.f, best = 0.f;
  uint32_t pick = builtin;
  int32_t st = time_of(builtin, &base);
  best = base;
  for (uint32_t i = 0; i < n_cands && !st; i++) {
    if (cands[i] == builtin) continue;
    float ms = 0.f;
    st = time_of(cands[i], &ms);
    if (!st && ms < best) {
      best = ms;
      pick = cands[i];
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st) return st;
  *choice = best < 0.97f * base ? pick : builtin;
  tune_record(site, key, *choice);
  return STWO_OK;
}

// At most this many distinct points (mask offsets) per planned evaluation or quotient group.
constexpr uint32_t EP_MAX_POINTS = 8;
struct EvalPlan {
  uint32_t n_evals = 0, n_points = 0, n_blocks = 0;
  unsigned char* d = nullptr;
  size_t off_polyof = 0, off_pointof = 0, off_work = 0, off_acc = 0, off_vals = 0, off_tables = 0;
};
int32_t eval_plan_build(const uint32_t* const* coeffs, const uint32_t* log_sizes, uint32_t n_polys,
                        const uint32_t* poly_of, const uint32_t* point_of, uint32_t n_evals, uint32_t n_points,
                        cudaStream_t s, EvalPlan* plan);
// Also leaves the values in device memory (eval_plan_values: 4 words per evaluation) until freed.
int32_t eval_plan_run(const EvalPlan& plan, const stwo_qm31_point* points, stwo_qm31* out, cudaStream_t s);
inline const uint32_t* eval_plan_values(const EvalPlan& plan) {
  return reinterpret_cast<const uint32_t*>(plan.d + plan.off_vals);
}
void eval_plan_free(EvalPlan& plan, cudaStream_t s);

// A quotient group (accumulate_quotients) whose samples — which column at which point id, and
// which planned OODS evaluation holds its value — are known before the points are: quot_plan_build
// uploads them; quot_plan_run takes the points, the batch order (point ids in the reference's order
// of point values), the random coefficient and the values in device memory.
struct QuotPlan {
  uint32_t log_n = 0, log_blowup = 0, n_points = 0, n_samples = 0;
  std::vector<const uint32_t*> cols;
  std::vector<uint32_t> s_first;
  unsigned char* d = nullptr;
  size_t off_samples = 0, off_batches = 0, off_entries = 0, off_sub = 0;
};
int32_t quot_plan_build(uint32_t log_n, const uint32_t* const* cols, uint32_t n_cols, const uint32_t* sample_col,
                        const uint32_t* sample_eval, const uint32_t* sample_point, uint32_t n_samples, uint32_t n_points,
                        uint32_t log_blowup, cudaStream_t s, QuotPlan* plan);
int32_t quot_plan_run(const QuotPlan& plan, const uint32_t* d_vals, const stwo_qm31_point* points, const uint32_t* order,
                      uint32_t n_batches, stwo_qm31 rc, uint32_t* const out[4], cudaStream_t s);
void quot_plan_free(QuotPlan& plan, cudaStream_t s);

// Pinned host words mapped into the device address space, one growable buffer per host thread:
// kernels write small results straight into host memory, read after a stream synchronisation.
struct Mapped {
  uint32_t* host = nullptr;
  uint32_t* dev = nullptr;
  size_t words = 0;
};
int32_t mapped_words(size_t words, Mapped& m);
// 64 pinned bytes of the calling host thread, separate from mapped_words (nullptr on failure).
unsigned long long* small_pinned();

}  // namespace stwo
