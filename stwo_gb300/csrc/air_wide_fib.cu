// Wide-Fibonacci AIR on the device (crates/prover/src/examples/wide_fibonacci/mod.rs:22-68):
// N columns per row with c = a^2 + b^2, constraints c - (a^2 + b^2) for columns 2..N-1.
//
// Composition kernel: one thread per row of the evaluation domain streams the N columns
// (coalesced), accumulates sum_k coeff_k * C_k in four 64-bit lanes (partial reduction every
// three terms) and writes row_res * denom_inv as four coordinate columns (or adds it to them).
#include "common.cuh"
#include "prover.cuh"

namespace stwo {

__device__ __forceinline__ uint32_t fold64_(unsigned long long x) {
  x = (x & P) + (x >> 31);
  x = (x & P) + (x >> 31);
  uint32_t r = (uint32_t)x;
  return r >= P ? r - P : r;
}

__global__ void __launch_bounds__(256) k_wide_fib_composition(ConstColPtrs cols, uint32_t n_cols, uint32_t n_rows,
                                                              uint32_t trace_log, const uint32_t* __restrict__ coeffs,
                                                              const uint32_t* __restrict__ dinv, uint32_t accumulate,
                                                              uint32_t* o0, uint32_t* o1, uint32_t* o2, uint32_t* o3) {
  pdl_enter();
  extern __shared__ uint32_t s_coeffs[];
  for (uint32_t i = threadIdx.x; i < 4 * (n_cols - 2); i += blockDim.x) s_coeffs[i] = coeffs[i];
  __syncthreads();
  uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_rows) return;
  uint32_t a = __ldg(cols.p[0] + r), b = __ldg(cols.p[1] + r);
  unsigned long long acc0 = 0, acc1 = 0, acc2 = 0, acc3 = 0;
  uint32_t cnt = 0;
  for (uint32_t i = 2; i < n_cols; i++) {
    uint32_t c = __ldg(cols.p[i] + r);
    uint32_t cons = m31_sub(c, m31_add(m31_sqr(a), m31_sqr(b)));
    const uint32_t* k = s_coeffs + 4 * (i - 2);
    acc0 += (unsigned long long)k[0] * cons;
    acc1 += (unsigned long long)k[1] * cons;
    acc2 += (unsigned long long)k[2] * cons;
    acc3 += (unsigned long long)k[3] * cons;
    // Products are at most (P - 1)^2 and a folded sum is below 2^33 + 2^31: four products fit
    // between folds without passing 2^64.
    if (++cnt == 4) {
      acc0 = (acc0 & P) + (acc0 >> 31);
      acc1 = (acc1 & P) + (acc1 >> 31);
      acc2 = (acc2 & P) + (acc2 >> 31);
      acc3 = (acc3 & P) + (acc3 >> 31);
      cnt = 0;
    }
    a = b;
    b = c;
  }
  uint32_t d = __ldg(dinv + (r >> trace_log));
  uint32_t v0 = m31_mul(fold64_(acc0), d), v1 = m31_mul(fold64_(acc1), d);
  uint32_t v2 = m31_mul(fold64_(acc2), d), v3 = m31_mul(fold64_(acc3), d);
  if (accumulate) {
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

// Trace of generate_trace (wide_fibonacci/mod.rs:46-68): row r starts from (a[r], b[r]).
__global__ void k_wide_fib_trace(const uint32_t* a, const uint32_t* b, uint32_t n_rows, ColPtrs cols,
                                 uint32_t n_cols) {
  pdl_enter();
  uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_rows) return;
  uint32_t x = a[r], y = b[r];
  cols.p[0][r] = x;
  cols.p[1][r] = y;
  for (uint32_t c = 2; c < n_cols; c++) {
    uint32_t z = m31_add(m31_sqr(x), m31_sqr(y));
    x = y;
    y = z;
    cols.p[c][r] = z;
  }
}

struct WideFibGpuAir : GpuAir {
  uint32_t log_n, n_cols;
  WideFibGpuAir(uint32_t l, uint32_t n) : log_n(l), n_cols(n) {}
  uint32_t log_size() const override { return log_n; }
  uint32_t max_constraint_log_degree_bound() const override { return log_n + 1; }
  size_t n_constraints() const override { return n_cols - 2; }
  std::vector<std::vector<std::vector<int>>> mask_offsets() const override {
    std::vector<std::vector<std::vector<int>>> m(2);
    m[1].assign(n_cols, {0});
    return m;
  }
  int32_t eval_composition(const std::vector<std::vector<const uint32_t*>>& cols, const uint32_t* coeffs,
                           const uint32_t* dinv, uint32_t* const acc[4], bool accumulate,
                           cudaStream_t s) const override {
    STWO_REQUIRE(cols.size() >= 2 && cols[1].size() == n_cols, "trace tree mismatch");
    ConstColPtrs cp;
    for (uint32_t i = 0; i < n_cols; i++) cp.p[i] = cols[1][i];
    uint32_t n_rows = 1u << (log_n + 1);
    size_t smem = (size_t)4 * (n_cols - 2) * 4;
    launch_pdl(k_wide_fib_composition, dim3((n_rows + 255) / 256), dim3(256), smem, s, cp, n_cols, n_rows, log_n, coeffs,
               dinv, accumulate ? 1u : 0u, acc[0], acc[1], acc[2], acc[3]);
    note_launch();
    STWO_LAUNCH_CHECK();
    return STWO_OK;
  }
  hq eval_at_point(const std::vector<std::vector<std::vector<hq>>>& mask, hq rc, hq denom_inv) const override {
    hq acc = hq_make(0, 0, 0, 0);
    const auto& t = mask[1];
    hq a = t[0][0], b = t[1][0];
    for (uint32_t i = 2; i < n_cols; i++) {
      hq c = t[i][0];
      hq cons = hq_sub(c, hq_add(hq_mul(a, a), hq_mul(b, b)));
      acc = hq_add(hq_mul(acc, rc), cons);  // denom_inv factored out of the sum
      a = b;
      b = c;
    }
    return hq_mul(acc, denom_inv);
  }
};

GpuAir* new_wide_fib_air(uint32_t log_n, uint32_t n_cols) { return new WideFibGpuAir(log_n, n_cols); }

}  // namespace stwo

using namespace stwo;

extern "C" {

stwo_status stwo_gen_wide_fib_trace(uint32_t log_n_rows, uint32_t n_cols, const uint32_t* d_a, const uint32_t* d_b,
                                    uint32_t* const* d_cols, void* stream) {
  STWO_REQUIRE(n_cols >= 2 && n_cols <= MAX_PARAM_COLS, "n_cols must be in [2, %d]", MAX_PARAM_COLS);
  STWO_REQUIRE(log_n_rows <= 28, "log_n_rows too large");
  ColPtrs cp;
  for (uint32_t i = 0; i < n_cols; i++) cp.p[i] = d_cols[i];
  uint32_t n = 1u << log_n_rows;
  launch_pdl(k_wide_fib_trace, dim3((n + 255) / 256), dim3(256), 0, as_stream(stream), d_a, d_b, n, cp, n_cols);
  note_launch();
  STWO_LAUNCH_CHECK();
  return STWO_OK;
}

stwo_status stwo_prove_wide_fib(uint32_t log_n_rows, uint32_t n_cols, uint32_t* const* d_trace, stwo_pcs_config cfg,
                                uint8_t* h_proof, size_t capacity, size_t* h_len, void* stream) {
  STWO_REQUIRE(n_cols >= 3 && n_cols <= MAX_PARAM_COLS, "n_cols must be in [3, %d]", MAX_PARAM_COLS);
  STWO_REQUIRE(log_n_rows >= 1 && log_n_rows + 1 + cfg.log_blowup_factor <= 28, "bad log_n_rows");
  STWO_REQUIRE(cfg.log_blowup_factor >= 1 && cfg.log_blowup_factor <= 16, "log_blowup_factor out of [1, 16]");
  STWO_REQUIRE(cfg.log_last_layer_degree_bound <= 10, "log_last_layer_degree_bound > 10");
  STWO_REQUIRE(h_len, "null length");
  cudaStream_t s = as_stream(stream);
  std::vector<uint8_t> bytes;
  int32_t st;
  {
    Prover pv(cfg, log_n_rows + 1 + cfg.log_blowup_factor, s);
    if (pv.init_status) return pv.init_status;
    st = pv.commit_polys({}, {});
    if (!st) st = pv.commit_evals(std::vector<uint32_t*>(d_trace, d_trace + n_cols), log_n_rows);
    if (!st) {
      WideFibGpuAir air(log_n_rows, n_cols);
      st = pv.prove(air, bytes);
    }
    cudaStreamSynchronize(s);
  }
  if (st) return st;
  *h_len = bytes.size();
  STWO_REQUIRE(bytes.size() <= capacity, "proof buffer too small (%zu bytes needed)", bytes.size());
  if (h_proof) memcpy(h_proof, bytes.data(), bytes.size());
  return STWO_OK;
}

}  // extern "C"
