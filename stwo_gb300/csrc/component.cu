// Per-component constraint evaluation behind the C ABI: ComponentProver::
// evaluate_constraint_quotients_on_domain (crates/prover/src/core/air/mod.rs:59-62) for the
// configured AIRs, so that the reference's prove() can drive this backend component by component.
//
// The reference's SIMD implementation (crates/prover/src/constraint_framework/component.rs:278-416)
// extends the component's trace to the evaluation domain, computes the vanishing inverses of the
// 2^log_expand cosets, takes its slice of random-coefficient powers from the accumulator, reverses
// it, and adds row_res * denom_inv to the accumulation column. Here the caller does the extension
// with stwo_evaluate_columns (the same step the reference times as "Extension") and passes the
// accumulator slice as it receives it; this entry point does the rest with the AIR's constraint
// kernel in its accumulating mode.
#include "common.cuh"
#include "prover.cuh"
#include <memory>

namespace stwo {

static int32_t make_air(const stwo_component* c, std::unique_ptr<GpuAir>& out) {
  STWO_REQUIRE(c, "null component");
  auto q = [](const stwo_qm31& v) { return hq_make(v.v[0], v.v[1], v.v[2], v.v[3]); };
  switch (c->air) {
    case STWO_AIR_WIDE_FIB:
      STWO_REQUIRE(c->n_cols >= 3 && c->n_cols <= MAX_PARAM_COLS, "wide-Fibonacci n_cols must be in [3, %d]",
                   MAX_PARAM_COLS);
      STWO_REQUIRE(c->log_n_rows >= 1 && c->log_n_rows <= 27, "log_n_rows out of range");
      out.reset(new_wide_fib_air(c->log_n_rows, c->n_cols));
      return STWO_OK;
    case STWO_AIR_POSEIDON:
      STWO_REQUIRE(c->h_elements && c->n_elements == 2, "Poseidon2 takes 2 relation elements (z, alpha)");
      STWO_REQUIRE(c->log_n_rows >= 3 && c->log_n_rows <= 26, "log_n_rows out of range");
      out.reset(new_poseidon_air(c->log_n_rows, q(c->h_elements[0]), q(c->h_elements[1]), q(c->claimed_sum)));
      return STWO_OK;
    case STWO_AIR_BLAKE_ROUND: {
      STWO_REQUIRE(c->h_elements && c->n_elements == 12,
                   "the Blake2s round takes 12 relation elements (z, alpha of the round and of 5 XOR relations)");
      STWO_REQUIRE(c->log_n_rows >= 4 && c->log_n_rows <= 26, "log_n_rows out of range");
      hq e[12];
      for (int i = 0; i < 12; i++) e[i] = q(c->h_elements[i]);
      out.reset(new_blake_round_air(c->log_n_rows, e, q(c->claimed_sum)));
      return STWO_OK;
    }
  }
  STWO_REQUIRE(false, "unknown AIR id %u", c->air);
}

}  // namespace stwo

using namespace stwo;

extern "C" {

stwo_status stwo_component_info(const stwo_component* component, uint32_t* h_n_constraints, uint32_t* h_eval_log_size,
                                uint32_t* h_n_trees, uint32_t h_tree_n_cols[3]) {
  std::unique_ptr<GpuAir> air;
  int32_t st = make_air(component, air);
  if (st) return st;
  const auto mask = air->mask_offsets();
  if (h_n_constraints) *h_n_constraints = (uint32_t)air->n_constraints();
  if (h_eval_log_size) *h_eval_log_size = air->max_constraint_log_degree_bound();
  if (h_n_trees) *h_n_trees = (uint32_t)mask.size();
  if (h_tree_n_cols)
    for (size_t t = 0; t < 3; t++) h_tree_n_cols[t] = t < mask.size() ? (uint32_t)mask[t].size() : 0u;
  return STWO_OK;
}

stwo_status stwo_eval_constraints(const stwo_component* component, const uint32_t* const* d_cols, uint32_t n_cols,
                                  const stwo_qm31* h_coeff_powers, uint32_t n_coeff_powers, uint32_t* const d_accum[4],
                                  void* stream) {
  std::unique_ptr<GpuAir> air;
  int32_t st = make_air(component, air);
  if (st) return st;
  const auto mask = air->mask_offsets();
  size_t want = 0;
  for (auto& t : mask) want += t.size();
  STWO_REQUIRE(n_cols == want, "the component reads %zu columns, %u given", want, n_cols);
  STWO_REQUIRE(d_cols || n_cols == 0, "null column table");
  const size_t n = air->n_constraints();
  STWO_REQUIRE(n_coeff_powers == n, "the component has %zu constraints, %u coefficient powers given", n,
               n_coeff_powers);
  STWO_REQUIRE(h_coeff_powers && d_accum && d_accum[0] && d_accum[1] && d_accum[2] && d_accum[3],
               "null argument");
  for (uint32_t i = 0; i < n_cols; i++) STWO_REQUIRE(d_cols[i], "null column %u", i);
  std::vector<std::vector<const uint32_t*>> cols(mask.size());
  size_t k = 0;
  for (size_t t = 0; t < mask.size(); t++)
    for (size_t c = 0; c < mask[t].size(); c++) cols[t].push_back(d_cols[k++]);

  cudaStream_t s = as_stream(stream);
  const std::vector<uint32_t> dinv = composition_denom_inv(air->log_size(), air->max_constraint_log_degree_bound());
  // The accumulator's slice reversed (component.rs:331): constraint i gets power n - 1 - i.
  std::vector<uint32_t> host(4 * n + dinv.size());
  for (size_t i = 0; i < n; i++)
    for (int j = 0; j < 4; j++) host[4 * i + j] = h_coeff_powers[n - 1 - i].v[j];
  for (size_t i = 0; i < dinv.size(); i++) host[4 * n + i] = dinv[i];
  uint32_t* d = nullptr;
  st = scratch_alloc((void**)&d, host.size() * 4, s);
  if (st) return st;
  cudaError_t e = cudaMemcpyAsync(d, host.data(), host.size() * 4, cudaMemcpyHostToDevice, s);
  if (e) {
    scratch_free(d, s);
    set_error("eval_constraints: %s", cudaGetErrorString(e));
    return STWO_ERR_CUDA;
  }
  st = air->eval_composition(cols, d, d + 4 * n, d_accum, true, s);
  scratch_free(d, s);
  return st;
}

}  // extern "C"
