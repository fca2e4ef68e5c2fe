// Declarations of the GPU prover host (prover.cu) and of the AIR interface its constraint
// kernels implement.
#pragma once
#include <functional>
#include <map>
#include <vector>
#include "common.cuh"
#include "host_channel.h"
#include "dchannel.cuh"

namespace stwo {

// Device memory of one proof, released together at its end. Small requests are carved from
// 32 MiB chunks (256-byte aligned) so that a proof makes a few dozen pool allocations rather
// than hundreds; large ones get their own.
struct Arena {
  static constexpr size_t CHUNK = 32u << 20;
  cudaStream_t s;
  std::vector<void*> ptrs;
  char* chunk = nullptr;
  size_t chunk_used = 0;
  bool failed = false;
  explicit Arena(cudaStream_t st) : s(st) {}
  ~Arena();
  uint32_t* alloc(size_t words);
};

// Words to read back from HBM, collected while walking decommitment structures on the host and
// fetched in one launch per word size.
// A value request takes one result slot of vres; a run of `count` columns that lie `stride` words
// apart (one column block) takes `count` consecutive slots with one request.
struct Gather {
  std::vector<unsigned long long> vreq;  // (column, index, slot) per single value
  std::vector<unsigned long long> rreq;  // (first column, stride, index, slot | count << 32) per run
  std::vector<unsigned long long> hptr, hidx;
  std::vector<uint32_t> vres, hres;
  size_t n_slots = 0;
  size_t val(const uint32_t* col, size_t i) {
    vreq.push_back((unsigned long long)(uintptr_t)col);
    vreq.push_back(i);
    vreq.push_back(n_slots);
    return n_slots++;
  }
  // Slots of col0[i], col0[stride + i], ..., col0[(count - 1) stride + i]: the first is returned.
  size_t vals_strided(const uint32_t* col0, size_t stride, uint32_t count, size_t i) {
    rreq.push_back((unsigned long long)(uintptr_t)col0);
    rreq.push_back(stride);
    rreq.push_back(i);
    rreq.push_back((unsigned long long)n_slots | ((unsigned long long)count << 32));
    const size_t first = n_slots;
    n_slots += count;
    return first;
  }
  size_t hash(const uint32_t* layer, size_t node) {
    hptr.push_back((unsigned long long)(uintptr_t)layer);
    hidx.push_back(node);
    return hptr.size() - 1;
  }
  int32_t run(cudaStream_t s);
};

struct ColRef {
  const uint32_t* p;
  uint32_t log;
};

// A Merkle decommitment as indices into a Gather's results.
struct DecommitRecipe {
  std::vector<size_t> hash_witness, column_witness, queried;
};

// MerkleProver (crates/prover/src/core/vcs/prover.rs:13-154) with layers resident in HBM.
struct DevMerkle {
  std::vector<uint32_t*> layers;  // layers[l]: 2^l hashes of 8 words
  std::vector<ColRef> sorted;     // columns, stable-sorted by descending log size
  Digest root;
  // With read_root false the root stays on the device (layers[0]) and `root` is left unset. With
  // `ch` set, the launch that writes the root also mixes it into that device channel and draws
  // the next alpha into alpha_out, when the root comes from a node-only run (channel_fused).
  int32_t commit(const std::vector<ColRef>& columns, Arena& arena, cudaStream_t s, bool read_root = true,
                 DevChannel* ch = nullptr, uint32_t* alpha_out = nullptr);
  // Waits for the stream and copies the root (layers[0]) into `root`.
  int32_t read_root(cudaStream_t s);
  // A tree of equal-size columns whose leaf level is already in `all` (written by the FRI fold
  // that produced the columns); `all` holds every layer, as commit lays them out.
  int32_t commit_from_leaves(const std::vector<ColRef>& columns, uint32_t* all, cudaStream_t s,
                             DevChannel* ch = nullptr, uint32_t* alpha_out = nullptr);
  bool channel_fused = false;
  void decommit(const std::map<uint32_t, std::vector<size_t>>& queries, Gather& g, DecommitRecipe& out) const;
};

struct SecureCols {
  uint32_t* c[4];
};

// One FrameworkComponent-like AIR (constraint_framework/component.rs:126-416).
struct GpuAir {
  virtual ~GpuAir() {}
  virtual uint32_t log_size() const = 0;
  virtual uint32_t max_constraint_log_degree_bound() const = 0;
  virtual size_t n_constraints() const = 0;
  // [tree][column] -> mask offsets (tree 0 = preprocessed, 1 = trace, 2 = interaction).
  virtual std::vector<std::vector<std::vector<int>>> mask_offsets() const = 0;
  // Writes row_res * denom_inv for every row of the evaluation domain into acc (4 coordinate
  // columns), or adds it to acc's words when `accumulate` is set; `cols[tree][col]` are the trace
  // columns on that domain, `coeffs` the reversed powers of the random coefficient (4 words each,
  // device), `dinv` the bit-reversed denominator inverses (device).
  virtual int32_t eval_composition(const std::vector<std::vector<const uint32_t*>>& cols, const uint32_t* coeffs,
                                   const uint32_t* dinv, uint32_t* const acc[4], bool accumulate,
                                   cudaStream_t s) const = 0;
  // The constraint quotient sum at a point from the sampled mask values (PointEvaluator).
  virtual hq eval_at_point(const std::vector<std::vector<std::vector<hq>>>& mask, hq rc, hq denom_inv) const = 0;
};

// The configured AIRs, for callers outside their translation units. Relation elements are given
// as drawn: Poseidon2 (z, alpha); the Blake2s round (z, alpha) of the round relation, then of the
// XOR relations of widths 12, 9, 8, 7, 4.
GpuAir* new_wide_fib_air(uint32_t log_n, uint32_t n_cols);
GpuAir* new_poseidon_air(uint32_t log_n, const hq& z, const hq& alpha, const hq& claimed_sum);
GpuAir* new_blake_round_air(uint32_t log_n, const hq* z_alpha, const hq& claimed_sum);

// 1 / coset_vanishing(trace coset, eval_domain.at(i)) for the 2^(eval_log - trace_log) cosets,
// bit-reversed (constraint_framework/component.rs:323-328).
std::vector<uint32_t> composition_denom_inv(uint32_t trace_log, uint32_t eval_log);

struct Tree;

// CommitmentSchemeProver + prove() for one AIR.
struct Prover {
  stwo_pcs_config cfg;
  cudaStream_t s;
  Arena arena;
  TwiddleTree* tree = nullptr;
  int32_t init_status = 0;
  HostChannel ch;
  std::vector<Tree> trees;
  // Run once by the next commit_polys, after its launches and before it waits for the root.
  std::function<void()> before_root_wait;

  Prover(const stwo_pcs_config& c, uint32_t max_log, cudaStream_t st);
  ~Prover();
  // `evals`, when given, are the polynomials' evaluations on the blown-up domains already.
  int32_t commit_polys(std::vector<uint32_t*> polys, std::vector<uint32_t> logs,
                       const std::vector<uint32_t*>* evals = nullptr);
  int32_t commit_evals(const std::vector<uint32_t*>& cols, uint32_t log_size);
  int32_t commit_composition(const GpuAir& air, hq rc);
  int32_t prove(const GpuAir& air, std::vector<uint8_t>& out);
};

std::vector<hq> line_interpolate_host(stwo_coset dom, std::vector<hq> v);

// LogupTraceGenerator::finalize_last on the device (air_poseidon.cu): claimed sum, shift and
// coset-order prefix sum of the last secure column (four contiguous coordinate columns).
int32_t logup_finalize_last(uint32_t* last, uint32_t log_n, Arena& arena, cudaStream_t s, hq* claimed);

template <class T>
inline void bit_reverse_host(std::vector<T>& v) {
  size_t n = v.size();
  uint32_t log = 0;
  while (((size_t)1 << log) < n) log++;
  for (size_t i = 0; i < n; i++) {
    size_t r = 0;
    for (uint32_t b = 0; b < log; b++) r |= ((i >> b) & 1) << (log - 1 - b);
    if (r > i) std::swap(v[i], v[r]);
  }
}

}  // namespace stwo
