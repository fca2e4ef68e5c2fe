/*
 * stwo_cuda.h — C ABI of the GB300 (sm_103a) prover backend.
 *
 * Each entry point replaces one method of the reference's backend trait family
 * (crates/prover/src/core/backend/mod.rs:19-65 and the trait homes cited per function).
 * Conventions:
 *   - Every function returns stwo_status; nothing aborts and nothing throws across the ABI.
 *     Preconditions the reference `assert!`s return STWO_ERR_INVALID_ARG.
 *   - `d_` pointers are device (HBM) pointers owned by the caller; `h_` pointers are host.
 *     Base-field columns are arrays of canonical M31 words (u32 < 2^31 - 1). A secure
 *     (QM31) column is four such coordinate columns, as SecureColumnByCoords
 *     (crates/prover/src/core/fields/secure_column.rs:15).
 *   - `stream` is a cudaStream_t (NULL = legacy default stream). Calls are stream ordered;
 *     results written to host memory are complete when the call returns.
 *   - Evaluations are in bit-reversed circle-domain order, as the reference's
 *     CircleEvaluation<_, _, BitReversedOrder>; coefficients are in the reference CPU
 *     backend's order (crates/prover/src/core/backend/cpu/circle.rs:18-135).
 */
#ifndef STWO_CUDA_H
#define STWO_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t stwo_status;
#define STWO_OK 0
#define STWO_ERR_INVALID_ARG 1
#define STWO_ERR_OOM 2
#define STWO_ERR_TIMEOUT 3
#define STWO_ERR_CUDA 4
#define STWO_ERR_UNSUPPORTED 5

/* Coset `initial + <step>` of size 2^log_size, by circle-group indices modulo 2^31
 * (crates/prover/src/core/circle.rs:307-330). A CircleDomain is given by its half coset
 * (crates/prover/src/core/poly/circle/domain.rs:14-20). */
typedef struct {
  uint32_t initial_index;
  uint32_t step_size;
  uint32_t log_size;
} stwo_coset;

/* QM31 element (a + b i) + (c + d i) u as {a, b, c, d} (crates/prover/src/core/fields/qm31.rs:21-45). */
typedef struct {
  uint32_t v[4];
} stwo_qm31;

/* CirclePoint<SecureField> (crates/prover/src/core/circle.rs:13-17). */
typedef struct {
  stwo_qm31 x;
  stwo_qm31 y;
} stwo_qm31_point;

typedef struct stwo_twiddle_tree_s* stwo_twiddle_tree;

/* ------------------------------------------------------------------ runtime */
const char* stwo_status_string(stwo_status status);
/* Detail of the last failure on the calling host thread. */
const char* stwo_last_error(void);
/* Selects the device for the calling thread and warms the context. */
stwo_status stwo_device_init(int device);
stwo_status stwo_sync(void* stream);
/* Diagnostic without a reference counterpart: kernels launched by this library so far
 * (benchmarks report the count inside their timed region). */
uint64_t stwo_kernel_launches(void);
/* Diagnostics without a reference counterpart: per-stage device times of the prover on the
 * calling thread, named after the reference's tracing spans ("Extension", "Merkle", ...).
 * stwo_set_stage_timing(1) enables recording (and clears earlier records); stwo_stage_times
 * returns the number of distinct stages and fills up to `cap` names / summed milliseconds. */
stwo_status stwo_set_stage_timing(int enable);
uint32_t stwo_stage_times(const char** names, float* ms, uint32_t cap);
/* Autotuner without a reference counterpart: launch shapes of some operations (a Merkle leaf
 * layer's kernel variant and block size; rows per lane of the quotient pass) chosen per size key.
 * mode 0: the built-in choices; 1: the table's entry where there is one; 2: as 1, and a key not in
 * the table is measured on the call's own data (each candidate timed as the best of three runs after
 * a warm-up; another shape replaces the built-in one when it is at least 3% faster; the operation's
 * results are unchanged). The table is process-wide:
 * stwo_autotune_entries copies up to `cap` entries and returns how many there are, set_entry adds
 * or replaces one (entries saved by a caller can be loaded back), clear empties it. */
stwo_status stwo_autotune_mode(int mode);
uint32_t stwo_autotune_entries(uint32_t* sites, uint64_t* keys, uint32_t* choices, uint32_t cap);
stwo_status stwo_autotune_set_entry(uint32_t site, uint64_t key, uint32_t choice);
stwo_status stwo_autotune_clear(void);
/* Diagnostic without a reference counterpart: the circle-FFT butterfly of the library's FFT
 * kernels with every operand in registers (one full wave of blocks, `rounds` rounds of 32
 * butterflies per thread, on `stream`). `h_butterflies_per_s` is its rate from event timing;
 * `h_cycles_per_warp_butterfly` (may be null) is its issue cost from the SM cycle counter: SM
 * cycles per warp-wide butterfly on one of the SM's four schedulers, independent of the clock;
 * `h_probe_sm_mhz` (may be null) is the SM clock the probe ran at (cycle counter over the global
 * timer). The integer-datapath bound of an FFT pass at SM clock f is 4 x SMs x f x 32 / cost. */
stwo_status stwo_butterfly_rate(uint32_t rounds, double* h_butterflies_per_s, double* h_cycles_per_warp_butterfly,
                                double* h_probe_sm_mhz, void* stream);
/* Diagnostic without a reference counterpart: the same for the BLAKE2s compression of the Merkle
 * leaf kernels (each thread chains `rounds` compressions of a message held in registers): the
 * event-timed rate in compressions per second, the issue cost in SM cycles per warp-wide
 * compression on one scheduler, and the SM clock the probe ran at. */
stwo_status stwo_blake2s_rate(uint32_t rounds, double* h_compressions_per_s, double* h_cycles_per_warp_compression,
                              double* h_probe_sm_mhz, void* stream);

/* Column storage: Column::zeros / uninitialized / to_cpu / at
 * (crates/prover/src/core/backend/mod.rs:46-65). */
stwo_status stwo_buf_alloc(void** d_ptr, size_t bytes, void* stream);
stwo_status stwo_buf_free(void* d_ptr, void* stream);
stwo_status stwo_buf_upload(void* d_dst, const void* h_src, size_t bytes, void* stream);
stwo_status stwo_buf_download(void* h_dst, const void* d_src, size_t bytes, void* stream);
stwo_status stwo_buf_zero(void* d_dst, size_t bytes, void* stream);
/* Column::at for a list of indices (Merkle decommitment reads,
 * crates/prover/src/core/vcs/prover.rs:80-149). */
stwo_status stwo_read_words(const uint32_t* d_col, const uint64_t* h_idx, size_t n, uint32_t* h_out,
                            void* stream);
/* Column::at for the same indices of several columns, in one transfer: h_out[c * n + i] =
 * h_cols[c][h_idx[i]] (the values a Merkle layer's decommitment reads, vcs/prover.rs:80-149). */
stwo_status stwo_read_words_cols(const uint32_t* const* h_cols, size_t n_cols, const uint64_t* h_idx, size_t n,
                                 uint32_t* h_out, void* stream);

/* ------------------------------------------------------------------ twiddles */
/* PolyOps::precompute_twiddles (crates/prover/src/core/poly/circle/ops.rs:68;
 * layout of crates/prover/src/core/backend/cpu/circle.rs:137-188, not doubled). */
stwo_status stwo_twiddles_precompute(stwo_coset root, stwo_twiddle_tree* out, void* stream);
stwo_status stwo_twiddles_free(stwo_twiddle_tree tree);
stwo_status stwo_twiddles_info(stwo_twiddle_tree tree, stwo_coset* root, const uint32_t** d_twiddles,
                               const uint32_t** d_itwiddles, size_t* size);

/* ------------------------------------------------------------------ PolyOps */
/* PolyOps::interpolate_columns (crates/prover/src/core/poly/circle/ops.rs:20-33), in place:
 * each column holds 2^(domain.log_size+1) bit-reversed evaluations and receives the
 * coefficients. `domain_half_coset` must be a doubling of the tree's root coset. */
stwo_status stwo_interpolate_columns(stwo_twiddle_tree tree, stwo_coset domain_half_coset,
                                     uint32_t* const* d_cols, uint32_t n_cols, void* stream);
/* PolyOps::evaluate_polynomials / evaluate (ops.rs:41-65): polynomials with 2^coeff_log_size
 * coefficients evaluated on the circle domain of `domain_half_coset` (log size >= coeff_log_size). */
stwo_status stwo_evaluate_columns(stwo_twiddle_tree tree, stwo_coset domain_half_coset,
                                  const uint32_t* const* d_coeffs, uint32_t coeff_log_size,
                                  uint32_t* const* d_out, uint32_t n_cols, void* stream);
/* PolyOps::extend (ops.rs:39-40): coefficients zero-padded to 2^log_size. */
stwo_status stwo_extend(const uint32_t* d_coeffs, uint32_t coeff_log_size, uint32_t* d_out, uint32_t log_size,
                        void* stream);
/* PolyOps::eval_at_point (ops.rs:37) batched: h_out[i] = poly[poly_of[i]](points[i]). */
stwo_status stwo_eval_at_points(const uint32_t* const* d_coeffs, const uint32_t* h_log_sizes, uint32_t n_polys,
                                const uint32_t* h_poly_of, const stwo_qm31_point* h_points, uint32_t n_evals,
                                stwo_qm31* h_out, void* stream);

/* No counterpart in the reference. The same result as stwo_eval_at_points for callers that
 * cannot allocate device memory (their HBM is owned by a pool manager that forbids other
 * allocations, or an allocation would stall or synchronise work they run on other streams). It
 * calls no cudaMalloc/cudaFree or allocating library routine: its scratch is a fixed
 * 256-byte-aligned static device array of about 200 KB, held by every GPU that loads this library
 * until the process exits. Limits: n_evals <= STWO_NOALLOC_MAX_EVALS and
 * n_polys <= STWO_NOALLOC_MAX_POLYS, else STWO_ERR_INVALID_ARG. Every call looks up the array's
 * device address (cudaGetSymbolAddress, which allocates nothing) in the current device's context,
 * so the first call on a device also loads the module there; make that first call before any
 * stream capture. All calls share the one array and it keeps the last call's contents (the call
 * clears its accumulators itself): calls that overlap on the GPU (other streams, other host
 * threads) race and must be serialised by the caller. */
#define STWO_NOALLOC_MAX_EVALS 2048
#define STWO_NOALLOC_MAX_POLYS 2048
stwo_status stwo_eval_at_points_noalloc(const uint32_t* const* d_coeffs, const uint32_t* h_log_sizes,
                                        uint32_t n_polys, const uint32_t* h_poly_of, const stwo_qm31_point* h_points,
                                        uint32_t n_evals, stwo_qm31* h_out, void* stream);

/* ColumnOps::bit_reverse_column (crates/prover/src/core/backend/mod.rs:40). */
stwo_status stwo_bit_reverse_column(uint32_t* d_col, uint32_t log_size, void* stream);

/* ------------------------------------------------------------------ MerkleOps */
/* MerkleOps<Blake2sMerkleHasher>::commit_on_layer (crates/prover/src/core/vcs/ops.rs:41-45;
 * backend/simd/blake2s.rs:60-145). Hashes are 8 little-endian u32 words. `d_prev_layer` is
 * NULL for the leaf layer, else 2^(log_size+1) hashes. Columns have 2^log_size values. */
stwo_status stwo_merkle_commit_layer(uint32_t log_size, const uint32_t* d_prev_layer,
                                     const uint32_t* const* d_cols, uint32_t n_cols, uint32_t* d_out,
                                     void* stream);

/* MerkleOps<Poseidon252MerkleHasher>::commit_on_layer (crates/prover/src/core/vcs/ops.rs:41-45; hasher
 * crates/prover/src/core/vcs/poseidon252_merkle.rs:17-45, CPU backend backend/cpu/poseidon252.rs:9-25),
 * the Merkle half of BackendForChannel<Poseidon252MerkleChannel> (backend/simd/mod.rs:34-35). Hashes
 * are FieldElement252 values, each 8 little-endian u32 limbs of the canonical integer below
 * p = 2^251 + 17 * 2^192 + 1. `d_prev_layer` is NULL for the leaf layer, else 2^(log_size+1) hashes. */
stwo_status stwo_merkle_commit_layer_poseidon252(uint32_t log_size, const uint32_t* d_prev_layer,
                                                 const uint32_t* const* d_cols, uint32_t n_cols, uint32_t* d_out,
                                                 void* stream);

/* ------------------------------------------------------------------ FriOps */
/* FriOps::fold_line (crates/prover/src/core/fri.rs:103-107): evaluation on the line domain
 * `line_domain` (2^log_size values) folded into 2^(log_size-1) values. */
stwo_status stwo_fri_fold_line(stwo_twiddle_tree tree, stwo_coset line_domain, const uint32_t* const d_eval[4],
                               stwo_qm31 alpha, uint32_t* const d_out[4], void* stream);
/* FriOps::fold_circle_into_line (fri.rs:124-129): dst = dst * alpha^2 + fold(src). */
stwo_status stwo_fri_fold_circle_into_line(stwo_twiddle_tree tree, stwo_coset src_half_coset,
                                           uint32_t* const d_dst[4], const uint32_t* const d_src[4],
                                           stwo_qm31 alpha, void* stream);
/* FriOps::decompose (fri.rs:136-138; backend/simd/fri.rs:111-161). */
stwo_status stwo_fri_decompose(const uint32_t* const d_eval[4], uint32_t log_size, uint32_t* const d_g[4],
                               stwo_qm31* h_lambda, void* stream);

/* ------------------------------------------------------------------ QuotientOps */
/* One ColumnSampleBatch (crates/prover/src/core/pcs/quotients.rs:37-68). */
typedef struct {
  stwo_qm31_point point;
  uint32_t n_columns;
  const uint32_t* h_column_indices;
  const stwo_qm31* h_values;
} stwo_sample_batch;
/* QuotientOps::accumulate_quotients (pcs/quotients.rs:21-35; backend/simd/quotients.rs:31-100),
 * on CanonicCoset(domain_log_size).circle_domain(). Columns hold 2^domain_log_size values. */
stwo_status stwo_accumulate_quotients(uint32_t domain_log_size, const uint32_t* const* d_cols, uint32_t n_cols,
                                      stwo_qm31 random_coeff, const stwo_sample_batch* h_batches,
                                      uint32_t n_batches, uint32_t log_blowup_factor, uint32_t* const d_out[4],
                                      void* stream);

/* ------------------------------------------------------------------ AccumulationOps */
/* AccumulationOps::accumulate (crates/prover/src/core/air/accumulation.rs:151-158). */
stwo_status stwo_secure_accumulate(uint32_t* const d_acc[4], const uint32_t* const d_other[4], size_t n,
                                   void* stream);
/* AccumulationOps::generate_secure_powers (accumulation.rs:156-157). */
stwo_status stwo_generate_secure_powers(stwo_qm31 felt, uint32_t n_powers, stwo_qm31* h_out, void* stream);

/* ------------------------------------------------------------------ GkrOps / MleOps */
/* Mle columns (crates/prover/src/core/lookups/mle.rs:16-19) hold values on the boolean hypercube,
 * first variable = most significant index bit. Layer kinds of gkr_prover.rs:94-108: */
#define STWO_GKR_GRAND_PRODUCT 0u        /* d_num = the secure column, d_den unused */
#define STWO_GKR_LOGUP_GENERIC 1u        /* d_num, d_den secure */
#define STWO_GKR_LOGUP_MULTIPLICITIES 2u /* d_num[0] = base-field numerators, d_den secure */
#define STWO_GKR_LOGUP_SINGLES 3u        /* numerators implicitly 1 (d_num unused), d_den secure */

/* GkrOps::gen_eq_evals (gkr_prover.rs:28; backend/simd/lookups/gkr.rs:22-54): eq(x, y) * v for
 * every x in {0,1}^n_y (n_y <= 30), into 2^n_y secure values. */
stwo_status stwo_gkr_gen_eq_evals(const stwo_qm31* h_y, uint32_t n_y, stwo_qm31 v, uint32_t* const d_out[4],
                                  void* stream);
/* GkrOps::next_layer (gkr_prover.rs:31; backend/simd/lookups/gkr.rs:56-74): the layer of
 * 2^(log_n-1) gates above a layer of 2^log_n. A grand product writes d_next_num only; every LogUp
 * kind writes a generic layer (d_next_num, d_next_den). */
stwo_status stwo_gkr_next_layer(uint32_t kind, uint32_t log_n, const uint32_t* const d_num[4],
                                const uint32_t* const d_den[4], uint32_t* const d_next_num[4],
                                uint32_t* const d_next_den[4], void* stream);
/* GkrOps::sum_as_poly_in_first_variable (gkr_prover.rs:36-41; backend/simd/lookups/gkr.rs:76-127)
 * for the GkrMultivariatePolyOracle (gkr_prover.rs:285-318) of a layer of 2^log_n gates (log_n >=
 * 2): eq evaluations d_eq_evals (at least 2^(log_n-2) values) generated from y = h_y[0..n_y),
 * lambda and eq_fixed_var_correction. Writes the round polynomial's monomial coefficients
 * (leading zeros dropped, at most 4) and their count. Synchronous. */
stwo_status stwo_gkr_sum_as_poly_in_first_variable(uint32_t kind, uint32_t log_n, const uint32_t* const d_num[4],
                                                   const uint32_t* const d_den[4],
                                                   const uint32_t* const d_eq_evals[4], const stwo_qm31* h_y,
                                                   uint32_t n_y, stwo_qm31 lambda,
                                                   stwo_qm31 eq_fixed_var_correction, stwo_qm31 claim,
                                                   stwo_qm31* h_coeffs, uint32_t* h_n_coeffs, void* stream);
/* MleOps<BaseField>::fix_first_variable (mle.rs:9-14; backend/simd/lookups/mle.rs:14-45):
 * out[i] = a * (in[i + h] - in[i]) + in[i], h = 2^(log_n-1), into a secure column. */
stwo_status stwo_mle_fix_first_variable_base(uint32_t log_n, const uint32_t* d_mle, stwo_qm31 assignment,
                                             uint32_t* const d_out[4], void* stream);
/* MleOps<SecureField>::fix_first_variable (backend/simd/lookups/mle.rs:47-91); d_out may equal
 * d_mle (the reference folds in place). */
stwo_status stwo_mle_fix_first_variable_secure(uint32_t log_n, const uint32_t* const d_mle[4], stwo_qm31 assignment,
                                               uint32_t* const d_out[4], void* stream);
/* gkr_prover::prove_batch (gkr_prover.rs:401-506) over n_instances input layers: instance i has
 * kind h_kinds[i], 2^h_log_sizes[i] gates (log size >= 1), numerators h_num[4i..4i+4) and
 * denominators h_den[4i..4i+4) (device pointers; entries a kind does not use may be NULL). The
 * Blake2s channel starts from digest h_digest_in (NULL: the default channel) and its final digest is
 * written to h_digest_out (if not NULL). Writes the canonical bytes of the GkrBatchProof followed by
 * the GkrArtifact (u64 lengths, QM31 as four LE u32 words, fields in struct order). Inputs are not
 * modified. Synchronous. */
stwo_status stwo_gkr_prove_batch(uint32_t n_instances, const uint32_t* h_kinds, const uint32_t* h_log_sizes,
                                 const uint32_t* const* h_num, const uint32_t* const* h_den,
                                 const uint8_t* h_digest_in, uint8_t* h_out, size_t capacity, size_t* h_len,
                                 uint8_t* h_digest_out, void* stream);

/* ------------------------------------------------------------------ GrindOps */
/* GrindOps<Blake2sChannel>::grind (crates/prover/src/core/proof_of_work.rs:3-7;
 * backend/simd/grind.rs:21-63): the smallest nonce whose raw Blake2s compression of
 * (digest, [nonce_lo, nonce_hi, 0...]) has >= pow_bits trailing zeros in word 0. */
stwo_status stwo_grind_blake2s(const uint32_t h_digest[8], uint32_t pow_bits, uint64_t* h_nonce, void* stream);

/* GrindOps<Poseidon252Channel>::grind (crates/prover/src/core/backend/simd/grind.rs:65-79): the smallest
 * nonce for which poseidon_hash(digest, nonce) has >= pow_bits trailing zeros as
 * Poseidon252Channel::trailing_zeros counts them (channel/poseidon252.rs:59-62). h_digest is the channel
 * digest as 8 little-endian u32 limbs; pow_bits <= 32. */
stwo_status stwo_grind_poseidon252(const uint32_t h_digest[8], uint32_t pow_bits, uint64_t* h_nonce, void* stream);

/* ------------------------------------------------------------------ proving */
/* PcsConfig { pow_bits, fri_config: FriConfig { log_last_layer_degree_bound, log_blowup_factor,
 * n_queries } } (crates/prover/src/core/pcs/mod.rs:33-59, fri.rs:37-70). */
typedef struct {
  uint32_t pow_bits;
  uint32_t log_blowup_factor;
  uint32_t log_last_layer_degree_bound;
  uint32_t n_queries;
} stwo_pcs_config;

/* generate_trace of the wide-Fibonacci example (crates/prover/src/examples/wide_fibonacci/mod.rs:46-68):
 * row r of the n_cols device columns starts from (d_a[r], d_b[r]). */
stwo_status stwo_gen_wide_fib_trace(uint32_t log_n_rows, uint32_t n_cols, const uint32_t* d_a, const uint32_t* d_b,
                                    uint32_t* const* d_cols, void* stream);
/* prove::<CudaBackend, Blake2sMerkleChannel> (crates/prover/src/core/prover/mod.rs:27-79) of the
 * wide-Fibonacci AIR, with an empty preprocessed tree and the trace committed as in
 * test_wide_fib_prove_with_blake (wide_fibonacci/mod.rs:174-227). The trace columns (bit-reversed
 * evaluations) are consumed: they hold the trace coefficients afterwards. Writes the canonical
 * proof bytes (u32 words and u64 lengths little-endian, fields in StarkProof order) to h_proof and
 * their count to *h_len (also when the buffer is too small, which returns INVALID_ARG). */
stwo_status stwo_prove_wide_fib(uint32_t log_n_rows, uint32_t n_cols, uint32_t* const* d_trace, stwo_pcs_config cfg,
                                uint8_t* h_proof, size_t capacity, size_t* h_len, void* stream);

/* prove_poseidon (crates/prover/src/examples/poseidon/mod.rs:327-389): 2^log_n_rows rows of 8
 * Poseidon2 permutations. d_init holds the initial states (word ((row * 8 + rep) * 16 + i)), or is
 * NULL for the reference's deterministic inputs (row + i + rep). It may be device memory or pinned
 * host memory (cudaHostAlloc / cudaHostRegister), which the trace kernel reads once, coalesced,
 * across the host link. Trace, lookup elements, LogUp
 * interaction trace and proof are produced on the device; the claimed LogUp sum (part of the
 * statement the verifier needs) is returned in *h_claimed_sum. */
stwo_status stwo_prove_poseidon(uint32_t log_n_rows, const uint32_t* d_init, stwo_pcs_config cfg, uint8_t* h_proof,
                                size_t capacity, size_t* h_len, stwo_qm31* h_claimed_sum, void* stream);

/* The Blake2s round AIR: BlakeRoundComponent (crates/prover/src/examples/blake/round/) proved on
 * its own, one BLAKE2s round per row over 2^log_n_rows rows (log_n_rows >= 4). d_inputs holds per
 * row the 16 state words then the 16 message words (word row * 32 + i), or is NULL for the
 * reference test's inputs (v_i = i, m_i = i + 1, round/mod.rs:60-110). The transcript follows the
 * Blake example's statements (blake/air.rs:83-183): an empty preprocessed tree, the log size
 * mixed, the trace committed, RoundElements then the five XOR relations drawn, the claimed LogUp
 * sum mixed, the interaction trace committed, then prove(). The claimed sum is returned in
 * *h_claimed_sum. */
stwo_status stwo_prove_blake_round(uint32_t log_n_rows, const uint32_t* d_inputs, stwo_pcs_config cfg,
                                   uint8_t* h_proof, size_t capacity, size_t* h_len, stwo_qm31* h_claimed_sum,
                                   void* stream);

/* A framework component's constraints at one point (constraint_framework/point.rs:15-70), on the
 * host, from its recorded expressions compiled to a small program (values: inputs, then one per
 * op; ops add, sub, mul, neg, inv, partial-evals, relation combine); *acc = acc * rc + denom_inv * c
 * for each output constraint c. The program format is written beside the function. */
stwo_status stwo_point_program_eval(const uint32_t* program, size_t program_len, const stwo_qm31* inputs,
                                    size_t n_inputs, stwo_qm31 rc, stwo_qm31 denom_inv, stwo_qm31* acc);

/* The trace of the full Blake example (prove_blake, crates/prover/src/examples/blake/air.rs:363-400;
 * generators scheduler/gen.rs:45-118, round/gen.rs:206-235, xor_table/mod.rs:60-90) for 2^log_n
 * BLAKE2s instances, generated in HBM. d_trace receives, column after column in commit order, the
 * scheduler's 384 columns of 2^log_n words, the two round components' 384 columns of 2^(log_n+3)
 * and 2^(log_n+1) words, then the XOR tables' multiplicity columns (12/4: 256 of 2^16 words,
 * 9/2: 16 of 2^14, 8/2: 16 of 2^12, 7/2: 16 of 2^10, 4/0: 1 of 2^8): 4224 * 2^log_n + 17,121,536
 * words. d_scratch holds the round inputs, 320 * 2^log_n words. log_n in [4, 20]. */
stwo_status stwo_gen_blake_example_trace(uint32_t log_n, uint32_t* d_trace, uint32_t* d_scratch, void* stream);

/* ------------------------------------------------------------------ batched and served proving */
/* No counterpart in the reference, which proves one statement per call (prover/mod.rs:27-79).
 * A server owns a pool of host workers, each with its own CUDA stream, that run whole-proof jobs
 * (stwo_prove_wide_fib / stwo_prove_poseidon / stwo_prove_blake_round) concurrently. A job starts when its estimated
 * device bytes (stwo_job_hbm_bytes) fit in the HBM budget beside the running jobs; among queued
 * jobs the first in submission order that fits starts next. Proof bytes equal those of the
 * single-call entry points. */
#define STWO_AIR_WIDE_FIB 0u
#define STWO_AIR_POSEIDON 1u
#define STWO_AIR_BLAKE_ROUND 2u
typedef struct {
  uint32_t air;
  uint32_t log_n_rows;
  uint32_t n_cols;        /* wide-Fibonacci columns */
  const uint32_t* d_a;    /* wide-Fibonacci: per-row first two values (device, 2^log_n_rows each) */
  const uint32_t* d_b;
  const uint32_t* d_init; /* Poseidon2 initial states or Blake2s round inputs (device), or NULL for
                             the reference inputs */
  stwo_pcs_config cfg;
  uint8_t* h_proof;       /* host buffer for the proof bytes */
  size_t capacity;
} stwo_proof_job;
typedef struct {
  stwo_status status;
  size_t len;
  stwo_qm31 claimed_sum;  /* Poseidon2 LogUp claimed sum */
  double queue_ms;        /* submission to start */
  double run_ms;          /* start to completion */
  double latency_ms;      /* submission to completion */
  char error[256];
} stwo_proof_result;
typedef struct stwo_server_s* stwo_server;

/* n_workers workers on `device`; hbm_budget_bytes = 0 takes 90% of the free device memory. Each
 * worker owns one stream per priority level: jobs under 256 MB of estimated device bytes run at
 * the highest priority, jobs under 2 GB at the next, and larger jobs below those, each below the
 * large jobs already running, so that small proofs are not queued behind the blocks of large
 * ones and overlapping large proofs finish in arrival order. */
stwo_status stwo_server_create(uint32_t n_workers, size_t hbm_budget_bytes, int device, stwo_server* out);
/* Queues a job (its buffers must stay valid until its wait returns); returns at once. */
stwo_status stwo_server_submit(stwo_server server, const stwo_proof_job* job, uint64_t* ticket);
/* Blocks until the job of `ticket` has finished; each ticket is waited for once. */
stwo_status stwo_server_wait(stwo_server server, uint64_t ticket, stwo_proof_result* out);
/* Runs every queued job to completion, then stops the workers. */
stwo_status stwo_server_destroy(stwo_server server);
/* The admission estimate of a job, in bytes. */
size_t stwo_job_hbm_bytes(const stwo_proof_job* job);
/* All n_jobs on a temporary server without stream priorities, submitted largest first (by
 * stwo_job_hbm_bytes); results[i] belongs to jobs[i]. Returns the first failure. */
stwo_status stwo_prove_batch(const stwo_proof_job* jobs, uint32_t n_jobs, uint32_t n_workers,
                             size_t hbm_budget_bytes, stwo_proof_result* results);

/* ------------------------------------------------------------------ components */
/* One component of a configured AIR: the FrameworkComponent<E> of the wide-Fibonacci, Poseidon2 or
 * Blake2s-round example (crates/prover/src/constraint_framework/component.rs:126-200). Relation
 * elements are given as the channel drew them (LookupElements::draw, logup.rs:74-88): Poseidon2
 * takes 2 (z, alpha); the Blake2s round takes 12: (z, alpha) of the round relation, then of the XOR
 * relations of widths 12, 9, 8, 7 and 4. claimed_sum is the LogUp claimed sum (unused by
 * wide-Fibonacci). */
typedef struct {
  uint32_t air;                /* STWO_AIR_WIDE_FIB, STWO_AIR_POSEIDON or STWO_AIR_BLAKE_ROUND */
  uint32_t log_n_rows;         /* trace log size */
  uint32_t n_cols;             /* wide-Fibonacci columns */
  stwo_qm31 claimed_sum;
  const stwo_qm31* h_elements;
  uint32_t n_elements;
} stwo_component;

/* Component::n_constraints, max_constraint_log_degree_bound and trace_log_degree_bounds
 * (crates/prover/src/core/air/mod.rs:17-40): the constraint count, the log size of the evaluation
 * domain CanonicCoset(eval_log_size).circle_domain(), and how many columns the component reads from
 * each tree (tree 0 preprocessed, 1 trace, 2 interaction; *h_n_trees of them). */
stwo_status stwo_component_info(const stwo_component* component, uint32_t* h_n_constraints, uint32_t* h_eval_log_size,
                                uint32_t* h_n_trees, uint32_t h_tree_n_cols[3]);

/* ComponentProver::evaluate_constraint_quotients_on_domain (crates/prover/src/core/air/mod.rs:59-62;
 * SimdBackend implementation crates/prover/src/constraint_framework/component.rs:278-416), after its
 * extension step:
 *   d_cols          the component's columns on the evaluation domain (bit-reversed evaluations),
 *                   tree by tree in stwo_component_info's counts; the caller extends the committed
 *                   polynomials with stwo_evaluate_columns where the domains differ. Poseidon2 and
 *                   Blake2s-round columns must form one contiguous block per tree (column c at the
 *                   tree's first column + c * 2^eval_log_size words).
 *   h_coeff_powers  the n_constraints random-coefficient powers that
 *                   DomainEvaluationAccumulator::columns hands the component
 *                   (crates/prover/src/core/air/accumulation.rs:71-93), in that order.
 *   d_accum         the accumulation column of the evaluation domain's log size: every row adds
 *                   row_res / coset_vanishing(trace coset, row point).
 * Stream ordered. */
stwo_status stwo_eval_constraints(const stwo_component* component, const uint32_t* const* d_cols, uint32_t n_cols,
                                  const stwo_qm31* h_coeff_powers, uint32_t n_coeff_powers,
                                  uint32_t* const d_accum[4], void* stream);

/* ---- Generated constraint kernels (constraint framework's expr module,
 * crates/prover/src/constraint_framework/expr/evaluator.rs:54-227, evaluated on the domain as
 * SimdDomainEvaluator does, constraint_framework/simd_domain.rs:24-114). A component written
 * against the framework is recorded as expressions and emitted as CUDA source defining
 * `extern "C" __global__ void stwo_generated_constraints(stwo::GenArgs)` (the argument block of
 * stwo_gb300/csrc/codegen_rt.cuh, which the source may include together with field.cuh). */
typedef struct stwo_codegen_component_s* stwo_codegen_component;

/* Compiles kernel_source with NVRTC for sm_103a (no device needed) and, when load_now is set,
 * loads it on the current device (otherwise the first evaluation loads it). n_cols, n_params and
 * n_constraints are the component's column count (all interactions), parameter count and
 * constraint count, checked on every call. A source that does not compile returns
 * STWO_ERR_INVALID_ARG with the compiler log in stwo_last_error(). */
stwo_status stwo_codegen_compile(const char* kernel_source, uint32_t n_cols, uint32_t n_params,
                                 uint32_t n_constraints, int load_now, stwo_codegen_component* out);
/* The compiled cubin: its size in *h_size, and a copy in h_dst when h_dst is given (capacity must
 * cover it). With stwo_codegen_from_cubin, a caller can cache compiled components across
 * processes (NVRTC takes tens of seconds for a component of a thousand constraints). */
stwo_status stwo_codegen_cubin(stwo_codegen_component component, void* h_dst, size_t capacity, size_t* h_size);
/* A component from a cubin that stwo_codegen_cubin returned for the same source and sizes. */
stwo_status stwo_codegen_from_cubin(const void* h_cubin, size_t size, uint32_t n_cols, uint32_t n_params,
                                    uint32_t n_constraints, int load_now, stwo_codegen_component* out);
stwo_status stwo_codegen_destroy(stwo_codegen_component component);

/* The LogUp interaction trace of a generated component (LogupTraceGenerator,
 * crates/prover/src/constraint_framework/logup.rs:123-260): `component` was compiled from the source
 * of its fraction kernel (stwo_gb300/codegen.py generate_fractions; n_constraints = the number of
 * LogUp batches B), d_cols are its preprocessed then trace columns on the trace domain (2^log_size
 * bit-reversed evaluations), d_out 4 B contiguous columns of 2^log_size words: batch b's column holds
 * the running sum over batches 0..b of num/den, the last one finalised (claimed sum subtracted as
 * claimed_sum / 2^log_size, inclusive prefix sum in coset order). The claimed sum is returned in
 * h_claimed_sum (the call synchronises the stream). */
stwo_status stwo_logup_interaction_codegen(stwo_codegen_component component, uint32_t log_size,
                                          const uint32_t* const* d_cols, uint32_t n_cols, const stwo_qm31* h_params,
                                          uint32_t n_params, uint32_t* d_out, stwo_qm31* h_claimed_sum,
                                          void* stream);

/* ComponentProver::evaluate_constraint_quotients_on_domain (crates/prover/src/core/air/mod.rs:59-62;
 * SimdBackend implementation crates/prover/src/constraint_framework/component.rs:278-416) for a
 * generated component, after its extension step:
 *   d_cols          the columns on the evaluation domain (bit-reversed), interaction 0 (preprocessed,
 *                   in the order the component requests them), then the trace, then the interaction
 *                   trace, each in mask order;
 *   h_params        the values of the component's formal parameters, in the generator's order
 *                   (relation elements, claimed_sum, column_size = 2^trace_log_size, ...), 4 words
 *                   each (a base-field parameter in word 0);
 *   h_coeff_powers  the n_constraints powers DomainEvaluationAccumulator::columns hands the
 *                   component (crates/prover/src/core/air/accumulation.rs:71-93), in that order;
 *   d_accum         the accumulation column of size 2^eval_log_size: every row adds
 *                   row_res / coset_vanishing(trace coset, row point).
 * Stream ordered. */
stwo_status stwo_eval_constraints_codegen(stwo_codegen_component component, uint32_t trace_log_size,
                                          uint32_t eval_log_size, const uint32_t* const* d_cols, uint32_t n_cols,
                                          const stwo_qm31* h_params, uint32_t n_params,
                                          const stwo_qm31* h_coeff_powers, uint32_t n_coeff_powers,
                                          uint32_t* const d_accum[4], void* stream);

#ifdef __cplusplus
}
#endif
#endif /* STWO_CUDA_H */
