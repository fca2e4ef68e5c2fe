// ORACLE — test infrastructure only. CPU-baseline timing of the oracle on bounded samples of
// the benchmark workloads, parallelised with OpenMP over columns / rows. Used only by bench.py's
// CPU-baseline leg and its `--impl reference` arm.
#include "ops.h"
#include <chrono>
#include <omp.h>

using namespace oracle;

namespace {

// Benchmark input generator shared with bench.py: word i of column c of workload k is
// splitmix64(k + (c * 2^32 + i + 1) * 0x9E3779B97F4A7C15) mod P (uniform up to a 2^-33 bias).
inline uint64_t splitmix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
inline uint32_t gen_word(uint64_t k, uint64_t c, uint64_t i) {
  return (uint32_t)(splitmix64(k + ((c << 32) + i + 1) * 0x9E3779B97F4A7C15ull) % P);
}

double now() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

extern "C" {

void oracle_gen_words(uint64_t k, uint64_t c, uint64_t n, uint32_t* out) {
  for (uint64_t i = 0; i < n; i++) out[i] = gen_word(k, c, i);
}

}  // extern "C"

namespace {

// Kernel-microbench sample: `n_cols` columns of 2^log words (workload k = 1) interpolated on the
// canonic domain, evaluated at log + blowup, committed in a Blake2s Merkle tree; plus one FRI
// fold chain of a 2^fri_log QM31 circle evaluation (columns 1000..1003) down to 2^4 with seeded
// alphas. Returns compute seconds (input generation and twiddles excluded); writes the Merkle
// root (8 words) and the last FRI layer (4 x 16 words). With `fri_layers_out` set, every folded
// FRI layer is written there too (4 coordinate columns per layer, largest layer first).
double cfg2_pass(uint32_t n_cols, uint32_t log, uint32_t blowup, uint32_t fri_log, int threads, uint32_t* root_out,
                 uint32_t* fri_out, uint32_t* fri_layers_out) {
  if (threads > 0) omp_set_num_threads(threads);
  const uint32_t L = log + blowup;
  size_t n = (size_t)1 << log, N = (size_t)1 << L;
  std::vector<Column> cols(n_cols, Column(n));
#pragma omp parallel for schedule(static)
  for (long c = 0; c < (long)n_cols; c++)
    for (size_t i = 0; i < n; i++) cols[c][i] = M31(gen_word(1, c, i));
  SecureColumn fsrc((size_t)1 << fri_log);
  for (int k = 0; k < 4; k++)
    for (size_t i = 0; i < fsrc.size(); i++) fsrc.c[k][i] = M31(gen_word(1, 1000 + k, i));
  std::vector<QM31> alphas;
  for (uint32_t j = 0; j < fri_log; j++)
    alphas.push_back(QM31::from_u32(gen_word(1, 2000, 4 * j), gen_word(1, 2000, 4 * j + 1),
                                    gen_word(1, 2000, 4 * j + 2), gen_word(1, 2000, 4 * j + 3)));
  CircleDomain big = canonic_domain(L), small = canonic_domain(log);
  TwiddleTree tw = precompute_twiddles(big.half_coset);
  CircleDomain fdom = canonic_domain(fri_log);
  TwiddleTree ftw = precompute_twiddles(fdom.half_coset);
  (void)ftw;

  double t0 = now();
  std::vector<Column> evals(n_cols);
#pragma omp parallel for schedule(dynamic)
  for (long c = 0; c < (long)n_cols; c++) {
    std::vector<M31> coeffs = interpolate(small, cols[c], tw);
    evals[c] = evaluate(big, coeffs, tw);
  }
  // Merkle: leaf layer parallel over nodes, then the node layers.
  std::vector<std::vector<Hash32>> layers;
  {
    std::vector<Hash32> leaf(N);
#pragma omp parallel
    {
      std::vector<uint32_t> vals(n_cols);
#pragma omp for schedule(static)
      for (long i = 0; i < (long)N; i++) {
        for (uint32_t c = 0; c < n_cols; c++) vals[c] = evals[c][i].v;
        leaf[i] = hash_node(nullptr, nullptr, vals.data(), n_cols);
      }
    }
    layers.push_back(std::move(leaf));
    for (int lg = (int)L - 1; lg >= 0; lg--) {
      const std::vector<Hash32>& prev = layers.back();
      std::vector<Hash32> cur((size_t)1 << lg);
#pragma omp parallel for schedule(static)
      for (long i = 0; i < (long)cur.size(); i++) cur[i] = hash_node(&prev[2 * i], &prev[2 * i + 1], nullptr, 0);
      layers.push_back(std::move(cur));
    }
  }
  // FRI fold chain.
  SecureColumn line((size_t)1 << (fri_log - 1));
  fold_circle_into_line(line, fsrc, fdom, alphas[0]);
  auto keep = [&](const SecureColumn& l) {
    if (!fri_layers_out) return;
    for (int k = 0; k < 4; k++)
      for (size_t i = 0; i < l.size(); i++) *fri_layers_out++ = l.c[k][i].v;
  };
  keep(line);
  Coset ld = fdom.half_coset;
  for (uint32_t j = 1; line.size() > 16; j++) {
    line = fold_line(line, ld, alphas[j]);
    ld = ld.dbl();
    keep(line);
  }
  double t1 = now();
  layers.back()[0].words(root_out);
  for (int k = 0; k < 4; k++)
    for (size_t i = 0; i < line.size() && i < 16; i++) fri_out[16 * k + i] = line.c[k][i].v;
  return t1 - t0;
}

}  // namespace

extern "C" {

double oracle_bench_cfg2(uint32_t n_cols, uint32_t log, uint32_t blowup, uint32_t fri_log, int threads,
                         uint32_t* root_out, uint32_t* fri_out) {
  return cfg2_pass(n_cols, log, blowup, fri_log, threads, root_out, fri_out, nullptr);
}

// The same pass with every folded FRI layer written to `fri_layers_out`: 4 x 2^(fri_log-1) words
// for the circle fold, then 4 x 2^(k-1) for each line fold down to 2^4 points.
double oracle_cfg2_outputs(uint32_t n_cols, uint32_t log, uint32_t blowup, uint32_t fri_log, int threads,
                           uint32_t* root_out, uint32_t* fri_out, uint32_t* fri_layers_out) {
  return cfg2_pass(n_cols, log, blowup, fri_log, threads, root_out, fri_out, fri_layers_out);
}

}  // extern "C"
