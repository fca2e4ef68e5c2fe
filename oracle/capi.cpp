// ORACLE — test infrastructure only. C entry points over the oracle restatement, loaded by the
// tests (ctypes) as the checker for the CUDA backend and by bench.py as the CPU baseline.
// Nothing in the product links this library.
#include "ops.h"
#include <cstring>
#include <memory>

using namespace oracle;

static Coset mk_coset(const uint32_t c[3]) { return Coset::raw(c[0], c[1], c[2]); }
static QM31 q_of(const uint32_t* v) { return QM31::from_u32(v[0], v[1], v[2], v[3]); }
static void q_to(QM31 q, uint32_t* v) {
  v[0] = q.a.a.v; v[1] = q.a.b.v; v[2] = q.b.a.v; v[3] = q.b.b.v;
}
static Column col_of(const uint32_t* p, size_t n) {
  Column c(n);
  for (size_t i = 0; i < n; i++) c[i] = M31(p[i]);
  return c;
}

extern "C" {

// Twiddle tree of `root` (size 2^root.log_size): x-coordinates and inverses.
void oracle_twiddles(const uint32_t root[3], uint32_t* tw, uint32_t* itw) {
  TwiddleTree t = precompute_twiddles(mk_coset(root));
  for (size_t i = 0; i < t.twiddles.size(); i++) {
    tw[i] = t.twiddles[i].v;
    itw[i] = t.itwiddles[i].v;
  }
}

// In-place interpolation of n = 2^(half.log_size+1) bit-reversed values on the domain with
// half coset `half`, using the tree of `tree_root`.
int oracle_interpolate(const uint32_t half[3], const uint32_t tree_root[3], uint32_t* values) {
  try {
    CircleDomain d{mk_coset(half)};
    TwiddleTree t = precompute_twiddles(mk_coset(tree_root));
    std::vector<M31> v = interpolate(d, col_of(values, d.size()), t);
    for (size_t i = 0; i < v.size(); i++) values[i] = v[i].v;
    return 0;
  } catch (...) {
    return 1;
  }
}

int oracle_evaluate(const uint32_t half[3], const uint32_t tree_root[3], const uint32_t* coeffs,
                    uint32_t coeff_log, uint32_t* out) {
  try {
    CircleDomain d{mk_coset(half)};
    TwiddleTree t = precompute_twiddles(mk_coset(tree_root));
    std::vector<M31> v = evaluate(d, col_of(coeffs, (size_t)1 << coeff_log), t);
    for (size_t i = 0; i < v.size(); i++) out[i] = v[i].v;
    return 0;
  } catch (...) {
    return 1;
  }
}

void oracle_eval_at_point(const uint32_t* coeffs, uint32_t log_size, const uint32_t point[8], uint32_t out[4]) {
  CirclePointQM31 p{q_of(point), q_of(point + 4)};
  q_to(eval_at_point(col_of(coeffs, (size_t)1 << log_size), p), out);
}

// Merkle layer: prev (8 words per hash, 2^(log+1) hashes) or NULL.
void oracle_commit_on_layer(uint32_t log_size, const uint32_t* prev, const uint32_t* const* cols, uint32_t n_cols,
                            uint32_t* out) {
  size_t n = (size_t)1 << log_size;
  std::vector<Column> cs;
  for (uint32_t c = 0; c < n_cols; c++) cs.push_back(col_of(cols[c], n));
  std::vector<const Column*> cp;
  for (auto& c : cs) cp.push_back(&c);
  std::vector<Hash32> pv;
  if (prev) {
    pv.resize(2 * n);
    for (size_t i = 0; i < 2 * n; i++) pv[i] = Hash32::from_words(prev + 8 * i);
  }
  std::vector<Hash32> r = commit_on_layer(log_size, prev ? &pv : nullptr, cp);
  for (size_t i = 0; i < n; i++) r[i].words(out + 8 * i);
}

void oracle_blake2s(const uint8_t* data, size_t len, uint8_t out[32]) {
  Hash32 h = Blake2s::hash(data, len);
  std::memcpy(out, h.b, 32);
}

void oracle_fold_line(const uint32_t domain[3], const uint32_t* const src[4], const uint32_t alpha[4],
                      uint32_t* const out[4]) {
  Coset d = mk_coset(domain);
  size_t n = d.size();
  SecureColumn e(n);
  for (int k = 0; k < 4; k++) e.c[k] = col_of(src[k], n);
  SecureColumn r = fold_line(e, d, q_of(alpha));
  for (int k = 0; k < 4; k++)
    for (size_t i = 0; i < n / 2; i++) out[k][i] = r.c[k][i].v;
}

void oracle_fold_circle_into_line(const uint32_t half[3], uint32_t* const dst[4], const uint32_t* const src[4],
                                  const uint32_t alpha[4]) {
  CircleDomain d{mk_coset(half)};
  size_t n = d.size();
  SecureColumn s(n), t(n / 2);
  for (int k = 0; k < 4; k++) {
    s.c[k] = col_of(src[k], n);
    t.c[k] = col_of(dst[k], n / 2);
  }
  fold_circle_into_line(t, s, d, q_of(alpha));
  for (int k = 0; k < 4; k++)
    for (size_t i = 0; i < n / 2; i++) dst[k][i] = t.c[k][i].v;
}

void oracle_decompose(const uint32_t* const src[4], uint32_t log_size, uint32_t* const g[4], uint32_t lambda[4]) {
  size_t n = (size_t)1 << log_size;
  SecureColumn e(n);
  for (int k = 0; k < 4; k++) e.c[k] = col_of(src[k], n);
  auto r = decompose(e);
  for (int k = 0; k < 4; k++)
    for (size_t i = 0; i < n; i++) g[k][i] = r.first.c[k][i].v;
  q_to(r.second, lambda);
}

// Quotients on CanonicCoset(log_n).circle_domain(). Batches: n_batches points (8 words each),
// batch_offsets[n_batches+1] into entry_cols / entry_values (4 words each).
void oracle_accumulate_quotients(uint32_t log_n, const uint32_t* const* cols, uint32_t n_cols,
                                 const uint32_t random_coeff[4], uint32_t n_batches, const uint32_t* batch_points,
                                 const uint32_t* batch_offsets, const uint32_t* entry_cols,
                                 const uint32_t* entry_values, uint32_t log_blowup, uint32_t* const out[4]) {
  size_t n = (size_t)1 << log_n;
  std::vector<Column> cs;
  for (uint32_t c = 0; c < n_cols; c++) cs.push_back(col_of(cols[c], n));
  std::vector<const Column*> cp;
  for (auto& c : cs) cp.push_back(&c);
  std::vector<ColumnSampleBatch> batches;
  for (uint32_t b = 0; b < n_batches; b++) {
    ColumnSampleBatch sb;
    sb.point = {q_of(batch_points + 8 * b), q_of(batch_points + 8 * b + 4)};
    for (uint32_t e = batch_offsets[b]; e < batch_offsets[b + 1]; e++)
      sb.columns_and_values.push_back({entry_cols[e], q_of(entry_values + 4 * e)});
    batches.push_back(sb);
  }
  SecureColumn r = accumulate_quotients(canonic_domain(log_n), cp, q_of(random_coeff), batches, log_blowup);
  for (int k = 0; k < 4; k++)
    for (size_t i = 0; i < n; i++) out[k][i] = r.c[k][i].v;
}

void oracle_secure_powers(const uint32_t felt[4], uint32_t n, uint32_t* out) {
  auto v = generate_secure_powers(q_of(felt), n);
  for (uint32_t i = 0; i < n; i++) q_to(v[i], out + 4 * i);
}

uint64_t oracle_grind(const uint32_t digest[8], uint32_t pow_bits) { return grind(digest, pow_bits); }

void oracle_raw_compress(const uint32_t h[8], const uint32_t m[16], uint32_t t0, uint32_t t1, uint32_t f0,
                         uint32_t f1, uint32_t out[8]) {
  auto r = b2s_compress(h, m, t0, t1, f0, f1);
  for (int i = 0; i < 8; i++) out[i] = r[i];
}

void oracle_qm31_mul(const uint32_t a[4], const uint32_t b[4], uint32_t out[4]) { q_to(q_of(a) * q_of(b), out); }
void oracle_qm31_inv(const uint32_t a[4], uint32_t out[4]) { q_to(inv(q_of(a)), out); }

// Circle point i * M31_CIRCLE_GEN.
void oracle_index_to_point(uint32_t idx, uint32_t out[2]) {
  CirclePointM31 p = index_to_point(idx);
  out[0] = p.x.v;
  out[1] = p.y.v;
}

}  // extern "C"

// ---------------------------------------------------------------- proofs
#include "air_wide_fib.h"

extern "C" {

// Proves the wide-Fibonacci AIR (log_n rows, n_cols columns, row r starting from (a[r], b[r])) as
// the reference's test_wide_fib_prove_with_blake does; writes the canonical proof bytes.
// Returns the proof length, or 0 on failure (message in err).
size_t oracle_prove_wide_fib(uint32_t log_n, uint32_t n_cols, const uint32_t* a, const uint32_t* b,
                             const uint32_t cfg[4], uint8_t* out, size_t cap, char* err, size_t err_cap) {
  try {
    PcsConfig config{cfg[0], cfg[1], cfg[2], cfg[3]};
    TwiddleTree tw = precompute_twiddles(canonic_domain(log_n + 1 + config.log_blowup).half_coset);
    Channel ch;
    CommitmentSchemeProver pcs;
    pcs.config = config;
    pcs.twiddles = &tw;
    pcs.commit({}, ch);
    pcs.commit_evals(wide_fib_trace(log_n, n_cols, a, b), log_n, ch);
    WideFibAir air(log_n, n_cols);
    StarkProof proof = prove(air, ch, pcs);
    std::vector<uint8_t> bytes = serialize(proof);
    if (bytes.size() > cap) throw std::runtime_error("output buffer too small");
    std::memcpy(out, bytes.data(), bytes.size());
    return bytes.size();
  } catch (const std::exception& e) {
    snprintf(err, err_cap, "%s", e.what());
    return 0;
  }
}

// Verifies canonical proof bytes of the wide-Fibonacci AIR; returns 1 when accepted.
int oracle_verify_wide_fib(uint32_t log_n, uint32_t n_cols, const uint8_t* proof, size_t len, char* err,
                           size_t err_cap) {
  try {
    StarkProof p;
    if (!deserialize(proof, len, p)) throw std::runtime_error("malformed proof bytes");
    Channel ch;
    WideFibAir air(log_n, n_cols);
    std::string r = verify(air, ch, p, {{}, std::vector<uint32_t>(n_cols, log_n)});
    if (!r.empty()) throw std::runtime_error(r);
    return 1;
  } catch (const std::exception& e) {
    snprintf(err, err_cap, "%s", e.what());
    return 0;
  }
}

}  // extern "C"

#include "air_poseidon.h"

extern "C" {

// The Poseidon2 linear layers of the example (poseidon/mod.rs apply_m4, apply_internal_round_matrix,
// apply_external_round_matrix), in place on canonical words.
void oracle_poseidon_apply_m4(uint32_t x[4]) {
  M31 v[4];
  for (int i = 0; i < 4; i++) v[i] = M31(x[i]);
  apply_m4(v);
  for (int i = 0; i < 4; i++) x[i] = v[i].v;
}
void oracle_poseidon_apply_internal(uint32_t x[16]) {
  M31 v[16];
  for (int i = 0; i < 16; i++) v[i] = M31(x[i]);
  apply_internal_round_matrix(v);
  for (int i = 0; i < 16; i++) x[i] = v[i].v;
}
void oracle_poseidon_apply_external(uint32_t x[16]) {
  M31 v[16];
  for (int i = 0; i < 16; i++) v[i] = M31(x[i]);
  apply_external_round_matrix(v);
  for (int i = 0; i < 16; i++) x[i] = v[i].v;
}

// Proves the Poseidon2 AIR (2^log_n rows, 8 permutations per row) as prove_poseidon does
// (poseidon/mod.rs:327-389). `init` holds the initial states ((row * 8 + rep) * 16 + i), or is NULL
// for the reference's deterministic inputs. Writes the proof bytes; claimed_sum (4 words) out.
size_t oracle_prove_poseidon(uint32_t log_n, const uint32_t* init, const uint32_t cfg[4], uint8_t* out, size_t cap,
                             uint32_t claimed_sum[4], char* err, size_t err_cap) {
  try {
    PcsConfig config{cfg[0], cfg[1], cfg[2], cfg[3]};
    std::vector<uint32_t> ref;
    if (!init) {
      ref = poseidon_reference_inputs(log_n);
      init = ref.data();
    }
    TwiddleTree tw = precompute_twiddles(canonic_domain(log_n + PS_LOG_EXPAND + config.log_blowup).half_coset);
    Channel ch;
    CommitmentSchemeProver pcs;
    pcs.config = config;
    pcs.twiddles = &tw;
    pcs.commit({}, ch);
    std::vector<std::vector<M31>> lookups;
    pcs.commit_evals(poseidon_trace(log_n, init, lookups), log_n, ch);
    LookupElements le = LookupElements::draw(ch);
    QM31 cs;
    pcs.commit_evals(poseidon_interaction_trace(log_n, lookups, le, cs), log_n, ch);
    PoseidonAir air(log_n, le, cs);
    StarkProof proof = prove(air, ch, pcs);
    std::vector<uint8_t> bytes = serialize(proof);
    if (bytes.size() > cap) throw std::runtime_error("output buffer too small");
    std::memcpy(out, bytes.data(), bytes.size());
    q_to(cs, claimed_sum);
    return bytes.size();
  } catch (const std::exception& e) {
    snprintf(err, err_cap, "%s", e.what());
    return 0;
  }
}

int oracle_verify_poseidon(uint32_t log_n, const uint32_t claimed_sum[4], const uint8_t* proof, size_t len, char* err,
                           size_t err_cap) {
  try {
    StarkProof p;
    if (!deserialize(proof, len, p)) throw std::runtime_error("malformed proof bytes");
    Channel ch;
    PoseidonAir air(log_n, LookupElements{}, q_of(claimed_sum));
    auto hook = [&](size_t t, Channel& c) {
      if (t == 1) air.le = LookupElements::draw(c);
    };
    std::string r = verify(air, ch, p,
                           {{}, std::vector<uint32_t>(PS_COLUMNS, log_n), std::vector<uint32_t>(32, log_n)}, hook);
    if (!r.empty()) throw std::runtime_error(r);
    return 1;
  } catch (const std::exception& e) {
    snprintf(err, err_cap, "%s", e.what());
    return 0;
  }
}

}  // extern "C"

#include "gkr.h"

namespace {
std::vector<QM31> secure_of(const uint32_t* soa, size_t n) {
  std::vector<QM31> v(n);
  for (size_t i = 0; i < n; i++) v[i] = QM31::from_u32(soa[i], soa[n + i], soa[2 * n + i], soa[3 * n + i]);
  return v;
}
void secure_to(const std::vector<QM31>& v, uint32_t* soa) {
  size_t n = v.size();
  for (size_t i = 0; i < n; i++) {
    soa[i] = v[i].a.a.v;
    soa[n + i] = v[i].a.b.v;
    soa[2 * n + i] = v[i].b.a.v;
    soa[3 * n + i] = v[i].b.b.v;
  }
}
std::vector<QM31> qs_of(const uint32_t* aos, size_t n) {
  std::vector<QM31> v(n);
  for (size_t i = 0; i < n; i++) v[i] = q_of(aos + 4 * i);
  return v;
}
// Reads one layer from `data`: the grand-product column, or numerators then denominators, each
// secure column as four coordinate arrays and the multiplicities as one base array.
GkrLayer layer_of(uint32_t kind, uint32_t log_n, const uint32_t*& data) {
  size_t n = (size_t)1 << log_n;
  GkrLayer l;
  l.kind = (GkrKind)kind;
  if (kind == GKR_GRAND_PRODUCT || kind == GKR_LOGUP_GENERIC) {
    l.num = secure_of(data, n);
    data += 4 * n;
  } else if (kind == GKR_LOGUP_MULTIPLICITIES) {
    for (size_t i = 0; i < n; i++) l.num_base.push_back(M31(data[i]));
    data += n;
  }
  if (kind != GKR_GRAND_PRODUCT) {
    l.den = secure_of(data, n);
    data += 4 * n;
  }
  return l;
}
std::vector<GkrLayer> layers_of(size_t n_inst, const uint32_t* kinds, const uint32_t* logs, const uint32_t* data) {
  std::vector<GkrLayer> v;
  for (size_t i = 0; i < n_inst; i++) v.push_back(layer_of(kinds[i], logs[i], data));
  return v;
}
}  // namespace

extern "C" {

// GkrOps::gen_eq_evals: eq(x, y) * v over {0,1}^n_y into four coordinate arrays of 2^n_y.
void oracle_gkr_gen_eq_evals(const uint32_t* y, uint32_t n_y, const uint32_t v[4], uint32_t* out) {
  secure_to(gen_eq_evals(qs_of(y, n_y), q_of(v)), out);
}

// GkrOps::next_layer for a layer of 2^log_n gates; writes the next layer's columns in the same
// packing (a grand product stays one column, every LogUp kind becomes generic: numerators then
// denominators).
void oracle_gkr_next_layer(uint32_t kind, uint32_t log_n, const uint32_t* data, uint32_t* out) {
  GkrLayer l = next_layer(layer_of(kind, log_n, data));
  secure_to(l.num, out);
  if (l.kind != GKR_GRAND_PRODUCT) secure_to(l.den, out + 4 * l.num.size());
}

// GkrOps::sum_as_poly_in_first_variable for the oracle of a layer of 2^log_n gates with eq
// evaluations generated from y (EqEvals::generate), lambda and the accumulated eq correction.
// Writes the round polynomial's coefficients (up to 4) and returns their number.
uint32_t oracle_gkr_sum_as_poly(uint32_t kind, uint32_t log_n, const uint32_t* data, const uint32_t* y, uint32_t n_y,
                                const uint32_t lambda[4], const uint32_t correction[4], const uint32_t claim[4],
                                uint32_t* coeffs) {
  EqEvals eq = EqEvals::generate(qs_of(y, n_y));
  GkrPolyOracle o;
  o.eq = &eq;
  o.layer = layer_of(kind, log_n, data);
  o.lambda = q_of(lambda);
  o.correction = q_of(correction);
  UPoly p = o.sum_as_poly_in_first_variable(q_of(claim));
  for (size_t i = 0; i < p.size(); i++) q_to(p[i], coeffs + 4 * i);
  return (uint32_t)p.size();
}

// MleOps::fix_first_variable of a base (is_base = 1, one array) or secure (four coordinate
// arrays) column of 2^log_n values; writes 2^(log_n-1) secure values.
void oracle_mle_fix_first_variable(int is_base, uint32_t log_n, const uint32_t* in, const uint32_t a[4],
                                   uint32_t* out) {
  size_t n = (size_t)1 << log_n;
  if (is_base) {
    std::vector<M31> m(n);
    for (size_t i = 0; i < n; i++) m[i] = M31(in[i]);
    secure_to(fix_first_variable(m, q_of(a)), out);
  } else {
    secure_to(fix_first_variable(secure_of(in, n), q_of(a)), out);
  }
}

// gkr_prover::prove_batch over n_inst input layers (kinds / log sizes / packed data as above)
// on a channel whose digest is `digest` (NULL: the default channel). Writes the proof followed by
// the artifact; returns the byte count, or 0 with `err` set.
size_t oracle_gkr_prove(size_t n_inst, const uint32_t* kinds, const uint32_t* logs, const uint32_t* data,
                        const uint8_t* digest, uint8_t* out, size_t cap, uint8_t* digest_out, char* err,
                        size_t err_cap) {
  try {
    Channel ch;
    if (digest) std::memcpy(ch.digest.b, digest, 32);
    auto [proof, art] = gkr_prove_batch(ch, layers_of(n_inst, kinds, logs, data));
    Writer w;
    write_gkr(w, proof, art);
    if (w.b.size() > cap) throw std::runtime_error("output buffer too small");
    std::memcpy(out, w.b.data(), w.b.size());
    if (digest_out) std::memcpy(digest_out, ch.digest.b, 32);
    return w.b.size();
  } catch (const std::exception& e) {
    snprintf(err, err_cap, "%s", e.what());
    return 0;
  }
}

// partially_verify_batch on the proof bytes, then the checks of the reference's GKR tests: the
// recomputed artifact equals the one written after the proof, and each instance's claims equal
// its input layer's columns at the artifact's point (gkr.rs tests, cpu/lookups/gkr.rs:315-470).
// `data` may be NULL to skip the input-layer check. Returns 1 on success.
int oracle_gkr_verify(size_t n_inst, const uint32_t* kinds, const uint32_t* logs, const uint32_t* data,
                      const uint8_t* digest, const uint8_t* bytes, size_t len, char* err, size_t err_cap) {
  try {
    GkrBatchProof proof;
    GkrArtifact claimed, art;
    if (!read_gkr(bytes, len, proof, claimed)) throw std::runtime_error("malformed proof bytes");
    Channel ch;
    if (digest) std::memcpy(ch.digest.b, digest, 32);
    std::vector<GkrGate> gates;
    for (size_t i = 0; i < n_inst; i++) gates.push_back(kinds[i] == GKR_GRAND_PRODUCT ? GATE_GRAND_PRODUCT : GATE_LOGUP);
    std::string r = gkr_partially_verify_batch(gates, proof, ch, art);
    if (!r.empty()) throw std::runtime_error(r);
    if (art.ood_point != claimed.ood_point || art.claims_to_verify_by_instance != claimed.claims_to_verify_by_instance ||
        art.n_variables_by_instance != claimed.n_variables_by_instance)
      throw std::runtime_error("artifact differs from the verifier's");
    if (data) {
      std::vector<GkrLayer> layers = layers_of(n_inst, kinds, logs, data);
      size_t n_layers = 0;
      for (auto& l : layers) n_layers = std::max(n_layers, l.n_variables());
      for (size_t i = 0; i < n_inst; i++) {
        const GkrLayer& l = layers[i];
        std::vector<QM31> pt(art.ood_point.begin() + (n_layers - l.n_variables()), art.ood_point.end());
        std::vector<QM31> want;
        if (l.kind == GKR_GRAND_PRODUCT) {
          want = {mle_eval_at_point(l.num, pt)};
        } else {
          std::vector<QM31> num;
          if (l.kind == GKR_LOGUP_SINGLES) num.assign(l.den.size(), q_one());
          else if (l.kind == GKR_LOGUP_MULTIPLICITIES) for (auto x : l.num_base) num.push_back(QM31(x));
          else num = l.num;
          want = {mle_eval_at_point(num, pt), mle_eval_at_point(l.den, pt)};
        }
        if (want != art.claims_to_verify_by_instance[i]) throw std::runtime_error("input layer claim mismatch");
      }
    }
    return 1;
  } catch (const std::exception& e) {
    snprintf(err, err_cap, "%s", e.what());
    return 0;
  }
}

// Draws n secure felts from the default channel (test_channel().draw_felts(n)), four words each.
void oracle_channel_draw_felts(size_t n, uint32_t* out) {
  Channel ch;
  std::vector<QM31> v = ch.draw_felts(n);
  for (size_t i = 0; i < n; i++) q_to(v[i], out + 4 * i);
}

}  // extern "C"

#include "air_blake_round.h"
#include "air_examples.h"
#include "components.h"
#include "air_blake_full.h"

extern "C" {

// Proves the Blake2s round AIR (2^log_n rows, one BLAKE2s round per row): empty preprocessed
// tree, the log size mixed into the channel, the trace, the relation elements, the claimed sum
// mixed, the LogUp interaction trace, then prove(). `inputs` holds per row the 16 state words and
// the 16 message words (row * 32 + i), or is NULL for the reference test's inputs.
size_t oracle_prove_blake_round(uint32_t log_n, const uint32_t* inputs, const uint32_t cfg[4], uint8_t* out,
                                size_t cap, uint32_t claimed_sum[4], char* err, size_t err_cap) {
  try {
    PcsConfig config{cfg[0], cfg[1], cfg[2], cfg[3]};
    std::vector<uint32_t> ref;
    if (!inputs) {
      ref = blake_round_reference_inputs(log_n);
      inputs = ref.data();
    }
    TwiddleTree tw = precompute_twiddles(canonic_domain(log_n + 1 + config.log_blowup).half_coset);
    Channel ch;
    CommitmentSchemeProver pcs;
    pcs.config = config;
    pcs.twiddles = &tw;
    pcs.commit({}, ch);
    ch.mix_u64(log_n);
    std::vector<BrXorLookup> xl;
    std::vector<std::vector<M31>> round;
    pcs.commit_evals(blake_round_trace(log_n, inputs, xl, round), log_n, ch);
    BlakeRoundElements el = BlakeRoundElements::draw(ch);
    QM31 cs;
    std::vector<Column> inter = blake_round_interaction_trace(log_n, xl, round, el, cs);
    ch.mix_felts({cs});
    pcs.commit_evals(inter, log_n, ch);
    BlakeRoundAir air(log_n, el, cs);
    StarkProof proof = prove(air, ch, pcs);
    std::vector<uint8_t> bytes = serialize(proof);
    if (bytes.size() > cap) throw std::runtime_error("output buffer too small");
    std::memcpy(out, bytes.data(), bytes.size());
    q_to(cs, claimed_sum);
    return bytes.size();
  } catch (const std::exception& e) {
    snprintf(err, err_cap, "%s", e.what());
    return 0;
  }
}

int oracle_verify_blake_round(uint32_t log_n, const uint32_t claimed_sum[4], const uint8_t* proof, size_t len,
                              char* err, size_t err_cap) {
  try {
    StarkProof p;
    if (!deserialize(proof, len, p)) throw std::runtime_error("malformed proof bytes");
    Channel ch;
    BlakeRoundAir air(log_n, BlakeRoundElements{}, q_of(claimed_sum));
    auto hook = [&](size_t t, Channel& c) {
      if (t == 0) c.mix_u64(log_n);
      if (t == 1) {
        air.el = BlakeRoundElements::draw(c);
        c.mix_felts({air.claimed_sum});
      }
    };
    std::string r = verify(air, ch, p,
                           {{}, std::vector<uint32_t>(BR_TRACE_COLS, log_n),
                            std::vector<uint32_t>(4 * BR_INTERACTION_SECURE, log_n)},
                           hook);
    if (!r.empty()) throw std::runtime_error(r);
    return 1;
  } catch (const std::exception& e) {
    snprintf(err, err_cap, "%s", e.what());
    return 0;
  }
}

// ComponentProver::evaluate_constraint_quotients_on_domain after the extension step
// (constraint_framework/component.rs:322-416): acc[r] += row_res(r) / coset_vanishing(trace coset,
// point r) on CanonicCoset(eval log).circle_domain(). `cols` lists the component's columns on that
// domain tree by tree (trace, then interaction); `coeffs` are the accumulator's powers in the order
// it hands them (reversed here, as the component does). air: 0 wide-Fibonacci, 1 Poseidon2,
// 2 Blake2s round, 3 Plonk, 4 / 5 state-machine transition of coordinate 0 / 1; `elements` as
// drawn (z, alpha pairs). Returns 0, or 1 on bad input.
int oracle_eval_constraints(uint32_t air_id, uint32_t log_n, uint32_t n_cols, const uint32_t claimed_sum[4],
                            const uint32_t* elements, uint32_t n_elements, const uint32_t* const* cols,
                            uint32_t n_cols_total, const uint32_t* coeffs, uint32_t n_coeffs, uint32_t* const acc[4]) {
  try {
    auto rel_powers = [](QM31 alpha, QM31* out, size_t n) {
      QM31 cur(M31(1));
      for (size_t i = 0; i < n; i++) {
        out[i] = cur;
        cur = cur * alpha;
      }
    };
    std::unique_ptr<Air> air;
    std::vector<size_t> tree_cols;
    BlakeAllElements all;  // outlives the Blake scheduler / XOR-table AIRs, which point into it
    auto set_rel = [&](auto& r, int k, size_t n) {
      r.z = q_of(elements + 8 * k);
      r.alpha = q_of(elements + 8 * k + 4);
      rel_powers(r.alpha, r.alpha_powers, n);
    };
    if (air_id == 0) {
      air.reset(new WideFibAir(log_n, n_cols));
      tree_cols = {0, n_cols};
    } else if (air_id == 1) {
      if (n_elements != 2) return 1;
      LookupElements le;
      le.z = q_of(elements);
      le.alpha = q_of(elements + 4);
      rel_powers(le.alpha, le.alpha_powers, PS_STATE);
      air.reset(new PoseidonAir(log_n, le, q_of(claimed_sum)));
      tree_cols = {0, PS_COLUMNS, 4 * PS_INSTANCES_PER_ROW};
    } else if (air_id == 2) {
      if (n_elements != 12) return 1;
      BlakeRoundElements el;
      auto set = [&](auto& r, int k, size_t n) {
        r.z = q_of(elements + 8 * k);
        r.alpha = q_of(elements + 8 * k + 4);
        rel_powers(r.alpha, r.alpha_powers, n);
      };
      set(el.round, 0, BR_ROUND_FELTS);
      set(el.xor_.xor12, 1, 3);
      set(el.xor_.xor9, 2, 3);
      set(el.xor_.xor8, 3, 3);
      set(el.xor_.xor7, 4, 3);
      set(el.xor_.xor4, 5, 3);
      air.reset(new BlakeRoundAir(log_n, el, q_of(claimed_sum)));
      tree_cols = {0, BR_TRACE_COLS, 4 * BR_INTERACTION_SECURE};
    } else if (air_id == 3 || air_id == 4 || air_id == 5) {
      if (n_elements != 2) return 1;
      Relation<2> r;
      r.z = q_of(elements);
      r.alpha = q_of(elements + 4);
      rel_powers(r.alpha, r.alpha_powers, 2);
      if (air_id == 3) {
        air.reset(new PlonkAir(log_n, r, q_of(claimed_sum)));
        tree_cols = {4, 4, 8};
      } else {
        air.reset(new StateTransitionAir(air_id - 4, log_n, r, q_of(claimed_sum)));
        tree_cols = {0, 2, 4};
      }
    } else if (air_id == 6) {
      // The full Blake example's scheduler: elements (Blake, Round).
      if (n_elements != 4) return 1;
      set_rel(all.blake, 0, BR_ROUND_FELTS);
      set_rel(all.round.round, 1, BR_ROUND_FELTS);
      air.reset(new BlakeSchedulerAir(log_n, &all, q_of(claimed_sum)));
      tree_cols = {0, BF_SCHED_COLS, 4 * BF_SCHED_BATCHES};
    } else if (air_id == 7) {
      // An XOR table of the full Blake example: n_cols = its element bits; elements (XorElements).
      if (n_elements != 2) return 1;
      size_t t = xor_table_index(n_cols);
      const XorTableShape& sh = BF_XOR_TABLES[t];
      Relation<3>& r = const_cast<Relation<3>&>(all.round.xor_.of(n_cols));
      set_rel(r, 0, 3);
      air.reset(new XorTableAir(sh, &r, q_of(claimed_sum)));
      tree_cols = {3, sh.n_mult_cols(), 4 * sh.n_batches()};
    } else {
      return 1;
    }
    size_t total = 0;
    for (size_t t : tree_cols) total += t;
    if (total != n_cols_total || n_coeffs != air->n_constraints()) return 1;
    const uint32_t trace_log = air->log_size(), eval_log = air->max_constraint_log_degree_bound();
    const size_t N = (size_t)1 << eval_log;
    std::vector<std::vector<Column>> own(tree_cols.size());
    std::vector<std::vector<const Column*>> tr(tree_cols.size());
    size_t k = 0;
    for (size_t t = 0; t < tree_cols.size(); t++) {
      for (size_t c = 0; c < tree_cols[t]; c++) own[t].push_back(col_of(cols[k++], N));
      for (auto& c : own[t]) tr[t].push_back(&c);
    }
    std::vector<QM31> rc;
    for (size_t i = n_coeffs; i-- > 0;) rc.push_back(q_of(coeffs + 4 * i));
    CircleDomain ed = canonic_domain(eval_log);
    Coset tc = canonic_coset(trace_log);
    std::vector<M31> dinv;
    for (size_t i = 0; i < ((size_t)1 << (eval_log - trace_log)); i++) dinv.push_back(inv(coset_vanishing(tc, ed.at(i))));
    bit_reverse(dinv);
#pragma omp parallel for schedule(static)
    for (long r = 0; r < (long)N; r++) {
      DomainEvaluator e(&tr, r, trace_log, eval_log, rc.data());
      QM31 v = air->eval_row(e) * dinv[r >> trace_log];
      QM31 a = QM31::from_u32(acc[0][r], acc[1][r], acc[2][r], acc[3][r]) + v;
      uint32_t w[4];
      q_to(a, w);
      for (int j = 0; j < 4; j++) acc[j][r] = w[j];
    }
    return 0;
  } catch (...) {
    return 1;
  }
}

// prove_fibonacci_plonk (plonk/mod.rs:153-266) with the canonical proof bytes; returns the length
// (0 on error).
size_t oracle_prove_plonk(uint32_t log_n, const uint32_t cfg[4], uint8_t* out, size_t cap, uint32_t claimed[4],
                          char* err, size_t err_cap) {
  try {
    QM31 cs;
    std::vector<uint8_t> bytes = serialize(prove_plonk(log_n, PcsConfig{cfg[0], cfg[1], cfg[2], cfg[3]}, &cs));
    q_to(cs, claimed);
    if (bytes.size() > cap) throw std::runtime_error("output buffer too small");
    std::memcpy(out, bytes.data(), bytes.size());
    return bytes.size();
  } catch (const std::exception& e) {
    snprintf(err, err_cap, "%s", e.what());
    return 0;
  }
}

// Verification of a prove_fibonacci_plonk proof (prover/mod.rs:81-127) given the claimed sum.
int oracle_verify_plonk(uint32_t log_n, const uint32_t claimed_sum[4], const uint8_t* proof, size_t len, char* err,
                        size_t err_cap) {
  try {
    StarkProof p;
    if (!deserialize(proof, len, p)) throw std::runtime_error("malformed proof bytes");
    Channel ch;
    PlonkAir air(log_n, Relation<2>{}, q_of(claimed_sum));
    auto hook = [&](size_t t, Channel& c) {
      if (t == 1) air.rel = Relation<2>::draw(c);
    };
    std::vector<uint32_t> four(4, log_n);
    std::string r = verify_components(place({&air}, {{0, 1, 2, 3}}), ch, p, {four, four, std::vector<uint32_t>(8, log_n)},
                                      hook);
    if (!r.empty()) throw std::runtime_error(r);
    return 1;
  } catch (const std::exception& e) {
    snprintf(err, err_cap, "%s", e.what());
    return 0;
  }
}

// Verification of a prove_state_machine stark proof given the two claimed sums: the statements are
// mixed where the prover mixed them (the log sizes after the empty preprocessed root, the claimed
// sums after the relation elements are drawn).
int oracle_verify_state_machine(uint32_t log_n, const uint32_t claimed[8], const uint8_t* proof, size_t len,
                                char* err, size_t err_cap) {
  try {
    StarkProof p;
    if (!deserialize(proof, len, p)) throw std::runtime_error("malformed proof bytes");
    Channel ch;
    mix_config(p.config, ch);
    const uint32_t logs[2] = {log_n, log_n - 1};
    QM31 cs[2] = {q_of(claimed), q_of(claimed + 4)};
    StateTransitionAir a0(0, logs[0], Relation<2>{}, cs[0]), a1(1, logs[1], Relation<2>{}, cs[1]);
    auto hook = [&](size_t t, Channel& c) {
      if (t == 0) {
        c.mix_u64(logs[0]);
        c.mix_u64(logs[1]);
      } else if (t == 1) {
        a0.rel = a1.rel = Relation<2>::draw(c);
        c.mix_felts({cs[0], cs[1]});
      }
    };
    std::string r = verify_components(place({&a0, &a1}, {{}, {}}), ch, p,
                                      {{}, {logs[0], logs[0], logs[1], logs[1]},
                                       {logs[0], logs[0], logs[0], logs[0], logs[1], logs[1], logs[1], logs[1]}},
                                      hook);
    if (!r.empty()) throw std::runtime_error(r);
    return 1;
  } catch (const std::exception& e) {
    snprintf(err, err_cap, "%s", e.what());
    return 0;
  }
}

// prove_state_machine (state_machine/mod.rs:26-135): the stark proof's canonical bytes and the two
// components' claimed sums.
size_t oracle_prove_state_machine(uint32_t log_n, const uint32_t initial[2], const uint32_t cfg[4], uint8_t* out,
                                  size_t cap, uint32_t claimed[8], char* err, size_t err_cap) {
  try {
    QM31 cs[2];
    std::vector<uint8_t> bytes =
        serialize(prove_state_machine(log_n, initial, PcsConfig{cfg[0], cfg[1], cfg[2], cfg[3]}, cs));
    if (bytes.size() > cap) throw std::runtime_error("output buffer too small");
    std::memcpy(out, bytes.data(), bytes.size());
    q_to(cs[0], claimed);
    q_to(cs[1], claimed + 4);
    return bytes.size();
  } catch (const std::exception& e) {
    snprintf(err, err_cap, "%s", e.what());
    return 0;
  }
}

}  // extern "C"

extern "C" {

// prove_blake (blake/air.rs:308-460) for 2^log_n instances: the stark proof's canonical bytes and
// the eight claimed sums (scheduler, round 0, round 1, XOR tables 12, 9, 8, 7, 4).
size_t oracle_prove_blake(uint32_t log_n, const uint32_t cfg[4], uint8_t* out, size_t cap, uint32_t sums[32],
                          char* err, size_t err_cap) {
  try {
    QM31 cs[8];
    std::vector<uint8_t> bytes = serialize(prove_blake(log_n, PcsConfig{cfg[0], cfg[1], cfg[2], cfg[3]}, cs));
    if (bytes.size() > cap) throw std::runtime_error("output buffer too small");
    std::memcpy(out, bytes.data(), bytes.size());
    for (int i = 0; i < 8; i++) q_to(cs[i], sums + 4 * i);
    return bytes.size();
  } catch (const std::exception& e) {
    snprintf(err, err_cap, "%s", e.what());
    return 0;
  }
}

// verify_blake (blake/air.rs:462-520) given the eight claimed sums.
int oracle_verify_blake(uint32_t log_n, const uint32_t sums[32], const uint8_t* proof, size_t len, char* err,
                        size_t err_cap) {
  try {
    StarkProof p;
    if (!deserialize(proof, len, p)) throw std::runtime_error("malformed proof bytes");
    QM31 cs[8];
    for (int i = 0; i < 8; i++) cs[i] = q_of(sums + 4 * i);
    std::string r = verify_blake(log_n, cs, p);
    if (!r.empty()) throw std::runtime_error(r);
    return 1;
  } catch (const std::exception& e) {
    snprintf(err, err_cap, "%s", e.what());
    return 0;
  }
}

// r rounds of BLAKE2s on the 16-word state v with message m (the scheduler's round function),
// in place.
void oracle_blake2s_rounds(uint32_t v[16], const uint32_t m[16], uint32_t rounds) {
  for (uint32_t r = 0; r < rounds; r++) blake2s_round_words(v, m, r);
}

// The trace tree of prove_blake (the preprocessed columns, then the trace columns), in commit order,
// written to `out` column after column; returns the number of words (0 on error or if cap is short).
size_t oracle_blake_traces(uint32_t log_n, uint32_t* out, size_t cap, uint32_t* n_cols) {
  try {
    BlakeFullTraces T = blake_full_traces(log_n);
    size_t w = 0, k = 0;
    for (const auto* tree : {&T.preprocessed, &T.trace})
      for (const Column& c : *tree) {
        if (w + c.size() > cap) return 0;
        for (const M31& x : c) out[w++] = x.v;
        k++;
      }
    *n_cols = (uint32_t)k;
    return w;
  } catch (...) {
    return 0;
  }
}

}  // extern "C"

#include "poseidon252.h"

extern "C" {

// Poseidon252: felts cross this interface as 8 little-endian u32 limbs of the canonical integer.
void oracle_p252_hash(const uint32_t x[8], const uint32_t y[8], uint32_t out[8]) {
  f252_to_words(poseidon_hash(f252_from_words(x), f252_from_words(y)), out);
}
void oracle_p252_hash_many(const uint32_t* v, size_t n, uint32_t out[8]) {
  std::vector<F252> in;
  for (size_t i = 0; i < n; i++) in.push_back(f252_from_words(v + 8 * i));
  f252_to_words(poseidon_hash_many(in), out);
}
void oracle_p252_hash_node(const uint32_t* left, const uint32_t* right, const uint32_t* vals, size_t n,
                           uint32_t out[8]) {
  F252 l, r;
  if (left) {
    l = f252_from_words(left);
    r = f252_from_words(right);
  }
  f252_to_words(p252_hash_node(left ? &l : nullptr, left ? &r : nullptr, vals, n), out);
}
// MerkleOps<Poseidon252MerkleHasher>::commit_on_layer (backend/cpu/poseidon252.rs:9-25).
void oracle_p252_commit_on_layer(uint32_t log_size, const uint32_t* prev, const uint32_t* const* cols,
                                 uint32_t n_cols, uint32_t* out) {
  const size_t n = (size_t)1 << log_size;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < (long)n; i++) {
    std::vector<uint32_t> vals(n_cols);
    for (uint32_t c = 0; c < n_cols; c++) vals[c] = cols[c][i];
    F252 l, r;
    if (prev) {
      l = f252_from_words(prev + 16 * i);
      r = f252_from_words(prev + 16 * i + 8);
    }
    f252_to_words(p252_hash_node(prev ? &l : nullptr, prev ? &r : nullptr, vals.data(), n_cols), out + 8 * i);
  }
}
uint64_t oracle_p252_grind(const uint32_t digest[8], uint32_t pow_bits) {
  Poseidon252Channel ch;
  ch.digest = f252_from_words(digest);
  return p252_grind(ch, pow_bits);
}
uint32_t oracle_p252_trailing_zeros(const uint32_t digest[8]) {
  Poseidon252Channel ch;
  ch.digest = f252_from_words(digest);
  return ch.trailing_zeros();
}
// A channel script: from `digest`, mix `n_felts` QM31 values (if any), then draw `n_draw` felts;
// writes the draws and the final digest.
void oracle_p252_channel(const uint32_t digest[8], const uint32_t* felts, size_t n_felts, size_t n_draw,
                         uint32_t* draws, uint32_t digest_out[8]) {
  Poseidon252Channel ch;
  ch.digest = f252_from_words(digest);
  if (n_felts) {
    std::vector<QM31> f;
    for (size_t i = 0; i < n_felts; i++) f.push_back(q_of(felts + 4 * i));
    ch.mix_felts(f);
  }
  auto d = ch.draw_felts(n_draw);
  for (size_t i = 0; i < d.size(); i++) q_to(d[i], draws + 4 * i);
  f252_to_words(ch.digest, digest_out);
}

}  // extern "C"
