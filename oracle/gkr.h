// ORACLE — test infrastructure only (see field.h).
// GKR batch prover and verifier for grand-product and LogUp circuits, together with the backend
// operations beneath them, restated from the reference:
//   GkrOps, EqEvals, Layer          crates/prover/src/core/lookups/gkr_prover.rs:22-260
//   GkrMultivariatePolyOracle       crates/prover/src/core/lookups/gkr_prover.rs:272-372
//   prove_batch, gen_layers         crates/prover/src/core/lookups/gkr_prover.rs:401-516
//   correct_sum_as_poly_in_first_variable  crates/prover/src/core/lookups/gkr_prover.rs:527-566
//   sum-check                       crates/prover/src/core/lookups/sumcheck.rs:62-160
//   partially_verify_batch, GkrMask crates/prover/src/core/lookups/gkr_verifier.rs:17-246
//   eq, UnivariatePoly, Fraction    crates/prover/src/core/lookups/utils.rs:12-286
//   CPU backend operations          crates/prover/src/core/backend/cpu/lookups/gkr.rs:16-265,
//                                   crates/prover/src/core/backend/cpu/lookups/mle.rs:11-45
// Mle columns hold evaluations over the boolean hypercube with the first variable as the most
// significant index bit (mle.rs:16-19), so fixing the first variable folds the two halves.
// The reference serialises GkrBatchProof with serde only; the byte format here (u32 words, u64
// lengths, fields in struct order) is this project's own, applied identically to oracle and GPU.
#pragma once
#include "protocol.h"
#include <array>

namespace oracle {

enum GkrKind : uint32_t {
  GKR_GRAND_PRODUCT = 0,
  GKR_LOGUP_GENERIC = 1,
  GKR_LOGUP_MULTIPLICITIES = 2,
  GKR_LOGUP_SINGLES = 3,
};

inline QM31 q_one() { return QM31(M31(1)); }
inline QM31 q_two() { return QM31(M31(2)); }

// utils.rs:160-167: lagrange kernel of the boolean hypercube.
inline QM31 eq_eval(const std::vector<QM31>& x, const std::vector<QM31>& y) {
  if (x.size() != y.size()) throw std::runtime_error("eq: length mismatch");
  QM31 r = q_one();
  for (size_t i = 0; i < x.size(); i++) r = r * (x[i] * y[i] + (q_one() - x[i]) * (q_one() - y[i]));
  return r;
}

// utils.rs:170-176: eq(0, a) * e0 + eq(1, a) * e1.
inline QM31 fold_mle_evals(QM31 a, QM31 e0, QM31 e1) { return a * (e1 - e0) + e0; }

// ------------------------------------------------------------ univariate polynomials (utils.rs:12-150)
using UPoly = std::vector<QM31>;  // monomial coefficients, constant first

inline void upoly_trunc(UPoly& p) {
  while (!p.empty() && p.back().is_zero()) p.pop_back();
}
inline UPoly upoly_new(UPoly p) {
  upoly_trunc(p);
  return p;
}
inline QM31 upoly_eval(const UPoly& p, QM31 x) {
  QM31 acc;
  for (size_t i = p.size(); i-- > 0;) acc = acc * x + p[i];
  return acc;
}
// Degree as the reference reports it: length - 1, saturating (utils.rs:51-55).
inline size_t upoly_degree(const UPoly& p) { return p.empty() ? 0 : p.size() - 1; }
inline bool upoly_is_zero(const UPoly& p) {
  for (auto& c : p)
    if (!c.is_zero()) return false;
  return true;
}
// Sum keeps the longer length (no truncation), as Add does.
inline UPoly upoly_add(const UPoly& a, const UPoly& b) {
  UPoly r(std::max(a.size(), b.size()));
  for (size_t i = 0; i < r.size(); i++) {
    if (i < a.size() && i < b.size()) r[i] = a[i] + b[i];
    else r[i] = i < a.size() ? a[i] : b[i];
  }
  return r;
}
inline UPoly upoly_scale(UPoly a, QM31 s) {
  for (auto& c : a) c = c * s;
  return a;
}
inline UPoly upoly_mul(UPoly a, UPoly b) {
  if (upoly_is_zero(a) || upoly_is_zero(b)) return {};
  upoly_trunc(a);
  upoly_trunc(b);
  UPoly r(a.size() + b.size() - 1);
  for (size_t i = 0; i < a.size(); i++)
    for (size_t j = 0; j < b.size(); j++) r[i + j] = r[i + j] + a[i] * b[j];
  return upoly_new(r);
}
// utils.rs:24-49.
inline UPoly interpolate_lagrange(const std::vector<QM31>& xs, const std::vector<QM31>& ys) {
  if (xs.size() != ys.size()) throw std::runtime_error("interpolate_lagrange: length mismatch");
  UPoly acc;
  for (size_t i = 0; i < xs.size(); i++) {
    QM31 prod = ys[i];
    for (size_t j = 0; j < xs.size(); j++)
      if (i != j) prod = prod * inv(xs[i] - xs[j]);
    UPoly term = upoly_new({prod});
    for (size_t j = 0; j < xs.size(); j++) {
      if (i == j) continue;
      UPoly lin = upoly_add({QM31(), q_one()}, upoly_scale(upoly_new({xs[j]}), -q_one()));
      term = upoly_mul(term, lin);
    }
    acc = upoly_add(acc, term);
  }
  upoly_trunc(acc);
  return acc;
}
// sumcheck.rs:128-135: p_0 + alpha p_1 + ... folded from the last polynomial.
inline UPoly upoly_rlc(const std::vector<UPoly>& ps, QM31 alpha) {
  UPoly acc;
  for (size_t i = ps.size(); i-- > 0;) acc = upoly_add(upoly_scale(acc, alpha), ps[i]);
  return acc;
}
// utils.rs:154-157.
inline QM31 rlc(const std::vector<QM31>& v, QM31 alpha) { return upoly_eval(v, alpha); }

// ------------------------------------------------------------ backend operations
// cpu/lookups/gkr.rs:214-230: eq(x, y) * v for x in {0,1}^|y|, first variable most significant.
inline std::vector<QM31> gen_eq_evals(const std::vector<QM31>& y, QM31 v) {
  std::vector<QM31> e{v};
  e.reserve(size_t(1) << y.size());
  for (size_t k = y.size(); k-- > 0;) {
    size_t n = e.size();
    e.resize(2 * n);
#pragma omp parallel for if (n >= 4096)
    for (size_t j = 0; j < n; j++) {
      QM31 t = e[j] * y[k];
      e[n + j] = t;
      e[j] = e[j] - t;
    }
  }
  return e;
}

// cpu/lookups/mle.rs:11-40: fix the first variable of a base or secure column.
inline std::vector<QM31> fix_first_variable(const std::vector<QM31>& m, QM31 a) {
  size_t h = m.size() / 2;
  std::vector<QM31> r(h);
#pragma omp parallel for if (h >= 4096)
  for (size_t i = 0; i < h; i++) r[i] = fold_mle_evals(a, m[i], m[i + h]);
  return r;
}
inline std::vector<QM31> fix_first_variable(const std::vector<M31>& m, QM31 a) {
  size_t h = m.size() / 2;
  std::vector<QM31> r(h);
#pragma omp parallel for if (h >= 4096)
  for (size_t i = 0; i < h; i++) r[i] = fold_mle_evals(a, QM31(m[i]), QM31(m[i + h]));
  return r;
}

// gkr_prover.rs:94-108: one layer of a binary-tree circuit. `num` holds the grand-product column
// or the secure numerators, `num_base` the base-field multiplicities; singles have no numerators.
struct GkrLayer {
  GkrKind kind = GKR_GRAND_PRODUCT;
  std::vector<QM31> num;
  std::vector<M31> num_base;
  std::vector<QM31> den;
  size_t len() const { return kind == GKR_GRAND_PRODUCT ? num.size() : den.size(); }
  size_t n_variables() const {
    size_t n = len(), l = 0;
    while ((size_t(1) << l) < n) l++;
    return l;
  }
  QM31 numer(size_t i) const {
    if (kind == GKR_LOGUP_SINGLES) return q_one();
    if (kind == GKR_LOGUP_MULTIPLICITIES) return QM31(num_base[i]);
    return num[i];
  }
};

// cpu/lookups/gkr.rs:232-262 and utils.rs:190-205: pairwise products or fraction sums.
inline GkrLayer next_layer(const GkrLayer& l) {
  GkrLayer r;
  size_t h = l.len() / 2;
  if (l.kind == GKR_GRAND_PRODUCT) {
    r.kind = GKR_GRAND_PRODUCT;
    r.num.resize(h);
#pragma omp parallel for if (h >= 4096)
    for (size_t i = 0; i < h; i++) r.num[i] = l.num[2 * i] * l.num[2 * i + 1];
    return r;
  }
  r.kind = GKR_LOGUP_GENERIC;
  r.num.resize(h);
  r.den.resize(h);
#pragma omp parallel for if (h >= 4096)
  for (size_t i = 0; i < h; i++) {
    QM31 n0 = l.numer(2 * i), n1 = l.numer(2 * i + 1), d0 = l.den[2 * i], d1 = l.den[2 * i + 1];
    r.num[i] = d1 * n0 + d0 * n1;
    r.den[i] = d0 * d1;
  }
  return r;
}

// gkr_prover.rs:167-195.
inline GkrLayer layer_fix_first_variable(const GkrLayer& l, QM31 x0) {
  if (l.n_variables() == 0) return l;
  GkrLayer r;
  switch (l.kind) {
    case GKR_GRAND_PRODUCT:
      r.kind = GKR_GRAND_PRODUCT;
      r.num = fix_first_variable(l.num, x0);
      break;
    case GKR_LOGUP_GENERIC:
      r.kind = GKR_LOGUP_GENERIC;
      r.num = fix_first_variable(l.num, x0);
      r.den = fix_first_variable(l.den, x0);
      break;
    case GKR_LOGUP_MULTIPLICITIES:
      r.kind = GKR_LOGUP_GENERIC;
      r.num = fix_first_variable(l.num_base, x0);
      r.den = fix_first_variable(l.den, x0);
      break;
    case GKR_LOGUP_SINGLES:
      r.kind = GKR_LOGUP_SINGLES;
      r.den = fix_first_variable(l.den, x0);
      break;
  }
  return r;
}

// gkr_prover.rs:137-164.
inline std::vector<QM31> output_layer_values(const GkrLayer& l) {
  if (l.n_variables() != 0) throw std::runtime_error("not an output layer");
  if (l.kind == GKR_GRAND_PRODUCT) return {l.num[0]};
  return {l.numer(0), l.den[0]};
}

// gkr_prover.rs:52-73.
struct EqEvals {
  std::vector<QM31> y;
  std::vector<QM31> evals;
  static EqEvals generate(const std::vector<QM31>& y) {
    EqEvals e;
    e.y = y;
    if (y.empty()) {
      e.evals = {q_one()};
      return e;
    }
    std::vector<QM31> rest(y.begin() + 1, y.end());
    e.evals = gen_eq_evals(rest, eq_eval({QM31()}, {y[0]}));
    return e;
  }
};

// gkr_prover.rs:527-566.
inline UPoly correct_sum_as_poly_in_first_variable(QM31 f0, QM31 f2, QM31 claim, const std::vector<QM31>& y,
                                                   size_t k) {
  size_t n = y.size();
  if (k == 0 || k > n) throw std::runtime_error("correct_sum: bad k");
  std::vector<QM31> zeros(n - k + 1), head(y.begin(), y.begin() + (n - k + 1));
  QM31 a = inv(eq_eval(zeros, head));
  QM31 yk = y[n - k];
  QM31 b = (q_one() - yk) * inv(q_one() - (yk + yk));
  QM31 r0 = f0 * eq_eval({QM31()}, {yk}) * a;
  QM31 r1 = claim - r0;
  QM31 r2 = f2 * eq_eval({q_two()}, {yk}) * a;
  return interpolate_lagrange({QM31(), q_one(), q_two(), b}, {r0, r1, r2, QM31()});
}

// cpu/lookups/gkr.rs:38-212: (f(0), f(2)) of sum_x eq((0, x), y) * P(t, x) before correction.
inline std::pair<QM31, QM31> gkr_eval_sums(const std::vector<QM31>& eq_evals, const GkrLayer& l, QM31 lambda) {
  size_t n_terms = l.len() / 4;
  QM31 e0, e2;
  // Field sums are exact, so any split across threads gives the same result.
#pragma omp parallel if (n_terms >= 4096)
  {
  QM31 s0, s2;
#pragma omp for nowait
  for (size_t i = 0; i < n_terms; i++) {
    size_t a0 = 2 * i, a1 = 2 * i + 1, b0 = 2 * (n_terms + i), b1 = 2 * (n_terms + i) + 1;
    QM31 eqv = eq_evals[i];
    if (l.kind == GKR_GRAND_PRODUCT) {
      QM31 r2a = l.num[b0] + l.num[b0] - l.num[a0];
      QM31 r2b = l.num[b1] + l.num[b1] - l.num[a1];
      s0 = s0 + eqv * (l.num[a0] * l.num[a1]);
      s2 = s2 + eqv * (r2a * r2b);
      continue;
    }
    QM31 n00 = l.numer(a0), n01 = l.numer(a1), n10 = l.numer(b0), n11 = l.numer(b1);
    QM31 d00 = l.den[a0], d01 = l.den[a1], d10 = l.den[b0], d11 = l.den[b1];
    QM31 n20 = n10 + n10 - n00, n21 = n11 + n11 - n01;
    QM31 d20 = d10 + d10 - d00, d21 = d11 + d11 - d01;
    QM31 num0 = d01 * n00 + d00 * n01, den0 = d00 * d01;
    QM31 num2 = d21 * n20 + d20 * n21, den2 = d20 * d21;
    s0 = s0 + eqv * (num0 + lambda * den0);
    s2 = s2 + eqv * (num2 + lambda * den2);
  }
#pragma omp critical
  {
    e0 = e0 + s0;
    e2 = e2 + s2;
  }
  }
  return {e0, e2};
}

// gkr_prover.rs:285-372: the sum-check oracle of one layer.
struct GkrPolyOracle {
  const EqEvals* eq = nullptr;
  GkrLayer layer;
  QM31 correction = q_one();
  QM31 lambda;
  size_t n_variables() const { return layer.n_variables() - 1; }
  UPoly sum_as_poly_in_first_variable(QM31 claim) const {
    size_t k = n_variables();
    if (k == 0) throw std::runtime_error("sum_as_poly on a constant oracle");
    auto [e0, e2] = gkr_eval_sums(eq->evals, layer, lambda);
    return correct_sum_as_poly_in_first_variable(e0 * correction, e2 * correction, claim, eq->y, k);
  }
  GkrPolyOracle fix_first_variable(QM31 c) const {
    if (n_variables() == 0) return *this;
    GkrPolyOracle r = *this;
    QM31 z0 = eq->y[eq->y.size() - n_variables()];
    r.correction = correction * eq_eval({c}, {z0});
    r.layer = layer_fix_first_variable(layer, c);
    return r;
  }
};

// gkr_verifier.rs:215-241.
struct GkrMask {
  std::vector<std::array<QM31, 2>> columns;
  std::vector<QM31> reduce_at_point(QM31 x) const {
    std::vector<QM31> r;
    for (auto& c : columns) r.push_back(fold_mle_evals(x, c[0], c[1]));
    return r;
  }
};

// gkr_prover.rs:320-346.
inline GkrMask try_into_mask(const GkrPolyOracle& o) {
  if (o.n_variables() != 0) throw std::runtime_error("polynomial is not constant");
  const GkrLayer& l = o.layer;
  GkrMask m;
  switch (l.kind) {
    case GKR_GRAND_PRODUCT: m.columns.push_back({l.num[0], l.num[1]}); break;
    case GKR_LOGUP_GENERIC:
      m.columns.push_back({l.num[0], l.num[1]});
      m.columns.push_back({l.den[0], l.den[1]});
      break;
    case GKR_LOGUP_SINGLES:
      m.columns.push_back({q_one(), q_one()});
      m.columns.push_back({l.den[0], l.den[1]});
      break;
    default: throw std::runtime_error("multiplicities layer as a mask");
  }
  return m;
}

struct SumcheckProof {
  std::vector<UPoly> round_polys;
};

// sumcheck.rs:62-126.
struct SumcheckResult {
  SumcheckProof proof;
  std::vector<QM31> assignment;
  std::vector<GkrPolyOracle> oracles;
  std::vector<QM31> claims;
};
inline SumcheckResult sumcheck_prove_batch(std::vector<QM31> claims, std::vector<GkrPolyOracle> polys, QM31 lambda,
                                           Channel& ch) {
  size_t n_vars = 0;
  for (auto& p : polys) n_vars = std::max(n_vars, p.n_variables());
  if (claims.size() != polys.size()) throw std::runtime_error("sumcheck: claims / polys mismatch");
  for (size_t i = 0; i < polys.size(); i++) claims[i] = claims[i] * M31(1u << (n_vars - polys[i].n_variables()));
  SumcheckResult res;
  const QM31 half = QM31(inv(M31(2)));
  for (size_t round = 0; round < n_vars; round++) {
    size_t remaining = n_vars - round;
    std::vector<UPoly> this_round;
    for (size_t i = 0; i < polys.size(); i++) {
      UPoly rp = remaining == polys[i].n_variables() ? polys[i].sum_as_poly_in_first_variable(claims[i])
                                                      : upoly_new({claims[i] * half});
      if (upoly_eval(rp, QM31()) + upoly_eval(rp, q_one()) != claims[i])
        throw std::runtime_error("sumcheck: round polynomial inconsistent with its claim");
      if (upoly_degree(rp) > 3) throw std::runtime_error("sumcheck: round polynomial degree too high");
      this_round.push_back(rp);
    }
    UPoly rp = upoly_rlc(this_round, lambda);
    ch.mix_felts(rp);
    QM31 c = ch.draw_felt();
    for (size_t i = 0; i < polys.size(); i++) {
      claims[i] = upoly_eval(this_round[i], c);
      if (remaining == polys[i].n_variables()) polys[i] = polys[i].fix_first_variable(c);
    }
    res.proof.round_polys.push_back(rp);
    res.assignment.push_back(c);
  }
  res.oracles = std::move(polys);
  res.claims = std::move(claims);
  return res;
}

// sumcheck.rs:137-160.
inline std::string sumcheck_partially_verify(QM31 claim, const SumcheckProof& p, Channel& ch,
                                             std::vector<QM31>& assignment, QM31& eval) {
  assignment.clear();
  for (size_t r = 0; r < p.round_polys.size(); r++) {
    const UPoly& rp = p.round_polys[r];
    if (upoly_degree(rp) > 3) return "sum-check degree invalid in round " + std::to_string(r);
    if (upoly_eval(rp, QM31()) + upoly_eval(rp, q_one()) != claim)
      return "sum-check sum invalid in round " + std::to_string(r);
    ch.mix_felts(rp);
    QM31 c = ch.draw_felt();
    claim = upoly_eval(rp, c);
    assignment.push_back(c);
  }
  eval = claim;
  return "";
}

struct GkrBatchProof {
  std::vector<SumcheckProof> sumcheck_proofs;
  std::vector<std::vector<GkrMask>> layer_masks_by_instance;
  std::vector<std::vector<QM31>> output_claims_by_instance;
};
struct GkrArtifact {
  std::vector<QM31> ood_point;
  std::vector<std::vector<QM31>> claims_to_verify_by_instance;
  std::vector<uint64_t> n_variables_by_instance;
};

// gkr_prover.rs:401-516.
inline std::pair<GkrBatchProof, GkrArtifact> gkr_prove_batch(Channel& ch, const std::vector<GkrLayer>& inputs) {
  size_t n_inst = inputs.size();
  std::vector<size_t> n_layers_by(n_inst);
  size_t n_layers = 0;
  std::vector<std::vector<GkrLayer>> layers(n_inst);  // output layer first
  for (size_t i = 0; i < n_inst; i++) {
    n_layers_by[i] = inputs[i].n_variables();
    n_layers = std::max(n_layers, n_layers_by[i]);
    layers[i].push_back(inputs[i]);
    while (layers[i].back().n_variables() > 0) layers[i].push_back(next_layer(layers[i].back()));
    std::reverse(layers[i].begin(), layers[i].end());
  }
  std::vector<size_t> cursor(n_inst, 0);
  GkrBatchProof proof;
  proof.layer_masks_by_instance.resize(n_inst);
  proof.output_claims_by_instance.resize(n_inst);
  std::vector<bool> active(n_inst, false);
  std::vector<std::vector<QM31>> claims_to_verify(n_inst);
  std::vector<QM31> ood_point;
  for (size_t layer = 0; layer < n_layers; layer++) {
    size_t remaining = n_layers - layer;
    for (size_t i = 0; i < n_inst; i++) {
      if (n_layers_by[i] == remaining) {
        std::vector<QM31> out = output_layer_values(layers[i][cursor[i]++]);
        claims_to_verify[i] = out;
        proof.output_claims_by_instance[i] = out;
        active[i] = true;
      }
    }
    for (size_t i = 0; i < n_inst; i++)
      if (active[i]) ch.mix_felts(claims_to_verify[i]);
    EqEvals eq = EqEvals::generate(ood_point);
    QM31 alpha = ch.draw_felt();
    QM31 lambda = ch.draw_felt();
    std::vector<GkrPolyOracle> oracles;
    std::vector<QM31> claims;
    std::vector<size_t> insts;
    for (size_t i = 0; i < n_inst; i++) {
      if (!active[i]) continue;
      GkrPolyOracle o;
      o.eq = &eq;
      o.layer = layers[i][cursor[i]++];
      o.lambda = lambda;
      oracles.push_back(std::move(o));
      claims.push_back(rlc(claims_to_verify[i], lambda));
      insts.push_back(i);
    }
    SumcheckResult sc = sumcheck_prove_batch(claims, std::move(oracles), alpha, ch);
    proof.sumcheck_proofs.push_back(sc.proof);
    std::vector<GkrMask> masks;
    for (auto& o : sc.oracles) masks.push_back(try_into_mask(o));
    for (size_t j = 0; j < insts.size(); j++) {
      std::vector<QM31> flat;
      for (auto& c : masks[j].columns) {
        flat.push_back(c[0]);
        flat.push_back(c[1]);
      }
      ch.mix_felts(flat);
      proof.layer_masks_by_instance[insts[j]].push_back(masks[j]);
    }
    QM31 challenge = ch.draw_felt();
    ood_point = sc.assignment;
    ood_point.push_back(challenge);
    for (size_t j = 0; j < insts.size(); j++) claims_to_verify[insts[j]] = masks[j].reduce_at_point(challenge);
  }
  GkrArtifact art;
  art.ood_point = ood_point;
  art.claims_to_verify_by_instance = claims_to_verify;
  for (auto n : n_layers_by) art.n_variables_by_instance.push_back(n);
  return {proof, art};
}

enum GkrGate : uint32_t { GATE_LOGUP = 0, GATE_GRAND_PRODUCT = 1 };

// gkr_verifier.rs:17-175. Returns "" and fills `art` on success, the failure otherwise.
inline std::string gkr_partially_verify_batch(const std::vector<GkrGate>& gates, const GkrBatchProof& proof,
                                              Channel& ch, GkrArtifact& art) {
  size_t n_inst = proof.layer_masks_by_instance.size();
  if (n_inst != proof.output_claims_by_instance.size() || n_inst == 0) return "malformed proof";
  size_t n_layers = 0;
  for (auto& m : proof.layer_masks_by_instance) n_layers = std::max(n_layers, m.size());
  if (n_layers != proof.sumcheck_proofs.size()) return "malformed proof";
  if (gates.size() != n_inst) return "instance count mismatch";
  auto inst_layers = [&](size_t i) { return proof.layer_masks_by_instance[i].size(); };
  std::vector<QM31> ood_point;
  std::vector<bool> active(n_inst, false);
  std::vector<std::vector<QM31>> claims_to_verify(n_inst);
  for (size_t layer = 0; layer < n_layers; layer++) {
    size_t remaining = n_layers - layer;
    for (size_t i = 0; i < n_inst; i++)
      if (inst_layers(i) == remaining) {
        claims_to_verify[i] = proof.output_claims_by_instance[i];
        active[i] = true;
      }
    for (size_t i = 0; i < n_inst; i++)
      if (active[i]) ch.mix_felts(claims_to_verify[i]);
    QM31 alpha = ch.draw_felt();
    QM31 lambda = ch.draw_felt();
    std::vector<QM31> sc_claims;
    std::vector<size_t> insts;
    for (size_t i = 0; i < n_inst; i++) {
      if (!active[i]) continue;
      size_t unused = n_layers - inst_layers(i);
      sc_claims.push_back(rlc(claims_to_verify[i], lambda) * M31(1u << unused));
      insts.push_back(i);
    }
    QM31 sc_claim = rlc(sc_claims, alpha);
    std::vector<QM31> sc_point;
    QM31 sc_eval;
    std::string e = sumcheck_partially_verify(sc_claim, proof.sumcheck_proofs[layer], ch, sc_point, sc_eval);
    if (!e.empty()) return "layer " + std::to_string(layer) + ": " + e;
    std::vector<QM31> layer_evals;
    for (size_t i : insts) {
      size_t unused = n_layers - inst_layers(i);
      const GkrMask& m = proof.layer_masks_by_instance[i][layer - unused];
      std::vector<QM31> out;
      if (gates[i] == GATE_LOGUP) {
        if (m.columns.size() != 2) return "invalid mask";
        QM31 na = m.columns[0][0], nb = m.columns[0][1], da = m.columns[1][0], db = m.columns[1][1];
        out = {db * na + da * nb, da * db};
      } else {
        if (m.columns.size() != 1) return "invalid mask";
        out = {m.columns[0][0] * m.columns[0][1]};
      }
      std::vector<QM31> a(ood_point.begin() + unused, ood_point.end()), b(sc_point.begin() + unused, sc_point.end());
      layer_evals.push_back(eq_eval(a, b) * rlc(out, lambda));
    }
    if (sc_eval != rlc(layer_evals, alpha)) return "circuit check failed in layer " + std::to_string(layer);
    for (size_t i : insts) {
      size_t unused = n_layers - inst_layers(i);
      const GkrMask& m = proof.layer_masks_by_instance[i][layer - unused];
      std::vector<QM31> flat;
      for (auto& c : m.columns) {
        flat.push_back(c[0]);
        flat.push_back(c[1]);
      }
      ch.mix_felts(flat);
    }
    QM31 challenge = ch.draw_felt();
    ood_point = sc_point;
    ood_point.push_back(challenge);
    for (size_t i : insts) {
      size_t unused = n_layers - inst_layers(i);
      claims_to_verify[i] = proof.layer_masks_by_instance[i][layer - unused].reduce_at_point(challenge);
    }
  }
  art.ood_point = ood_point;
  art.claims_to_verify_by_instance = claims_to_verify;
  art.n_variables_by_instance.clear();
  for (size_t i = 0; i < n_inst; i++) art.n_variables_by_instance.push_back(inst_layers(i));
  return "";
}

// mle.rs:84-101 (test helper): multilinear evaluation at a point, first variable first.
inline QM31 mle_eval_at_point(std::vector<QM31> e, const std::vector<QM31>& p) {
  for (auto& x : p) e = fix_first_variable(e, x);
  return e.at(0);
}

// ------------------------------------------------------------ canonical bytes
inline void write_gkr(Writer& w, const GkrBatchProof& p, const GkrArtifact& a) {
  w.u64(p.sumcheck_proofs.size());
  for (auto& s : p.sumcheck_proofs) {
    w.u64(s.round_polys.size());
    for (auto& rp : s.round_polys) w.qs(rp);
  }
  w.u64(p.layer_masks_by_instance.size());
  for (auto& ms : p.layer_masks_by_instance) {
    w.u64(ms.size());
    for (auto& m : ms) {
      w.u64(m.columns.size());
      for (auto& c : m.columns) {
        w.q(c[0]);
        w.q(c[1]);
      }
    }
  }
  w.u64(p.output_claims_by_instance.size());
  for (auto& c : p.output_claims_by_instance) w.qs(c);
  // The artifact follows the proof: the verifier recomputes it, so a reader can compare.
  w.qs(a.ood_point);
  w.u64(a.claims_to_verify_by_instance.size());
  for (auto& c : a.claims_to_verify_by_instance) w.qs(c);
  w.u64(a.n_variables_by_instance.size());
  for (auto n : a.n_variables_by_instance) w.u64(n);
}

inline bool read_gkr(const uint8_t* data, size_t n, GkrBatchProof& p, GkrArtifact& a) {
  Reader r{data, n};
  uint64_t ns = r.len();
  for (uint64_t i = 0; i < ns && r.ok; i++) {
    SumcheckProof s;
    uint64_t nr = r.len();
    for (uint64_t j = 0; j < nr && r.ok; j++) s.round_polys.push_back(r.qs());
    p.sumcheck_proofs.push_back(s);
  }
  uint64_t ni = r.len();
  for (uint64_t i = 0; i < ni && r.ok; i++) {
    std::vector<GkrMask> ms;
    uint64_t nm = r.len();
    for (uint64_t j = 0; j < nm && r.ok; j++) {
      GkrMask m;
      uint64_t nc = r.len();
      for (uint64_t c = 0; c < nc && r.ok; c++) {
        QM31 x = r.q(), y = r.q();
        m.columns.push_back({x, y});
      }
      ms.push_back(m);
    }
    p.layer_masks_by_instance.push_back(ms);
  }
  uint64_t no = r.len();
  for (uint64_t i = 0; i < no && r.ok; i++) p.output_claims_by_instance.push_back(r.qs());
  a.ood_point = r.qs();
  uint64_t nc = r.len();
  for (uint64_t i = 0; i < nc && r.ok; i++) a.claims_to_verify_by_instance.push_back(r.qs());
  uint64_t nv = r.len();
  for (uint64_t i = 0; i < nv && r.ok; i++) a.n_variables_by_instance.push_back(r.u64());
  return r.ok && r.i == r.n;
}

}  // namespace oracle
