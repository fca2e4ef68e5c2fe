// ORACLE — test infrastructure only (see field.h).
// AIR components, the composition polynomial, prove() and verify(), restated from the reference:
//   FrameworkComponent  crates/prover/src/constraint_framework/component.rs:126-416
//   evaluators          constraint_framework/cpu_domain.rs:17-100, point.rs:15-70
//   accumulators        crates/prover/src/core/air/accumulation.rs:20-149
//   prove / verify      crates/prover/src/core/prover/mod.rs:27-127
//   PCS verifier        crates/prover/src/core/pcs/verifier.rs:13-120, pcs/quotients.rs:103-165
//   FRI verifier        crates/prover/src/core/fri.rs:338-590, :767-1100
#pragma once
#include "protocol.h"

namespace oracle {

using Mask = std::vector<std::vector<std::vector<int>>>;                 // [tree][col] -> offsets
using MaskValues = std::vector<std::vector<std::vector<QM31>>>;          // [tree][col][offset]

// Evaluates constraints at one row of the evaluation domain (CpuDomainEvaluator).
struct DomainEvaluator {
  using F = M31;
  using EF = QM31;
  const std::vector<std::vector<const Column*>>* trace;  // [tree][col], on the eval domain
  size_t row;
  uint32_t trace_log, eval_log;
  const QM31* coeffs;
  QM31 row_res = QM31();
  size_t ci = 0;
  std::vector<size_t> col;
  DomainEvaluator(const std::vector<std::vector<const Column*>>* t, size_t r, uint32_t tl, uint32_t el,
                  const QM31* c)
      : trace(t), row(r), trace_log(tl), eval_log(el), coeffs(c), col(t->size(), 0) {}
  std::vector<M31> next_interaction_mask(size_t tree, const std::vector<int>& offsets) {
    const Column* c = (*trace)[tree][col[tree]++];
    std::vector<M31> out;
    for (int off : offsets) {
      size_t r = off == 0 ? row : offset_bit_reversed_circle_domain_index(row, trace_log, eval_log, off);
      out.push_back((*c)[r]);
    }
    return out;
  }
  M31 next_trace_mask() { return next_interaction_mask(1, {0})[0]; }
  // Four consecutive columns combined into QM31 values (EvalAtRow::next_extension_interaction_mask).
  std::vector<QM31> next_extension_interaction_mask(size_t tree, const std::vector<int>& offsets) {
    std::vector<M31> c[4];
    for (int k = 0; k < 4; k++) c[k] = next_interaction_mask(tree, offsets);
    std::vector<QM31> out;
    for (size_t j = 0; j < offsets.size(); j++) {
      M31 v[4] = {c[0][j], c[1][j], c[2][j], c[3][j]};
      out.push_back(combine_ef(v));
    }
    return out;
  }
  template <class G>
  void add_constraint(const G& c) { row_res = row_res + coeffs[ci++] * c; }
  static QM31 combine_ef(const M31 v[4]) { return QM31::from_m31(v[0], v[1], v[2], v[3]); }
};

// PointEvaluator: accumulates denom_inverse * constraint into acc = acc * rc + value.
struct PointEvaluator {
  using F = QM31;
  using EF = QM31;
  const MaskValues* mask;
  QM31* acc;
  QM31 rc, denom_inv;
  std::vector<size_t> col;
  PointEvaluator(const MaskValues* m, QM31* a, QM31 r, QM31 d) : mask(m), acc(a), rc(r), denom_inv(d), col(m->size(), 0) {}
  std::vector<QM31> next_interaction_mask(size_t tree, const std::vector<int>& offsets) {
    const std::vector<QM31>& v = (*mask)[tree][col[tree]++];
    if (v.size() != offsets.size()) throw std::runtime_error("mask size mismatch");
    return v;
  }
  QM31 next_trace_mask() { return next_interaction_mask(1, {0})[0]; }
  std::vector<QM31> next_extension_interaction_mask(size_t tree, const std::vector<int>& offsets) {
    std::vector<QM31> c[4];
    for (int k = 0; k < 4; k++) c[k] = next_interaction_mask(tree, offsets);
    std::vector<QM31> out;
    for (size_t j = 0; j < offsets.size(); j++) {
      QM31 v[4] = {c[0][j], c[1][j], c[2][j], c[3][j]};
      out.push_back(combine_ef(v));
    }
    return out;
  }
  void add_constraint(const QM31& c) { *acc = *acc * rc + denom_inv * c; }
  static QM31 combine_ef(const QM31 v[4]) {
    // QM31::from_partial_evals (fields/qm31.rs:52-58)
    return v[0] + v[1] * QM31::from_u32(0, 1, 0, 0) + v[2] * QM31::from_u32(0, 0, 1, 0) +
           v[3] * QM31::from_u32(0, 0, 0, 1);
  }
};

// A single FrameworkComponent-like AIR over one log size.
struct Air {
  virtual ~Air() {}
  virtual uint32_t log_size() const = 0;
  virtual uint32_t max_constraint_log_degree_bound() const = 0;
  virtual size_t n_constraints() const = 0;
  virtual Mask mask_offsets() const = 0;
  virtual QM31 eval_row(DomainEvaluator& e) const = 0;
  virtual void eval_point(PointEvaluator& e) const = 0;
};

inline CirclePointQM31 pt_add_q(const CirclePointQM31& a, const CirclePointM31& b) {
  CirclePointQM31 bq = to_qm31(b);
  return pt_add(a, bq);
}

// FrameworkComponent::mask_points (component.rs:236-249): point + trace_step * offset.
inline std::vector<std::vector<std::vector<CirclePointQM31>>> mask_points(const Air& air, CirclePointQM31 p) {
  Mask m = air.mask_offsets();
  uint32_t step = subgroup_gen(air.log_size());
  std::vector<std::vector<std::vector<CirclePointQM31>>> out(m.size());
  for (size_t t = 0; t < m.size(); t++)
    for (auto& offs : m[t]) {
      std::vector<CirclePointQM31> pts;
      for (int off : offs) {
        uint32_t idx = idx_reduce((uint64_t)step * (uint64_t)(off >= 0 ? off : -off));
        if (off < 0) idx = idx_reduce((1ull << 31) - idx);
        pts.push_back(pt_add_q(p, index_to_point(idx)));
      }
      out[t].push_back(pts);
    }
  return out;
}

// ComponentProvers::compute_composition_polynomial for one component: the four coordinate
// polynomials of log size max_constraint_log_degree_bound.
inline std::vector<Column> composition_polynomial(const Air& air, const CommitmentSchemeProver& pcs, QM31 rc) {
  size_t n = air.n_constraints();
  std::vector<QM31> coeffs = generate_secure_powers(rc, n);
  std::reverse(coeffs.begin(), coeffs.end());
  uint32_t trace_log = air.log_size(), eval_log = air.max_constraint_log_degree_bound();
  CircleDomain ed = canonic_domain(eval_log);
  Mask m = air.mask_offsets();
  // Trace columns on the evaluation domain (extension when it differs from the committed one).
  std::vector<std::vector<Column>> ext(m.size());
  std::vector<std::vector<const Column*>> tr(m.size());
  TwiddleTree etw;
  bool have_etw = false;
  for (size_t t = 0; t < m.size(); t++) {
    for (size_t c = 0; c < m[t].size(); c++) {
      const Column& ev = pcs.trees[t].evals[c];
      if (ev.size() == ed.size()) {
        tr[t].push_back(&ev);
      } else {
        ext[t].emplace_back();
      }
    }
    if (!ext[t].empty()) {
      if (!have_etw) { etw = precompute_twiddles(ed.half_coset); have_etw = true; }
#pragma omp parallel for schedule(dynamic)
      for (long c = 0; c < (long)ext[t].size(); c++) ext[t][c] = evaluate(ed, pcs.trees[t].polys[c], etw);
    }
    if (!ext[t].empty()) {
      tr[t].clear();
      for (auto& e : ext[t]) tr[t].push_back(&e);
    }
  }
  // Denominator inverses on the 2^(eval_log - trace_log) cosets, bit-reversed.
  uint32_t expand = eval_log - trace_log;
  Coset tc = canonic_coset(trace_log);
  std::vector<M31> dinv;
  for (size_t i = 0; i < ((size_t)1 << expand); i++) dinv.push_back(inv(coset_vanishing(tc, ed.at(i))));
  bit_reverse(dinv);
  SecureColumn acc(ed.size());
#pragma omp parallel for schedule(static)
  for (long r = 0; r < (long)ed.size(); r++) {
    DomainEvaluator e(&tr, r, trace_log, eval_log, coeffs.data());
    QM31 rr = air.eval_row(e);
    acc.set(r, rr * dinv[r >> trace_log]);
  }
  TwiddleTree ftw = precompute_twiddles(ed.half_coset);
  std::vector<Column> polys;
  for (int k = 0; k < 4; k++) polys.push_back(interpolate(ed, acc.c[k], ftw));
  return polys;
}

inline QM31 eval_composition_at_point(const Air& air, CirclePointQM31 p, const MaskValues& mask, QM31 rc) {
  QM31 acc;
  QM31 dinv = inv(coset_vanishing(canonic_coset(air.log_size()), p));
  PointEvaluator e(&mask, &acc, rc, dinv);
  air.eval_point(e);
  return acc;
}

// prover/mod.rs:27-79. `pcs` holds the preprocessed and trace trees already.
inline StarkProof prove(const Air& air, Channel& ch, CommitmentSchemeProver& pcs) {
  QM31 rc = ch.draw_felt();
  pcs.commit(composition_polynomial(air, pcs, rc), ch);
  CirclePointQM31 oods = random_point(ch);
  auto pts = mask_points(air, oods);
  while (pts.size() < pcs.trees.size() - 1) pts.emplace_back();
  // Preprocessed columns (tree 0) are not sampled by these AIRs.
  pts[0].assign(pcs.trees[0].polys.size(), {});
  pts.push_back(std::vector<std::vector<CirclePointQM31>>(4, {oods}));
  StarkProof proof = pcs.prove_values(pts, ch);
  MaskValues mv(proof.sampled_values.begin(), proof.sampled_values.end() - 1);
  const auto& comp = proof.sampled_values.back();
  QM31 parts[4] = {comp[0][0], comp[1][0], comp[2][0], comp[3][0]};
  if (PointEvaluator::combine_ef(parts) != eval_composition_at_point(air, oods, mv, rc))
    throw std::runtime_error("ConstraintsNotSatisfied");
  return proof;
}

// ---------------------------------------------------------------- verifier
// Rebuilds the 2-element cosets around `queries` from query evaluations and witness values
// (fri.rs:989-1031). Returns false when the witness runs short.
inline bool rebuild_evals(const std::vector<size_t>& queries, const std::vector<QM31>& query_evals,
                          const std::vector<QM31>& witness, size_t& wi, std::vector<size_t>& positions,
                          std::vector<std::array<QM31, 2>>& subsets, std::vector<size_t>& starts) {
  size_t qe = 0, i = 0;
  while (i < queries.size()) {
    size_t start = (queries[i] >> 1) << 1;
    size_t j = i;
    while (j < queries.size() && (queries[j] >> 1) == (queries[i] >> 1)) j++;
    std::array<QM31, 2> ev;
    size_t k = i;
    for (size_t pos = start; pos < start + 2; pos++) {
      positions.push_back(pos);
      if (k < j && queries[k] == pos) {
        k++;
        if (qe >= query_evals.size()) return false;
        ev[pos - start] = query_evals[qe++];
      } else {
        if (wi >= witness.size()) return false;
        ev[pos - start] = witness[wi++];
      }
    }
    subsets.push_back(ev);
    starts.push_back(start);
    i = j;
  }
  return true;
}

// Full verification (prover/mod.rs:81-127 with pcs/verifier.rs and the FRI verifier).
// `trace_log_sizes[t]` are the committed trees' column log sizes before blowup (trees before
// the composition tree). Returns "" on success, else the failure reason.
// The component-specific parts of verify(): the composition's log size, the mask points of every
// committed tree at the out-of-domain point, and the composition value those samples imply.
struct VerifyAir {
  uint32_t composition_log;
  std::function<std::vector<std::vector<std::vector<CirclePointQM31>>>(CirclePointQM31)> mask_points;
  std::function<QM31(CirclePointQM31, const MaskValues&, QM31)> composition_at;
};

inline std::string verify_with(const VerifyAir& va, Channel& ch, const StarkProof& proof,
                               const std::vector<std::vector<uint32_t>>& trace_log_sizes,
                               const std::function<void(size_t, Channel&)>& after_tree);

inline std::string verify(const Air& air, Channel& ch, const StarkProof& proof,
                          const std::vector<std::vector<uint32_t>>& trace_log_sizes,
                          const std::function<void(size_t, Channel&)>& after_tree = nullptr) {
  VerifyAir va;
  va.composition_log = air.max_constraint_log_degree_bound();
  const size_t n_trees = trace_log_sizes.size(), n_pre = trace_log_sizes[0].size();
  va.mask_points = [&air, n_trees, n_pre](CirclePointQM31 oods) {
    auto pts = mask_points(air, oods);
    while (pts.size() < n_trees) pts.emplace_back();
    pts[0].assign(n_pre, {});
    return pts;
  };
  va.composition_at = [&air](CirclePointQM31 oods, const MaskValues& mv, QM31 rc) {
    return eval_composition_at_point(air, oods, mv, rc);
  };
  return verify_with(va, ch, proof, trace_log_sizes, after_tree);
}

inline std::string verify_with(const VerifyAir& va, Channel& ch, const StarkProof& proof,
                               const std::vector<std::vector<uint32_t>>& trace_log_sizes,
                               const std::function<void(size_t, Channel&)>& after_tree) {
  const PcsConfig& cfg = proof.config;
  size_t n_trees = trace_log_sizes.size();
  if (proof.commitments.size() != n_trees + 1) return "commitments";
  std::vector<std::vector<uint32_t>> tree_logs;  // extended log sizes
  for (size_t t = 0; t < n_trees; t++) {
    ch.mix_root(proof.commitments[t]);
    if (after_tree) after_tree(t, ch);
    std::vector<uint32_t> l;
    for (auto x : trace_log_sizes[t]) l.push_back(x + cfg.log_blowup);
    tree_logs.push_back(l);
  }
  QM31 rc = ch.draw_felt();
  ch.mix_root(proof.commitments[n_trees]);
  tree_logs.push_back(std::vector<uint32_t>(4, va.composition_log + cfg.log_blowup));
  CirclePointQM31 oods = random_point(ch);
  auto pts = va.mask_points(oods);
  pts.push_back(std::vector<std::vector<CirclePointQM31>>(4, {oods}));
  if (proof.sampled_values.size() != pts.size()) return "sampled structure";
  for (size_t t = 0; t < pts.size(); t++) {
    if (proof.sampled_values[t].size() != pts[t].size()) return "sampled structure";
    for (size_t c = 0; c < pts[t].size(); c++)
      if (proof.sampled_values[t][c].size() != pts[t][c].size()) return "sampled structure";
  }
  MaskValues mv(proof.sampled_values.begin(), proof.sampled_values.end() - 1);
  const auto& comp = proof.sampled_values.back();
  QM31 parts[4] = {comp[0][0], comp[1][0], comp[2][0], comp[3][0]};
  if (PointEvaluator::combine_ef(parts) != va.composition_at(oods, mv, rc)) return "OodsNotMatching";

  // verify_values
  std::vector<QM31> flat;
  for (auto& t : proof.sampled_values)
    for (auto& c : t) flat.insert(flat.end(), c.begin(), c.end());
  ch.mix_felts(flat);
  QM31 qrc = ch.draw_felt();
  std::set<uint32_t, std::greater<uint32_t>> logs;
  for (auto& t : tree_logs) logs.insert(t.begin(), t.end());
  std::vector<uint32_t> col_logs(logs.begin(), logs.end());  // commitment domain log sizes, desc
  // FRI commitment phase.
  const FriProof& fp = proof.fri;
  ch.mix_root(fp.first_layer.commitment);
  QM31 first_alpha = ch.draw_felt();
  uint32_t layer_bound = col_logs[0] - cfg.log_blowup - 1;
  Coset layer_dom = Coset::half_odds(layer_bound + cfg.log_blowup);
  std::vector<QM31> alphas;
  std::vector<Coset> doms;
  std::vector<uint32_t> bounds;
  for (auto& l : fp.inner_layers) {
    ch.mix_root(l.commitment);
    alphas.push_back(ch.draw_felt());
    doms.push_back(layer_dom);
    bounds.push_back(layer_bound);
    if (layer_bound < 1) return "InvalidNumFriLayers";
    layer_bound -= 1;
    layer_dom = layer_dom.dbl();
  }
  if (layer_bound != cfg.log_last_layer) return "InvalidNumFriLayers";
  if (fp.last_layer_poly.size() > ((size_t)1 << cfg.log_last_layer)) return "LastLayerDegreeInvalid";
  ch.mix_felts(fp.last_layer_poly);
  ch.mix_u64(proof.proof_of_work);
  if (ch.trailing_zeros() < cfg.pow_bits) return "ProofOfWork";
  Queries q = Queries::generate(ch, col_logs[0], cfg.n_queries);
  std::map<uint32_t, std::vector<size_t>> by_log;
  for (auto l : col_logs) by_log[l] = q.fold(col_logs[0] - l).positions;
  // Merkle decommitments of the trees.
  if (proof.decommitments.size() != tree_logs.size() || proof.queried_values.size() != tree_logs.size())
    return "decommitment structure";
  for (size_t t = 0; t < tree_logs.size(); t++) {
    std::map<uint32_t, std::vector<size_t>> qs;
    for (auto l : tree_logs[t]) qs[l] = by_log[l];
    if (!merkle_verify(proof.commitments[t], tree_logs[t], qs, proof.queried_values[t], proof.decommitments[t]))
      return "MerkleVerification";
  }
  // FRI answers (pcs/quotients.rs:103-165).
  std::vector<std::pair<uint32_t, const std::vector<CirclePointQM31>*>> cols;
  std::vector<std::vector<PointSample>> samples_flat;
  std::vector<uint32_t> logs_flat;
  for (size_t t = 0; t < tree_logs.size(); t++)
    for (size_t c = 0; c < tree_logs[t].size(); c++) {
      std::vector<PointSample> s;
      for (size_t k = 0; k < pts[t][c].size(); k++) s.push_back({pts[t][c][k], proof.sampled_values[t][c][k]});
      samples_flat.push_back(s);
      logs_flat.push_back(tree_logs[t][c]);
    }
  std::vector<size_t> order(logs_flat.size());
  for (size_t i = 0; i < order.size(); i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return logs_flat[a] > logs_flat[b]; });
  std::vector<size_t> qv_pos(tree_logs.size(), 0);
  std::vector<std::vector<QM31>> answers;  // per FRI column (desc log)
  for (size_t i = 0; i < order.size();) {
    uint32_t log = logs_flat[order[i]];
    size_t j = i;
    std::vector<std::vector<PointSample>> gs;
    while (j < order.size() && logs_flat[order[j]] == log) gs.push_back(samples_flat[order[j++]]);
    auto batches = column_sample_batches(gs);
    QuotientConstants qc = quotient_constants(batches, qrc);
    CircleDomain dom = canonic_domain(log);
    std::vector<QM31> ans;
    for (size_t qpos : by_log[log]) {
      CirclePointM31 p = dom.at(bit_reverse_index(qpos, log));
      std::vector<M31> row;
      for (size_t t = 0; t < tree_logs.size(); t++) {
        size_t nc = 0;
        for (auto l : tree_logs[t]) nc += l == log;
        for (size_t k = 0; k < nc; k++) {
          if (qv_pos[t] >= proof.queried_values[t].size()) return "queried values";
          row.push_back(proof.queried_values[t][qv_pos[t]++]);
        }
      }
      ans.push_back(accumulate_row_quotients(batches, row, qc, p));
    }
    answers.push_back(ans);
    i = j;
  }
  // FRI decommitment: first layer.
  size_t wi = 0;
  std::vector<std::vector<std::array<QM31, 2>>> first_subsets(col_logs.size());
  std::vector<std::vector<size_t>> first_starts(col_logs.size());
  std::map<uint32_t, std::vector<size_t>> dpos;
  std::vector<M31> dvals;
  for (size_t c = 0; c < col_logs.size(); c++) {
    Queries cq = q.fold(col_logs[0] - col_logs[c]);
    std::vector<size_t> pos;
    if (!rebuild_evals(cq.positions, answers[c], fp.first_layer.fri_witness, wi, pos, first_subsets[c], first_starts[c]))
      return "FirstLayerEvaluationsInvalid";
    dpos[col_logs[c]] = pos;
    for (auto& s : first_subsets[c])
      for (auto& v : s)
        for (int k = 0; k < 4; k++) dvals.push_back(v.coord(k));
  }
  if (wi != fp.first_layer.fri_witness.size()) return "FirstLayerEvaluationsInvalid";
  std::vector<uint32_t> fl_logs;
  for (auto l : col_logs)
    for (int k = 0; k < 4; k++) fl_logs.push_back(l);
  if (!merkle_verify(fp.first_layer.commitment, fl_logs, dpos, dvals, fp.first_layer.decommitment))
    return "FirstLayerCommitmentInvalid";
  // Inner layers.
  Queries lq = q.fold(1);
  std::vector<QM31> levals(lq.positions.size(), QM31());
  size_t next_col = 0;
  QM31 prev_alpha = first_alpha;
  for (size_t li = 0; li < fp.inner_layers.size(); li++) {
    while (next_col < col_logs.size() && col_logs[next_col] - cfg.log_blowup - 1 == bounds[li]) {
      CircleDomain cd = canonic_domain(col_logs[next_col]);
      std::vector<CirclePointM31> pts_c = cd.points();
      QM31 a2 = prev_alpha * prev_alpha;
      for (size_t s = 0; s < first_subsets[next_col].size(); s++) {
        CirclePointM31 p = pts_c[bit_reverse_index(first_starts[next_col][s], col_logs[next_col])];
        QM31 f0 = first_subsets[next_col][s][0], f1 = first_subsets[next_col][s][1];
        ibutterfly(f0, f1, inv(p.y));
        QM31 folded = prev_alpha * f1 + f0;
        if (s >= levals.size()) return "fold structure";
        levals[s] = levals[s] * a2 + folded;
      }
      next_col++;
    }
    const FriLayerProof& L = fp.inner_layers[li];
    size_t w = 0;
    std::vector<size_t> pos, starts;
    std::vector<std::array<QM31, 2>> subsets;
    if (!rebuild_evals(lq.positions, levals, L.fri_witness, w, pos, subsets, starts) || w != L.fri_witness.size())
      return "InnerLayerEvaluationsInvalid";
    std::vector<M31> vals;
    for (auto& s : subsets)
      for (auto& v : s)
        for (int k = 0; k < 4; k++) vals.push_back(v.coord(k));
    std::map<uint32_t, std::vector<size_t>> m;
    m[doms[li].log_size] = pos;
    if (!merkle_verify(L.commitment, std::vector<uint32_t>(4, doms[li].log_size), m, vals, L.decommitment))
      return "InnerLayerCommitmentInvalid";
    std::vector<CirclePointM31> dp = doms[li].points();
    std::vector<QM31> next_evals;
    for (size_t s = 0; s < subsets.size(); s++) {
      M31 x = dp[bit_reverse_index(starts[s], doms[li].log_size)].x;
      QM31 f0 = subsets[s][0], f1 = subsets[s][1];
      ibutterfly(f0, f1, inv(x));
      next_evals.push_back(f0 + alphas[li] * f1);
    }
    levals = next_evals;
    lq = lq.fold(1);
    prev_alpha = alphas[li];
  }
  if (next_col != col_logs.size()) return "FRI columns not consumed";
  // Last layer.
  std::vector<CirclePointM31> lp = layer_dom.points();
  for (size_t i = 0; i < lq.positions.size(); i++) {
    M31 x = lp[bit_reverse_index(lq.positions[i], layer_dom.log_size)].x;
    if (levals[i] != line_poly_eval_at_point(fp.last_layer_poly, QM31(x))) return "LastLayerEvaluationsInvalid";
  }
  return "";
}

}  // namespace oracle
