// ORACLE — test infrastructure only (see field.h).
// The Plonk and state-machine example AIRs, restated from the reference for checking generated
// constraint kernels:
//   PlonkEval            crates/prover/src/examples/plonk/mod.rs:40-95
//   StateTransitionEval  crates/prover/src/examples/state_machine/components.rs:33-66
//   finalize_logup_in_pairs (finalize_logup_batched with batch(n) = n / 2),
//                        crates/prover/src/constraint_framework/mod.rs:165-240
// E is DomainEvaluator (F = M31) or PointEvaluator (F = QM31).
#pragma once
#include "air_blake_round.h"

namespace oracle {

inline QM31 to_q(const M31& x) { return QM31(x); }
inline QM31 to_q(const QM31& x) { return x; }

template <class E>
inline void finalize_logup_in_pairs(E& e, const std::vector<Frac>& fracs, QM31 cumsum_shift) {
  const size_t n_batches = (fracs.size() + 1) / 2;
  auto batch_frac = [&](size_t b) {
    Frac f = fracs[2 * b];
    if (2 * b + 1 < fracs.size()) f = frac_add(f, fracs[2 * b + 1]);
    return f;
  };
  QM31 prev_col;
  for (size_t b = 0; b + 1 < n_batches; b++) {
    Frac f = batch_frac(b);
    QM31 cur = e.next_extension_interaction_mask(2, {0})[0];
    QM31 diff = cur - prev_col;
    prev_col = cur;
    e.add_constraint(diff * f.den - f.num);
  }
  Frac f = batch_frac(n_batches - 1);
  auto pc = e.next_extension_interaction_mask(2, {-1, 0});
  QM31 fixed = pc[1] - pc[0] - prev_col + cumsum_shift;
  e.add_constraint(fixed * f.den - f.num);
}

template <class E>
inline void plonk_evaluate(E& e, const Relation<2>& rel, QM31 cumsum_shift) {
  using F = typename E::F;
  // Preprocessed wires and op, read as the next columns of tree 0 (get_preprocessed_column).
  F a_wire = e.next_interaction_mask(0, {0})[0];
  F b_wire = e.next_interaction_mask(0, {0})[0];
  F c_wire = e.next_interaction_mask(0, {0})[0];
  F op = e.next_interaction_mask(0, {0})[0];
  F mult = e.next_trace_mask();
  F a_val = e.next_trace_mask();
  F b_val = e.next_trace_mask();
  F c_val = e.next_trace_mask();
  const F one(M31(1));
  e.add_constraint(c_val - op * (a_val + b_val) + (one - op) * a_val * b_val);
  std::vector<Frac> fracs;
  F va[2] = {a_wire, a_val}, vb[2] = {b_wire, b_val}, vc[2] = {c_wire, c_val};
  fracs.push_back({QM31(M31(1)), rel.combine(va, 2)});
  fracs.push_back({QM31(M31(1)), rel.combine(vb, 2)});
  fracs.push_back({to_q(F() - mult), rel.combine(vc, 2)});
  finalize_logup_in_pairs(e, fracs, cumsum_shift);
}

struct PlonkAir : Air {
  uint32_t log_n;
  Relation<2> rel;
  QM31 claimed_sum;
  PlonkAir(uint32_t l, const Relation<2>& r, QM31 cs) : log_n(l), rel(r), claimed_sum(cs) {}
  uint32_t log_size() const override { return log_n; }
  uint32_t max_constraint_log_degree_bound() const override { return log_n + 1; }
  size_t n_constraints() const override { return 3; }
  Mask mask_offsets() const override {
    Mask m(3);
    m[0].assign(4, {0});
    m[1].assign(4, {0});
    for (int k = 0; k < 4; k++) m[2].push_back({0});
    for (int k = 0; k < 4; k++) m[2].push_back({-1, 0});
    return m;
  }
  QM31 shift() const { return claimed_sum * inv(M31(1u << log_n)); }
  QM31 eval_row(DomainEvaluator& e) const override {
    plonk_evaluate(e, rel, shift());
    return e.row_res;
  }
  void eval_point(PointEvaluator& e) const override { plonk_evaluate(e, rel, shift()); }
};

template <class E>
inline void state_transition_evaluate(E& e, size_t coordinate, const Relation<2>& rel, QM31 cumsum_shift) {
  using F = typename E::F;
  F in[2] = {e.next_trace_mask(), e.next_trace_mask()};
  F out[2] = {in[0], in[1]};
  out[coordinate] = out[coordinate] + F(M31(1));
  std::vector<Frac> fracs;
  fracs.push_back({QM31(M31(1)), rel.combine(in, 2)});
  fracs.push_back({-QM31(M31(1)), rel.combine(out, 2)});
  finalize_logup_in_pairs(e, fracs, cumsum_shift);
}

struct StateTransitionAir : Air {
  size_t coordinate;
  uint32_t log_n;
  Relation<2> rel;
  QM31 claimed_sum;
  StateTransitionAir(size_t c, uint32_t l, const Relation<2>& r, QM31 cs) : coordinate(c), log_n(l), rel(r), claimed_sum(cs) {}
  uint32_t log_size() const override { return log_n; }
  uint32_t max_constraint_log_degree_bound() const override { return log_n + 1; }
  size_t n_constraints() const override { return 1; }
  Mask mask_offsets() const override {
    Mask m(3);
    m[1].assign(2, {0});
    for (int k = 0; k < 4; k++) m[2].push_back({-1, 0});
    return m;
  }
  QM31 shift() const { return claimed_sum * inv(M31(1u << log_n)); }
  QM31 eval_row(DomainEvaluator& e) const override {
    state_transition_evaluate(e, coordinate, rel, shift());
    return e.row_res;
  }
  void eval_point(PointEvaluator& e) const override { state_transition_evaluate(e, coordinate, rel, shift()); }
};

}  // namespace oracle
