// ORACLE — test infrastructure only (see field.h).
// Poseidon2 AIR with its LogUp interaction trace, restated from
// crates/prover/src/examples/poseidon/mod.rs:30-389 and the LogUp machinery of
// crates/prover/src/constraint_framework/logup.rs:17-260 and constraint_framework/mod.rs:182-248
// (finalize_logup_batched), prefix sum of crates/prover/src/core/backend/simd/prefix_sum.rs:122-139,
// Fraction arithmetic of crates/prover/src/core/lookups/utils.rs:198-251.
#pragma once
#include "air.h"

namespace oracle {

constexpr size_t PS_INSTANCES_PER_ROW = 8;
constexpr size_t PS_STATE = 16;
constexpr size_t PS_PARTIAL_ROUNDS = 14;
constexpr size_t PS_HALF_FULL_ROUNDS = 4;
constexpr size_t PS_COLUMNS_PER_REP = PS_STATE * (1 + 2 * PS_HALF_FULL_ROUNDS) + PS_PARTIAL_ROUNDS;  // 158
constexpr size_t PS_COLUMNS = PS_INSTANCES_PER_ROW * PS_COLUMNS_PER_REP;                            // 1264
constexpr uint32_t PS_LOG_EXPAND = 2;
// Round constants of the reference example (all 1234).
inline M31 ps_external_const(size_t, size_t) { return M31(1234); }
inline M31 ps_internal_const(size_t) { return M31(1234); }

template <class F>
inline void apply_m4(F* x) {
  F t0 = x[0] + x[1];
  F t02 = t0 + t0;
  F t1 = x[2] + x[3];
  F t12 = t1 + t1;
  F t2 = x[1] + x[1] + t1;
  F t3 = x[3] + x[3] + t0;
  F t4 = t12 + t12 + t3;
  F t5 = t02 + t02 + t2;
  F t6 = t3 + t5;
  F t7 = t2 + t4;
  x[0] = t6;
  x[1] = t5;
  x[2] = t7;
  x[3] = t4;
}
template <class F>
inline void apply_external_round_matrix(F* s) {
  for (int i = 0; i < 4; i++) apply_m4(s + 4 * i);
  for (int j = 0; j < 4; j++) {
    F t = s[j] + s[j + 4] + s[j + 8] + s[j + 12];
    for (int i = 0; i < 4; i++) s[4 * i + j] = s[4 * i + j] + t;
  }
}
template <class F>
inline void apply_internal_round_matrix(F* s) {
  F sum = s[0];
  for (int i = 1; i < 16; i++) sum = sum + s[i];
  for (int i = 0; i < 16; i++) s[i] = s[i] * M31(1u << (i + 1)) + sum;
}
template <class F>
inline F pow5(const F& x) {
  F x2 = x * x;
  F x4 = x2 * x2;
  return x4 * x;
}

struct LookupElements {
  QM31 z, alpha;
  QM31 alpha_powers[PS_STATE];
  // LookupElements::draw (logup.rs:74-88)
  static LookupElements draw(Channel& ch) {
    LookupElements le;
    auto v = ch.draw_felts(2);
    le.z = v[0];
    le.alpha = v[1];
    QM31 cur(M31(1));
    for (size_t i = 0; i < PS_STATE; i++) {
      le.alpha_powers[i] = cur;
      cur = cur * le.alpha;
    }
    return le;
  }
  template <class F>
  QM31 combine(const F* v) const {
    QM31 acc;
    for (size_t i = 0; i < PS_STATE; i++) acc = acc + alpha_powers[i] * v[i];
    return acc - z;
  }
};

struct Frac {
  QM31 num, den;
};
inline Frac frac_add(const Frac& a, const Frac& b) { return {b.den * a.num + a.den * b.num, a.den * b.den}; }

// Constraints of eval_poseidon_constraints (poseidon/mod.rs:141-197) followed by
// finalize_logup_in_pairs. E is DomainEvaluator (F = M31) or PointEvaluator (F = QM31).
template <class E>
inline void poseidon_evaluate(E& e, const LookupElements& le, QM31 cumsum_shift) {
  using F = typename E::F;
  std::vector<Frac> fracs;
  for (size_t rep = 0; rep < PS_INSTANCES_PER_ROW; rep++) {
    F state[PS_STATE];
    for (size_t i = 0; i < PS_STATE; i++) state[i] = e.next_trace_mask();
    F initial[PS_STATE];
    for (size_t i = 0; i < PS_STATE; i++) initial[i] = state[i];
    for (size_t round = 0; round < PS_HALF_FULL_ROUNDS; round++) {
      for (size_t i = 0; i < PS_STATE; i++) state[i] = state[i] + ps_external_const(round, i);
      apply_external_round_matrix(state);
      for (size_t i = 0; i < PS_STATE; i++) state[i] = pow5(state[i]);
      for (size_t i = 0; i < PS_STATE; i++) {
        F m = e.next_trace_mask();
        e.add_constraint(state[i] - m);
        state[i] = m;
      }
    }
    for (size_t round = 0; round < PS_PARTIAL_ROUNDS; round++) {
      state[0] = state[0] + ps_internal_const(round);
      apply_internal_round_matrix(state);
      state[0] = pow5(state[0]);
      F m = e.next_trace_mask();
      e.add_constraint(state[0] - m);
      state[0] = m;
    }
    for (size_t round = 0; round < PS_HALF_FULL_ROUNDS; round++) {
      for (size_t i = 0; i < PS_STATE; i++) state[i] = state[i] + ps_external_const(round + PS_HALF_FULL_ROUNDS, i);
      apply_external_round_matrix(state);
      for (size_t i = 0; i < PS_STATE; i++) state[i] = pow5(state[i]);
      for (size_t i = 0; i < PS_STATE; i++) {
        F m = e.next_trace_mask();
        e.add_constraint(state[i] - m);
        state[i] = m;
      }
    }
    fracs.push_back({QM31(M31(1)), le.combine(initial)});
    fracs.push_back({-QM31(M31(1)), le.combine(state)});
  }
  // finalize_logup_batched with batches (0, 0, 1, 1, ...) (constraint_framework/mod.rs:182-248).
  size_t n_batches = fracs.size() / 2;
  QM31 prev_col;
  for (size_t b = 0; b + 1 < n_batches; b++) {
    Frac f = frac_add(fracs[2 * b], fracs[2 * b + 1]);
    QM31 cur = e.next_extension_interaction_mask(2, {0})[0];
    QM31 diff = cur - prev_col;
    prev_col = cur;
    e.add_constraint(diff * f.den - f.num);
  }
  Frac f = frac_add(fracs[2 * (n_batches - 1)], fracs[2 * (n_batches - 1) + 1]);
  auto pc = e.next_extension_interaction_mask(2, {-1, 0});
  QM31 diff = pc[1] - pc[0] - prev_col;
  QM31 fixed = diff + cumsum_shift;
  e.add_constraint(fixed * f.den - f.num);
}

struct PoseidonAir : Air {
  uint32_t log_n;
  LookupElements le;
  QM31 claimed_sum;
  PoseidonAir(uint32_t l, const LookupElements& e, QM31 cs) : log_n(l), le(e), claimed_sum(cs) {}
  uint32_t log_size() const override { return log_n; }
  uint32_t max_constraint_log_degree_bound() const override { return log_n + PS_LOG_EXPAND; }
  size_t n_constraints() const override {
    return PS_INSTANCES_PER_ROW * (2 * PS_HALF_FULL_ROUNDS * PS_STATE + PS_PARTIAL_ROUNDS) + PS_INSTANCES_PER_ROW;
  }
  Mask mask_offsets() const override {
    Mask m(3);
    m[1].assign(PS_COLUMNS, {0});
    for (size_t b = 0; b + 1 < PS_INSTANCES_PER_ROW; b++)
      for (int k = 0; k < 4; k++) m[2].push_back({0});
    for (int k = 0; k < 4; k++) m[2].push_back({-1, 0});
    return m;
  }
  QM31 shift() const { return claimed_sum * inv(M31(1u << log_n)); }
  QM31 eval_row(DomainEvaluator& e) const override {
    poseidon_evaluate(e, le, shift());
    return e.row_res;
  }
  void eval_point(PointEvaluator& e) const override { poseidon_evaluate(e, le, shift()); }
};

// gen_trace (poseidon/mod.rs:203-290) from explicit initial states: init[(row * 8 + rep) * 16 + i].
// Returns the 1264 trace columns and, per rep, the initial and final states (for the lookups).
inline std::vector<Column> poseidon_trace(uint32_t log_n, const uint32_t* init, std::vector<std::vector<M31>>& lookups) {
  size_t n = (size_t)1 << log_n;
  std::vector<Column> t(PS_COLUMNS, Column(n));
  lookups.assign(PS_INSTANCES_PER_ROW * 2 * PS_STATE, std::vector<M31>(n));
#pragma omp parallel for schedule(static)
  for (long r = 0; r < (long)n; r++) {
    size_t col = 0;
    for (size_t rep = 0; rep < PS_INSTANCES_PER_ROW; rep++) {
      M31 s[PS_STATE];
      for (size_t i = 0; i < PS_STATE; i++) {
        s[i] = M31(init[((size_t)r * PS_INSTANCES_PER_ROW + rep) * PS_STATE + i]);
        t[col++][r] = s[i];
        lookups[(rep * 2) * PS_STATE + i][r] = s[i];
      }
      for (size_t round = 0; round < PS_HALF_FULL_ROUNDS; round++) {
        for (size_t i = 0; i < PS_STATE; i++) s[i] = s[i] + ps_external_const(round, i);
        apply_external_round_matrix(s);
        for (size_t i = 0; i < PS_STATE; i++) s[i] = pow5(s[i]);
        for (size_t i = 0; i < PS_STATE; i++) t[col++][r] = s[i];
      }
      for (size_t round = 0; round < PS_PARTIAL_ROUNDS; round++) {
        s[0] = s[0] + ps_internal_const(round);
        apply_internal_round_matrix(s);
        s[0] = pow5(s[0]);
        t[col++][r] = s[0];
      }
      for (size_t round = 0; round < PS_HALF_FULL_ROUNDS; round++) {
        for (size_t i = 0; i < PS_STATE; i++) s[i] = s[i] + ps_external_const(round + PS_HALF_FULL_ROUNDS, i);
        apply_external_round_matrix(s);
        for (size_t i = 0; i < PS_STATE; i++) s[i] = pow5(s[i]);
        for (size_t i = 0; i < PS_STATE; i++) t[col++][r] = s[i];
      }
      for (size_t i = 0; i < PS_STATE; i++) lookups[(rep * 2 + 1) * PS_STATE + i][r] = s[i];
    }
  }
  return t;
}

// The reference's deterministic inputs: state_i of rep at row r = r + state_i + rep.
inline std::vector<uint32_t> poseidon_reference_inputs(uint32_t log_n) {
  size_t n = (size_t)1 << log_n;
  std::vector<uint32_t> v(n * PS_INSTANCES_PER_ROW * PS_STATE);
  for (size_t r = 0; r < n; r++)
    for (size_t rep = 0; rep < PS_INSTANCES_PER_ROW; rep++)
      for (size_t i = 0; i < PS_STATE; i++) v[(r * PS_INSTANCES_PER_ROW + rep) * PS_STATE + i] = (uint32_t)(r + i + rep);
  return v;
}

// Inclusive prefix sum in coset order of a bit-reversed circle-domain column
// (prefix_sum.rs:122-139, utils.rs:96-115).
inline Column inclusive_prefix_sum(const Column& col) {
  size_t n = col.size();
  uint32_t log = ilog2(n);
  std::vector<M31> nat(n);
  for (size_t i = 0; i < n; i++) nat[i] = col[bit_reverse_index(i, log)];
  std::vector<M31> coset(n);
  for (size_t i = 0; i < n / 2; i++) {
    coset[2 * i] = nat[i];
    coset[2 * i + 1] = nat[n - 1 - i];
  }
  M31 acc(0);
  for (size_t k = 0; k < n; k++) {
    acc = acc + coset[k];
    coset[k] = acc;
  }
  for (size_t i = 0; i < n / 2; i++) {
    nat[i] = coset[2 * i];
    nat[n - 1 - i] = coset[2 * i + 1];
  }
  Column out(n);
  for (size_t i = 0; i < n; i++) out[bit_reverse_index(i, log)] = nat[i];
  return out;
}

// gen_interaction_trace (poseidon/mod.rs:292-325) with LogupTraceGenerator (logup.rs:123-260):
// per rep a cumulative secure column of (1/d0 - 1/d1); the last one shifted and prefix-summed.
inline std::vector<Column> poseidon_interaction_trace(uint32_t log_n, const std::vector<std::vector<M31>>& lookups,
                                                      const LookupElements& le, QM31& claimed_sum) {
  size_t n = (size_t)1 << log_n;
  std::vector<SecureColumn> cols;
  SecureColumn prev(n);
  for (size_t rep = 0; rep < PS_INSTANCES_PER_ROW; rep++) {
    SecureColumn c(n);
#pragma omp parallel for schedule(static)
    for (long r = 0; r < (long)n; r++) {
      M31 a[PS_STATE], b[PS_STATE];
      for (size_t i = 0; i < PS_STATE; i++) {
        a[i] = lookups[(rep * 2) * PS_STATE + i][r];
        b[i] = lookups[(rep * 2 + 1) * PS_STATE + i][r];
      }
      QM31 d0 = le.combine(a), d1 = le.combine(b);
      QM31 v = (d1 - d0) * inv(d0 * d1);
      c.set(r, v + (rep ? prev.at(r) : QM31()));
    }
    prev = c;
    cols.push_back(c);
  }
  SecureColumn& last = cols.back();
  M31 sums[4] = {M31(0), M31(0), M31(0), M31(0)};
  for (int k = 0; k < 4; k++)
    for (size_t r = 0; r < n; r++) sums[k] = sums[k] + last.c[k][r];
  claimed_sum = QM31::from_m31(sums[0], sums[1], sums[2], sums[3]);
  QM31 shift = claimed_sum * inv(M31((uint32_t)n));
  for (size_t r = 0; r < n; r++) last.set(r, last.at(r) - shift);
  for (int k = 0; k < 4; k++) last.c[k] = inclusive_prefix_sum(last.c[k]);
  std::vector<Column> out;
  for (auto& c : cols)
    for (int k = 0; k < 4; k++) out.push_back(c.c[k]);
  return out;
}

}  // namespace oracle
