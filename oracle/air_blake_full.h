// ORACLE — test infrastructure only (see field.h).
// The full Blake example: the scheduler, two round components and five XOR-table components in
// one proof, with preprocessed XOR tables. Restated from
//   prove_blake / verify_blake   crates/prover/src/examples/blake/air.rs:308-540
//   statements, components       crates/prover/src/examples/blake/air.rs:30-305
//   scheduler constraints        crates/prover/src/examples/blake/scheduler/constraints.rs:10-61
//   scheduler trace generation   crates/prover/src/examples/blake/scheduler/gen.rs:45-172
//   XOR table component          crates/prover/src/examples/blake/xor_table/{mod,constraints,gen}.rs
//   preprocessed XOR table       crates/prover/src/examples/blake/preprocessed_columns.rs:13-82
//   round component              air_blake_round.h (round/constraints.rs, round/gen.rs)
// The round component is the one of air_blake_round.h; here its inputs come from the scheduler
// (ROUND_LOG_SPLIT = [3, 1]: the first 2^(L+3) round inputs, then the next 2^(L+1)) and its XOR
// lookups are balanced by the XOR tables, so the claimed sums of all eight components add to zero.
#pragma once
#include "components.h"

namespace oracle {

constexpr uint32_t BF_ROUNDS = 10;
constexpr size_t BF_SCHED_COLS = 2 * BR_STATE * (1 + BF_ROUNDS + 1);  // m, v0, v1..v10: 384
constexpr size_t BF_SCHED_LOOKUPS = BF_ROUNDS + 1;                   // ten Round entries, one Blake
constexpr size_t BF_SCHED_BATCHES = (BF_SCHED_LOOKUPS + 1) / 2;      // 6

// One of the five XOR tables: (elem_bits, expand_bits) = (12, 4), (9, 2), (8, 2), (7, 2), (4, 0).
struct XorTableShape {
  uint32_t elem_bits, expand_bits;
  uint32_t limb_bits() const { return elem_bits - expand_bits; }
  uint32_t column_bits() const { return 2 * limb_bits(); }
  size_t n_mult_cols() const { return (size_t)1 << (2 * expand_bits); }
  size_t n_batches() const { return (n_mult_cols() + 1) / 2; }
};
inline constexpr XorTableShape BF_XOR_TABLES[5] = {{12, 4}, {9, 2}, {8, 2}, {7, 2}, {4, 0}};

// AllElements (air.rs:119-133): the Blake, Round and XOR relations, drawn in that order.
struct BlakeAllElements {
  Relation<BR_ROUND_FELTS> blake;
  BlakeRoundElements round;  // .round and .xor_
  static BlakeAllElements draw(Channel& ch) {
    BlakeAllElements a;
    a.blake = Relation<BR_ROUND_FELTS>::draw(ch);
    a.round.round = Relation<BR_ROUND_FELTS>::draw(ch);
    a.round.xor_ = BlakeXorRelations::draw(ch);
    return a;
  }
};

// eval_blake_scheduler_constraints: messages, then the 11 states; one Round entry (multiplicity 1)
// per round with the SIGMA-permuted messages, one Blake entry with multiplicity 0; in pairs.
template <class E>
inline void blake_scheduler_evaluate(E& e, const BlakeAllElements& el, QM31 cumsum_shift) {
  using F = typename E::F;
  F msg[2 * BR_STATE];
  for (auto& x : msg) x = e.next_trace_mask();
  std::vector<std::vector<F>> st(BF_ROUNDS + 1, std::vector<F>(2 * BR_STATE));
  for (auto& s : st)
    for (auto& x : s) x = e.next_trace_mask();
  std::vector<Frac> fracs;
  F vals[BR_ROUND_FELTS];
  for (uint32_t r = 0; r < BF_ROUNDS; r++) {
    size_t k = 0;
    for (size_t i = 0; i < 2 * BR_STATE; i++) vals[k++] = st[r][i];
    for (size_t i = 0; i < 2 * BR_STATE; i++) vals[k++] = st[r + 1][i];
    for (size_t i = 0; i < BR_STATE; i++) {
      vals[k++] = msg[2 * B2S_SIGMA[r][i]];
      vals[k++] = msg[2 * B2S_SIGMA[r][i] + 1];
    }
    fracs.push_back({QM31(M31(1)), el.round.round.combine(vals, BR_ROUND_FELTS)});
  }
  size_t k = 0;
  for (size_t i = 0; i < 2 * BR_STATE; i++) vals[k++] = st[0][i];
  for (size_t i = 0; i < 2 * BR_STATE; i++) vals[k++] = st[BF_ROUNDS][i];
  for (size_t i = 0; i < 2 * BR_STATE; i++) vals[k++] = msg[i];
  fracs.push_back({QM31(), el.blake.combine(vals, BR_ROUND_FELTS)});
  finalize_logup_in_pairs(e, fracs, cumsum_shift);
}

inline Mask logup_mask(Mask m, size_t n_batches) {
  for (size_t b = 0; b + 1 < n_batches; b++)
    for (int k = 0; k < 4; k++) m[2].push_back({0});
  for (int k = 0; k < 4; k++) m[2].push_back({-1, 0});
  return m;
}

struct BlakeSchedulerAir : Air {
  uint32_t log_n;
  const BlakeAllElements* el;
  QM31 claimed_sum;
  BlakeSchedulerAir(uint32_t l, const BlakeAllElements* e, QM31 cs) : log_n(l), el(e), claimed_sum(cs) {}
  uint32_t log_size() const override { return log_n; }
  uint32_t max_constraint_log_degree_bound() const override { return log_n + 1; }
  size_t n_constraints() const override { return BF_SCHED_BATCHES; }
  Mask mask_offsets() const override {
    Mask m(3);
    m[1].assign(BF_SCHED_COLS, {0});
    return logup_mask(m, BF_SCHED_BATCHES);
  }
  QM31 shift() const { return claimed_sum * inv(M31(1u << log_n)); }
  QM31 eval_row(DomainEvaluator& e) const override {
    blake_scheduler_evaluate(e, *el, shift());
    return e.row_res;
  }
  void eval_point(PointEvaluator& e) const override { blake_scheduler_evaluate(e, *el, shift()); }
};

// The round component with the drawn elements of the whole example (held by pointer, since the
// verifier draws them after placing the components).
struct BlakeRoundFullAir : Air {
  uint32_t log_n;
  const BlakeAllElements* el;
  QM31 claimed_sum;
  BlakeRoundFullAir(uint32_t l, const BlakeAllElements* e, QM31 cs) : log_n(l), el(e), claimed_sum(cs) {}
  uint32_t log_size() const override { return log_n; }
  uint32_t max_constraint_log_degree_bound() const override { return log_n + 1; }
  size_t n_constraints() const override { return BR_N_CONSTRAINTS; }
  Mask mask_offsets() const override {
    Mask m(3);
    m[1].assign(BR_TRACE_COLS, {0});
    return logup_mask(m, BR_INTERACTION_SECURE);
  }
  QM31 shift() const { return claimed_sum * inv(M31(1u << log_n)); }
  QM31 eval_row(DomainEvaluator& e) const override {
    BlakeRoundEvaluator<DomainEvaluator> ev(e, el->round);
    ev.eval(shift());
    return e.row_res;
  }
  void eval_point(PointEvaluator& e) const override {
    BlakeRoundEvaluator<PointEvaluator> ev(e, el->round);
    ev.eval(shift());
  }
};

// XorTableEvalAtRow::eval (xor_table/constraints.rs:1-61): the preprocessed (al, bl, al ^ bl), and
// per multiplicity column (ah, bh) the entry (al + ah 2^limb, bl + bh 2^limb, cl + (ah ^ bh) 2^limb)
// with multiplicity -mult; in pairs.
template <class E>
inline void xor_table_evaluate(E& e, const XorTableShape& s, const Relation<3>& rel, QM31 cumsum_shift) {
  using F = typename E::F;
  F al = e.next_interaction_mask(0, {0})[0];
  F bl = e.next_interaction_mask(0, {0})[0];
  F cl = e.next_interaction_mask(0, {0})[0];
  const uint32_t lb = s.limb_bits();
  std::vector<Frac> fracs;
  for (uint32_t i = 0; i < (uint32_t)s.n_mult_cols(); i++) {
    uint32_t ih = i >> s.expand_bits, jh = i & ((1u << s.expand_bits) - 1);
    F mult = e.next_trace_mask();
    F v[3] = {al + F(M31(ih << lb)), bl + F(M31(jh << lb)), cl + F(M31((ih ^ jh) << lb))};
    fracs.push_back({to_q(F() - mult), rel.combine(v, 3)});
  }
  finalize_logup_in_pairs(e, fracs, cumsum_shift);
}

struct XorTableAir : Air {
  XorTableShape s;
  const Relation<3>* rel;
  QM31 claimed_sum;
  XorTableAir(XorTableShape sh, const Relation<3>* r, QM31 cs) : s(sh), rel(r), claimed_sum(cs) {}
  uint32_t log_size() const override { return s.column_bits(); }
  uint32_t max_constraint_log_degree_bound() const override { return s.column_bits() + 1; }
  size_t n_constraints() const override { return s.n_batches(); }
  Mask mask_offsets() const override {
    Mask m(3);
    m[0].assign(3, {0});
    m[1].assign(s.n_mult_cols(), {0});
    return logup_mask(m, s.n_batches());
  }
  QM31 shift() const { return claimed_sum * inv(M31(1u << log_size())); }
  QM31 eval_row(DomainEvaluator& e) const override {
    xor_table_evaluate(e, s, *rel, shift());
    return e.row_res;
  }
  void eval_point(PointEvaluator& e) const override { xor_table_evaluate(e, s, *rel, shift()); }
};

// LogupTraceGenerator from a per-(batch, row) fraction, rows in parallel: each column the running
// sum over batches of num / den; the last shifted by claimed_sum / n and prefix-summed.
template <class FracAt>
inline std::vector<Column> logup_trace_fn(size_t n_batches, size_t n, const FracAt& frac_at, QM31& claimed_sum) {
  std::vector<SecureColumn> cols(n_batches, SecureColumn(n));
#pragma omp parallel for schedule(static)
  for (long r = 0; r < (long)n; r++) {
    QM31 run;
    for (size_t b = 0; b < n_batches; b++) {
      Frac f = frac_at(b, (size_t)r);
      run = run + f.num * inv(f.den);
      cols[b].set(r, run);
    }
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

// The whole example's traces, the lookups the interaction trace needs, and the claimed sums.
struct BlakeFullTraces {
  uint32_t log_n;
  std::vector<Column> preprocessed, trace, interaction;
  std::vector<BrXorLookup> rxl[2];
  std::vector<std::vector<M31>> rround[2];
  std::vector<std::vector<Column>> mults;  // per XOR table, its multiplicity columns
  QM31 scheduler_sum, round_sums[2], xor_sums[5];
};

// The preprocessed tree (air.rs:343-361): IsFirst(L), IsFirst(L+3), IsFirst(L+1), then per XOR
// table its (al, bl, al ^ bl) columns in natural index order and an IsFirst of its size.
inline std::vector<Column> blake_preprocessed(uint32_t log_n) {
  std::vector<Column> out;
  auto is_first = [](uint32_t log) {
    Column c((size_t)1 << log, M31(0));
    c[0] = M31(1);
    return c;
  };
  out.push_back(is_first(log_n));
  out.push_back(is_first(log_n + 3));
  out.push_back(is_first(log_n + 1));
  for (const XorTableShape& s : BF_XOR_TABLES) {
    size_t n = (size_t)1 << s.column_bits();
    const uint32_t lb = s.limb_bits(), mask = (1u << lb) - 1;
    Column a(n), b(n), c(n);
    for (size_t i = 0; i < n; i++) {
      a[i] = M31((uint32_t)(i >> lb));
      b[i] = M31((uint32_t)i & mask);
      c[i] = M31((uint32_t)(i >> lb) ^ ((uint32_t)i & mask));
    }
    out.push_back(a);
    out.push_back(b);
    out.push_back(c);
    out.push_back(is_first(s.column_bits()));
  }
  return out;
}

// The inputs of prove_blake (air.rs:331-338): instance s = 16 vec_row + lane has every state word
// vec_row + 2 lane and every message word vec_row + 2 lane + 1.
inline void blake_example_input(size_t s, uint32_t v[16], uint32_t m[16]) {
  uint32_t vec_row = (uint32_t)(s >> 4), lane = (uint32_t)(s & 15);
  for (int k = 0; k < 16; k++) {
    v[k] = vec_row + 2 * lane;
    m[k] = vec_row + 2 * lane + 1;
  }
}

// One BLAKE2s round on 16 words with the round's SIGMA (blake2s::round, simd/blake2s.rs:180-270).
inline void blake2s_round_words(uint32_t v[16], const uint32_t m[16], uint32_t r) {
  const uint8_t* s = B2S_SIGMA[r];
  auto G = [&](int a, int b, int c, int d, uint32_t x, uint32_t y) {
    v[a] = v[a] + v[b] + x;
    v[d] = rotr32(v[d] ^ v[a], 16);
    v[c] = v[c] + v[d];
    v[b] = rotr32(v[b] ^ v[c], 12);
    v[a] = v[a] + v[b] + y;
    v[d] = rotr32(v[d] ^ v[a], 8);
    v[c] = v[c] + v[d];
    v[b] = rotr32(v[b] ^ v[c], 7);
  };
  G(0, 4, 8, 12, m[s[0]], m[s[1]]);
  G(1, 5, 9, 13, m[s[2]], m[s[3]]);
  G(2, 6, 10, 14, m[s[4]], m[s[5]]);
  G(3, 7, 11, 15, m[s[6]], m[s[7]]);
  G(0, 5, 10, 15, m[s[8]], m[s[9]]);
  G(1, 6, 11, 12, m[s[10]], m[s[11]]);
  G(2, 7, 8, 13, m[s[12]], m[s[13]]);
  G(3, 4, 9, 14, m[s[14]], m[s[15]]);
}

// Index of table w among BF_XOR_TABLES.
inline size_t xor_table_index(uint32_t w) {
  for (size_t t = 0; t < 5; t++)
    if (BF_XOR_TABLES[t].elem_bits == w) return t;
  throw std::runtime_error("invalid xor width");
}

// The scheduler trace (gen.rs:45-118) and the round inputs it hands on: round input p = 10 vec_row
// + r holds, for each of its 16 lanes, the state before round r and the SIGMA[r]-permuted messages.
// Round-component row p_local 16 + lane therefore takes instance 16 (p / 10) + lane, round p % 10.
inline std::vector<Column> blake_scheduler_trace(uint32_t log_n, std::vector<uint32_t>& round_inputs) {
  const size_t n = (size_t)1 << log_n;
  std::vector<Column> t(BF_SCHED_COLS, Column(n));
  round_inputs.assign(n * BF_ROUNDS * 32, 0);
  for (size_t s = 0; s < n; s++) {
    uint32_t v[16], m[16];
    blake_example_input(s, v, m);
    size_t col = 0;
    auto put = [&](const uint32_t* w) {
      for (int k = 0; k < 16; k++) {
        t[col++][s] = M31(w[k] & 0xffffu);
        t[col++][s] = M31(w[k] >> 16);
      }
    };
    put(m);
    put(v);
    const size_t vec_row = s >> 4, lane = s & 15;
    for (uint32_t r = 0; r < BF_ROUNDS; r++) {
      size_t row = ((vec_row * BF_ROUNDS + r) << 4) + lane;
      uint32_t* in = &round_inputs[row * 32];
      for (int k = 0; k < 16; k++) {
        in[k] = v[k];
        in[16 + k] = m[B2S_SIGMA[r][k]];
      }
      blake2s_round_words(v, m, r);
      put(v);
    }
  }
  return t;
}

// prove_blake's traces (air.rs:363-460). The XOR multiplicities are accumulated from the rounds'
// lookups as XorAccumulator::add_input does (xor_table/mod.rs:60-90): column (ah << e) + bh, row
// (al << limb) + bl.
inline BlakeFullTraces blake_full_traces(uint32_t log_n) {
  BlakeFullTraces T;
  T.log_n = log_n;
  T.preprocessed = blake_preprocessed(log_n);
  std::vector<uint32_t> rin;
  std::vector<Column> sched = blake_scheduler_trace(log_n, rin);
  const uint32_t rlog[2] = {log_n + 3, log_n + 1};
  std::vector<Column> rtrace[2];
  std::vector<BrXorLookup>* rxl = T.rxl;
  size_t first = 0;
  for (int c = 0; c < 2; c++) {
    rtrace[c] = blake_round_trace(rlog[c], rin.data() + first * 32, rxl[c], T.rround[c]);
    first += (size_t)1 << rlog[c];
  }
  std::vector<std::vector<Column>>& mults = T.mults;
  mults.resize(5);
  for (size_t t = 0; t < 5; t++)
    mults[t].assign(BF_XOR_TABLES[t].n_mult_cols(), Column((size_t)1 << BF_XOR_TABLES[t].column_bits(), M31(0)));
  for (int c = 0; c < 2; c++)
    for (const BrXorLookup& l : rxl[c]) {
      size_t t = xor_table_index(l.w);
      const XorTableShape& s = BF_XOR_TABLES[t];
      const uint32_t lb = s.limb_bits(), mask = (1u << lb) - 1;
      for (size_t r = 0; r < l.a.size(); r++) {
        uint32_t a = l.a[r].v, b = l.b[r].v;
        size_t col = ((size_t)(a >> lb) << s.expand_bits) + (b >> lb);
        size_t off = ((size_t)(a & mask) << lb) + (b & mask);
        mults[t][col][off] = mults[t][col][off] + M31(1);
      }
    }
  for (auto& c : sched) T.trace.push_back(std::move(c));
  for (int c = 0; c < 2; c++)
    for (auto& col : rtrace[c]) T.trace.push_back(std::move(col));
  for (auto& tab : mults)
    for (auto& col : tab) T.trace.push_back(col);
  return T;
}

// The interaction trees of prove_blake (air.rs:402-446) and the claimed sums.
inline void blake_full_interaction(BlakeFullTraces& T, const BlakeAllElements& el) {
  const uint32_t log_n = T.log_n;
  const uint32_t rlog[2] = {log_n + 3, log_n + 1};
  const std::vector<std::vector<Column>>& mults = T.mults;
  T.interaction.clear();

  // Scheduler interaction (gen.rs:120-172): round lookups in pairs, then the Blake lookup alone
  // with numerator 0.
  const size_t n = (size_t)1 << log_n;
  const std::vector<Column>& st = T.trace;  // the scheduler's columns come first
  auto round_combine = [&](uint32_t r, size_t row) {
    M31 vals[BR_ROUND_FELTS];
    size_t k = 0;
    for (size_t i = 0; i < 2 * BR_STATE; i++) vals[k++] = st[2 * BR_STATE * (1 + r) + i][row];
    for (size_t i = 0; i < 2 * BR_STATE; i++) vals[k++] = st[2 * BR_STATE * (2 + r) + i][row];
    for (size_t i = 0; i < BR_STATE; i++) {
      vals[k++] = st[2 * B2S_SIGMA[r][i]][row];
      vals[k++] = st[2 * B2S_SIGMA[r][i] + 1][row];
    }
    return el.round.round.combine(vals, BR_ROUND_FELTS);
  };
  auto sched_frac = [&](size_t b, size_t row) -> Frac {
    if (b + 1 < BF_SCHED_BATCHES) {
      QM31 p0 = round_combine((uint32_t)(2 * b), row), p1 = round_combine((uint32_t)(2 * b + 1), row);
      return {p0 + p1, p0 * p1};
    }
    M31 vals[BR_ROUND_FELTS];
    size_t k = 0;
    for (size_t i = 0; i < 2 * BR_STATE; i++) vals[k++] = st[2 * BR_STATE + i][row];
    for (size_t i = 0; i < 2 * BR_STATE; i++) vals[k++] = st[2 * BR_STATE * (1 + BF_ROUNDS) + i][row];
    for (size_t i = 0; i < 2 * BR_STATE; i++) vals[k++] = st[i][row];
    return {QM31(), el.blake.combine(vals, BR_ROUND_FELTS)};
  };
  for (auto& c : logup_trace_fn(BF_SCHED_BATCHES, n, sched_frac, T.scheduler_sum)) T.interaction.push_back(c);
  for (int c = 0; c < 2; c++)
    for (auto& col : blake_round_interaction_trace(rlog[c], T.rxl[c], T.rround[c], el.round, T.round_sums[c]))
      T.interaction.push_back(col);
  // XOR tables (xor_table/gen.rs:40-140): pairs of multiplicity columns, -(m0/p0 + m1/p1); an
  // odd last column alone.
  for (size_t t = 0; t < 5; t++) {
    const XorTableShape& s = BF_XOR_TABLES[t];
    const Relation<3>& rel = el.round.xor_.of(s.elem_bits);
    const uint32_t lb = s.limb_bits(), mask = (1u << lb) - 1;
    auto p_of = [&](size_t col, size_t row) {
      uint32_t ah = (uint32_t)col >> s.expand_bits, bh = (uint32_t)col & ((1u << s.expand_bits) - 1);
      uint32_t a = (ah << lb) | (uint32_t)(row >> lb), b = (bh << lb) | ((uint32_t)row & mask);
      M31 v[3] = {M31(a), M31(b), M31(a ^ b)};
      return rel.combine(v, 3);
    };
    auto xor_frac = [&](size_t b, size_t row) -> Frac {
      size_t c0 = 2 * b;
      QM31 p0 = p_of(c0, row);
      QM31 m0 = QM31(mults[t][c0][row]);
      if (c0 + 1 >= s.n_mult_cols()) return {-m0, p0};
      QM31 p1 = p_of(c0 + 1, row);
      QM31 m1 = QM31(mults[t][c0 + 1][row]);
      return {-(p1 * m0 + p0 * m1), p0 * p1};
    };
    for (auto& col : logup_trace_fn(s.n_batches(), (size_t)1 << s.column_bits(), xor_frac, T.xor_sums[t]))
      T.interaction.push_back(col);
  }
}

// The eight components in air.rs's order, placed with their preprocessed columns (air.rs:185-305).
struct BlakeFullComponents {
  BlakeSchedulerAir sched;
  BlakeRoundFullAir r0, r1;
  std::vector<XorTableAir> xors;
  BlakeFullComponents(uint32_t log_n, const BlakeAllElements* el, QM31 sched_sum, const QM31 round_sums[2],
                      const QM31 xor_sums[5])
      : sched(log_n, el, sched_sum), r0(log_n + 3, el, round_sums[0]), r1(log_n + 1, el, round_sums[1]) {
    for (size_t t = 0; t < 5; t++)
      xors.emplace_back(BF_XOR_TABLES[t], &el->round.xor_.of(BF_XOR_TABLES[t].elem_bits), xor_sums[t]);
  }
  std::vector<Placed> placed() const {
    std::vector<const Air*> airs = {&sched, &r0, &r1};
    std::vector<std::vector<size_t>> pre = {{}, {}, {}};
    for (size_t t = 0; t < 5; t++) {
      airs.push_back(&xors[t]);
      pre.push_back({3 + 4 * t, 4 + 4 * t, 5 + 4 * t});
    }
    return place(airs, pre);
  }
};

// BlakeStatement1::mix_into (air.rs:146-162).
inline void blake_mix_sums(Channel& ch, QM31 sched, const QM31 rounds[2], const QM31 xors[5]) {
  ch.mix_felts({sched, xors[0], xors[1], xors[2], xors[3], xors[4], rounds[0], rounds[1]});
}

// BlakeStatement0::log_sizes (air.rs:87-125): the column log sizes of the three trees.
inline std::vector<std::vector<uint32_t>> blake_log_sizes(uint32_t log_n) {
  std::vector<std::vector<uint32_t>> ls(3);
  ls[0] = {log_n, log_n + 3, log_n + 1};
  for (const XorTableShape& s : BF_XOR_TABLES) ls[0].insert(ls[0].end(), 4, s.column_bits());
  ls[1].insert(ls[1].end(), BF_SCHED_COLS, log_n);
  ls[1].insert(ls[1].end(), BR_TRACE_COLS, log_n + 3);
  ls[1].insert(ls[1].end(), BR_TRACE_COLS, log_n + 1);
  for (const XorTableShape& s : BF_XOR_TABLES) ls[1].insert(ls[1].end(), s.n_mult_cols(), s.column_bits());
  ls[2].insert(ls[2].end(), 4 * BF_SCHED_BATCHES, log_n);
  ls[2].insert(ls[2].end(), 4 * BR_INTERACTION_SECURE, log_n + 3);
  ls[2].insert(ls[2].end(), 4 * BR_INTERACTION_SECURE, log_n + 1);
  for (const XorTableShape& s : BF_XOR_TABLES) ls[2].insert(ls[2].end(), 4 * s.n_batches(), s.column_bits());
  return ls;
}

// prove_blake (air.rs:308-460) for 2^log_n instances. `sums` receives the statement's claimed sums:
// scheduler, round 0, round 1, then the XOR tables 12, 9, 8, 7, 4.
inline StarkProof prove_blake(uint32_t log_n, const PcsConfig& config, QM31 sums[8]) {
  if (log_n < 4) throw std::runtime_error("prove_blake needs log_n >= 4 (LOG_N_LANES)");
  const uint32_t log_max_rows = std::max(log_n + 3, 16u);
  TwiddleTree tw = precompute_twiddles(canonic_domain(log_max_rows + 1 + config.log_blowup).half_coset);
  Channel ch;
  CommitmentSchemeProver pcs;
  pcs.config = config;
  pcs.twiddles = &tw;
  BlakeFullTraces T = blake_full_traces(log_n);
  commit_evals_mixed(pcs, T.preprocessed, ch);
  ch.mix_u64(log_n);
  commit_evals_mixed(pcs, T.trace, ch);
  BlakeAllElements el = BlakeAllElements::draw(ch);
  blake_full_interaction(T, el);
  const BlakeFullTraces& I = T;
  blake_mix_sums(ch, I.scheduler_sum, I.round_sums, I.xor_sums);
  commit_evals_mixed(pcs, I.interaction, ch);
  sums[0] = I.scheduler_sum;
  sums[1] = I.round_sums[0];
  sums[2] = I.round_sums[1];
  for (int t = 0; t < 5; t++) sums[3 + t] = I.xor_sums[t];
  BlakeFullComponents comps(log_n, &el, I.scheduler_sum, I.round_sums, I.xor_sums);
  return prove_components(comps.placed(), ch, pcs);
}

// verify_blake (air.rs:462-520): the claimed sums must add to zero, then verify().
inline std::string verify_blake(uint32_t log_n, const QM31 sums[8], const StarkProof& proof) {
  QM31 total;
  for (int i = 0; i < 8; i++) total = total + sums[i];
  if (total != QM31()) return "claimed sums do not add to zero";
  Channel ch;
  BlakeAllElements el;
  const QM31 rounds[2] = {sums[1], sums[2]};
  const QM31 xors[5] = {sums[3], sums[4], sums[5], sums[6], sums[7]};
  BlakeFullComponents comps(log_n, &el, sums[0], rounds, xors);
  auto hook = [&](size_t t, Channel& c) {
    if (t == 0) {
      c.mix_u64(log_n);
    } else if (t == 1) {
      el = BlakeAllElements::draw(c);
      blake_mix_sums(c, sums[0], rounds, xors);
    }
  };
  return verify_components(comps.placed(), ch, proof, blake_log_sizes(log_n), hook);
}

}  // namespace oracle
