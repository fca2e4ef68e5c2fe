// ORACLE — test infrastructure only (see field.h).
// The Blake2s round AIR: the reference's BlakeRoundComponent proved on its own. Restated from
//   constraints        crates/prover/src/examples/blake/round/constraints.rs:22-206
//   trace generation   crates/prover/src/examples/blake/round/gen.rs:34-235
//   interaction trace  crates/prover/src/examples/blake/round/gen.rs:237-280 with
//                      LogupTraceGenerator (constraint_framework/logup.rs:123-260)
//   relations          crates/prover/src/examples/blake/mod.rs:55-121 (BlakeXorElements),
//                      blake/round/mod.rs:15 (RoundElements), LookupElements (logup.rs:74-121)
//   LogUp constraints  finalize_logup_in_pairs (constraint_framework/mod.rs:180-243)
// The component's XOR lookups and its Round relation entry are not balanced by the scheduler and
// XOR-table components of the full Blake example, so the claimed sum is a public output of the
// proof, as Poseidon2's is. Statement mixing follows the example's statements
// (blake/air.rs:83-183): the log size before the trace commitment, the claimed sum before the
// interaction commitment. The relation elements are drawn in AllElements order without the
// scheduler's (round elements, then the five XOR relations).
#pragma once
#include "air_poseidon.h"

namespace oracle {

constexpr size_t BR_STATE = 16;
constexpr size_t BR_ROUND_FELTS = (BR_STATE + BR_STATE + BR_STATE) * 2;  // 96
constexpr size_t BR_XOR_LOOKUPS = 8 * 4 * 4;                             // 128 xor() calls per row
constexpr size_t BR_TRACE_COLS = 2 * (BR_STATE + BR_STATE) + 8 * 40;     // 384
constexpr size_t BR_INTERACTION_SECURE = BR_XOR_LOOKUPS / 2 + 1;          // 65
constexpr size_t BR_N_CONSTRAINTS = 8 * 4 * 2 + BR_INTERACTION_SECURE;   // 129

// LookupElements<N> (logup.rs:74-121): draw z, alpha; combine = sum alpha^i v_i - z.
template <size_t N>
struct Relation {
  QM31 z, alpha;
  QM31 alpha_powers[N];
  static Relation draw(Channel& ch) {
    Relation r;
    auto v = ch.draw_felts(2);
    r.z = v[0];
    r.alpha = v[1];
    QM31 cur(M31(1));
    for (size_t i = 0; i < N; i++) {
      r.alpha_powers[i] = cur;
      cur = cur * r.alpha;
    }
    return r;
  }
  template <class F>
  QM31 combine(const F* v, size_t n) const {
    QM31 acc;
    for (size_t i = 0; i < n; i++) acc = acc + alpha_powers[i] * v[i];
    return acc - z;
  }
};

// BlakeXorElements (blake/mod.rs:55-121): one 3-element relation per XOR width.
struct BlakeXorRelations {
  Relation<3> xor12, xor9, xor8, xor7, xor4;
  static BlakeXorRelations draw(Channel& ch) {
    BlakeXorRelations r;
    r.xor12 = Relation<3>::draw(ch);
    r.xor9 = Relation<3>::draw(ch);
    r.xor8 = Relation<3>::draw(ch);
    r.xor7 = Relation<3>::draw(ch);
    r.xor4 = Relation<3>::draw(ch);
    return r;
  }
  const Relation<3>& of(uint32_t w) const {
    switch (w) {
      case 12: return xor12;
      case 9: return xor9;
      case 8: return xor8;
      case 7: return xor7;
      case 4: return xor4;
    }
    throw std::runtime_error("invalid xor width");
  }
};

struct BlakeRoundElements {
  Relation<BR_ROUND_FELTS> round;
  BlakeXorRelations xor_;
  static BlakeRoundElements draw(Channel& ch) {
    BlakeRoundElements e;
    e.round = Relation<BR_ROUND_FELTS>::draw(ch);
    e.xor_ = BlakeXorRelations::draw(ch);
    return e;
  }
};

// The round's constraints (round/constraints.rs:22-206) and its LogUp relation entries, then
// finalize_logup_in_pairs. E is DomainEvaluator (F = M31) or PointEvaluator (F = QM31).
template <class E>
struct BlakeRoundEvaluator {
  using F = typename E::F;
  E& e;
  const BlakeRoundElements& el;
  std::vector<Frac> fracs;
  BlakeRoundEvaluator(E& ev, const BlakeRoundElements& l) : e(ev), el(l) {}

  static F c(uint32_t x) { return F(M31(x)); }
  struct U32 {
    F l, h;
  };
  U32 next_u32() {
    F l = e.next_trace_mask();
    F h = e.next_trace_mask();
    return {l, h};
  }
  U32 add2(const U32& a, const U32& b) {
    F sl = e.next_trace_mask(), sh = e.next_trace_mask();
    F carry_l = (a.l + b.l - sl) * M31(1u << 15);  // INV16 = 2^-16 = 2^15 mod P
    e.add_constraint(carry_l * carry_l - carry_l);
    F carry_h = (a.h + b.h + carry_l - sh) * M31(1u << 15);
    e.add_constraint(carry_h * carry_h - carry_h);
    return {sl, sh};
  }
  U32 add3(const U32& a, const U32& b, const U32& d) {
    F sl = e.next_trace_mask(), sh = e.next_trace_mask();
    F carry_l = (a.l + b.l + d.l - sl) * M31(1u << 15);
    e.add_constraint(carry_l * (carry_l - c(1)) * (carry_l - c(2)));
    F carry_h = (a.h + b.h + d.h + carry_l - sh) * M31(1u << 15);
    e.add_constraint(carry_h * (carry_h - c(1)) * (carry_h - c(2)));
    return {sl, sh};
  }
  // (l, h) with a = l + h * 2^r, h from the trace.
  void split(const F& a, uint32_t r, F& l, F& h) {
    h = e.next_trace_mask();
    l = a - h * M31(1u << r);
  }
  void xor2(uint32_t w, const F a[2], const F b[2], F out[2]) {
    out[0] = e.next_trace_mask();
    out[1] = e.next_trace_mask();
    const Relation<3>& rel = el.xor_.of(w);
    for (int k = 0; k < 2; k++) {
      F v[3] = {a[k], b[k], out[k]};
      fracs.push_back({QM31(M31(1)), rel.combine(v, 3)});
    }
  }
  U32 xor_rotr(const U32& a, const U32& b, uint32_t r) {
    F all, alh, ahl, ahh, bll, blh, bhl, bhh;
    split(a.l, r, all, alh);
    split(a.h, r, ahl, ahh);
    split(b.l, r, bll, blh);
    split(b.h, r, bhl, bhh);
    F x0[2], x1[2];
    {
      F aa[2] = {all, ahl}, bb[2] = {bll, bhl};
      xor2(r, aa, bb, x0);
    }
    {
      F aa[2] = {alh, ahh}, bb[2] = {blh, bhh};
      xor2(16 - r, aa, bb, x1);
    }
    // x0 = [xorll, xorhl], x1 = [xorlh, xorhh]
    return {x0[1] * M31(1u << (16 - r)) + x1[0], x0[0] * M31(1u << (16 - r)) + x1[1]};
  }
  U32 xor_rotr16(const U32& a, const U32& b) {
    F all, alh, ahl, ahh, bll, blh, bhl, bhh;
    split(a.l, 8, all, alh);
    split(a.h, 8, ahl, ahh);
    split(b.l, 8, bll, blh);
    split(b.h, 8, bhl, bhh);
    F x0[2], x1[2];
    {
      F aa[2] = {all, ahl}, bb[2] = {bll, bhl};
      xor2(8, aa, bb, x0);
    }
    {
      F aa[2] = {alh, ahh}, bb[2] = {blh, bhh};
      xor2(8, aa, bb, x1);
    }
    // x0 = [xorll, xorhl], x1 = [xorlh, xorhh]: l = xorhh * 2^8 + xorhl, h = xorlh * 2^8 + xorll
    return {x1[1] * M31(1u << 8) + x0[1], x1[0] * M31(1u << 8) + x0[0]};
  }
  void g(U32& a, U32& b, U32& cc, U32& d, const U32& m0, const U32& m1) {
    a = add3(a, b, m0);
    d = xor_rotr16(a, d);
    cc = add2(cc, d);
    b = xor_rotr(b, cc, 12);
    a = add3(a, b, m1);
    d = xor_rotr(a, d, 8);
    cc = add2(cc, d);
    b = xor_rotr(b, cc, 7);
  }
  void eval(QM31 cumsum_shift) {
    U32 v[BR_STATE], m[BR_STATE];
    for (size_t i = 0; i < BR_STATE; i++) v[i] = next_u32();
    U32 in[BR_STATE];
    for (size_t i = 0; i < BR_STATE; i++) in[i] = v[i];
    for (size_t i = 0; i < BR_STATE; i++) m[i] = next_u32();
    g(v[0], v[4], v[8], v[12], m[0], m[1]);
    g(v[1], v[5], v[9], v[13], m[2], m[3]);
    g(v[2], v[6], v[10], v[14], m[4], m[5]);
    g(v[3], v[7], v[11], v[15], m[6], m[7]);
    g(v[0], v[5], v[10], v[15], m[8], m[9]);
    g(v[1], v[6], v[11], v[12], m[10], m[11]);
    g(v[2], v[7], v[8], v[13], m[12], m[13]);
    g(v[3], v[4], v[9], v[14], m[14], m[15]);
    // Round(input_v, output_v, message) with multiplicity -1.
    F vals[BR_ROUND_FELTS];
    size_t k = 0;
    for (size_t i = 0; i < BR_STATE; i++) vals[k++] = in[i].l, vals[k++] = in[i].h;
    for (size_t i = 0; i < BR_STATE; i++) vals[k++] = v[i].l, vals[k++] = v[i].h;
    for (size_t i = 0; i < BR_STATE; i++) vals[k++] = m[i].l, vals[k++] = m[i].h;
    fracs.push_back({-QM31(M31(1)), el.round.combine(vals, BR_ROUND_FELTS)});
    finalize_in_pairs(cumsum_shift);
  }
  // finalize_logup_batched with batch(n) = n / 2 (constraint_framework/mod.rs:180-243).
  void finalize_in_pairs(QM31 cumsum_shift) {
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
};

struct BlakeRoundAir : Air {
  uint32_t log_n;
  BlakeRoundElements el;
  QM31 claimed_sum;
  BlakeRoundAir(uint32_t l, const BlakeRoundElements& e, QM31 cs) : log_n(l), el(e), claimed_sum(cs) {}
  uint32_t log_size() const override { return log_n; }
  uint32_t max_constraint_log_degree_bound() const override { return log_n + 1; }
  size_t n_constraints() const override { return BR_N_CONSTRAINTS; }
  Mask mask_offsets() const override {
    Mask m(3);
    m[1].assign(BR_TRACE_COLS, {0});
    for (size_t b = 0; b + 1 < BR_INTERACTION_SECURE; b++)
      for (int k = 0; k < 4; k++) m[2].push_back({0});
    for (int k = 0; k < 4; k++) m[2].push_back({-1, 0});
    return m;
  }
  QM31 shift() const { return claimed_sum * inv(M31(1u << log_n)); }
  QM31 eval_row(DomainEvaluator& e) const override {
    BlakeRoundEvaluator<DomainEvaluator> ev(e, el);
    ev.eval(shift());
    return e.row_res;
  }
  void eval_point(PointEvaluator& e) const override {
    BlakeRoundEvaluator<PointEvaluator> ev(e, el);
    ev.eval(shift());
  }
};

// One XOR lookup of the trace generator: width and the (a, b, a ^ b) columns.
struct BrXorLookup {
  uint32_t w;
  std::vector<M31> a, b, c;
};

// TraceGeneratorRow::generate (round/gen.rs:75-204) for row r, writing the trace columns, the
// 128 XOR lookups and the 96 Round lookup values.
struct BrRowGen {
  std::vector<Column>& t;
  std::vector<BrXorLookup>& xl;
  std::vector<std::vector<M31>>& round;
  size_t r, col = 0, xi = 0;
  void felt(uint32_t v) { t[col++][r] = M31(v); }
  void u32(uint32_t v) {
    felt(v & 0xffffu);
    felt(v >> 16);
  }
  uint32_t add2(uint32_t a, uint32_t b) {
    uint32_t s = a + b;
    u32(s);
    return s;
  }
  uint32_t add3(uint32_t a, uint32_t b, uint32_t c) {
    uint32_t s = a + b + c;
    u32(s);
    return s;
  }
  void split(uint32_t a, uint32_t rr, uint32_t& l, uint32_t& h) {
    h = a >> rr;
    l = a & ((1u << rr) - 1);
    felt(h);
  }
  uint32_t xor1(uint32_t w, uint32_t a, uint32_t b) {
    uint32_t c = a ^ b;
    felt(c);
    BrXorLookup& L = xl[xi++];
    L.w = w;
    L.a[r] = M31(a);
    L.b[r] = M31(b);
    L.c[r] = M31(c);
    return c;
  }
  uint32_t xor_rotr(uint32_t a, uint32_t b, uint32_t rr) {
    uint32_t c = a ^ b;
    uint32_t cr = (c >> rr) | (c << (32 - rr));
    uint32_t all, alh, ahl, ahh, bll, blh, bhl, bhh;
    split(a & 0xffffu, rr, all, alh);
    split(a >> 16, rr, ahl, ahh);
    split(b & 0xffffu, rr, bll, blh);
    split(b >> 16, rr, bhl, bhh);
    xor1(rr, all, bll);
    xor1(rr, ahl, bhl);
    xor1(16 - rr, alh, blh);
    xor1(16 - rr, ahh, bhh);
    return cr;
  }
  uint32_t xor_rotr16(uint32_t a, uint32_t b) {
    uint32_t c = a ^ b;
    uint32_t cr = (c >> 16) | (c << 16);
    uint32_t all, alh, ahl, ahh, bll, blh, bhl, bhh;
    split(a & 0xffffu, 8, all, alh);
    split(a >> 16, 8, ahl, ahh);
    split(b & 0xffffu, 8, bll, blh);
    split(b >> 16, 8, bhl, bhh);
    xor1(8, all, bll);
    xor1(8, ahl, bhl);
    xor1(8, alh, blh);
    xor1(8, ahh, bhh);
    return cr;
  }
  void g(uint32_t& a, uint32_t& b, uint32_t& c, uint32_t& d, uint32_t m0, uint32_t m1) {
    a = add3(a, b, m0);
    d = xor_rotr16(a, d);
    c = add2(c, d);
    b = xor_rotr(b, c, 12);
    a = add3(a, b, m1);
    d = xor_rotr(a, d, 8);
    c = add2(c, d);
    b = xor_rotr(b, c, 7);
  }
  void generate(const uint32_t* vin, const uint32_t* m) {
    uint32_t v[BR_STATE];
    for (size_t i = 0; i < BR_STATE; i++) v[i] = vin[i];
    for (size_t i = 0; i < BR_STATE; i++) u32(v[i]);
    for (size_t i = 0; i < BR_STATE; i++) u32(m[i]);
    g(v[0], v[4], v[8], v[12], m[0], m[1]);
    g(v[1], v[5], v[9], v[13], m[2], m[3]);
    g(v[2], v[6], v[10], v[14], m[4], m[5]);
    g(v[3], v[7], v[11], v[15], m[6], m[7]);
    g(v[0], v[5], v[10], v[15], m[8], m[9]);
    g(v[1], v[6], v[11], v[12], m[10], m[11]);
    g(v[2], v[7], v[8], v[13], m[12], m[13]);
    g(v[3], v[4], v[9], v[14], m[14], m[15]);
    size_t k = 0;
    auto put = [&](uint32_t x) {
      round[k++][r] = M31(x & 0xffffu);
      round[k++][r] = M31(x >> 16);
    };
    for (size_t i = 0; i < BR_STATE; i++) put(vin[i]);
    for (size_t i = 0; i < BR_STATE; i++) put(v[i]);
    for (size_t i = 0; i < BR_STATE; i++) put(m[i]);
  }
};

// generate_trace (round/gen.rs:206-235) from explicit inputs: inputs[(row * 32) + i], the 16 state
// words then the 16 message words of row `row`.
inline std::vector<Column> blake_round_trace(uint32_t log_n, const uint32_t* inputs, std::vector<BrXorLookup>& xl,
                                             std::vector<std::vector<M31>>& round) {
  size_t n = (size_t)1 << log_n;
  std::vector<Column> t(BR_TRACE_COLS, Column(n));
  xl.assign(BR_XOR_LOOKUPS, BrXorLookup{0, std::vector<M31>(n), std::vector<M31>(n), std::vector<M31>(n)});
  round.assign(BR_ROUND_FELTS, std::vector<M31>(n));
#pragma omp parallel for schedule(static)
  for (long r = 0; r < (long)n; r++) {
    BrRowGen g{t, xl, round, (size_t)r};
    g.generate(inputs + (size_t)r * 32, inputs + (size_t)r * 32 + 16);
  }
  return t;
}

// The reference test's inputs (round/mod.rs:60-110): v_i = i, m_i = i + 1 on every row.
inline std::vector<uint32_t> blake_round_reference_inputs(uint32_t log_n) {
  size_t n = (size_t)1 << log_n;
  std::vector<uint32_t> v(n * 32);
  for (size_t r = 0; r < n; r++)
    for (size_t i = 0; i < 16; i++) {
      v[r * 32 + i] = (uint32_t)i;
      v[r * 32 + 16 + i] = (uint32_t)(i + 1);
    }
  return v;
}

// generate_interaction_trace (round/gen.rs:237-280): one column per pair of XOR lookups
// (1/p0 + 1/p1 = (p0 + p1) / (p0 p1)), then one for the Round relation (-1 / p), each added to
// the previous column; the last one shifted by claimed_sum / 2^log_n and prefix-summed
// (LogupTraceGenerator::finalize_last, logup.rs:150-190).
inline std::vector<Column> blake_round_interaction_trace(uint32_t log_n, const std::vector<BrXorLookup>& xl,
                                                         const std::vector<std::vector<M31>>& round,
                                                         const BlakeRoundElements& el, QM31& claimed_sum) {
  size_t n = (size_t)1 << log_n;
  std::vector<SecureColumn> cols;
  for (size_t p = 0; p + 1 < BR_INTERACTION_SECURE; p++) {
    const BrXorLookup& l0 = xl[2 * p];
    const BrXorLookup& l1 = xl[2 * p + 1];
    SecureColumn c(n);
#pragma omp parallel for schedule(static)
    for (long r = 0; r < (long)n; r++) {
      M31 v0[3] = {l0.a[r], l0.b[r], l0.c[r]}, v1[3] = {l1.a[r], l1.b[r], l1.c[r]};
      QM31 p0 = el.xor_.of(l0.w).combine(v0, 3), p1 = el.xor_.of(l1.w).combine(v1, 3);
      QM31 val = (p0 + p1) * inv(p0 * p1);
      c.set(r, val + (cols.empty() ? QM31() : cols.back().at(r)));
    }
    cols.push_back(c);
  }
  {
    SecureColumn c(n);
#pragma omp parallel for schedule(static)
    for (long r = 0; r < (long)n; r++) {
      M31 v[BR_ROUND_FELTS];
      for (size_t k = 0; k < BR_ROUND_FELTS; k++) v[k] = round[k][r];
      QM31 p = el.round.combine(v, BR_ROUND_FELTS);
      c.set(r, -QM31(M31(1)) * inv(p) + cols.back().at(r));
    }
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
