// ORACLE — test infrastructure only (see field.h).
// prove() for several components, and the Plonk and state-machine example provers, restated from
// the reference:
//   prove                      crates/prover/src/core/prover/mod.rs:27-79
//   Components                 crates/prover/src/core/air/components.rs:15-137
//   DomainEvaluationAccumulator crates/prover/src/core/air/accumulation.rs:49-149
//   TraceLocationAllocator     crates/prover/src/constraint_framework/component.rs:45-175
//   LogupTraceGenerator        crates/prover/src/constraint_framework/logup.rs:123-260
//   prove_fibonacci_plonk      crates/prover/src/examples/plonk/mod.rs:153-266
//   prove_state_machine        crates/prover/src/examples/state_machine/mod.rs:26-135, gen.rs:20-89
#pragma once
#include "air_examples.h"

namespace oracle {

// A component placed in the trees: its columns [start, end) of each tree t >= 1 (allocated in
// component order), and the indices of the preprocessed columns it reads.
struct Placed {
  const Air* air;
  std::vector<std::pair<size_t, size_t>> spans;
  std::vector<size_t> preprocessed;
};

inline std::vector<Placed> place(const std::vector<const Air*>& airs, const std::vector<std::vector<size_t>>& pre) {
  std::vector<Placed> out;
  std::vector<size_t> next;
  for (size_t k = 0; k < airs.size(); k++) {
    Placed p{airs[k], {}, pre[k]};
    Mask m = airs[k]->mask_offsets();
    for (size_t t = 1; t < m.size(); t++) {
      if (next.size() <= t) next.resize(t + 1, 0);
      p.spans.push_back({next[t], next[t] + m[t].size()});
      next[t] += m[t].size();
    }
    out.push_back(p);
  }
  return out;
}

// coset_index_to_circle_domain_index (crates/prover/src/core/utils.rs:137-143).
inline size_t coset_index_to_circle_domain_index(size_t i, uint32_t log) {
  return i % 2 == 0 ? i / 2 : ((((size_t)2) << log) - i) / 2;
}

// PcsConfig::mix_into (crates/prover/src/core/pcs/mod.rs:42-49, fri.rs:80-89).
inline void mix_config(const PcsConfig& c, Channel& ch) {
  ch.mix_u64(c.pow_bits);
  ch.mix_u64(c.log_blowup);
  ch.mix_u64(c.n_queries);
  ch.mix_u64(c.log_last_layer);
}

inline QM31 from_partial_evals(const QM31 v[4]) {
  return v[0] + v[1] * QM31::from_u32(0, 1, 0, 0) + v[2] * QM31::from_u32(0, 0, 1, 0) + v[3] * QM31::from_u32(0, 0, 0, 1);
}

// prove() over several components. `pcs` holds the preprocessed, trace and interaction trees.
inline StarkProof prove_components(const std::vector<Placed>& comps, Channel& ch, CommitmentSchemeProver& pcs) {
  QM31 rc = ch.draw_felt();
  size_t total = 0;
  uint32_t comp_log = 0;
  for (auto& c : comps) {
    total += c.air->n_constraints();
    comp_log = std::max(comp_log, c.air->max_constraint_log_degree_bound());
  }
  std::vector<QM31> powers = generate_secure_powers(rc, total);
  std::map<uint32_t, SecureColumn> sub;
  for (auto& c : comps) {
    const Air& air = *c.air;
    size_t n = air.n_constraints();
    // DomainEvaluationAccumulator::columns: the last n powers, reversed by the component.
    std::vector<QM31> coeffs(powers.end() - n, powers.end());
    powers.resize(powers.size() - n);
    std::reverse(coeffs.begin(), coeffs.end());
    uint32_t trace_log = air.log_size(), eval_log = air.max_constraint_log_degree_bound();
    CircleDomain ed = canonic_domain(eval_log);
    TwiddleTree etw = precompute_twiddles(ed.half_coset);
    Mask m = air.mask_offsets();
    std::vector<std::vector<Column>> ext(m.size());
    std::vector<std::vector<const Column*>> tr(m.size());
    for (size_t t = 0; t < m.size(); t++) {
      std::vector<const Column*> polys;
      if (t == 0)
        for (size_t idx : c.preprocessed) polys.push_back(&pcs.trees[0].polys[idx]);
      else
        for (size_t i = c.spans[t - 1].first; i < c.spans[t - 1].second; i++) polys.push_back(&pcs.trees[t].polys[i]);
      ext[t].resize(polys.size());
#pragma omp parallel for schedule(dynamic)
      for (long i = 0; i < (long)polys.size(); i++) ext[t][i] = evaluate(ed, *polys[i], etw);
      for (auto& e : ext[t]) tr[t].push_back(&e);
    }
    uint32_t expand = eval_log - trace_log;
    Coset tc = canonic_coset(trace_log);
    std::vector<M31> dinv;
    for (size_t i = 0; i < ((size_t)1 << expand); i++) dinv.push_back(inv(coset_vanishing(tc, ed.at(i))));
    bit_reverse(dinv);
    auto it = sub.find(eval_log);
    if (it == sub.end()) it = sub.emplace(eval_log, SecureColumn(ed.size())).first;
    SecureColumn& acc = it->second;
#pragma omp parallel for schedule(static)
    for (long r = 0; r < (long)ed.size(); r++) {
      DomainEvaluator e(&tr, r, trace_log, eval_log, coeffs.data());
      acc.set(r, acc.at(r) + air.eval_row(e) * dinv[r >> trace_log]);
    }
  }
  // DomainEvaluationAccumulator::finalize: smallest size first; each polynomial is evaluated on the
  // next size's domain and added there, then that size is interpolated.
  TwiddleTree ftw = precompute_twiddles(canonic_domain(comp_log).half_coset);
  std::vector<Column> cur;
  for (auto& [log, vals] : sub) {
    CircleDomain d = canonic_domain(log);
    if (!cur.empty())
      for (int k = 0; k < 4; k++) {
        Column e = evaluate(d, cur[k], ftw);
        for (size_t r = 0; r < e.size(); r++) vals.c[k][r] = vals.c[k][r] + e[r];
      }
    cur.clear();
    for (int k = 0; k < 4; k++) cur.push_back(interpolate(d, vals.c[k], ftw));
  }
  pcs.commit(cur, ch);
  // Components::mask_points (components.rs:30-50).
  CirclePointQM31 oods = random_point(ch);
  std::vector<std::vector<std::vector<CirclePointQM31>>> pts(pcs.trees.size());
  pts[0].assign(pcs.trees[0].polys.size(), {});
  for (auto& c : comps) {
    auto mp = mask_points(*c.air, oods);
    for (size_t t = 1; t < mp.size(); t++)
      for (auto& col : mp[t]) pts[t].push_back(col);
    for (size_t idx : c.preprocessed) pts[0][idx] = {oods};
  }
  pts.back() = std::vector<std::vector<CirclePointQM31>>(4, {oods});
  StarkProof proof = pcs.prove_values(pts, ch);
  // Components::eval_composition_polynomial_at_point: one accumulator across the components.
  QM31 acc;
  for (auto& c : comps) {
    MaskValues mv(c.air->mask_offsets().size());
    for (size_t idx : c.preprocessed) mv[0].push_back(proof.sampled_values[0][idx]);
    for (size_t t = 1; t < mv.size(); t++)
      for (size_t i = c.spans[t - 1].first; i < c.spans[t - 1].second; i++) mv[t].push_back(proof.sampled_values[t][i]);
    QM31 dinv = inv(coset_vanishing(canonic_coset(c.air->log_size()), oods));
    PointEvaluator e(&mv, &acc, rc, dinv);
    c.air->eval_point(e);
  }
  const auto& comp = proof.sampled_values.back();
  QM31 parts[4] = {comp[0][0], comp[1][0], comp[2][0], comp[3][0]};
  if (from_partial_evals(parts) != acc) throw std::runtime_error("ConstraintsNotSatisfied");
  return proof;
}

// verify() for placed components (prover/mod.rs:81-127 with Components' mask points and
// composition at the point). `trace_log_sizes[t]` are the committed trees' column log sizes.
inline std::string verify_components(const std::vector<Placed>& comps, Channel& ch, const StarkProof& proof,
                                     const std::vector<std::vector<uint32_t>>& trace_log_sizes,
                                     const std::function<void(size_t, Channel&)>& after_tree) {
  VerifyAir va;
  va.composition_log = 0;
  for (auto& c : comps) va.composition_log = std::max(va.composition_log, c.air->max_constraint_log_degree_bound());
  va.mask_points = [&](CirclePointQM31 oods) {
    std::vector<std::vector<std::vector<CirclePointQM31>>> pts(trace_log_sizes.size());
    pts[0].assign(trace_log_sizes[0].size(), {});
    for (auto& c : comps) {
      auto mp = mask_points(*c.air, oods);
      for (size_t t = 1; t < mp.size(); t++)
        for (auto& col : mp[t]) pts[t].push_back(col);
      for (size_t idx : c.preprocessed) pts[0][idx] = {oods};
    }
    return pts;
  };
  va.composition_at = [&](CirclePointQM31 oods, const MaskValues& all, QM31 rc) {
    QM31 acc;
    for (auto& c : comps) {
      MaskValues mv(c.air->mask_offsets().size());
      for (size_t idx : c.preprocessed) mv[0].push_back(all[0][idx]);
      for (size_t t = 1; t < mv.size(); t++)
        for (size_t i = c.spans[t - 1].first; i < c.spans[t - 1].second; i++) mv[t].push_back(all[t][i]);
      QM31 dinv = inv(coset_vanishing(canonic_coset(c.air->log_size()), oods));
      PointEvaluator e(&mv, &acc, rc, dinv);
      c.air->eval_point(e);
    }
    return acc;
  };
  return verify_with(va, ch, proof, trace_log_sizes, after_tree);
}

inline void commit_evals_mixed(CommitmentSchemeProver& pcs, const std::vector<Column>& evals, Channel& ch) {
  std::vector<Column> polys(evals.size());
#pragma omp parallel for schedule(dynamic)
  for (long i = 0; i < (long)evals.size(); i++)
    polys[i] = interpolate(canonic_domain(ilog2(evals[i].size())), evals[i], *pcs.twiddles);
  pcs.commit(std::move(polys), ch);
}

// LogupTraceGenerator (logup.rs:123-260) from per-batch fractions: each column the running sum
// over batches of num / den; the last one shifted by claimed_sum / n and prefix-summed in coset
// order.
inline std::vector<Column> logup_trace(const std::vector<std::vector<Frac>>& batches, size_t n, QM31& claimed_sum) {
  std::vector<SecureColumn> cols;
  for (size_t b = 0; b < batches.size(); b++) {
    SecureColumn c(n);
    for (size_t r = 0; r < n; r++) {
      QM31 v = batches[b][r].num * inv(batches[b][r].den);
      c.set(r, v + (b ? cols.back().at(r) : QM31()));
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

// prove_fibonacci_plonk (plonk/mod.rs:153-266): a Fibonacci circuit of 2^log_n gates.
inline StarkProof prove_plonk(uint32_t log_n, const PcsConfig& config, QM31* claimed = nullptr) {
  size_t n = (size_t)1 << log_n;
  std::vector<M31> fib = {M31(1), M31(1)};
  for (size_t i = 0; i < n; i++) fib.push_back(fib[fib.size() - 1] + fib[fib.size() - 2]);
  Column mult(n), a_wire(n), b_wire(n), c_wire(n), op(n), a_val(n), b_val(n), c_val(n);
  for (size_t i = 0; i < n; i++) {
    mult[i] = M31(2);
    a_wire[i] = M31((uint32_t)i);
    b_wire[i] = M31((uint32_t)(i + 1));
    c_wire[i] = M31((uint32_t)(i + 2));
    op[i] = M31(1);
    a_val[i] = fib[i];
    b_val[i] = fib[i + 1];
    c_val[i] = fib[i + 2];
  }
  mult[n - 1] = M31(0);
  mult[n - 2] = M31(1);
  TwiddleTree tw = precompute_twiddles(canonic_domain(log_n + config.log_blowup + 1).half_coset);
  Channel ch;
  CommitmentSchemeProver pcs;
  pcs.config = config;
  pcs.twiddles = &tw;
  pcs.commit_evals({a_wire, b_wire, c_wire, op}, log_n, ch);
  pcs.commit_evals({mult, a_val, b_val, c_val}, log_n, ch);
  Relation<2> rel = Relation<2>::draw(ch);
  // gen_interaction_trace (plonk/mod.rs:111-151): (a, b) lookups in one column, c in the next.
  std::vector<std::vector<Frac>> batches(2, std::vector<Frac>(n));
  for (size_t r = 0; r < n; r++) {
    M31 va[2] = {a_wire[r], a_val[r]}, vb[2] = {b_wire[r], b_val[r]}, vc[2] = {c_wire[r], c_val[r]};
    QM31 q0 = rel.combine(va, 2), q1 = rel.combine(vb, 2), q2 = rel.combine(vc, 2);
    batches[0][r] = {q0 + q1, q0 * q1};
    batches[1][r] = {QM31(M31(0) - mult[r]), q2};
  }
  QM31 cs;
  pcs.commit_evals(logup_trace(batches, n, cs), log_n, ch);
  if (claimed) *claimed = cs;
  PlonkAir air(log_n, rel, cs);
  return prove_components(place({&air}, {{0, 1, 2, 3}}), ch, pcs);
}

// prove_state_machine (state_machine/mod.rs:26-135): transitions of coordinate 0 over 2^log_n rows,
// then of coordinate 1 over 2^(log_n - 1) rows.
inline StarkProof prove_state_machine(uint32_t log_n, const uint32_t initial[2], const PcsConfig& config,
                                      QM31 claimed[2]) {
  const uint32_t logs[2] = {log_n, log_n - 1};
  M31 state[2] = {M31(initial[0]), M31(initial[1])};
  std::vector<Column> traces[2];
  for (int k = 0; k < 2; k++) {
    // gen_trace (gen.rs:20-48): row i holds the state plus i in coordinate k, stored at the
    // bit-reversed circle-domain position of coset index i.
    size_t n = (size_t)1 << logs[k];
    traces[k].assign(2, Column(n));
    M31 cur[2] = {state[0], state[1]};
    for (size_t i = 0; i < n; i++) {
      size_t pos = bit_reverse_index(coset_index_to_circle_domain_index(i, logs[k]), logs[k]);
      traces[k][0][pos] = cur[0];
      traces[k][1][pos] = cur[1];
      cur[k] = cur[k] + M31(1);
    }
    state[k] = state[k] + M31((uint32_t)n);
  }
  TwiddleTree tw = precompute_twiddles(canonic_domain(log_n + config.log_blowup + 1).half_coset);
  Channel ch;
  mix_config(config, ch);
  CommitmentSchemeProver pcs;
  pcs.config = config;
  pcs.twiddles = &tw;
  pcs.commit({}, ch);
  ch.mix_u64(logs[0]);
  ch.mix_u64(logs[1]);
  commit_evals_mixed(pcs, {traces[0][0], traces[0][1], traces[1][0], traces[1][1]}, ch);
  Relation<2> rel = Relation<2>::draw(ch);
  std::vector<Column> inter;
  for (int k = 0; k < 2; k++) {
    size_t n = (size_t)1 << logs[k];
    std::vector<std::vector<Frac>> b(1, std::vector<Frac>(n));
    for (size_t r = 0; r < n; r++) {
      M31 in[2] = {traces[k][0][r], traces[k][1][r]}, out[2] = {in[0], in[1]};
      out[k] = out[k] + M31(1);
      QM31 di = rel.combine(in, 2), dout = rel.combine(out, 2);
      b[0][r] = {dout - di, di * dout};
    }
    for (auto& c : logup_trace(b, n, claimed[k])) inter.push_back(c);
  }
  ch.mix_felts({claimed[0], claimed[1]});
  commit_evals_mixed(pcs, inter, ch);
  StateTransitionAir a0(0, logs[0], rel, claimed[0]), a1(1, logs[1], rel, claimed[1]);
  return prove_components(place({&a0, &a1}, {{}, {}}), ch, pcs);
}

}  // namespace oracle
