// ORACLE — test infrastructure only (see field.h).
// Fiat-Shamir channel, polynomial commitment scheme, FRI, prove / verify and the canonical proof
// serialisation, restated from the reference:
//   channel     crates/prover/src/core/channel/blake2s.rs:15-110, vcs/blake2_merkle.rs:36-45
//   queries     crates/prover/src/core/queries.rs:21-52
//   FRI         crates/prover/src/core/fri.rs:168-336 (prover), :338-590 (verifier), :860-1031
//   PCS         crates/prover/src/core/pcs/prover.rs:25-243, pcs/verifier.rs:13-120,
//               pcs/quotients.rs:76-197
//   composition crates/prover/src/core/air/accumulation.rs:49-149, air/components.rs:122-137,
//               constraint_framework/component.rs:278-416
//   prove       crates/prover/src/core/prover/mod.rs:27-127
// The reference serialises proofs with serde only; the byte format here (little-endian u32 words,
// u64 lengths, fields in struct order) is this project's canonical form, applied identically to
// oracle and GPU proofs.
#pragma once
#include "ops.h"
#include <set>
#include <stdexcept>
#include <cstring>
#include <functional>

namespace oracle {

// ---------------------------------------------------------------- channel
struct Channel {
  Hash32 digest{};
  uint64_t n_sent = 0;
  uint64_t n_challenges = 0;

  void update_digest(const Hash32& d) {
    digest = d;
    n_challenges++;
    n_sent = 0;
  }
  void mix_root(const Hash32& root) {
    Blake2s s;
    s.update(digest.b, 32);
    s.update(root.b, 32);
    update_digest(s.finalize());
  }
  void mix_felts(const std::vector<QM31>& felts) {
    Blake2s s;
    s.update(digest.b, 32);
    for (auto& f : felts) {
      uint32_t w[4] = {f.a.a.v, f.a.b.v, f.b.a.v, f.b.b.v};
      s.update(w, 16);
    }
    update_digest(s.finalize());
  }
  void mix_u64(uint64_t v) {
    uint32_t h[8], m[16] = {0};
    digest.words(h);
    m[0] = (uint32_t)v;
    m[1] = (uint32_t)(v >> 32);
    auto r = b2s_compress(h, m, 0, 0, 0, 0);
    update_digest(Hash32::from_words(r.data()));
  }
  Hash32 draw_random_bytes() {
    uint8_t in[64] = {0};
    std::memcpy(in, digest.b, 32);
    uint64_t c = n_sent;
    std::memcpy(in + 32, &c, 8);
    n_sent++;
    return Blake2s::hash(in, 64);
  }
  std::array<M31, 8> draw_base_felts() {
    while (true) {
      Hash32 h = draw_random_bytes();
      uint32_t w[8];
      h.words(w);
      bool ok = true;
      for (int i = 0; i < 8; i++) ok = ok && w[i] < 2 * P;
      if (ok) {
        std::array<M31, 8> r;
        for (int i = 0; i < 8; i++) r[i] = M31::reduce(w[i]);
        return r;
      }
    }
  }
  QM31 draw_felt() {
    auto f = draw_base_felts();
    return QM31::from_m31(f[0], f[1], f[2], f[3]);
  }
  std::vector<QM31> draw_felts(size_t n) {
    std::vector<QM31> out;
    while (out.size() < n) {
      auto f = draw_base_felts();
      out.push_back(QM31::from_m31(f[0], f[1], f[2], f[3]));
      if (out.size() < n) out.push_back(QM31::from_m31(f[4], f[5], f[6], f[7]));
    }
    return out;
  }
  uint32_t trailing_zeros() const {
    for (int i = 0; i < 16; i++)
      if (digest.b[i]) return 8 * i + (uint32_t)__builtin_ctz(digest.b[i]);
    return 128;
  }
};

// CirclePoint::get_random_point (circle.rs:170-183)
inline CirclePointQM31 random_point(Channel& ch) {
  QM31 t = ch.draw_felt();
  QM31 t2 = t * t;
  QM31 d = inv(t2 + M31(1));
  QM31 one(M31(1));
  return {(one - t2) * d, (t + t) * d};
}

// ---------------------------------------------------------------- config / proof
struct PcsConfig {
  uint32_t pow_bits = 5;
  uint32_t log_blowup = 1;
  uint32_t log_last_layer = 0;
  uint32_t n_queries = 3;
  size_t last_layer_domain_size() const { return (size_t)1 << (log_last_layer + log_blowup); }
};

struct FriLayerProof {
  std::vector<QM31> fri_witness;
  MerkleDecommitment decommitment;
  Hash32 commitment;
};
struct FriProof {
  FriLayerProof first_layer;
  std::vector<FriLayerProof> inner_layers;
  std::vector<QM31> last_layer_poly;  // LinePoly coefficients as stored (bit-reversed)
};
struct StarkProof {
  PcsConfig config;
  std::vector<Hash32> commitments;
  std::vector<std::vector<std::vector<QM31>>> sampled_values;  // [tree][col][sample]
  std::vector<MerkleDecommitment> decommitments;
  std::vector<std::vector<M31>> queried_values;
  uint64_t proof_of_work = 0;
  FriProof fri;
};

struct Writer {
  std::vector<uint8_t> b;
  void u32(uint32_t v) { for (int i = 0; i < 4; i++) b.push_back((uint8_t)(v >> (8 * i))); }
  void u64(uint64_t v) { for (int i = 0; i < 8; i++) b.push_back((uint8_t)(v >> (8 * i))); }
  void hash(const Hash32& h) { b.insert(b.end(), h.b, h.b + 32); }
  void q(const QM31& x) { u32(x.a.a.v); u32(x.a.b.v); u32(x.b.a.v); u32(x.b.b.v); }
  void qs(const std::vector<QM31>& v) { u64(v.size()); for (auto& x : v) q(x); }
  void ms(const std::vector<M31>& v) { u64(v.size()); for (auto& x : v) u32(x.v); }
  void dec(const MerkleDecommitment& d) {
    u64(d.hash_witness.size());
    for (auto& h : d.hash_witness) hash(h);
    ms(d.column_witness);
  }
  void layer(const FriLayerProof& l) { qs(l.fri_witness); dec(l.decommitment); hash(l.commitment); }
};

inline std::vector<uint8_t> serialize(const StarkProof& p) {
  Writer w;
  w.u32(p.config.pow_bits);
  w.u32(p.config.log_blowup);
  w.u32(p.config.log_last_layer);
  w.u64(p.config.n_queries);
  w.u64(p.commitments.size());
  for (auto& h : p.commitments) w.hash(h);
  w.u64(p.sampled_values.size());
  for (auto& t : p.sampled_values) {
    w.u64(t.size());
    for (auto& c : t) w.qs(c);
  }
  w.u64(p.decommitments.size());
  for (auto& d : p.decommitments) w.dec(d);
  w.u64(p.queried_values.size());
  for (auto& v : p.queried_values) w.ms(v);
  w.u64(p.proof_of_work);
  w.layer(p.fri.first_layer);
  w.u64(p.fri.inner_layers.size());
  for (auto& l : p.fri.inner_layers) w.layer(l);
  w.qs(p.fri.last_layer_poly);
  return w.b;
}

struct Reader {
  const uint8_t* p;
  size_t n, i = 0;
  bool ok = true;
  uint64_t take(int k) {
    if (i + k > n) { ok = false; return 0; }
    uint64_t v = 0;
    for (int j = 0; j < k; j++) v |= (uint64_t)p[i + j] << (8 * j);
    i += k;
    return v;
  }
  uint32_t u32() { return (uint32_t)take(4); }
  uint64_t u64() { return take(8); }
  uint64_t len() {
    uint64_t l = u64();
    if (l > n) ok = false;
    return ok ? l : 0;
  }
  Hash32 hash() {
    Hash32 h;
    if (i + 32 > n) { ok = false; return h; }
    std::memcpy(h.b, p + i, 32);
    i += 32;
    return h;
  }
  QM31 q() { uint32_t a = u32(), b = u32(), c = u32(), d = u32(); return QM31::from_u32(a, b, c, d); }
  std::vector<QM31> qs() { std::vector<QM31> v(len()); for (auto& x : v) x = q(); return v; }
  std::vector<M31> ms() { std::vector<M31> v(len()); for (auto& x : v) x = M31(u32()); return v; }
  MerkleDecommitment dec() {
    MerkleDecommitment d;
    d.hash_witness.resize(len());
    for (auto& h : d.hash_witness) h = hash();
    d.column_witness = ms();
    return d;
  }
  FriLayerProof layer() { FriLayerProof l; l.fri_witness = qs(); l.decommitment = dec(); l.commitment = hash(); return l; }
};

inline bool deserialize(const uint8_t* data, size_t n, StarkProof& p) {
  Reader r{data, n};
  p.config.pow_bits = r.u32();
  p.config.log_blowup = r.u32();
  p.config.log_last_layer = r.u32();
  p.config.n_queries = (uint32_t)r.u64();
  p.commitments.resize(r.len());
  for (auto& h : p.commitments) h = r.hash();
  p.sampled_values.resize(r.len());
  for (auto& t : p.sampled_values) {
    t.resize(r.len());
    for (auto& c : t) c = r.qs();
  }
  p.decommitments.resize(r.len());
  for (auto& d : p.decommitments) d = r.dec();
  p.queried_values.resize(r.len());
  for (auto& v : p.queried_values) v = r.ms();
  p.proof_of_work = r.u64();
  p.fri.first_layer = r.layer();
  p.fri.inner_layers.resize(r.len());
  for (auto& l : p.fri.inner_layers) l = r.layer();
  p.fri.last_layer_poly = r.qs();
  return r.ok && r.i == n;
}

// ---------------------------------------------------------------- queries
struct Queries {
  std::vector<size_t> positions;
  uint32_t log_domain_size = 0;
  static Queries generate(Channel& ch, uint32_t log_size, size_t n_queries) {
    std::set<size_t> qs;
    size_t cnt = 0;
    uint32_t mask = (uint32_t)((1ull << log_size) - 1);
    while (true) {
      Hash32 h = ch.draw_random_bytes();
      uint32_t w[8];
      h.words(w);
      for (int i = 0; i < 8; i++) {
        qs.insert(w[i] & mask);
        if (++cnt == n_queries) return Queries{std::vector<size_t>(qs.begin(), qs.end()), log_size};
      }
    }
  }
  Queries fold(uint32_t n) const {
    Queries q;
    q.log_domain_size = log_domain_size - n;
    for (size_t p : positions) {
      size_t v = p >> n;
      if (q.positions.empty() || q.positions.back() != v) q.positions.push_back(v);
    }
    return q;
  }
};

// fri.rs:943-976
inline void decommitment_positions_and_witness(const SecureColumn& col, const std::vector<size_t>& queries,
                                               std::vector<size_t>& positions, std::vector<QM31>& witness) {
  size_t i = 0;
  while (i < queries.size()) {
    size_t start = (queries[i] >> 1) << 1;
    size_t j = i;
    while (j < queries.size() && (queries[j] >> 1) == (queries[i] >> 1)) j++;
    size_t k = i;
    for (size_t pos = start; pos < start + 2; pos++) {
      positions.push_back(pos);
      if (k < j && queries[k] == pos) { k++; continue; }
      witness.push_back(col.at(pos));
    }
    i = j;
  }
}

// ---------------------------------------------------------------- FRI prover
struct FriLayer {
  SecureColumn eval;
  Coset domain;  // line domain
  MerkleProver tree;
};

struct FriProver {
  PcsConfig config;
  std::vector<const SecureColumn*> columns;  // first layer columns, descending sizes
  std::vector<uint32_t> column_log_sizes;
  MerkleProver first_tree;
  std::vector<FriLayer> inner;
  std::vector<QM31> last_layer_poly;

  static std::vector<const Column*> coord_cols(const std::vector<const SecureColumn*>& cs) {
    std::vector<const Column*> v;
    for (auto* c : cs)
      for (int k = 0; k < 4; k++) v.push_back(&c->c[k]);
    return v;
  }

  void commit(Channel& ch, const PcsConfig& cfg, const std::vector<const SecureColumn*>& cols) {
    config = cfg;
    columns = cols;
    for (auto* c : cols) column_log_sizes.push_back(ilog2(c->size()));
    for (size_t i = 1; i < cols.size(); i++)
      if (!(cols[i - 1]->size() > cols[i]->size())) throw std::runtime_error("column sizes not decreasing");
    first_tree = MerkleProver::commit(coord_cols(cols));
    ch.mix_root(first_tree.root());
    // Inner layers (fri.rs:215-263).
    uint32_t first_log = column_log_sizes[0] - 1;
    Coset dom = Coset::half_odds(first_log);
    SecureColumn layer(dom.size());
    size_t next = 0;
    QM31 alpha = ch.draw_felt();
    fold_circle_into_line(layer, *cols[next], canonic_domain(column_log_sizes[next]), alpha);
    next++;
    while (layer.size() > config.last_layer_domain_size()) {
      FriLayer L;
      L.eval = layer;
      L.domain = dom;
      std::vector<const Column*> lc;
      for (int k = 0; k < 4; k++) lc.push_back(&L.eval.c[k]);
      L.tree = MerkleProver::commit(lc);
      ch.mix_root(L.tree.root());
      alpha = ch.draw_felt();
      layer = fold_line(L.eval, dom, alpha);
      dom = dom.dbl();
      if (next < cols.size() && cols[next]->size() / 2 == layer.size()) {
        fold_circle_into_line(layer, *cols[next], canonic_domain(column_log_sizes[next]), alpha);
        next++;
      }
      inner.push_back(std::move(L));
      // The FriLayer's tree points at L.eval columns; re-anchor after the move.
    }
    if (next != cols.size()) throw std::runtime_error("not all FRI columns consumed");
    // Last layer (fri.rs:276-290).
    if (layer.size() != config.last_layer_domain_size()) throw std::runtime_error("last layer size");
    std::vector<QM31> vals(layer.size());
    for (size_t i = 0; i < layer.size(); i++) vals[i] = layer.at(i);
    std::vector<QM31> coeffs = line_interpolate(dom, vals);  // bit-reversed coefficient order
    bit_reverse(coeffs);                                     // ordered
    size_t bound = (size_t)1 << config.log_last_layer;
    for (size_t i = bound; i < coeffs.size(); i++)
      if (!coeffs[i].is_zero()) throw std::runtime_error("invalid degree");
    coeffs.resize(bound);
    bit_reverse(coeffs);
    last_layer_poly = coeffs;
    ch.mix_felts(last_layer_poly);
  }

  // fri.rs:295-334
  std::pair<FriProof, std::map<uint32_t, std::vector<size_t>>> decommit(Channel& ch) const {
    uint32_t max_log = column_log_sizes[0];
    Queries q = Queries::generate(ch, max_log, config.n_queries);
    std::map<uint32_t, std::vector<size_t>> by_log;
    for (uint32_t l : std::set<uint32_t>(column_log_sizes.begin(), column_log_sizes.end()))
      by_log[l] = q.fold(max_log - l).positions;
    FriProof proof;
    // First layer.
    std::map<uint32_t, std::vector<size_t>> dpos;
    for (size_t c = 0; c < columns.size(); c++) {
      Queries cq = q.fold(max_log - column_log_sizes[c]);
      std::vector<size_t> pos;
      decommitment_positions_and_witness(*columns[c], cq.positions, pos, proof.first_layer.fri_witness);
      dpos[column_log_sizes[c]] = pos;
    }
    proof.first_layer.decommitment = first_tree.decommit(dpos, coord_cols(columns)).second;
    proof.first_layer.commitment = first_tree.root();
    // Inner layers.
    Queries lq = q.fold(1);
    for (auto& L : inner) {
      FriLayerProof lp;
      std::vector<size_t> pos;
      decommitment_positions_and_witness(L.eval, lq.positions, pos, lp.fri_witness);
      std::vector<const Column*> lc;
      for (int k = 0; k < 4; k++) lc.push_back(&L.eval.c[k]);
      std::map<uint32_t, std::vector<size_t>> m;
      m[L.domain.log_size] = pos;
      lp.decommitment = L.tree.decommit(m, lc).second;
      lp.commitment = L.tree.root();
      proof.inner_layers.push_back(lp);
      lq = lq.fold(1);
    }
    proof.last_layer_poly = last_layer_poly;
    return {proof, by_log};
  }
};

// ---------------------------------------------------------------- commitment scheme prover
struct CommitmentTree {
  std::vector<Column> polys;
  std::vector<Column> evals;
  MerkleProver tree;
};

struct CommitmentSchemeProver {
  PcsConfig config;
  const TwiddleTree* twiddles = nullptr;
  std::vector<CommitmentTree> trees;

  // pcs/prover.rs:208-227
  void commit(std::vector<Column> polys, Channel& ch) {
    CommitmentTree t;
    t.polys = std::move(polys);
    t.evals.resize(t.polys.size());
#pragma omp parallel for schedule(dynamic)
    for (long i = 0; i < (long)t.polys.size(); i++) {
      uint32_t log = ilog2(t.polys[i].size()) + config.log_blowup;
      t.evals[i] = evaluate(canonic_domain(log), t.polys[i], *twiddles);
    }
    std::vector<const Column*> ec;
    for (auto& e : t.evals) ec.push_back(&e);
    t.tree = MerkleProver::commit(ec);
    ch.mix_root(t.tree.root());
    trees.push_back(std::move(t));
  }
  // TreeBuilder::extend_evals: interpolate then commit.
  void commit_evals(const std::vector<Column>& evals, uint32_t log_size, Channel& ch) {
    std::vector<Column> polys(evals.size());
#pragma omp parallel for schedule(dynamic)
    for (long i = 0; i < (long)evals.size(); i++) polys[i] = interpolate(canonic_domain(log_size), evals[i], *twiddles);
    commit(std::move(polys), ch);
  }

  // pcs/prover.rs:83-148
  StarkProof prove_values(const std::vector<std::vector<std::vector<CirclePointQM31>>>& points, Channel& ch) {
    StarkProof proof;
    proof.config = config;
    std::vector<std::vector<std::vector<PointSample>>> samples(trees.size());
    std::vector<QM31> flat;
    for (size_t t = 0; t < trees.size(); t++) {
      proof.sampled_values.emplace_back(trees[t].polys.size());
      samples[t].resize(trees[t].polys.size());
#pragma omp parallel for schedule(dynamic)
      for (long c = 0; c < (long)trees[t].polys.size(); c++) {
        for (auto& pt : points[t][c]) {
          QM31 v = eval_at_point(trees[t].polys[c], pt);
          samples[t][c].push_back({pt, v});
          proof.sampled_values[t][c].push_back(v);
        }
      }
      for (auto& col : proof.sampled_values[t]) flat.insert(flat.end(), col.begin(), col.end());
    }
    ch.mix_felts(flat);
    // compute_fri_quotients (pcs/quotients.rs:76-101): stable sort by descending log size.
    std::vector<std::pair<const Column*, const std::vector<PointSample>*>> cols;
    for (size_t t = 0; t < trees.size(); t++)
      for (size_t c = 0; c < trees[t].evals.size(); c++) cols.push_back({&trees[t].evals[c], &samples[t][c]});
    std::stable_sort(cols.begin(), cols.end(),
                     [](auto& a, auto& b) { return a.first->size() > b.first->size(); });
    QM31 rc = ch.draw_felt();
    std::vector<SecureColumn> quotients;
    for (size_t i = 0; i < cols.size();) {
      size_t j = i;
      while (j < cols.size() && cols[j].first->size() == cols[i].first->size()) j++;
      std::vector<const Column*> gc;
      std::vector<std::vector<PointSample>> gs;
      for (size_t k = i; k < j; k++) {
        gc.push_back(cols[k].first);
        gs.push_back(*cols[k].second);
      }
      uint32_t log = ilog2(cols[i].first->size());
      quotients.push_back(accumulate_quotients(canonic_domain(log), gc, rc, column_sample_batches(gs), config.log_blowup));
      i = j;
    }
    std::vector<const SecureColumn*> qp;
    for (auto& q : quotients) qp.push_back(&q);
    FriProver fri;
    fri.commit(ch, config, qp);
    uint32_t d[8];
    ch.digest.words(d);
    proof.proof_of_work = grind(d, config.pow_bits);
    ch.mix_u64(proof.proof_of_work);
    auto [fp, by_log] = fri.decommit(ch);
    proof.fri = fp;
    for (auto& t : trees) {
      std::vector<const Column*> ec;
      for (auto& e : t.evals) ec.push_back(&e);
      auto [vals, dec] = t.tree.decommit(by_log, ec);
      proof.queried_values.push_back(vals);
      proof.decommitments.push_back(dec);
      proof.commitments.push_back(t.tree.root());
    }
    return proof;
  }
};

}  // namespace oracle
