// ORACLE — test infrastructure only (see field.h).
// Backend operations other than the FFT, restated from the reference:
//   Merkle layer     crates/prover/src/core/backend/simd/blake2s.rs:60-145 (hash = blake2_merkle.rs:14-30)
//   Merkle tree      crates/prover/src/core/vcs/prover.rs:39-154, vcs/utils.rs:4-20
//   FRI folds        crates/prover/src/core/fri.rs:1132-1189
//   decompose        crates/prover/src/core/backend/simd/fri.rs:111-161
//   quotients        crates/prover/src/core/backend/simd/quotients.rs:31-100 (subdomain + extend),
//                    backend/cpu/quotients.rs:17-146 (row formula), constraints.rs:98-115,
//                    pcs/quotients.rs:37-68 (batch grouping)
//   accumulation     crates/prover/src/core/backend/simd/accumulation.rs:8-36
//   grind            crates/prover/src/core/backend/simd/grind.rs:21-63
#pragma once
#include "poly.h"
#include "blake2s.h"
#include <map>
#include <algorithm>
#include <functional>

namespace oracle {

// ---------------------------------------------------------------- Merkle
using Column = std::vector<M31>;

inline std::vector<Hash32> commit_on_layer(uint32_t log_size, const std::vector<Hash32>* prev,
                                           const std::vector<const Column*>& cols) {
  size_t n = (size_t)1 << log_size;
  std::vector<Hash32> out(n);
#pragma omp parallel for schedule(static)
  for (long i = 0; i < (long)n; i++) {
    std::vector<uint32_t> vals(cols.size());
    for (size_t c = 0; c < cols.size(); c++) vals[c] = (*cols[c])[i].v;
    if (prev) out[i] = hash_node(&(*prev)[2 * i], &(*prev)[2 * i + 1], vals.data(), vals.size());
    else out[i] = hash_node(nullptr, nullptr, vals.data(), vals.size());
  }
  return out;
}

inline uint32_t ilog2(size_t n) {
  uint32_t l = 0;
  while (((size_t)1 << (l + 1)) <= n) l++;
  return l;
}

// Stable descending sort by length, as `sorted_by_key(Reverse(len))`.
inline std::vector<const Column*> sort_desc(const std::vector<const Column*>& cols) {
  std::vector<const Column*> s = cols;
  std::stable_sort(s.begin(), s.end(), [](const Column* a, const Column* b) { return a->size() > b->size(); });
  return s;
}

struct MerkleDecommitment {
  std::vector<Hash32> hash_witness;
  std::vector<M31> column_witness;
};

struct MerkleProver {
  std::vector<std::vector<Hash32>> layers;  // layers[0] = root layer
  static MerkleProver commit(const std::vector<const Column*>& columns) {
    MerkleProver mp;
    if (columns.empty()) {
      mp.layers.push_back(commit_on_layer(0, nullptr, {}));
      return mp;
    }
    auto s = sort_desc(columns);
    uint32_t max_log = ilog2(s[0]->size());
    size_t ci = 0;
    std::vector<std::vector<Hash32>> rev;
    for (int log = (int)max_log; log >= 0; log--) {
      std::vector<const Column*> lc;
      while (ci < s.size() && ilog2(s[ci]->size()) == (uint32_t)log) lc.push_back(s[ci++]);
      rev.push_back(commit_on_layer((uint32_t)log, rev.empty() ? nullptr : &rev.back(), lc));
    }
    std::reverse(rev.begin(), rev.end());
    mp.layers = std::move(rev);
    return mp;
  }
  Hash32 root() const { return layers[0][0]; }

  // prover.rs:80-149
  std::pair<std::vector<M31>, MerkleDecommitment> decommit(
      const std::map<uint32_t, std::vector<size_t>>& queries_per_log_size,
      const std::vector<const Column*>& columns) const {
    std::vector<M31> queried;
    MerkleDecommitment dec;
    auto s = sort_desc(columns);
    size_t ci = 0;
    std::vector<size_t> last;
    for (int log = (int)layers.size() - 1; log >= 0; log--) {
      std::vector<size_t> total;
      std::vector<const Column*> lc;
      while (ci < s.size() && ilog2(s[ci]->size()) == (uint32_t)log) lc.push_back(s[ci++]);
      const std::vector<Hash32>* prev = (size_t)log + 1 < layers.size() ? &layers[log + 1] : nullptr;
      size_t pi = 0;
      static const std::vector<size_t> empty;
      auto it = queries_per_log_size.find((uint32_t)log);
      const std::vector<size_t>& cq = it == queries_per_log_size.end() ? empty : it->second;
      size_t qi = 0;
      while (true) {
        bool have = false;
        size_t node = 0;
        if (pi < last.size()) { node = last[pi] / 2; have = true; }
        if (qi < cq.size()) { node = have ? std::min(node, cq[qi]) : cq[qi]; have = true; }
        if (!have) break;
        if (prev) {
          if (pi < last.size() && last[pi] == 2 * node) pi++;
          else dec.hash_witness.push_back((*prev)[2 * node]);
          if (pi < last.size() && last[pi] == 2 * node + 1) pi++;
          else dec.hash_witness.push_back((*prev)[2 * node + 1]);
        }
        bool q = qi < cq.size() && cq[qi] == node;
        if (q) qi++;
        for (auto* c : lc) (q ? queried : dec.column_witness).push_back((*c)[node]);
        total.push_back(node);
      }
      last = total;
    }
    return {queried, dec};
  }
};

// verifier.rs:53-170. Returns true when the decommitment reproduces `root`.
inline bool merkle_verify(const Hash32& root, const std::vector<uint32_t>& column_log_sizes,
                          const std::map<uint32_t, std::vector<size_t>>& queries_per_log_size,
                          const std::vector<M31>& queried_values, const MerkleDecommitment& dec) {
  if (column_log_sizes.empty()) return true;
  uint32_t max_log = *std::max_element(column_log_sizes.begin(), column_log_sizes.end());
  std::map<uint32_t, size_t> ncols;
  for (auto l : column_log_sizes) ncols[l]++;
  size_t qv = 0, hw = 0, cw = 0;
  std::vector<std::pair<size_t, Hash32>> last;
  bool have_last = false;
  for (int log = (int)max_log; log >= 0; log--) {
    size_t nc = ncols.count((uint32_t)log) ? ncols[(uint32_t)log] : 0;
    std::vector<std::pair<size_t, Hash32>> cur;
    static const std::vector<size_t> empty;
    auto it = queries_per_log_size.find((uint32_t)log);
    const std::vector<size_t>& cq = it == queries_per_log_size.end() ? empty : it->second;
    size_t pq = 0, ph = 0, qi = 0;
    while (true) {
      bool have = false;
      size_t node = 0;
      if (pq < last.size()) { node = last[pq].first / 2; have = true; }
      if (qi < cq.size()) { node = have ? std::min(node, cq[qi]) : cq[qi]; have = true; }
      if (!have) break;
      while (pq < last.size() && last[pq].first / 2 == node) pq++;
      Hash32 l, r;
      bool has_children = have_last;
      if (has_children) {
        if (ph < last.size() && last[ph].first == 2 * node) l = last[ph++].second;
        else { if (hw >= dec.hash_witness.size()) return false; l = dec.hash_witness[hw++]; }
        if (ph < last.size() && last[ph].first == 2 * node + 1) r = last[ph++].second;
        else { if (hw >= dec.hash_witness.size()) return false; r = dec.hash_witness[hw++]; }
      }
      std::vector<uint32_t> vals;
      if (qi < cq.size() && cq[qi] == node) {
        qi++;
        for (size_t k = 0; k < nc; k++) { if (qv >= queried_values.size()) return false; vals.push_back(queried_values[qv++].v); }
      } else {
        for (size_t k = 0; k < nc; k++) { if (cw >= dec.column_witness.size()) return false; vals.push_back(dec.column_witness[cw++].v); }
      }
      cur.push_back({node, hash_node(has_children ? &l : nullptr, has_children ? &r : nullptr, vals.data(), vals.size())});
    }
    last = cur;
    have_last = true;
  }
  if (hw != dec.hash_witness.size() || cw != dec.column_witness.size() || qv != queried_values.size()) return false;
  if (last.size() != 1) return false;
  return last[0].second == root;
}

// ---------------------------------------------------------------- secure columns
struct SecureColumn {
  Column c[4];
  SecureColumn() = default;
  explicit SecureColumn(size_t n) { for (auto& x : c) x.assign(n, M31(0)); }
  size_t size() const { return c[0].size(); }
  QM31 at(size_t i) const { return QM31::from_m31(c[0][i], c[1][i], c[2][i], c[3][i]); }
  void set(size_t i, QM31 v) {
    c[0][i] = v.a.a; c[1][i] = v.a.b; c[2][i] = v.b.a; c[3][i] = v.b.b;
  }
};

// ---------------------------------------------------------------- FRI folds
// fri.rs:1132-1157. `domain` is the line domain coset of `eval`.
inline SecureColumn fold_line(const SecureColumn& eval, const Coset& domain, QM31 alpha) {
  size_t n = eval.size();
  SecureColumn out(n / 2);
  uint32_t log = domain.log_size;
  std::vector<CirclePointM31> pts = domain.points();
  for (size_t i = 0; i < n / 2; i++) {
    M31 x = pts[bit_reverse_index(i << 1, log)].x;
    QM31 f0 = eval.at(2 * i), f1 = eval.at(2 * i + 1);
    ibutterfly(f0, f1, inv(x));
    out.set(i, f0 + alpha * f1);
  }
  return out;
}

// fri.rs:1162-1189. `domain` is the circle domain of `src`.
inline void fold_circle_into_line(SecureColumn& dst, const SecureColumn& src, const CircleDomain& domain,
                                  QM31 alpha) {
  QM31 a2 = alpha * alpha;
  uint32_t log = domain.log_size();
  std::vector<CirclePointM31> pts = domain.points();
  for (size_t i = 0; i < src.size() / 2; i++) {
    CirclePointM31 p = pts[bit_reverse_index(i << 1, log)];
    QM31 f0 = src.at(2 * i), f1 = src.at(2 * i + 1);
    ibutterfly(f0, f1, inv(p.y));
    QM31 fp = alpha * f1 + f0;
    dst.set(i, dst.at(i) * a2 + fp);
  }
}

// simd/fri.rs:111-161: lambda = (sum of first half - sum of second half) / N.
inline std::pair<SecureColumn, QM31> decompose(const SecureColumn& eval) {
  size_t n = eval.size();
  M31 s[4] = {M31(0), M31(0), M31(0), M31(0)};
  for (size_t i = 0; i < n; i++)
    for (int k = 0; k < 4; k++) s[k] = i < n / 2 ? s[k] + eval.c[k][i] : s[k] - eval.c[k][i];
  QM31 lambda = QM31::from_m31(s[0], s[1], s[2], s[3]) * inv(M31((uint32_t)n));
  SecureColumn g(n);
  for (size_t i = 0; i < n; i++) g.set(i, i < n / 2 ? eval.at(i) - lambda : eval.at(i) + lambda);
  return {g, lambda};
}

// ---------------------------------------------------------------- quotients
struct ColumnSampleBatch {
  CirclePointQM31 point;
  std::vector<std::pair<size_t, QM31>> columns_and_values;
};
struct PointSample {
  CirclePointQM31 point;
  QM31 value;
};

// pcs/quotients.rs:49-68: group by point in the derived Ord of CirclePoint<QM31>.
inline std::vector<ColumnSampleBatch> column_sample_batches(const std::vector<std::vector<PointSample>>& samples) {
  std::map<CirclePointQM31, std::vector<std::pair<size_t, QM31>>> g;
  for (size_t c = 0; c < samples.size(); c++)
    for (auto& s : samples[c]) g[s.point].push_back({c, s.value});
  std::vector<ColumnSampleBatch> out;
  for (auto& kv : g) out.push_back({kv.first, kv.second});
  return out;
}

struct LineCoeffs { QM31 a, b, c; };

// constraints.rs:98-115
inline LineCoeffs complex_conjugate_line_coeffs(CirclePointQM31 point, QM31 value, QM31 alpha) {
  QM31 a = complex_conjugate(value) - value;
  QM31 c = complex_conjugate(point.y) - point.y;
  QM31 b = value * c - a * point.y;
  return {alpha * a, alpha * b, alpha * c};
}

struct QuotientConstants {
  std::vector<std::vector<LineCoeffs>> line_coeffs;
  std::vector<QM31> batch_random_coeffs;
};
inline QuotientConstants quotient_constants(const std::vector<ColumnSampleBatch>& batches, QM31 rc) {
  QuotientConstants q;
  for (auto& b : batches) {
    QM31 alpha(M31(1));
    std::vector<LineCoeffs> v;
    for (auto& cv : b.columns_and_values) {
      alpha = alpha * rc;
      v.push_back(complex_conjugate_line_coeffs(b.point, cv.second, alpha));
    }
    q.line_coeffs.push_back(v);
    q.batch_random_coeffs.push_back(qm31_pow(rc, b.columns_and_values.size()));
  }
  return q;
}

// cpu/quotients.rs:43-76
inline QM31 accumulate_row_quotients(const std::vector<ColumnSampleBatch>& batches, const std::vector<M31>& row,
                                     const QuotientConstants& qc, CirclePointM31 p) {
  std::vector<CM31> dens;
  for (auto& b : batches) {
    CM31 prx = b.point.x.a, pry = b.point.y.a, pix = b.point.x.b, piy = b.point.y.b;
    dens.push_back((prx - CM31(p.x)) * piy - (pry - CM31(p.y)) * pix);
  }
  std::vector<CM31> di = batch_inverse(dens);
  QM31 acc(M31(0));
  for (size_t k = 0; k < batches.size(); k++) {
    QM31 num(M31(0));
    for (size_t j = 0; j < batches[k].columns_and_values.size(); j++) {
      const LineCoeffs& lc = qc.line_coeffs[k][j];
      QM31 value = lc.c * row[batches[k].columns_and_values[j].first];
      QM31 lin = lc.a * p.y + lc.b;
      num = num + (value - lin);
    }
    acc = acc * qc.batch_random_coeffs[k] + num * di[k];
  }
  return acc;
}

inline SecureColumn accumulate_quotients_cpu(const CircleDomain& domain, const std::vector<const Column*>& cols,
                                             QM31 rc, const std::vector<ColumnSampleBatch>& batches) {
  SecureColumn out(domain.size());
  QuotientConstants qc = quotient_constants(batches, rc);
  std::vector<CirclePointM31> pts = domain_points_bitrev(domain);
  std::vector<M31> row(cols.size());
  for (size_t r = 0; r < domain.size(); r++) {
    for (size_t c = 0; c < cols.size(); c++) row[c] = (*cols[c])[r];
    out.set(r, accumulate_row_quotients(batches, row, qc, pts[r]));
  }
  return out;
}

// simd/quotients.rs:31-100: rows of the subdomain, then interpolate and evaluate on the shifts.
inline SecureColumn accumulate_quotients(const CircleDomain& domain, const std::vector<const Column*>& cols,
                                         QM31 rc, const std::vector<ColumnSampleBatch>& batches,
                                         uint32_t log_blowup) {
  CircleDomain sub = domain.split_sub(log_blowup);
  if (sub.log_size() < 6) return accumulate_quotients_cpu(domain, cols, rc, batches);
  std::vector<uint32_t> shifts;
  for (uint32_t i = 0; i < (1u << log_blowup); i++) shifts.push_back(domain.half_coset.step_size * i);
  bit_reverse(shifts);
  QuotientConstants qc = quotient_constants(batches, rc);
  std::vector<CirclePointM31> pts = domain_points_bitrev(sub);
  SecureColumn subv(sub.size());
#pragma omp parallel for schedule(static)
  for (long r = 0; r < (long)sub.size(); r++) {
    std::vector<M31> row(cols.size());
    for (size_t c = 0; c < cols.size(); c++) row[c] = (*cols[c])[r];
    subv.set(r, accumulate_row_quotients(batches, row, qc, pts[r]));
  }
  TwiddleTree tw = precompute_twiddles(sub.half_coset);
  std::vector<M31> polys[4];
  for (int k = 0; k < 4; k++) polys[k] = interpolate(sub, subv.c[k], tw);
  SecureColumn out(domain.size());
  for (size_t ci = 0; ci < shifts.size(); ci++) {
    CircleDomain sd = sub.shift(shifts[ci]);
    TwiddleTree t2 = precompute_twiddles(sd.half_coset);
    for (int k = 0; k < 4; k++) {
      std::vector<M31> e = evaluate(sd, polys[k], t2);
      std::copy(e.begin(), e.end(), out.c[k].begin() + ci * sub.size());
    }
  }
  return out;
}

// ---------------------------------------------------------------- accumulation
inline void accumulate(SecureColumn& a, const SecureColumn& b) {
  for (size_t i = 0; i < a.size(); i++) a.set(i, a.at(i) + b.at(i));
}
inline std::vector<QM31> generate_secure_powers(QM31 felt, size_t n) {
  std::vector<QM31> r;
  QM31 cur(M31(1));
  for (size_t i = 0; i < n; i++) {
    r.push_back(cur);
    cur = cur * felt;
  }
  return r;
}

// ---------------------------------------------------------------- grind
inline uint32_t grind_check(const uint32_t digest[8], uint64_t nonce) {
  uint32_t m[16] = {0};
  m[0] = (uint32_t)nonce;
  m[1] = (uint32_t)(nonce >> 32);
  auto r = b2s_compress(digest, m, 0, 0, 0, 0);
  return r[0] == 0 ? 32u : (uint32_t)__builtin_ctz(r[0]);
}
inline uint64_t grind(const uint32_t digest[8], uint32_t pow_bits) {
  for (uint64_t n = 0;; n++)
    if (grind_check(digest, n) >= pow_bits) return n;
}

}  // namespace oracle
