// ORACLE — test infrastructure only (see field.h).
// Twiddle trees and the circle FFT of the reference's CPU backend.
// Follows crates/prover/src/core/backend/cpu/circle.rs:15-232 (interpolate :18-71,
// eval_at_point :73-87, extend :89-95, evaluate :97-135, twiddles :137-188,
// fft_layer_loop :190-204, circle_twiddles_from_line_twiddles :209-229),
// core/fft.rs:5-21 (butterflies), poly/utils.rs:23-77 (fold, twiddle slicing),
// poly/line.rs:225-290 (line evaluation interpolation, line_ifft).
#pragma once
#include "circle.h"
#include <vector>
#include <stdexcept>
#include <algorithm>

namespace oracle {

template <class F>
inline void butterfly(F& v0, F& v1, M31 t) {
  F tmp = v1 * t;
  v1 = v0 - tmp;
  v0 = v0 + tmp;
}
template <class F>
inline void ibutterfly(F& v0, F& v1, M31 it) {
  F tmp = v0;
  v0 = tmp + v1;
  v1 = (tmp - v1) * it;
}

struct TwiddleTree {
  Coset root_coset;
  std::vector<M31> twiddles;   // size 2^root.log_size
  std::vector<M31> itwiddles;
};

// cpu/circle.rs:171-188
inline std::vector<M31> slow_precompute_twiddles(Coset coset) {
  std::vector<M31> tw;
  tw.reserve(coset.size());
  const uint32_t levels = coset.log_size;  // the Rust range is evaluated once
  for (uint32_t l = 0; l < levels; l++) {
    size_t i0 = tw.size();
    std::vector<CirclePointM31> pts = coset.points();
    for (size_t i = 0; i < coset.size() / 2; i++) tw.push_back(pts[i].x);
    bit_reverse(tw.data() + i0, tw.size() - i0);
    coset = coset.dbl();
  }
  tw.push_back(M31(1));
  return tw;
}

inline TwiddleTree precompute_twiddles(Coset coset) {
  TwiddleTree t;
  t.root_coset = coset;
  t.twiddles = slow_precompute_twiddles(coset);
  t.itwiddles.resize(t.twiddles.size());
  for (size_t i = 0; i < t.twiddles.size(); i++) t.itwiddles[i] = inv(t.twiddles[i]);
  return t;
}

// poly/utils.rs:62-77. Returns (offset, len) for each line layer, largest first.
inline std::vector<std::pair<size_t, size_t>> domain_line_twiddles_from_tree(uint32_t line_log_size,
                                                                             size_t buf_len) {
  if (((size_t)1 << line_log_size) > buf_len) throw std::runtime_error("Not enough twiddles!");
  std::vector<std::pair<size_t, size_t>> out;
  for (int i = (int)line_log_size - 1; i >= 0; i--) {
    size_t len = (size_t)1 << i;
    out.push_back({buf_len - 2 * len, len});
  }
  return out;
}

template <class F>
inline void fft_layer_loop(std::vector<F>& v, uint32_t i, size_t h, M31 t, bool inverse) {
  for (size_t l = 0; l < ((size_t)1 << i); l++) {
    size_t idx0 = (h << (i + 1)) + l;
    size_t idx1 = idx0 + ((size_t)1 << i);
    if (inverse) ibutterfly(v[idx0], v[idx1], t);
    else butterfly(v[idx0], v[idx1], t);
  }
}

inline std::vector<M31> circle_twiddles_from_line(const M31* lt, size_t n) {
  std::vector<M31> out;
  for (size_t j = 0; j + 1 < n; j += 2) {
    M31 x = lt[j], y = lt[j + 1];
    out.push_back(y);
    out.push_back(-y);
    out.push_back(-x);
    out.push_back(x);
  }
  return out;
}

// cpu/circle.rs:18-71. `values` are evaluations in bit-reversed order; returns coefficients.
inline std::vector<M31> interpolate(const CircleDomain& dom, std::vector<M31> values, const TwiddleTree& tw) {
  if (!dom.half_coset.is_doubling_of(tw.root_coset)) throw std::runtime_error("twiddle tree mismatch");
  uint32_t L = dom.log_size();
  if (values.size() != dom.size()) throw std::runtime_error("size mismatch");
  if (L == 1) {
    M31 y = dom.half_coset.initial().y;
    M31 n(2);
    M31 yn_inv = inv(y * n);
    M31 y_inv = yn_inv * n, n_inv = yn_inv * y;
    ibutterfly(values[0], values[1], y_inv);
    return {values[0] * n_inv, values[1] * n_inv};
  }
  if (L == 2) {
    CirclePointM31 p = dom.half_coset.initial();
    M31 n(4);
    M31 xyn_inv = inv(p.x * p.y * n);
    M31 x_inv = xyn_inv * p.y * n, y_inv = xyn_inv * p.x * n, n_inv = xyn_inv * p.x * p.y;
    ibutterfly(values[0], values[1], y_inv);
    ibutterfly(values[2], values[3], -y_inv);
    ibutterfly(values[0], values[2], x_inv);
    ibutterfly(values[1], values[3], x_inv);
    for (auto& v : values) v = v * n_inv;
    return values;
  }
  auto lt = domain_line_twiddles_from_tree(L - 1, tw.itwiddles.size());
  std::vector<M31> ct = circle_twiddles_from_line(&tw.itwiddles[lt[0].first], lt[0].second);
  for (size_t h = 0; h < ct.size(); h++) fft_layer_loop(values, 0, h, ct[h], true);
  for (size_t layer = 0; layer < lt.size(); layer++)
    for (size_t h = 0; h < lt[layer].second; h++)
      fft_layer_loop(values, (uint32_t)layer + 1, h, tw.itwiddles[lt[layer].first + h], true);
  M31 invn = inv(M31((uint32_t)dom.size()));
  for (auto& v : values) v = v * invn;
  return values;
}

// cpu/circle.rs:97-135. `coeffs` of log n <= domain log; returns bit-reversed evaluations.
inline std::vector<M31> evaluate(const CircleDomain& dom, const std::vector<M31>& coeffs, const TwiddleTree& tw) {
  if (!dom.half_coset.is_doubling_of(tw.root_coset)) throw std::runtime_error("twiddle tree mismatch");
  uint32_t L = dom.log_size();
  if (coeffs.size() > dom.size()) throw std::runtime_error("Can only evaluate on larger domains");
  std::vector<M31> values = coeffs;
  values.resize(dom.size(), M31(0));
  if (L == 1) {
    butterfly(values[0], values[1], dom.half_coset.initial().y);
    return values;
  }
  if (L == 2) {
    CirclePointM31 p = dom.half_coset.initial();
    butterfly(values[0], values[2], p.x);
    butterfly(values[1], values[3], p.x);
    butterfly(values[0], values[1], p.y);
    butterfly(values[2], values[3], -p.y);
    return values;
  }
  auto lt = domain_line_twiddles_from_tree(L - 1, tw.twiddles.size());
  std::vector<M31> ct = circle_twiddles_from_line(&tw.twiddles[lt[0].first], lt[0].second);
  for (int layer = (int)lt.size() - 1; layer >= 0; layer--)
    for (size_t h = 0; h < lt[layer].second; h++)
      fft_layer_loop(values, (uint32_t)layer + 1, h, tw.twiddles[lt[layer].first + h], false);
  for (size_t h = 0; h < ct.size(); h++) fft_layer_loop(values, 0, h, ct[h], false);
  return values;
}

// poly/utils.rs:23-34
template <class F, class E>
inline E fold(const F* values, size_t n, const E* factors) {
  if (n == 1) return E(values[0]);
  E l = fold(values, n / 2, factors + 1);
  E r = fold(values + n / 2, n / 2, factors + 1);
  return l + r * factors[0];
}
inline QM31 fold_qm31(const M31* values, size_t n, const QM31* factors) {
  if (n == 1) return QM31(values[0]);
  QM31 l = fold_qm31(values, n / 2, factors + 1);
  QM31 r = fold_qm31(values + n / 2, n / 2, factors + 1);
  return l + r * factors[0];
}
inline QM31 fold_qq(const QM31* values, size_t n, const QM31* factors) {
  if (n == 1) return values[0];
  QM31 l = fold_qq(values, n / 2, factors + 1);
  QM31 r = fold_qq(values + n / 2, n / 2, factors + 1);
  return l + r * factors[0];
}

// cpu/circle.rs:73-87
inline QM31 eval_at_point(const std::vector<M31>& coeffs, CirclePointQM31 point) {
  size_t n = coeffs.size();
  uint32_t log = 0;
  while (((size_t)1 << log) < n) log++;
  if (log == 0) return QM31(coeffs[0]);
  std::vector<QM31> mappings;
  mappings.push_back(point.y);
  QM31 x = point.x;
  for (uint32_t i = 1; i < log; i++) {
    mappings.push_back(x);
    x = double_x(x);
  }
  std::reverse(mappings.begin(), mappings.end());
  return fold_qm31(coeffs.data(), n, mappings.data());
}

// Line polynomial coefficients (bit-reversed, normalised) from natural-order-of-storage
// bit-reversed evaluations on `domain` (poly/line.rs:225-233, 255-266).
inline std::vector<QM31> line_interpolate(Coset domain, std::vector<QM31> values) {
  bit_reverse(values);
  Coset d = domain;
  while (d.size() > 1) {
    size_t half = d.size() / 2;
    std::vector<CirclePointM31> pts = d.points();
    for (size_t c = 0; c < values.size(); c += d.size()) {
      for (size_t i = 0; i < half; i++) ibutterfly(values[c + i], values[c + half + i], inv(pts[i].x));
    }
    d = d.dbl();
  }
  M31 li = inv(M31((uint32_t)values.size()));
  for (auto& v : values) v = v * li;
  return values;
}

// line.rs:134-142
inline QM31 line_poly_eval_at_point(const std::vector<QM31>& coeffs, QM31 x) {
  std::vector<QM31> d;
  size_t n = coeffs.size();
  uint32_t log = 0;
  while (((size_t)1 << log) < n) log++;
  for (uint32_t i = 0; i < log; i++) {
    d.push_back(x);
    x = double_x(x);
  }
  return fold_qq(coeffs.data(), n, d.data());
}

}  // namespace oracle
