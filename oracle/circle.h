// ORACLE — test infrastructure only (see field.h).
// Circle group, cosets and domains over M31.
// Follows crates/prover/src/core/circle.rs (points :13-140, generators :203-216,
// CirclePointIndex :221-305, Coset :307-430), poly/circle/domain.rs:14-110,
// poly/circle/canonic.rs:27-80, poly/line.rs:23-110, core/utils.rs:53-90.
#pragma once
#include "field.h"
#include <vector>

namespace oracle {

template <class F>
struct CirclePoint {
  F x, y;
  bool operator==(const CirclePoint& o) const { return x == o.x && y == o.y; }
  bool operator<(const CirclePoint& o) const { return x != o.x ? x < o.x : y < o.y; }
};
template <class F>
inline CirclePoint<F> pt_add(const CirclePoint<F>& a, const CirclePoint<F>& b) {
  return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <class F>
inline CirclePoint<F> pt_conj(const CirclePoint<F>& a) { return {a.x, -a.y}; }
template <class F>
inline CirclePoint<F> pt_double(const CirclePoint<F>& a) { return pt_add(a, a); }
template <class F>
inline F double_x(F x) {
  F sx = x * x;
  return sx + sx - F(M31(1));
}
inline M31 double_x(M31 x) {
  M31 sx = x * x;
  return sx + sx - M31(1);
}

using CirclePointM31 = CirclePoint<M31>;
using CirclePointQM31 = CirclePoint<QM31>;

inline const CirclePointM31 M31_CIRCLE_GEN = {M31(2), M31(1268011823)};
constexpr uint32_t M31_CIRCLE_LOG_ORDER = 31;
inline const CirclePointQM31 SECURE_FIELD_CIRCLE_GEN = {
    QM31::from_u32(1, 0, 478637715, 513582971),
    QM31::from_u32(992285211, 649143431, 740191619, 1186584352)};

inline CirclePointM31 pt_zero_m31() { return {M31(1), M31(0)}; }
inline CirclePointQM31 pt_zero_qm31() { return {QM31(M31(1)), QM31(M31(0))}; }

inline CirclePointM31 pt_mul(CirclePointM31 p, uint64_t s) {
  CirclePointM31 r = pt_zero_m31();
  while (s) {
    if (s & 1) r = pt_add(r, p);
    p = pt_double(p);
    s >>= 1;
  }
  return r;
}

inline CirclePointQM31 to_qm31(const CirclePointM31& p) { return {QM31(p.x), QM31(p.y)}; }

// Integer i representing i * M31_CIRCLE_GEN, modulo 2^31.
constexpr uint32_t IDX_MASK = (1u << 31) - 1;
inline uint32_t idx_reduce(uint64_t i) { return (uint32_t)(i & IDX_MASK); }
inline uint32_t subgroup_gen(uint32_t log_size) { return 1u << (31 - log_size); }

// Points of the generator tower: point(2^b) for b in 0..30, used to turn an index into a point.
struct GenTower {
  CirclePointM31 p[31];
  GenTower() {
    p[0] = M31_CIRCLE_GEN;
    for (int b = 1; b < 31; b++) p[b] = pt_double(p[b - 1]);
  }
};
inline const GenTower& gen_tower() {
  static GenTower t;
  return t;
}
inline CirclePointM31 index_to_point(uint32_t idx) {
  idx &= IDX_MASK;
  CirclePointM31 r = pt_zero_m31();
  const GenTower& t = gen_tower();
  for (int b = 0; b < 31; b++)
    if ((idx >> b) & 1) r = pt_add(r, t.p[b]);
  return r;
}

struct Coset {
  uint32_t initial_index = 0;
  uint32_t step_size = 0;
  uint32_t log_size = 0;
  Coset() = default;
  Coset(uint32_t init, uint32_t log) : initial_index(idx_reduce(init)), step_size(subgroup_gen(log)), log_size(log) {}
  static Coset raw(uint32_t init, uint32_t step, uint32_t log) {
    Coset c;
    c.initial_index = idx_reduce(init);
    c.step_size = idx_reduce(step);
    c.log_size = log;
    return c;
  }
  static Coset subgroup(uint32_t log) { return Coset(0, log); }
  static Coset odds(uint32_t log) { return Coset(subgroup_gen(log + 1), log); }
  static Coset half_odds(uint32_t log) { return Coset(subgroup_gen(log + 2), log); }
  size_t size() const { return (size_t)1 << log_size; }
  uint32_t index_at(size_t i) const { return idx_reduce((uint64_t)initial_index + (uint64_t)step_size * (uint64_t)i); }
  CirclePointM31 at(size_t i) const { return index_to_point(index_at(i)); }
  CirclePointM31 initial() const { return index_to_point(initial_index); }
  Coset dbl() const {
    return raw(initial_index * 2u, step_size * 2u, log_size ? log_size - 1 : 0);
  }
  Coset repeated_double(uint32_t n) const {
    Coset c = *this;
    for (uint32_t i = 0; i < n; i++) c = c.dbl();
    return c;
  }
  bool operator==(const Coset& o) const {
    return initial_index == o.initial_index && step_size == o.step_size && log_size == o.log_size;
  }
  bool is_doubling_of(const Coset& o) const {
    return log_size <= o.log_size && *this == o.repeated_double(o.log_size - log_size);
  }
  Coset shift(uint32_t s) const { return raw(initial_index + s, step_size, log_size); }
  Coset conjugate() const {
    return raw((1u << 31) - initial_index, (1u << 31) - step_size, log_size);
  }
  // Points of the coset in natural order, computed incrementally.
  std::vector<CirclePointM31> points() const {
    std::vector<CirclePointM31> out(size());
    CirclePointM31 cur = initial(), st = index_to_point(step_size);
    for (size_t i = 0; i < size(); i++) {
      out[i] = cur;
      cur = pt_add(cur, st);
    }
    return out;
  }
};

struct CircleDomain {
  Coset half_coset;
  uint32_t log_size() const { return half_coset.log_size + 1; }
  size_t size() const { return (size_t)1 << log_size(); }
  uint32_t index_at(size_t i) const {
    if (i < half_coset.size()) return half_coset.index_at(i);
    return idx_reduce((1ull << 31) - half_coset.index_at(i - half_coset.size()));
  }
  CirclePointM31 at(size_t i) const { return index_to_point(index_at(i)); }
  bool is_canonic() const { return idx_reduce((uint64_t)half_coset.initial_index * 4) == half_coset.step_size; }
  CircleDomain shift(uint32_t s) const { return CircleDomain{half_coset.shift(s)}; }
  // domain.rs:85-96
  CircleDomain split_sub(uint32_t log_parts) const {
    return CircleDomain{Coset(half_coset.initial_index, half_coset.log_size - log_parts)};
  }
  // All points in natural domain order.
  std::vector<CirclePointM31> points() const {
    std::vector<CirclePointM31> a = half_coset.points();
    std::vector<CirclePointM31> out(size());
    for (size_t i = 0; i < a.size(); i++) {
      out[i] = a[i];
      out[i + a.size()] = pt_conj(a[i]);
    }
    return out;
  }
};

inline Coset canonic_coset(uint32_t log) { return Coset::odds(log); }
inline CircleDomain canonic_domain(uint32_t log) { return CircleDomain{Coset::half_odds(log - 1)}; }

inline size_t bit_reverse_index(size_t i, uint32_t log) {
  if (log == 0) return i;
  size_t r = 0;
  for (uint32_t b = 0; b < log; b++) r |= ((i >> b) & 1) << (log - 1 - b);
  return r;
}
template <class T>
inline void bit_reverse(std::vector<T>& v) {
  size_t n = v.size();
  uint32_t log = 0;
  while (((size_t)1 << log) < n) log++;
  for (size_t i = 0; i < n; i++) {
    size_t j = bit_reverse_index(i, log);
    if (j > i) std::swap(v[i], v[j]);
  }
}
template <class T>
inline void bit_reverse(T* v, size_t n) {
  uint32_t log = 0;
  while (((size_t)1 << log) < n) log++;
  for (size_t i = 0; i < n; i++) {
    size_t j = bit_reverse_index(i, log);
    if (j > i) std::swap(v[i], v[j]);
  }
}

// Points of a domain in bit-reversed storage order.
inline std::vector<CirclePointM31> domain_points_bitrev(const CircleDomain& d) {
  std::vector<CirclePointM31> p = d.points();
  bit_reverse(p);
  return p;
}

// utils.rs:74-90
inline size_t offset_bit_reversed_circle_domain_index(size_t i, uint32_t domain_log_size,
                                                      uint32_t eval_log_size, int64_t offset) {
  int64_t prev = (int64_t)bit_reverse_index(i, eval_log_size);
  int64_t half = (int64_t)1 << (eval_log_size - 1);
  int64_t step = offset * ((int64_t)1 << (eval_log_size - domain_log_size - 1));
  auto rem = [](int64_t a, int64_t m) { int64_t r = a % m; return r < 0 ? r + m : r; };
  if (prev < half) prev = rem(prev + step, half);
  else prev = rem(prev - step, half) + half;
  return bit_reverse_index((size_t)prev, eval_log_size);
}

// constraints.rs:11-31
template <class F>
inline F coset_vanishing(const Coset& c, CirclePoint<F> p) {
  CirclePointM31 init = c.initial();
  CirclePointM31 half = index_to_point(c.step_size >> 1);
  CirclePointM31 shift = pt_add(pt_conj(init), half);  // -initial + step/2
  CirclePoint<F> s = {F(shift.x), F(shift.y)};
  p = pt_add(p, s);
  F x = p.x;
  for (uint32_t i = 1; i < c.log_size; i++) x = double_x(x);
  return x;
}
inline M31 coset_vanishing(const Coset& c, CirclePointM31 p) {
  CirclePointM31 init = c.initial();
  CirclePointM31 half = index_to_point(c.step_size >> 1);
  p = pt_add(p, pt_add(pt_conj(init), half));
  M31 x = p.x;
  for (uint32_t i = 1; i < c.log_size; i++) x = double_x(x);
  return x;
}

}  // namespace oracle
