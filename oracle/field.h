// ORACLE — test infrastructure only. Plain C++ restatement of the reference's
// scalar field arithmetic. Only tests/, __graft_entry__.smoke() and bench.py's
// cpu_baseline leg may load or run code from oracle/; the product never does.
//
// Follows:
//   M31  crates/prover/src/core/fields/m31.rs:32-140   (p = 2^31 - 1, reduce :58-60)
//   CM31 crates/prover/src/core/fields/cm31.rs:17-70   (i^2 = -1)
//   QM31 crates/prover/src/core/fields/qm31.rs:21-140  (u^2 = 2 + i, R = (2,1) :15)
//   batch inverse crates/prover/src/core/fields/mod.rs:40-120
#pragma once
#include <cstdint>
#include <cstddef>
#include <vector>
#include <cassert>

namespace oracle {

constexpr uint32_t P = 0x7fffffffu;

struct M31 {
  uint32_t v = 0;
  M31() = default;
  constexpr explicit M31(uint32_t x) : v(x) {}
  // m31.rs:58-60: val % P for val in [0, P^2).
  static constexpr M31 reduce(uint64_t val) {
    return M31((uint32_t)((((((val >> 31) + val + 1) >> 31) + val)) & (uint64_t)P));
  }
  static constexpr M31 from_u64(uint64_t x) { return M31((uint32_t)(x % P)); }
  bool operator==(const M31& o) const { return v == o.v; }
  bool operator!=(const M31& o) const { return v != o.v; }
  bool operator<(const M31& o) const { return v < o.v; }
  bool is_zero() const { return v == 0; }
};

inline M31 partial_reduce(uint32_t x) { return M31(x >= P ? x - P : x); }
inline M31 operator+(M31 a, M31 b) { return partial_reduce(a.v + b.v); }
inline M31 operator-(M31 a, M31 b) { return partial_reduce(a.v + P - b.v); }
inline M31 operator-(M31 a) { return partial_reduce(P - a.v); }
inline M31 operator*(M31 a, M31 b) { return M31::reduce((uint64_t)a.v * b.v); }
inline M31& operator+=(M31& a, M31 b) { return a = a + b; }
inline M31& operator-=(M31& a, M31 b) { return a = a - b; }
inline M31& operator*=(M31& a, M31 b) { return a = a * b; }

inline M31 m31_pow(M31 b, uint64_t e) {
  M31 r(1);
  while (e) {
    if (e & 1) r = r * b;
    b = b * b;
    e >>= 1;
  }
  return r;
}
inline M31 inv(M31 a) {
  assert(!a.is_zero());
  return m31_pow(a, P - 2);
}

struct CM31 {
  M31 a, b;  // a + b i
  CM31() = default;
  constexpr CM31(M31 x, M31 y) : a(x), b(y) {}
  explicit CM31(M31 x) : a(x), b(0) {}
  bool operator==(const CM31& o) const { return a == o.a && b == o.b; }
  bool operator!=(const CM31& o) const { return !(*this == o); }
  bool operator<(const CM31& o) const { return a.v != o.a.v ? a.v < o.a.v : b.v < o.b.v; }
  bool is_zero() const { return a.is_zero() && b.is_zero(); }
};
inline CM31 operator+(CM31 x, CM31 y) { return {x.a + y.a, x.b + y.b}; }
inline CM31 operator-(CM31 x, CM31 y) { return {x.a - y.a, x.b - y.b}; }
inline CM31 operator-(CM31 x) { return {-x.a, -x.b}; }
inline CM31 operator*(CM31 x, CM31 y) {
  return {x.a * y.a - x.b * y.b, x.a * y.b + x.b * y.a};
}
inline CM31 operator*(CM31 x, M31 y) { return {x.a * y, x.b * y}; }
inline CM31 inv(CM31 x) {
  // cm31.rs:67-71: (a - bi) / (a^2 + b^2)
  M31 d = inv(x.a * x.a + x.b * x.b);
  return {x.a * d, (-x.b) * d};
}

struct QM31 {
  CM31 a, b;  // a + b u
  QM31() = default;
  constexpr QM31(CM31 x, CM31 y) : a(x), b(y) {}
  explicit QM31(M31 x) : a(x), b(M31(0)) {}
  static QM31 from_u32(uint32_t x0, uint32_t x1, uint32_t x2, uint32_t x3) {
    return QM31(CM31(M31(x0), M31(x1)), CM31(M31(x2), M31(x3)));
  }
  static QM31 from_m31(M31 x0, M31 x1, M31 x2, M31 x3) { return QM31(CM31(x0, x1), CM31(x2, x3)); }
  M31 coord(int i) const {
    switch (i) { case 0: return a.a; case 1: return a.b; case 2: return b.a; default: return b.b; }
  }
  bool operator==(const QM31& o) const { return a == o.a && b == o.b; }
  bool operator!=(const QM31& o) const { return !(*this == o); }
  // Derived lexicographic Ord on ((a0,a1),(b0,b1)): used as BTreeMap key order.
  bool operator<(const QM31& o) const { return a != o.a ? a < o.a : b < o.b; }
  bool is_zero() const { return a.is_zero() && b.is_zero(); }
};
inline const CM31 QM31_R = CM31(M31(2), M31(1));
inline QM31 operator+(QM31 x, QM31 y) { return {x.a + y.a, x.b + y.b}; }
inline QM31 operator-(QM31 x, QM31 y) { return {x.a - y.a, x.b - y.b}; }
inline QM31 operator-(QM31 x) { return {-x.a, -x.b}; }
inline QM31 operator*(QM31 x, QM31 y) {
  // qm31.rs:84-91: (a + bu)(c + du) = (ac + R bd) + (ad + bc) u
  return {x.a * y.a + QM31_R * (x.b * y.b), x.a * y.b + x.b * y.a};
}
inline QM31 operator*(QM31 x, M31 y) { return {x.a * y, x.b * y}; }
inline QM31 operator*(QM31 x, CM31 y) { return {x.a * y, x.b * y}; }
inline QM31 operator+(QM31 x, M31 y) { return {x.a + CM31(y), x.b}; }
inline QM31 operator-(QM31 x, M31 y) { return {x.a - CM31(y), x.b}; }
inline QM31& operator+=(QM31& x, QM31 y) { return x = x + y; }
inline QM31& operator-=(QM31& x, QM31 y) { return x = x - y; }
inline QM31& operator*=(QM31& x, QM31 y) { return x = x * y; }
inline QM31 inv(QM31 x) {
  // qm31.rs:121-129
  CM31 b2 = x.b * x.b;
  CM31 ib2(-b2.b, b2.a);
  CM31 denom = x.a * x.a - (b2 + b2 + ib2);
  CM31 di = inv(denom);
  return {x.a * di, (-x.b) * di};
}
inline QM31 qm31_pow(QM31 b, uint64_t e) {
  QM31 r(M31(1));
  while (e) {
    if (e & 1) r = r * b;
    b = b * b;
    e >>= 1;
  }
  return r;
}
inline QM31 complex_conjugate(QM31 x) { return {x.a, -x.b}; }

// Montgomery batch inversion; the result equals elementwise inversion exactly.
template <class F>
std::vector<F> batch_inverse(const std::vector<F>& xs) {
  size_t n = xs.size();
  std::vector<F> out(n);
  if (!n) return out;
  std::vector<F> pre(n);
  pre[0] = xs[0];
  for (size_t i = 1; i < n; i++) pre[i] = pre[i - 1] * xs[i];
  F cur = inv(pre[n - 1]);
  for (size_t i = n - 1; i > 0; i--) {
    out[i] = pre[i - 1] * cur;
    cur = cur * xs[i];
  }
  out[0] = cur;
  return out;
}

}  // namespace oracle
