// ORACLE — test infrastructure only (see field.h).
// Wide-Fibonacci AIR (crates/prover/src/examples/wide_fibonacci/mod.rs:22-68): N columns per row,
// c = a^2 + b^2 along the row, one constraint per column after the first two.
#pragma once
#include "air.h"

namespace oracle {

template <class E>
inline void wide_fib_evaluate(E& e, size_t n_cols) {
  auto a = e.next_trace_mask();
  auto b = e.next_trace_mask();
  for (size_t i = 2; i < n_cols; i++) {
    auto c = e.next_trace_mask();
    e.add_constraint(c - (a * a + b * b));
    a = b;
    b = c;
  }
}

struct WideFibAir : Air {
  uint32_t log_n;
  size_t n_cols;
  WideFibAir(uint32_t l, size_t n) : log_n(l), n_cols(n) {}
  uint32_t log_size() const override { return log_n; }
  uint32_t max_constraint_log_degree_bound() const override { return log_n + 1; }
  size_t n_constraints() const override { return n_cols - 2; }
  Mask mask_offsets() const override {
    Mask m(2);
    m[1].assign(n_cols, {0});
    return m;
  }
  QM31 eval_row(DomainEvaluator& e) const override {
    wide_fib_evaluate(e, n_cols);
    return e.row_res;
  }
  void eval_point(PointEvaluator& e) const override { wide_fib_evaluate(e, n_cols); }
};

// Trace of generate_trace (wide_fibonacci/mod.rs:46-68): row r starts from (a_r, b_r).
inline std::vector<Column> wide_fib_trace(uint32_t log_n, size_t n_cols, const uint32_t* a, const uint32_t* b) {
  size_t n = (size_t)1 << log_n;
  std::vector<Column> t(n_cols, Column(n));
  for (size_t r = 0; r < n; r++) {
    M31 x(a[r]), y(b[r]);
    t[0][r] = x;
    t[1][r] = y;
    for (size_t c = 2; c < n_cols; c++) {
      M31 z = x * x + y * y;
      x = y;
      y = z;
      t[c][r] = z;
    }
  }
  return t;
}

}  // namespace oracle
