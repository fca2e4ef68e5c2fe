// PolyOps::eval_at_point / extend, ColumnOps::bit_reverse_column, AccumulationOps,
// and Column::at gathers.
//
// eval_at_point (crates/prover/src/core/backend/cpu/circle.rs:73-87): sum_i coeff_i * t_i(point),
// t_i = y^{i_0} x^{i_1} pi(x)^{i_2} ... pi^{L-2}(x)^{i_{L-1}}, pi(x) = 2x^2 - 1. The index is split
// as (top | mid 6 bits | low 8 bits): thread t of a block owns low = t, accumulates
// sum_mid coeff * Mid[mid] (4 IMAD per coefficient), multiplies once by Low[t]; the block sum is
// scaled by Top[block] and folded into 64-bit accumulators. The mappings and the Low and Mid
// products are computed once per distinct point (k_point_tables). One pass over the
// coefficients, coalesced; HBM-bound for large polynomials.
#include "common.cuh"
#include <array>
#include <map>

namespace stwo {

constexpr uint32_t EP_LOW = 8, EP_MID = 8;
// Chunks of 2^(8 + 6) coefficients when the point tables are precomputed: a block then starts
// loading at once, and a 2^16-coefficient polynomial is four blocks, which balances the waves.
constexpr uint32_t EP_MID_TABLES = 6;

struct EvalJob {
  const uint32_t* coeffs;
  uint32_t log_size;
  uint32_t pad;
};

__device__ __forceinline__ qm31 qm31_double_x(qm31 x) {
  qm31 s = qm31_mul(x, x);
  return qm31_sub(qm31_add(s, s), qm31_from_u32(1, 0, 0, 0));
}

// Mapping j of the point: j = 0 -> y, j >= 1 -> pi^{j-1}(x).
__device__ __forceinline__ void point_mappings(const stwo_qm31_point& pt, uint32_t L, qm31* m) {
  m[0] = qm31_from_u32(pt.y.v[0], pt.y.v[1], pt.y.v[2], pt.y.v[3]);
  qm31 x = qm31_from_u32(pt.x.v[0], pt.x.v[1], pt.x.v[2], pt.x.v[3]);
  for (uint32_t j = 1; j < L; j++) {
    m[j] = x;
    x = qm31_double_x(x);
  }
}

// Per distinct point, in global memory: its EP_MAPS mappings, then the products Low[t] over the
// set bits of t of mappings [0, EP_LOW), then Mid[m] over those of [EP_LOW, EP_LOW + EP_MID).
// They depend on the point only, not on the polynomial's size (for L < EP_LOW only Low[t < 2^L]
// is read, which uses mappings below L).
constexpr uint32_t EP_MAPS = 30;
constexpr uint32_t EP_TABLE = EP_MAPS + (1u << EP_LOW) + (1u << EP_MID);

__device__ __forceinline__ void point_tables_block(const stwo_qm31_point& pt, qm31* __restrict__ tables) {
  __shared__ qm31 s_map[EP_MAPS];
  if (threadIdx.x == 0) point_mappings(pt, EP_MAPS, s_map);
  __syncthreads();
  qm31* T = tables + (size_t)blockIdx.x * EP_TABLE;
  const uint32_t t = threadIdx.x;
  if (t < EP_MAPS) T[t] = s_map[t];
  qm31 lo = qm31_from_u32(1, 0, 0, 0), mid = lo;
  for (uint32_t b = 0; b < EP_LOW; b++)
    if ((t >> b) & 1) lo = qm31_mul(lo, s_map[b]);
  for (uint32_t b = 0; b < EP_MID; b++)
    if ((t >> b) & 1) mid = qm31_mul(mid, s_map[EP_LOW + b]);
  T[EP_MAPS + t] = lo;
  T[EP_MAPS + (1u << EP_LOW) + t] = mid;
}
__global__ void __launch_bounds__(256) k_point_tables(const stwo_qm31_point* __restrict__ points, qm31* __restrict__ tables) {
  pdl_enter();
  point_tables_block(points[blockIdx.x], tables);
}
// The same with the points in the launch parameters (at most EP_PARAM_POINTS).
constexpr uint32_t EP_PARAM_POINTS = EP_MAX_POINTS;
struct EvalPoints {
  stwo_qm31_point p[EP_PARAM_POINTS];
};
__global__ void __launch_bounds__(256) k_point_tables_param(EvalPoints pts, qm31* __restrict__ tables) {
  pdl_enter();
  point_tables_block(pts.p[blockIdx.x], tables);
}

// One block per (chunk of 2^(EP_LOW + mid_max) coefficients, evaluation). With `tables` the
// point's mappings and products come from k_point_tables (table_of[e] names the evaluation's
// entry); without, the block derives them from points[e].
// With `work`, block b evaluates chunk work[2b + 1] of evaluation work[2b] (a flat list of the
// chunks that exist, so polynomials of different sizes launch no idle blocks); without, the grid is
// (chunks of the largest polynomial, evaluations) and blocks past a polynomial's chunks return.
__global__ void __launch_bounds__(256) k_eval_at_point(const EvalJob* __restrict__ jobs, const uint32_t* __restrict__ poly_of,
                                                       const stwo_qm31_point* __restrict__ points,
                                                       const qm31* __restrict__ tables,
                                                       const uint32_t* __restrict__ table_of, uint32_t mid_max,
                                                       unsigned long long* __restrict__ acc,
                                                       const uint32_t* __restrict__ work = nullptr) {
  pdl_enter();
  __shared__ qm31 s_map[32];
  __shared__ qm31 s_mid[1 << EP_MID];
  __shared__ qm31 s_part[8];
  __shared__ EvalJob s_job;
  __shared__ uint32_t s_table, s_e, s_chunk;
  if (threadIdx.x == 0) {
    const uint32_t e0 = work ? work[2 * blockIdx.x] : blockIdx.y;
    s_e = e0;
    s_chunk = work ? work[2 * blockIdx.x + 1] : blockIdx.x;
    s_job = jobs[poly_of[e0]];  // one read of the (possibly host-mapped) tables
    if (tables) s_table = table_of[e0];
  }
  __syncthreads();
  const uint32_t e = s_e, chunk = s_chunk;
  const EvalJob job = s_job;
  const uint32_t L = job.log_size;
  const uint32_t lo_bits = L < EP_LOW ? L : EP_LOW;
  const uint32_t mid_bits = L - lo_bits < mid_max ? L - lo_bits : mid_max;
  const uint32_t chunk_bits = lo_bits + mid_bits;
  const uint32_t n_chunks = 1u << (L - chunk_bits);
  if (chunk >= n_chunks) return;
  const qm31* T = tables ? tables + (size_t)s_table * EP_TABLE : nullptr;
  if (T) {
    if (threadIdx.x < EP_MAPS) s_map[threadIdx.x] = T[threadIdx.x];
    if (threadIdx.x < (1u << mid_bits)) s_mid[threadIdx.x] = T[EP_MAPS + (1u << EP_LOW) + threadIdx.x];
  } else {
    if (threadIdx.x == 0) point_mappings(points[e], L, s_map);
    __syncthreads();
    if (threadIdx.x < (1u << mid_bits)) {
      qm31 t = qm31_from_u32(1, 0, 0, 0);
      for (uint32_t b = 0; b < mid_bits; b++)
        if ((threadIdx.x >> b) & 1) t = qm31_mul(t, s_map[lo_bits + b]);
      s_mid[threadIdx.x] = t;
    }
  }
  __syncthreads();
  qm31 res = qm31_zero();
  const uint32_t t = threadIdx.x;
  if (t < (1u << lo_bits)) {
    const uint32_t* c = job.coeffs + ((size_t)chunk << chunk_bits);
    unsigned long long a0 = 0, a1 = 0, a2 = 0, a3 = 0;
    // Products are at most (P - 1)^2 < 2^62 - 2^33 + 4, and a folded sum is below 2^33 + 2^31:
    // folding after every fourth product keeps the sums below 2^64. Eight coefficient loads are
    // issued before they are used.
    const uint32_t n_mid = 1u << mid_bits;
    uint32_t m = 0;
    for (; m + 8 <= n_mid; m += 8) {
      uint32_t v[8];
#pragma unroll
      for (int k = 0; k < 8; k++) v[k] = __ldg(c + ((m + k) << lo_bits) + t);
#pragma unroll
      for (int k = 0; k < 8; k++) {
        const qm31 w = s_mid[m + k];
        a0 += (unsigned long long)w.a.a * v[k];
        a1 += (unsigned long long)w.a.b * v[k];
        a2 += (unsigned long long)w.b.a * v[k];
        a3 += (unsigned long long)w.b.b * v[k];
        if ((k & 3) == 3) {
          a0 = (a0 & P) + (a0 >> 31);
          a1 = (a1 & P) + (a1 >> 31);
          a2 = (a2 & P) + (a2 >> 31);
          a3 = (a3 & P) + (a3 >> 31);
        }
      }
    }
    for (; m < n_mid; m++) {
      const uint32_t v = __ldg(c + (m << lo_bits) + t);
      const qm31 w = s_mid[m];
      a0 = (a0 & P) + (a0 >> 31) + (unsigned long long)w.a.a * v;
      a1 = (a1 & P) + (a1 >> 31) + (unsigned long long)w.a.b * v;
      a2 = (a2 & P) + (a2 >> 31) + (unsigned long long)w.b.a * v;
      a3 = (a3 & P) + (a3 >> 31) + (unsigned long long)w.b.b * v;
    }
    auto red = [](unsigned long long x) {
      x = (x & P) + (x >> 31);
      x = (x & P) + (x >> 31);
      uint32_t r = (uint32_t)x;
      return r >= P ? r - P : r;
    };
    res = qm31_from_u32(red(a0), red(a1), red(a2), red(a3));
    qm31 low;
    if (T) {
      low = T[EP_MAPS + t];
    } else {
      low = qm31_from_u32(1, 0, 0, 0);
      for (uint32_t b = 0; b < lo_bits; b++)
        if ((t >> b) & 1) low = qm31_mul(low, s_map[b]);
    }
    res = qm31_mul(res, low);
  }
  // Block reduction of the QM31 partials.
  uint32_t w[4] = {res.a.a, res.a.b, res.b.a, res.b.b};
#pragma unroll
  for (int q = 0; q < 4; q++)
    for (int o = 16; o > 0; o >>= 1) w[q] = m31_add(w[q], __shfl_xor_sync(0xffffffffu, w[q], o));
  if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = qm31_from_u32(w[0], w[1], w[2], w[3]);
  __syncthreads();
  if (threadIdx.x == 0) {
    qm31 sum = qm31_zero();
    for (uint32_t i = 0; i < blockDim.x / 32; i++) sum = qm31_add(sum, s_part[i]);
    qm31 top = qm31_from_u32(1, 0, 0, 0);
    for (uint32_t b = chunk_bits; b < L; b++)
      if ((chunk >> (b - chunk_bits)) & 1) top = qm31_mul(top, s_map[b]);
    sum = qm31_mul(sum, top);
    atomicAdd(acc + 4 * e + 0, (unsigned long long)sum.a.a);
    atomicAdd(acc + 4 * e + 1, (unsigned long long)sum.a.b);
    atomicAdd(acc + 4 * e + 2, (unsigned long long)sum.b.a);
    atomicAdd(acc + 4 * e + 3, (unsigned long long)sum.b.b);
  }
}

// Canonical words of the 64-bit accumulators into out (and into dev_out when it is set).
__global__ void k_reduce_acc(const unsigned long long* acc, uint32_t n, uint32_t* out, uint32_t* dev_out = nullptr) {
  pdl_enter();
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  unsigned long long x = acc[i];
  x = (x & P) + (x >> 31);
  x = (x & P) + (x >> 31);
  uint32_t r = (uint32_t)x;
  r = r >= P ? r - P : r;
  out[i] = r;
  if (dev_out) dev_out[i] = r;
}

int32_t eval_at_points(const uint32_t* const* coeffs, const uint32_t* log_sizes, uint32_t n_polys,
                       const uint32_t* poly_of, const stwo_qm31_point* points, uint32_t n_evals, stwo_qm31* out,
                       cudaStream_t s) {
  if (n_evals == 0) return STWO_OK;
  STWO_REQUIRE(coeffs && log_sizes && poly_of && points && out, "null argument");
  std::vector<EvalJob> jobs(n_polys);
  for (uint32_t i = 0; i < n_polys; i++) {
    STWO_REQUIRE(log_sizes[i] <= 30, "poly log size %u > 30", log_sizes[i]);
    jobs[i] = {coeffs[i], log_sizes[i], 0};
  }
  for (uint32_t e = 0; e < n_evals; e++) STWO_REQUIRE(poly_of[e] < n_polys, "poly index out of range");
  STWO_REQUIRE(n_evals <= 65535, "too many evaluations in one call");
  // Evaluations share a handful of points (the mask offsets of one OODS point): the point tables
  // are built once per distinct point.
  std::map<std::array<uint32_t, 8>, uint32_t> uniq;
  std::vector<stwo_qm31_point> upts;
  std::vector<uint32_t> table_of(n_evals);
  for (uint32_t e = 0; e < n_evals; e++) {
    std::array<uint32_t, 8> key;
    std::memcpy(key.data(), &points[e], sizeof(key));
    auto it = uniq.find(key);
    if (it == uniq.end()) {
      it = uniq.emplace(key, (uint32_t)upts.size()).first;
      upts.push_back(points[e]);
    }
    table_of[e] = it->second;
  }
  const uint32_t n_pts = (uint32_t)upts.size();
  // The job tables go to the kernels through mapped host memory (read once per block) and the
  // results come back the same way: no staging copies around the launches.
  const size_t w_jobs = (jobs.size() * sizeof(EvalJob) + 15) / 16 * 4;
  const size_t w_polyof = ((size_t)n_evals + 3) / 4 * 4;
  const size_t w_tabof = w_polyof;
  const size_t w_pts = (size_t)n_pts * sizeof(stwo_qm31_point) / 4;
  const size_t w_out = (size_t)n_evals * 4;
  std::vector<uint32_t> work;  // (evaluation, chunk) of every block
  for (uint32_t e = 0; e < n_evals; e++) {
    const uint32_t L = log_sizes[poly_of[e]];
    const uint32_t cb = std::min(L, EP_LOW) + std::min(L - std::min(L, EP_LOW), EP_MID_TABLES);
    for (uint32_t c = 0; c < (1u << (L - cb)); c++) {
      work.push_back(e);
      work.push_back(c);
    }
  }
  STWO_REQUIRE(work.size() / 2 <= 0x7fffffffu, "too many chunks");
  Mapped mp;
  int32_t st = mapped_words(w_jobs + w_polyof + w_tabof + w_pts + w_out + work.size(), mp);
  if (st) return st;
  uint32_t* h_polyof = mp.host + w_jobs;
  uint32_t* h_tabof = h_polyof + w_polyof;
  uint32_t* h_pts = h_tabof + w_tabof;
  uint32_t* h_out = h_pts + w_pts;
  uint32_t* h_work = h_out + w_out;
  std::memcpy(h_work, work.data(), work.size() * 4);
  std::memcpy(mp.host, jobs.data(), jobs.size() * sizeof(EvalJob));
  std::memcpy(h_polyof, poly_of, (size_t)n_evals * 4);
  std::memcpy(h_tabof, table_of.data(), (size_t)n_evals * 4);
  std::memcpy(h_pts, upts.data(), (size_t)n_pts * sizeof(stwo_qm31_point));
  auto dev = [&](const uint32_t* h) { return mp.dev + (h - mp.host); };
  // One stream-ordered block: the 64-bit accumulators, then the point tables.
  const size_t acc_bytes = (size_t)n_evals * 32;
  unsigned char* scratch = nullptr;
  st = scratch_alloc((void**)&scratch, acc_bytes + (size_t)n_pts * EP_TABLE * sizeof(qm31), s);
  if (st) return st;
  unsigned long long* acc = reinterpret_cast<unsigned long long*>(scratch);
  qm31* tables = reinterpret_cast<qm31*>(scratch + acc_bytes);
  cudaError_t err = cudaMemsetAsync(acc, 0, acc_bytes, s);
  if (!err) {
    launch_pdl(k_point_tables, dim3(n_pts), dim3(1u << EP_LOW), 0, s,
               reinterpret_cast<const stwo_qm31_point*>(dev(h_pts)), tables);
    note_launch();
    err = cudaGetLastError();
  }
  if (!err) {
    launch_pdl(k_eval_at_point, dim3((uint32_t)(work.size() / 2)), dim3(256), 0, s,
               reinterpret_cast<const EvalJob*>(mp.dev), dev(h_polyof), nullptr, tables, dev(h_tabof), EP_MID_TABLES,
               acc, dev(h_work));
    note_launch();
    err = cudaGetLastError();
  }
  if (!err) {
    launch_pdl(k_reduce_acc, dim3((n_evals * 4 + 255) / 256), dim3(256), 0, s, acc, n_evals * 4, dev(h_out),
               nullptr);
    note_launch();
    err = cudaGetLastError();
  }
  scratch_free(scratch, s);
  if (!err) err = cudaStreamSynchronize(s);
  if (err) {
    set_error("eval_at_points: %s", cudaGetErrorString(err));
    return STWO_ERR_CUDA;
  }
  std::memcpy(out, h_out, (size_t)n_evals * 16);
  return STWO_OK;
}

// ---------------------------------------------------------------- planned evaluation (the prover's OODS)
int32_t eval_plan_build(const uint32_t* const* coeffs, const uint32_t* log_sizes, uint32_t n_polys,
                        const uint32_t* poly_of, const uint32_t* point_of, uint32_t n_evals, uint32_t n_points,
                        cudaStream_t s, EvalPlan* plan) {
  STWO_REQUIRE(plan && coeffs && log_sizes && poly_of && point_of, "null argument");
  STWO_REQUIRE(n_evals >= 1, "no evaluations");
  STWO_REQUIRE(n_points >= 1 && n_points <= EP_PARAM_POINTS, "%u points (at most %u)", n_points, EP_PARAM_POINTS);
  std::vector<EvalJob> jobs(n_polys);
  for (uint32_t i = 0; i < n_polys; i++) {
    STWO_REQUIRE(log_sizes[i] <= 30, "poly log size %u > 30", log_sizes[i]);
    jobs[i] = {coeffs[i], log_sizes[i], 0};
  }
  std::vector<uint32_t> work;  // (evaluation, chunk) of every block
  for (uint32_t e = 0; e < n_evals; e++) {
    STWO_REQUIRE(poly_of[e] < n_polys && point_of[e] < n_points, "evaluation %u: index out of range", e);
    const uint32_t L = log_sizes[poly_of[e]];
    const uint32_t cb = std::min(L, EP_LOW) + std::min(L - std::min(L, EP_LOW), EP_MID_TABLES);
    for (uint32_t c = 0; c < (1u << (L - cb)); c++) {
      work.push_back(e);
      work.push_back(c);
    }
  }
  STWO_REQUIRE(work.size() / 2 <= 0x7fffffffu, "too many chunks");
  // One device block: jobs, poly_of, point_of, work (uploaded now), then the 64-bit accumulators
  // and the point tables (written at run time). Every part starts on a 16-byte boundary.
  auto up16 = [](size_t b) { return (b + 15) / 16 * 16; };
  EvalPlan p;
  p.n_evals = n_evals;
  p.n_points = n_points;
  p.n_blocks = (uint32_t)(work.size() / 2);
  p.off_polyof = up16(jobs.size() * sizeof(EvalJob));
  p.off_pointof = p.off_polyof + up16((size_t)n_evals * 4);
  p.off_work = p.off_pointof + up16((size_t)n_evals * 4);
  p.off_acc = p.off_work + up16(work.size() * 4);
  p.off_vals = p.off_acc + (size_t)n_evals * 32;
  p.off_tables = p.off_vals + up16((size_t)n_evals * 16);
  const size_t bytes = p.off_tables + (size_t)n_points * EP_TABLE * sizeof(qm31);
  std::vector<unsigned char> host(p.off_acc, 0);
  std::memcpy(host.data(), jobs.data(), jobs.size() * sizeof(EvalJob));
  std::memcpy(host.data() + p.off_polyof, poly_of, (size_t)n_evals * 4);
  std::memcpy(host.data() + p.off_pointof, point_of, (size_t)n_evals * 4);
  std::memcpy(host.data() + p.off_work, work.data(), work.size() * 4);
  int32_t st = scratch_alloc((void**)&p.d, bytes, s);
  if (st) return st;
  cudaError_t err = cudaMemcpyAsync(p.d, host.data(), host.size(), cudaMemcpyHostToDevice, s);
  if (err) {
    scratch_free(p.d, s);
    set_error("eval_plan_build: %s", cudaGetErrorString(err));
    return STWO_ERR_CUDA;
  }
  *plan = p;
  return STWO_OK;
}

int32_t eval_plan_run(const EvalPlan& p, const stwo_qm31_point* points, stwo_qm31* out, cudaStream_t s) {
  STWO_REQUIRE(p.d && points && out, "null argument");
  EvalPoints ep{};
  for (uint32_t i = 0; i < p.n_points; i++) ep.p[i] = points[i];
  Mapped mp;
  int32_t st = mapped_words((size_t)p.n_evals * 4, mp);
  if (st) return st;
  unsigned long long* acc = reinterpret_cast<unsigned long long*>(p.d + p.off_acc);
  qm31* tables = reinterpret_cast<qm31*>(p.d + p.off_tables);
  cudaError_t err = cudaMemsetAsync(acc, 0, (size_t)p.n_evals * 32, s);
  if (!err) {
    launch_pdl(k_point_tables_param, dim3(p.n_points), dim3(1u << EP_LOW), 0, s, ep, tables);
    note_launch();
    err = cudaGetLastError();
  }
  if (!err) {
    launch_pdl(k_eval_at_point, dim3(p.n_blocks), dim3(256), 0, s, reinterpret_cast<const EvalJob*>(p.d),
               reinterpret_cast<const uint32_t*>(p.d + p.off_polyof), nullptr, tables,
               reinterpret_cast<const uint32_t*>(p.d + p.off_pointof), EP_MID_TABLES, acc,
               reinterpret_cast<const uint32_t*>(p.d + p.off_work));
    note_launch();
    err = cudaGetLastError();
  }
  if (!err) {
    launch_pdl(k_reduce_acc, dim3((p.n_evals * 4 + 255) / 256), dim3(256), 0, s, acc, p.n_evals * 4, mp.dev,
               reinterpret_cast<uint32_t*>(p.d + p.off_vals));
    note_launch();
    err = cudaGetLastError();
  }
  if (!err) err = cudaStreamSynchronize(s);
  if (err) {
    set_error("eval_plan_run: %s", cudaGetErrorString(err));
    return STWO_ERR_CUDA;
  }
  std::memcpy(out, mp.host, (size_t)p.n_evals * 16);
  return STWO_OK;
}

void eval_plan_free(EvalPlan& p, cudaStream_t s) {
  if (p.d) scratch_free(p.d, s);
  p.d = nullptr;
}

// ---------------------------------------------------------------- eval_at_points without allocation
// Same computation as eval_at_points, for callers that must not allocate device memory: a process
// whose HBM is handed out by its own pool manager (a serving loop that reserves its budget up
// front and forbids any other allocation), or code running where cudaMalloc/cudaFree would stall
// other streams or device-wide synchronise. Its scratch is a fixed static device array instead of
// a stream-ordered allocation. Every GPU that loads this library keeps the array until exit.
constexpr uint32_t NOALLOC_MAX_EVALS = STWO_NOALLOC_MAX_EVALS;
constexpr uint32_t NOALLOC_MAX_POLYS = STWO_NOALLOC_MAX_POLYS;
constexpr size_t NA_OFF_JOBS = 0;
constexpr size_t NA_OFF_POLYOF = NA_OFF_JOBS + (size_t)NOALLOC_MAX_POLYS * sizeof(EvalJob);
constexpr size_t NA_OFF_PTS = NA_OFF_POLYOF + (size_t)NOALLOC_MAX_EVALS * 4;
constexpr size_t NA_OFF_ACC = NA_OFF_PTS + (size_t)NOALLOC_MAX_EVALS * sizeof(stwo_qm31_point);
constexpr size_t NA_OFF_OUT = NA_OFF_ACC + (size_t)NOALLOC_MAX_EVALS * 4 * 8;
constexpr size_t NA_BYTES = NA_OFF_OUT + (size_t)NOALLOC_MAX_EVALS * 16;
static_assert(NA_OFF_POLYOF % 8 == 0 && NA_OFF_PTS % 8 == 0 && NA_OFF_ACC % 8 == 0, "scratch alignment");

static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

// Device address of g_noalloc_scratch in the current device's context. It is looked up on every
// call (cudaGetSymbolAddress allocates nothing): a cached address would go stale after a device
// reset or when the caller makes a context current that is not the device's primary one. The
// host-side symbol is only a stand-in and must never reach a kernel.
static int32_t noalloc_scratch(unsigned char** out) {
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p) {
    set_error("cudaGetSymbolAddress of the no-alloc scratch: %s", cudaGetErrorString(e));
    return STWO_ERR_CUDA;
  }
  *out = reinterpret_cast<unsigned char*>(p);
  return STWO_OK;
}

int32_t eval_at_points_noalloc(const uint32_t* const* coeffs, const uint32_t* log_sizes, uint32_t n_polys,
                               const uint32_t* poly_of, const stwo_qm31_point* points, uint32_t n_evals,
                               stwo_qm31* out, cudaStream_t s) {
  if (n_evals == 0) return STWO_OK;
  STWO_REQUIRE(coeffs && log_sizes && poly_of && points && out, "null argument");
  STWO_REQUIRE(n_evals <= NOALLOC_MAX_EVALS, "n_evals %u exceeds the no-alloc maximum of %u", n_evals,
               NOALLOC_MAX_EVALS);
  STWO_REQUIRE(n_polys <= NOALLOC_MAX_POLYS, "n_polys %u exceeds the no-alloc maximum of %u", n_polys,
               NOALLOC_MAX_POLYS);
  EvalJob jobs[NOALLOC_MAX_POLYS];
  uint32_t max_chunks = 1;
  for (uint32_t i = 0; i < n_polys; i++) {
    STWO_REQUIRE(log_sizes[i] <= 30, "poly log size %u > 30", log_sizes[i]);
    jobs[i] = {coeffs[i], log_sizes[i], 0};
  }
  for (uint32_t e = 0; e < n_evals; e++) {
    STWO_REQUIRE(poly_of[e] < n_polys, "poly index out of range");
    uint32_t L = log_sizes[poly_of[e]];
    uint32_t cb = std::min(L, EP_LOW) + std::min(L - std::min(L, EP_LOW), EP_MID);
    max_chunks = std::max(max_chunks, 1u << (L - cb));
  }
  unsigned char* buf = nullptr;
  int32_t st = noalloc_scratch(&buf);
  if (st) return st;
  cudaError_t err = cudaSuccess;
  if (n_polys) err = cudaMemcpyAsync(buf + NA_OFF_JOBS, jobs, n_polys * sizeof(EvalJob), cudaMemcpyHostToDevice, s);
  if (!err) err = cudaMemcpyAsync(buf + NA_OFF_POLYOF, poly_of, (size_t)n_evals * 4, cudaMemcpyHostToDevice, s);
  if (!err) err = cudaMemcpyAsync(buf + NA_OFF_PTS, points, (size_t)n_evals * sizeof(stwo_qm31_point), cudaMemcpyHostToDevice, s);
  // The accumulators keep the previous call's sums: they must start at zero.
  if (!err) err = cudaMemsetAsync(buf + NA_OFF_ACC, 0, (size_t)n_evals * 32, s);
  if (!err) {
    dim3 grid(max_chunks, n_evals);
    launch_pdl(k_eval_at_point, grid, dim3(256), 0, s, reinterpret_cast<EvalJob*>(buf + NA_OFF_JOBS),
               reinterpret_cast<uint32_t*>(buf + NA_OFF_POLYOF), reinterpret_cast<stwo_qm31_point*>(buf + NA_OFF_PTS),
               nullptr, nullptr, EP_MID, reinterpret_cast<unsigned long long*>(buf + NA_OFF_ACC), nullptr);
    note_launch();
    err = cudaGetLastError();
  }
  if (!err) {
    launch_pdl(k_reduce_acc, dim3((n_evals * 4 + 255) / 256), dim3(256), 0, s,
               reinterpret_cast<unsigned long long*>(buf + NA_OFF_ACC), n_evals * 4,
               reinterpret_cast<uint32_t*>(buf + NA_OFF_OUT), nullptr);
    note_launch();
    err = cudaGetLastError();
  }
  if (!err) err = cudaMemcpyAsync(out, buf + NA_OFF_OUT, (size_t)n_evals * 16, cudaMemcpyDeviceToHost, s);
  if (!err) err = cudaStreamSynchronize(s);
  if (err) {
    set_error("eval_at_points_noalloc: %s", cudaGetErrorString(err));
    return STWO_ERR_CUDA;
  }
  return STWO_OK;
}

// ---------------------------------------------------------------- bit reverse
__global__ void k_bit_reverse(uint32_t* col, uint32_t log_n) {
  uint32_t n = 1u << log_n;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    uint32_t j = brev(i, log_n);
    if (i < j) {
      uint32_t a = col[i];
      col[i] = col[j];
      col[j] = a;
    }
  }
}

// ---------------------------------------------------------------- accumulation
__global__ void k_secure_accumulate(uint32_t* a0, uint32_t* a1, uint32_t* a2, uint32_t* a3, const uint32_t* b0,
                                    const uint32_t* b1, const uint32_t* b2, const uint32_t* b3, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    a0[i] = m31_add(a0[i], __ldg(b0 + i));
    a1[i] = m31_add(a1[i], __ldg(b1 + i));
    a2[i] = m31_add(a2[i], __ldg(b2 + i));
    a3[i] = m31_add(a3[i], __ldg(b3 + i));
  }
}

// out[j] = felt^i with j = i, or j = n - 1 - i when `reversed` (highest power first, the order of
// the composition's random coefficients).
__global__ void k_secure_powers(qm31 felt, uint32_t n, uint32_t reversed, uint32_t* out) {
  pdl_enter();
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  qm31 r = qm31_from_u32(1, 0, 0, 0), b = felt;
  uint32_t e = i;
  while (e) {
    if (e & 1) r = qm31_mul(r, b);
    b = qm31_mul(b, b);
    e >>= 1;
  }
  const uint32_t j = reversed ? n - 1 - i : i;
  out[4 * j] = r.a.a;
  out[4 * j + 1] = r.a.b;
  out[4 * j + 2] = r.b.a;
  out[4 * j + 3] = r.b.b;
}

int32_t secure_powers_reversed(const uint32_t felt[4], uint32_t n, uint32_t* out, cudaStream_t s) {
  if (n == 0) return STWO_OK;
  const qm31 f = {{felt[0], felt[1]}, {felt[2], felt[3]}};
  launch_pdl(k_secure_powers, dim3((n + 255) / 256), dim3(256), 0, s, f, n, 1u, out);
  note_launch();
  STWO_LAUNCH_CHECK();
  return STWO_OK;
}

__global__ void k_gather(const uint32_t* col, const unsigned long long* idx, size_t n, uint32_t* out) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = col[idx[i]];
}
// out[c * n + i] = cols[c][idx[i]] over total = n_cols * n words (decommitment reads of a
// Merkle layer's columns at the same positions).
__global__ void k_gather_cols(const uint32_t* const* cols, const unsigned long long* idx, size_t n, size_t total,
                              uint32_t* out) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < total) out[t] = __ldg(cols[t / n] + idx[t % n]);
}

static uint32_t grid_cap(size_t n, uint32_t threads) {
  size_t b = (n + threads - 1) / threads;
  size_t cap = (size_t)sm_count() * 16;
  return (uint32_t)std::max<size_t>(1, std::min(b, cap));
}

}  // namespace stwo

using namespace stwo;

extern "C" {

stwo_status stwo_eval_at_points(const uint32_t* const* d_coeffs, const uint32_t* h_log_sizes, uint32_t n_polys,
                                const uint32_t* h_poly_of, const stwo_qm31_point* h_points, uint32_t n_evals,
                                stwo_qm31* h_out, void* stream) {
  return eval_at_points(d_coeffs, h_log_sizes, n_polys, h_poly_of, h_points, n_evals, h_out, as_stream(stream));
}

stwo_status stwo_eval_at_points_noalloc(const uint32_t* const* d_coeffs, const uint32_t* h_log_sizes,
                                        uint32_t n_polys, const uint32_t* h_poly_of, const stwo_qm31_point* h_points,
                                        uint32_t n_evals, stwo_qm31* h_out, void* stream) {
  return eval_at_points_noalloc(d_coeffs, h_log_sizes, n_polys, h_poly_of, h_points, n_evals, h_out,
                                as_stream(stream));
}

stwo_status stwo_extend(const uint32_t* d_coeffs, uint32_t coeff_log_size, uint32_t* d_out, uint32_t log_size,
                        void* stream) {
  STWO_REQUIRE(log_size >= coeff_log_size && log_size <= 30, "extend to a smaller size");
  cudaStream_t s = as_stream(stream);
  size_t n0 = (size_t)1 << coeff_log_size, n1 = (size_t)1 << log_size;
  if (d_out != d_coeffs) STWO_CHECK_CUDA(cudaMemcpyAsync(d_out, d_coeffs, n0 * 4, cudaMemcpyDeviceToDevice, s));
  if (n1 > n0) STWO_CHECK_CUDA(cudaMemsetAsync(d_out + n0, 0, (n1 - n0) * 4, s));
  return STWO_OK;
}

stwo_status stwo_bit_reverse_column(uint32_t* d_col, uint32_t log_size, void* stream) {
  STWO_REQUIRE(log_size <= 30, "log size > 30");
  k_bit_reverse<<<grid_cap((size_t)1 << log_size, 256), 256, 0, as_stream(stream)>>>(d_col, log_size); note_launch();
  STWO_LAUNCH_CHECK();
  return STWO_OK;
}

stwo_status stwo_secure_accumulate(uint32_t* const d_acc[4], const uint32_t* const d_other[4], size_t n,
                                   void* stream) {
  if (n == 0) return STWO_OK;
  k_secure_accumulate<<<grid_cap(n, 256), 256, 0, as_stream(stream)>>>(d_acc[0], d_acc[1], d_acc[2], d_acc[3],
                                                                       d_other[0], d_other[1], d_other[2],
                                                                       d_other[3], n); note_launch();
  STWO_LAUNCH_CHECK();
  return STWO_OK;
}

stwo_status stwo_generate_secure_powers(stwo_qm31 felt, uint32_t n_powers, stwo_qm31* h_out, void* stream) {
  if (n_powers == 0) return STWO_OK;
  STWO_REQUIRE(h_out, "null output");
  cudaStream_t s = as_stream(stream);
  uint32_t* d = nullptr;
  int32_t st = scratch_alloc((void**)&d, (size_t)n_powers * 16, s);
  if (st) return st;
  qm31 f = {{felt.v[0], felt.v[1]}, {felt.v[2], felt.v[3]}};
  launch_pdl(k_secure_powers, dim3((n_powers + 255) / 256), dim3(256), 0, s, f, n_powers, 0u, d); note_launch();
  cudaError_t e = cudaGetLastError();
  if (!e) e = cudaMemcpyAsync(h_out, d, (size_t)n_powers * 16, cudaMemcpyDeviceToHost, s);
  scratch_free(d, s);
  if (!e) e = cudaStreamSynchronize(s);
  if (e) {
    set_error("secure powers: %s", cudaGetErrorString(e));
    return STWO_ERR_CUDA;
  }
  return STWO_OK;
}

stwo_status stwo_read_words_cols(const uint32_t* const* h_cols, size_t n_cols, const uint64_t* h_idx, size_t n,
                                 uint32_t* h_out, void* stream) {
  if (n == 0 || n_cols == 0) return STWO_OK;
  STWO_REQUIRE(h_cols && h_idx && h_out, "null argument");
  STWO_REQUIRE(n_cols * n <= ((size_t)1 << 31), "too many words");
  cudaStream_t s = as_stream(stream);
  const size_t tab = n_cols * 8, idx = n * 8, out = n_cols * n * 4;
  char* buf = nullptr;
  int32_t st = scratch_alloc((void**)&buf, tab + idx + out + 16, s);
  if (st) return st;
  const uint32_t** d_cols = reinterpret_cast<const uint32_t**>(buf);
  unsigned long long* d_idx = reinterpret_cast<unsigned long long*>(buf + tab);
  uint32_t* d_out = reinterpret_cast<uint32_t*>(buf + tab + idx);
  cudaError_t e = cudaMemcpyAsync(d_cols, h_cols, tab, cudaMemcpyHostToDevice, s);
  if (!e) e = cudaMemcpyAsync(d_idx, h_idx, idx, cudaMemcpyHostToDevice, s);
  if (!e) {
    const size_t total = n_cols * n;
    k_gather_cols<<<(uint32_t)((total + 255) / 256), 256, 0, s>>>(d_cols, d_idx, n, total, d_out); note_launch();
    e = cudaGetLastError();
  }
  if (!e) e = cudaMemcpyAsync(h_out, d_out, out, cudaMemcpyDeviceToHost, s);
  scratch_free(buf, s);
  if (!e) e = cudaStreamSynchronize(s);
  if (e) {
    set_error("read_words_cols: %s", cudaGetErrorString(e));
    return STWO_ERR_CUDA;
  }
  return STWO_OK;
}

stwo_status stwo_read_words(const uint32_t* d_col, const uint64_t* h_idx, size_t n, uint32_t* h_out, void* stream) {
  if (n == 0) return STWO_OK;
  STWO_REQUIRE(d_col && h_idx && h_out, "null argument");
  cudaStream_t s = as_stream(stream);
  char* buf = nullptr;
  int32_t st = scratch_alloc((void**)&buf, n * 12 + 16, s);
  if (st) return st;
  unsigned long long* d_idx = reinterpret_cast<unsigned long long*>(buf);
  uint32_t* d_out = reinterpret_cast<uint32_t*>(buf + n * 8);
  cudaError_t e = cudaMemcpyAsync(d_idx, h_idx, n * 8, cudaMemcpyHostToDevice, s);
  if (!e) {
    k_gather<<<(uint32_t)((n + 255) / 256), 256, 0, s>>>(d_col, d_idx, n, d_out); note_launch();
    e = cudaGetLastError();
  }
  if (!e) e = cudaMemcpyAsync(h_out, d_out, n * 4, cudaMemcpyDeviceToHost, s);
  scratch_free(buf, s);
  if (!e) e = cudaStreamSynchronize(s);
  if (e) {
    set_error("read_words: %s", cudaGetErrorString(e));
    return STWO_ERR_CUDA;
  }
  return STWO_OK;
}

}  // extern "C"
