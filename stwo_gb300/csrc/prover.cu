// GPU prover host: prove() of the reference (crates/prover/src/core/prover/mod.rs:27-79) over this
// backend, with every O(trace) stage on the device:
//   commitment trees  pcs/prover.rs:208-227  (FFT extension + Blake2s Merkle, trees kept in HBM)
//   composition       air/components.rs:122-137, constraint_framework/component.rs:278-416
//                     (one constraint kernel per AIR; accumulation, denominators, interpolation)
//   opening           pcs/prover.rs:83-148 (batched eval_at_point, quotients per log size)
//   FRI               fri.rs:168-336 (folds and layer Merkle trees on the device)
//   decommitment      vcs/prover.rs:80-149 and fri.rs:295-336: query positions and witness
//                     structure are computed on the host, the words themselves are gathered from
//                     HBM in one kernel launch
// The transcript (Blake2s channel) and the O(1)-size last FRI layer interpolation stay on the host,
// as in the reference. Proofs are written in the canonical byte form (little-endian u32 words,
// u64 lengths, struct order).
#include "common.cuh"
#include "host_channel.h"
#include "prover.cuh"
#include "dchannel.cuh"
#include <array>
#include <set>

namespace stwo {

int32_t fft_interpolate(const TwiddleTree* tree, stwo_coset half, uint32_t* const* cols, uint32_t n, cudaStream_t s);
int32_t fft_evaluate(const TwiddleTree* tree, stwo_coset half, const uint32_t* const* coeffs, uint32_t coeff_log,
                     uint32_t* const* out, uint32_t n, cudaStream_t s);
int32_t fft_interpolate_extend_begin(const TwiddleTree* tree_src, stwo_coset src_half, uint32_t* const* cols,
                                     uint32_t n, const TwiddleTree* tree_dst, stwo_coset dst_half,
                                     uint32_t* const* out, cudaStream_t s, bool* fused);
int32_t fft_interpolate_extend_end(const TwiddleTree* tree_dst, stwo_coset dst_half, uint32_t coeff_log,
                                   uint32_t* const* cols, uint32_t n, uint32_t* const* out, bool fused,
                                   cudaStream_t s);
int32_t merkle_commit_layer(uint32_t log_size, const uint32_t* prev, const uint32_t* const* cols, uint32_t n_cols,
                            uint32_t* out, cudaStream_t s);
int32_t merkle_node_layers(const uint32_t* prev, uint32_t first_log, uint32_t n_levels, uint32_t* const* out,
                           cudaStream_t s, DevChannel* ch = nullptr, uint32_t* alpha_out = nullptr);
int32_t accumulate_quotients(uint32_t log_n, const uint32_t* const* cols, uint32_t n_cols, stwo_qm31 rc_in,
                             const stwo_sample_batch* batches, uint32_t n_batches, uint32_t log_blowup,
                             uint32_t* const out[4], cudaStream_t s);
// With `leaves` set, the fold also writes the Merkle leaves of the next FRI layer (8 words per
// folded point), so that layer's tree starts at its first node level.
int32_t fri_fold_line(const TwiddleTree* tree, stwo_coset line_domain, const uint32_t* const src[4], qm31 alpha,
                      uint32_t* const out[4], cudaStream_t s, const uint32_t* alpha_dev, uint32_t* leaves);
int32_t fri_fold_circle(const TwiddleTree* tree, stwo_coset half, uint32_t* const dst[4], const uint32_t* const src[4],
                        qm31 alpha, cudaStream_t s, const uint32_t* alpha_dev, uint32_t* leaves);
int32_t fri_channel_step(DevChannel* ch, const uint32_t* root, uint32_t* alpha_out, cudaStream_t s);
int32_t fri_tail(const TwiddleTree* tree, const std::vector<stwo_coset>& doms,
                 const std::vector<std::array<uint32_t*, 4>>& evals, const std::vector<uint32_t*>& trees,
                 DevChannel* ch, uint32_t* alphas, cudaStream_t s);
// FRI layers of at most 2^FRI_TAIL_LOG points run in the single-launch tail (fri_tail).
constexpr uint32_t FRI_TAIL_LOG = 10;
int32_t channel_set(DevChannel* ch, const uint32_t digest[8], uint64_t n_sent, cudaStream_t s);

// Copies segments of device words into one destination (mapped host memory) in one launch.
constexpr int COLLECT_MAX = 48;
struct CollectList {
  const uint32_t* src[COLLECT_MAX];
  uint32_t n[COLLECT_MAX];
  uint32_t count;
};
__global__ void k_collect(CollectList l, uint32_t* out) {
  pdl_enter();
  uint32_t base = 0;
  for (uint32_t k = 0; k < l.count; k++) {
    for (uint32_t i = threadIdx.x; i < l.n[k]; i += blockDim.x) out[base + i] = l.src[k][i];
    base += l.n[k];
  }
}
// rc^(n-1), ..., rc, 1 as 4-word QM31 values into out (AccumulationOps::generate_secure_powers,
// reversed).
int32_t secure_powers_reversed(const uint32_t felt[4], uint32_t n, uint32_t* out, cudaStream_t s);

// ------------------------------------------------------------------------------------------------
Arena::~Arena() {
  for (void* p : ptrs) cudaFreeAsync(p, s);
}
uint32_t* Arena::alloc(size_t words) {
  const size_t bytes = (std::max<size_t>(words, 1) * 4 + 255) / 256 * 256;
  if (bytes > CHUNK / 4) {
    void* p = nullptr;
    if (scratch_alloc(&p, bytes, s) != STWO_OK) {
      failed = true;
      return nullptr;
    }
    ptrs.push_back(p);
    return reinterpret_cast<uint32_t*>(p);
  }
  if (!chunk || chunk_used + bytes > CHUNK) {
    void* p = nullptr;
    if (scratch_alloc(&p, CHUNK, s) != STWO_OK) {
      failed = true;
      return nullptr;
    }
    ptrs.push_back(p);
    chunk = reinterpret_cast<char*>(p);
    chunk_used = 0;
  }
  uint32_t* r = reinterpret_cast<uint32_t*>(chunk + chunk_used);
  chunk_used += bytes;
  return r;
}

// ------------------------------------------------------------------------------------------------
// Gather of words from HBM in one launch. Threads [0, nv) read one value each, [nv, nv + nh) one
// 8-word hash each; then one block per run reads its `count` strided words. Requests and results
// live in mapped host memory.
__global__ void k_gather(const unsigned long long* vreq, uint32_t nv, const unsigned long long* hreq, uint32_t nh,
                         const unsigned long long* rreq, uint32_t first_run_block, uint32_t* vout, uint32_t* hout) {
  pdl_enter();
  if (blockIdx.x >= first_run_block) {
    const unsigned long long* r = rreq + 4 * (size_t)(blockIdx.x - first_run_block);
    const uint32_t* base = reinterpret_cast<const uint32_t*>(r[0]);
    const size_t stride = r[1], idx = r[2];
    const uint32_t slot = (uint32_t)r[3], count = (uint32_t)(r[3] >> 32);
    for (uint32_t k = threadIdx.x; k < count; k += blockDim.x) vout[slot + k] = base[(size_t)k * stride + idx];
    return;
  }
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nv) {
    vout[vreq[3 * i + 2]] = reinterpret_cast<const uint32_t*>(vreq[3 * i])[vreq[3 * i + 1]];
  } else if (i < nv + nh) {
    const uint32_t j = i - nv;
    const uint4* p = reinterpret_cast<const uint4*>(reinterpret_cast<const uint32_t*>(hreq[2 * j]) + hreq[2 * j + 1] * 8);
    uint4 a = p[0], b = p[1];
    uint32_t* o = hout + (size_t)j * 8;
    o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w;
    o[4] = b.x; o[5] = b.y; o[6] = b.z; o[7] = b.w;
  }
}

int32_t Gather::run(cudaStream_t s) {
  const size_t nv = vreq.size() / 3, nh = hptr.size(), nr = rreq.size() / 4;
  vres.assign(n_slots, 0);
  hres.assign(nh * 8, 0);
  if (nv + nh + nr == 0) return STWO_OK;
  Mapped mp;
  const size_t w_req = 2 * (3 * nv + 2 * nh + 4 * nr);  // request words (u64 = 2 words)
  int32_t st = mapped_words(w_req + n_slots + 8 * nh, mp);
  if (st) return st;
  unsigned long long* req = reinterpret_cast<unsigned long long*>(mp.host);
  std::memcpy(req, vreq.data(), vreq.size() * 8);
  unsigned long long* hq_ = req + 3 * nv;
  for (size_t i = 0; i < nh; i++) {
    hq_[2 * i] = hptr[i];
    hq_[2 * i + 1] = hidx[i];
  }
  std::memcpy(hq_ + 2 * nh, rreq.data(), rreq.size() * 8);
  const unsigned long long* dreq = reinterpret_cast<const unsigned long long*>(mp.dev);
  uint32_t* dres = mp.dev + w_req;
  const uint32_t single_blocks = (uint32_t)((nv + nh + 127) / 128);
  launch_pdl(k_gather, dim3(single_blocks + (uint32_t)nr), dim3(128), 0, s, dreq, (uint32_t)nv, dreq + 3 * nv,
             (uint32_t)nh, dreq + 3 * nv + 2 * nh, single_blocks, dres, dres + n_slots);
  note_launch();
  cudaError_t e = cudaGetLastError();
  if (!e) e = cudaStreamSynchronize(s);
  if (e) {
    set_error("gather: %s", cudaGetErrorString(e));
    return STWO_ERR_CUDA;
  }
  const uint32_t* res = mp.host + w_req;
  std::memcpy(vres.data(), res, n_slots * 4);
  std::memcpy(hres.data(), res + n_slots, nh * 32);
  return STWO_OK;
}

// ------------------------------------------------------------------------------------------------

int32_t DevMerkle::commit(const std::vector<ColRef>& columns, Arena& arena, cudaStream_t s, bool read_root,
                          DevChannel* ch, uint32_t* alpha_out) {
  channel_fused = false;
  sorted = columns;
  std::stable_sort(sorted.begin(), sorted.end(), [](const ColRef& a, const ColRef& b) { return a.log > b.log; });
  uint32_t max_log = sorted.empty() ? 0 : sorted[0].log;
  layers.assign(max_log + 1, nullptr);
  // One block for all layers: 2^(max_log + 1) - 1 hashes.
  uint32_t* all = arena.alloc((size_t)8 * ((2ull << max_log) - 1));
  if (!all) return STWO_ERR_OOM;
  for (uint32_t lg = 0; lg <= max_log; lg++) layers[lg] = all + (size_t)8 * ((1ull << lg) - 1);
  size_t ci = 0;
  int lg = (int)max_log;
  while (lg >= 0) {
    std::vector<const uint32_t*> lc;
    while (ci < sorted.size() && sorted[ci].log == (uint32_t)lg) lc.push_back(sorted[ci++].p);
    // Columns that lie a fixed stride apart (one column block) are gathered as one run per node.
    size_t stride = 0;
    if (lc.size() >= 8 && lc[1] > lc[0]) {
      stride = (size_t)(lc[1] - lc[0]);
      for (size_t k = 2; k < lc.size() && stride; k++)
        if (lc[k] != lc[0] + k * stride) stride = 0;
    }
    const uint32_t* prev = (uint32_t)lg < max_log ? layers[lg + 1] : nullptr;
    if (!lc.empty() || !prev) {
      int32_t st = merkle_commit_layer((uint32_t)lg, prev, lc.data(), (uint32_t)lc.size(), layers[lg], s);
      if (st) return st;
      lg--;
      continue;
    }
    // A run of layers made only of child hashes, down to the next layer with columns.
    int stop = lg;
    while (stop - 1 >= 0 && !(ci < sorted.size() && sorted[ci].log == (uint32_t)(stop - 1))) stop--;
    std::vector<uint32_t*> outs;
    for (int l = lg; l >= stop; l--) outs.push_back(layers[l]);
    // The run that ends at the root can carry the FRI transcript step in its last launch.
    DevChannel* c = stop == 0 ? ch : nullptr;
    int32_t st = merkle_node_layers(prev, (uint32_t)lg, (uint32_t)outs.size(), outs.data(), s, c, alpha_out);
    if (st) return st;
    if (c) channel_fused = true;
    lg = stop - 1;
  }
  return read_root ? this->read_root(s) : STWO_OK;
}

int32_t DevMerkle::read_root(cudaStream_t s) {
  Mapped mp;
  int32_t st = mapped_words(8, mp);
  if (st) return st;
  STWO_CHECK_CUDA(cudaMemcpyAsync(mp.host, layers[0], 32, cudaMemcpyDeviceToHost, s));
  STWO_CHECK_CUDA(cudaStreamSynchronize(s));
  root = Digest::from_words(mp.host);
  return STWO_OK;
}

// The tree of columns whose leaf hashes are already in `all` (the layout of commit: layer lg at
// offset 8 (2^lg - 1)): only the node levels run, the last launch also taking the transcript step.
int32_t DevMerkle::commit_from_leaves(const std::vector<ColRef>& columns, uint32_t* all, cudaStream_t s,
                                      DevChannel* ch, uint32_t* alpha_out) {
  STWO_REQUIRE(!columns.empty() && all, "commit_from_leaves: no columns");
  const uint32_t k = columns[0].log;
  for (const ColRef& c : columns) STWO_REQUIRE(c.log == k, "commit_from_leaves: mixed column sizes");
  STWO_REQUIRE(k >= 1, "commit_from_leaves: a tree of one leaf");
  sorted = columns;
  layers.assign(k + 1, nullptr);
  for (uint32_t lg = 0; lg <= k; lg++) layers[lg] = all + (size_t)8 * ((1ull << lg) - 1);
  std::vector<uint32_t*> outs;
  for (int lg = (int)k - 1; lg >= 0; lg--) outs.push_back(layers[lg]);
  int32_t st = merkle_node_layers(layers[k], k - 1, k, outs.data(), s, ch, alpha_out);
  if (st) return st;
  channel_fused = ch != nullptr;
  return STWO_OK;
}

// vcs/prover.rs:80-149, recording gather requests instead of reading values.
void DevMerkle::decommit(const std::map<uint32_t, std::vector<size_t>>& queries, Gather& g, DecommitRecipe& out) const {
  size_t ci = 0;
  std::vector<size_t> last;
  static const std::vector<size_t> empty;
  for (int lg = (int)layers.size() - 1; lg >= 0; lg--) {
    std::vector<const uint32_t*> lc;
    while (ci < sorted.size() && sorted[ci].log == (uint32_t)lg) lc.push_back(sorted[ci++].p);
    // Columns that lie a fixed stride apart (one column block) are gathered as one run per node.
    size_t stride = 0;
    if (lc.size() >= 8 && lc[1] > lc[0]) {
      stride = (size_t)(lc[1] - lc[0]);
      for (size_t k = 2; k < lc.size() && stride; k++)
        if (lc[k] != lc[0] + k * stride) stride = 0;
    }
    const uint32_t* prev = (size_t)lg + 1 < layers.size() ? layers[lg + 1] : nullptr;
    auto it = queries.find((uint32_t)lg);
    const std::vector<size_t>& cq = it == queries.end() ? empty : it->second;
    std::vector<size_t> total;
    size_t pi = 0, qi = 0;
    while (true) {
      bool have = false;
      size_t node = 0;
      if (pi < last.size()) { node = last[pi] / 2; have = true; }
      if (qi < cq.size()) { node = have ? std::min(node, cq[qi]) : cq[qi]; have = true; }
      if (!have) break;
      if (prev) {
        if (pi < last.size() && last[pi] == 2 * node) pi++;
        else out.hash_witness.push_back(g.hash(prev, 2 * node));
        if (pi < last.size() && last[pi] == 2 * node + 1) pi++;
        else out.hash_witness.push_back(g.hash(prev, 2 * node + 1));
      }
      bool q = qi < cq.size() && cq[qi] == node;
      if (q) qi++;
      std::vector<size_t>& dst = q ? out.queried : out.column_witness;
      if (stride) {
        const size_t first = g.vals_strided(lc[0], stride, (uint32_t)lc.size(), node);
        for (size_t k = 0; k < lc.size(); k++) dst.push_back(first + k);
      } else {
        for (auto* c : lc) dst.push_back(g.val(c, node));
      }
      total.push_back(node);
    }
    last = total;
  }
}

// ------------------------------------------------------------------------------------------------
// Canonical proof bytes (same layout as the oracle's serialiser).
struct ByteWriter {
  std::vector<uint8_t> b;
  ByteWriter() { b.reserve(1 << 17); }
  template <class T>
  void le(T v) {  // little-endian bytes of an unsigned integer
    uint8_t t[sizeof(T)];
    for (size_t i = 0; i < sizeof(T); i++) t[i] = (uint8_t)(v >> (8 * i));
    b.insert(b.end(), t, t + sizeof(T));
  }
  void u32(uint32_t v) { le(v); }
  void u64(uint64_t v) { le(v); }
  void digest(const Digest& d) { b.insert(b.end(), d.b, d.b + 32); }
  void q(const hq& x) { for (int i = 0; i < 4; i++) u32(x.v[i]); }
  void hashes(const std::vector<size_t>& idx, const Gather& g) {
    u64(idx.size());
    for (size_t i : idx) {
      uint32_t w[8];
      for (int k = 0; k < 8; k++) w[k] = g.hres[8 * i + k];
      digest(Digest::from_words(w));
    }
  }
  void vals(const std::vector<size_t>& idx, const Gather& g) {
    u64(idx.size());
    size_t o = b.size();
    b.resize(o + 4 * idx.size());
    for (size_t i : idx) {
      const uint32_t v = g.vres[i];
      for (int k = 0; k < 4; k++) b[o++] = (uint8_t)(v >> (8 * k));
    }
  }
  void dec(const DecommitRecipe& d, const Gather& g) {
    hashes(d.hash_witness, g);
    vals(d.column_witness, g);
  }
};

// ------------------------------------------------------------------------------------------------
struct Queries {
  std::vector<size_t> pos;
  uint32_t log = 0;
  Queries fold(uint32_t n) const {
    Queries q;
    q.log = log - n;
    for (size_t p : pos) {
      size_t v = p >> n;
      if (q.pos.empty() || q.pos.back() != v) q.pos.push_back(v);
    }
    return q;
  }
};
static Queries generate_queries(HostChannel& ch, uint32_t log, uint32_t n_queries) {
  std::set<size_t> qs;
  uint32_t cnt = 0;
  uint32_t mask = (uint32_t)((1ull << log) - 1);
  while (true) {
    Digest d = ch.draw_random_bytes();
    uint32_t w[8];
    d.words(w);
    for (int i = 0; i < 8; i++) {
      qs.insert(w[i] & mask);
      if (++cnt == n_queries) return Queries{std::vector<size_t>(qs.begin(), qs.end()), log};
    }
  }
}

// Decommitment positions and witness requests of a 2-folding layer (fri.rs:943-976).
static void fri_positions_and_witness(const SecureCols& col, const std::vector<size_t>& queries, Gather& g,
                                      std::vector<size_t>& positions, std::vector<size_t>& witness) {
  size_t i = 0;
  while (i < queries.size()) {
    size_t start = (queries[i] >> 1) << 1;
    size_t j = i;
    while (j < queries.size() && (queries[j] >> 1) == (queries[i] >> 1)) j++;
    size_t k = i;
    for (size_t pos = start; pos < start + 2; pos++) {
      positions.push_back(pos);
      if (k < j && queries[k] == pos) {
        k++;
        continue;
      }
      for (int c = 0; c < 4; c++) witness.push_back(g.val(col.c[c], pos));
    }
    i = j;
  }
}

static stwo_qm31 to_sq(hq x) { stwo_qm31 r; for (int i = 0; i < 4; i++) r.v[i] = x.v[i]; return r; }
static hq from_sq(const stwo_qm31& x) { return hq_make(x.v[0], x.v[1], x.v[2], x.v[3]); }

// Circle point over QM31 on the host.
struct HPointQ { hq x, y; };
static HPointQ hpq_add_m31(const HPointQ& a, hpoint b) {
  hq bx = hq_make(b.x, 0, 0, 0), by = hq_make(b.y, 0, 0, 0);
  return {hq_sub(hq_mul(a.x, bx), hq_mul(a.y, by)), hq_add(hq_mul(a.x, by), hq_mul(a.y, bx))};
}
static bool hpq_less(const HPointQ& a, const HPointQ& b) {
  for (int i = 0; i < 4; i++) if (a.x.v[i] != b.x.v[i]) return a.x.v[i] < b.x.v[i];
  for (int i = 0; i < 4; i++) if (a.y.v[i] != b.y.v[i]) return a.y.v[i] < b.y.v[i];
  return false;
}
static bool hpq_eq(const HPointQ& a, const HPointQ& b) { return !hpq_less(a, b) && !hpq_less(b, a); }
static HPointQ random_point(HostChannel& ch) {
  hq t = ch.draw_felt();
  hq t2 = hq_mul(t, t);
  hq d = hq_inv(hq_add(t2, hq_make(1, 0, 0, 0)));
  return {hq_mul(hq_sub(hq_make(1, 0, 0, 0), t2), d), hq_mul(hq_add(t, t), d)};
}

// ------------------------------------------------------------------------------------------------
// Commitment scheme prover state on the device.
struct Tree {
  std::vector<uint32_t*> polys;     // device coefficient columns
  std::vector<uint32_t> poly_logs;
  std::vector<uint32_t*> evals;     // device evaluations on the blown-up canonic domains
  std::vector<uint32_t> eval_logs;
  DevMerkle merkle;
};

int32_t Prover::commit_polys(std::vector<uint32_t*> polys, std::vector<uint32_t> logs,
                             const std::vector<uint32_t*>* evals) {
  trees.emplace_back();
  Tree& t = trees.back();
  t.polys = std::move(polys);
  t.poly_logs = std::move(logs);
  std::vector<ColRef> refs;
  // Evaluate all polynomials of the same log size in one batched call (unless the caller has).
  std::map<uint32_t, std::vector<size_t>> by_log;
  for (size_t i = 0; i < t.polys.size(); i++) by_log[t.poly_logs[i]].push_back(i);
  t.evals.assign(t.polys.size(), nullptr);
  t.eval_logs.assign(t.polys.size(), 0);
  if (evals) {
    t.evals = *evals;
    for (size_t i = 0; i < t.polys.size(); i++) t.eval_logs[i] = t.poly_logs[i] + cfg.log_blowup_factor;
  } else {
    StageScope stage_ext("Extension", s);
    for (auto& kv : by_log) {
      uint32_t el = kv.first + cfg.log_blowup_factor;
      std::vector<const uint32_t*> src;
      std::vector<uint32_t*> dst;
      uint32_t* block = arena.alloc(kv.second.size() << el);
      if (!block) return STWO_ERR_OOM;
      for (size_t i : kv.second) {
        t.evals[i] = block + (dst.size() << el);
        t.eval_logs[i] = el;
        src.push_back(t.polys[i]);
        dst.push_back(t.evals[i]);
      }
      int32_t st =
          fft_evaluate(tree, canonic_half_coset(el), src.data(), kv.first, dst.data(), (uint32_t)src.size(), s);
      if (st) return st;
    }
  }
  for (size_t i = 0; i < t.evals.size(); i++) refs.push_back({t.evals[i], t.eval_logs[i]});
  StageScope stage_merkle("Merkle", s);
  int32_t st = t.merkle.commit(refs, arena, s, false);
  if (st) return st;
  if (before_root_wait) {
    // Host work that needs nothing from this commitment runs while the device computes it.
    std::function<void()> f = std::move(before_root_wait);
    before_root_wait = nullptr;
    f();
  }
  st = t.merkle.read_root(s);
  if (st) return st;
  ch.mix_root(t.merkle.root);
  return STWO_OK;
}

int32_t Prover::commit_evals(const std::vector<uint32_t*>& cols, uint32_t log_size) {
  // Interpolate in place (the evaluation is consumed, as PolyOps::interpolate takes it by value),
  // then evaluate on the blown-up domain; the pass the two transforms share runs fused where it
  // can (fft_interpolate_extend_begin), so the coefficients are read back from HBM once less.
  if (cols.empty()) return commit_polys({}, {});
  const uint32_t el = log_size + cfg.log_blowup_factor;
  uint32_t* block = arena.alloc(cols.size() << el);
  if (!block) return STWO_ERR_OOM;
  std::vector<uint32_t*> evals(cols.size());
  for (size_t i = 0; i < cols.size(); i++) evals[i] = block + (i << el);
  const uint32_t n = (uint32_t)cols.size();
  bool fused = false;
  {
    StageScope stage("Interpolation for commitment", s);
    int32_t st = fft_interpolate_extend_begin(tree, canonic_half_coset(log_size), cols.data(), n, tree,
                                              canonic_half_coset(el), evals.data(), s, &fused);
    if (st) return st;
  }
  {
    StageScope stage("Extension", s);
    int32_t st = fft_interpolate_extend_end(tree, canonic_half_coset(el), log_size, cols.data(), n, evals.data(),
                                            fused, s);
    if (st) return st;
  }
  return commit_polys(cols, std::vector<uint32_t>(cols.size(), log_size), &evals);
}

Prover::Prover(const stwo_pcs_config& c, uint32_t max_log, cudaStream_t st) : cfg(c), s(st), arena(st) {
  StageScope stage("Setup", s);
  init_status = get_tree(canonic_half_coset(max_log), s, &tree);
}
Prover::~Prover() = default;

// Composition polynomial (air/accumulation.rs:49-149 for one component): the AIR kernel
// accumulates row_res * denom_inv on the evaluation domain; the four coordinate columns are then
// interpolated and committed as a tree.
std::vector<uint32_t> composition_denom_inv(uint32_t trace_log, uint32_t eval_log) {
  // Denominator inverses: 1 / coset_vanishing(trace coset, eval_domain.at(i)), bit-reversed.
  const uint32_t expand = eval_log - trace_log;
  std::vector<uint32_t> dinv((size_t)1 << expand);
  stwo_coset tc = coset_new(1u << (31 - (trace_log + 1)), trace_log);  // Coset::odds(trace_log)
  hpoint init = h_index_to_point(tc.initial_index);
  hpoint half = h_index_to_point(tc.step_size >> 1);
  hpoint shift = h_padd({init.x, h_sub(0, init.y)}, half);
  stwo_coset eh = canonic_half_coset(eval_log);
  for (size_t i = 0; i < dinv.size(); i++) {
    uint32_t idx = idx_reduce((uint64_t)eh.initial_index + (uint64_t)eh.step_size * i);  // i < half size
    hpoint pt = h_padd(h_index_to_point(idx), shift);
    uint32_t x = pt.x;
    for (uint32_t k = 1; k < trace_log; k++) x = h_sub(h_add(h_mul(x, x), h_mul(x, x)), 1);
    dinv[i] = h_inv(x);
  }
  std::vector<uint32_t> tmp(dinv.size());
  for (size_t i = 0; i < dinv.size(); i++) {
    size_t r = 0;
    for (uint32_t b = 0; b < expand; b++) r |= ((i >> b) & 1) << (expand - 1 - b);
    tmp[r] = dinv[i];
  }
  return tmp;
}

int32_t Prover::commit_composition(const GpuAir& air, hq rc) {
  uint32_t eval_log = air.max_constraint_log_degree_bound();
  uint32_t trace_log = air.log_size();
  size_t n = air.n_constraints();
  const std::vector<uint32_t> dinv = composition_denom_inv(trace_log, eval_log);
  uint32_t* d_coeffs = arena.alloc(4 * n + dinv.size());
  if (!d_coeffs) return STWO_ERR_OOM;
  uint32_t* d_dinv = d_coeffs + 4 * n;
  // Random coefficient powers, highest first: constraint k gets rc^(n-1-k), computed on the device.
  int32_t pst = secure_powers_reversed(rc.v, (uint32_t)n, d_coeffs, s);
  if (pst) return pst;
  STWO_CHECK_CUDA(cudaMemcpyAsync(d_dinv, dinv.data(), dinv.size() * 4, cudaMemcpyHostToDevice, s));
  StageScope stage_cext("Composition extension", s);
  // Trace columns on the evaluation domain, per tree (extension when the committed domain differs).
  std::vector<std::vector<const uint32_t*>> tcols(trees.size());
  for (size_t ti = 0; ti < trees.size(); ti++) {
    Tree& t = trees[ti];
    std::vector<const uint32_t*> src;
    std::vector<uint32_t*> ext;
    size_t n_ext = 0;
    for (size_t c = 0; c < t.evals.size(); c++) n_ext += t.eval_logs[c] != eval_log;
    uint32_t* block = n_ext ? arena.alloc(n_ext << eval_log) : nullptr;
    if (n_ext && !block) return STWO_ERR_OOM;
    for (size_t c = 0; c < t.evals.size(); c++) {
      if (t.eval_logs[c] == eval_log) {
        tcols[ti].push_back(t.evals[c]);
      } else {
        uint32_t* e = block + (ext.size() << eval_log);
        src.push_back(t.polys[c]);
        ext.push_back(e);
        tcols[ti].push_back(e);
      }
    }
    if (!src.empty()) {
      // All columns of a component share one log size.
      int32_t st = fft_evaluate(tree, canonic_half_coset(eval_log), src.data(), t.poly_logs[0], ext.data(),
                                (uint32_t)src.size(), s);
      if (st) return st;
    }
  }
  uint32_t* acc[4];
  for (int k = 0; k < 4; k++) {
    acc[k] = arena.alloc((size_t)1 << eval_log);
    if (!acc[k]) return STWO_ERR_OOM;
  }
  StageScope stage_cons("Constraint point-wise eval", s);
  int32_t st = air.eval_composition(tcols, d_coeffs, d_dinv, acc, false, s);
  if (st) return st;
  StageScope stage_ci("Constraints interpolation", s);
  st = fft_interpolate(tree, canonic_half_coset(eval_log), acc, 4, s);
  if (st) return st;
  return commit_polys({acc[0], acc[1], acc[2], acc[3]}, std::vector<uint32_t>(4, eval_log));
}

static void write_config(ByteWriter& w, const stwo_pcs_config& c) {
  w.u32(c.pow_bits);
  w.u32(c.log_blowup_factor);
  w.u32(c.log_last_layer_degree_bound);
  w.u64(c.n_queries);
}

// Which columns are sampled at which mask offsets. It does not depend on the OODS point, so
// prove() builds it while the device computes the composition commitment. Columns are listed
// tree by tree, the composition tree's four columns last, each sampled at the OODS point (offset
// 0) as the reference samples them (prover/mod.rs:63-68).
struct SampleLayout {
  std::vector<int> offsets;          // distinct mask offsets, in order of first use
  std::vector<uint32_t> tree_first;  // first column of each tree; one entry per tree, plus the end
  std::vector<uint32_t> col_first;   // first sample of each column; one entry per column, plus the end
  std::vector<uint32_t> sample_off;  // the offset (index into `offsets`) of each sample
};

static SampleLayout sample_layout(const GpuAir& air, const std::vector<Tree>& trees) {
  SampleLayout L;
  const auto mask = air.mask_offsets();
  auto offset_id = [&](int off) -> uint32_t {
    for (size_t i = 0; i < L.offsets.size(); i++)
      if (L.offsets[i] == off) return (uint32_t)i;
    L.offsets.push_back(off);
    return (uint32_t)L.offsets.size() - 1;
  };
  for (size_t t = 0; t < trees.size(); t++) {
    L.tree_first.push_back((uint32_t)L.col_first.size());
    const bool comp = t + 1 == trees.size();
    for (size_t c = 0; c < trees[t].polys.size(); c++) {
      L.col_first.push_back((uint32_t)L.sample_off.size());
      if (comp) {
        L.sample_off.push_back(offset_id(0));
      } else if (t != 0 && t < mask.size()) {
        for (int off : mask[t][c]) L.sample_off.push_back(offset_id(off));
      }
    }
  }
  L.tree_first.push_back((uint32_t)L.col_first.size());
  L.col_first.push_back((uint32_t)L.sample_off.size());
  return L;
}

int32_t Prover::prove(const GpuAir& air, std::vector<uint8_t>& out) {
  // Composition polynomial and OODS point (prover/mod.rs:41-61). The sample layout is built
  // while the device commits the composition polynomial.
  SampleLayout lay;
  bool have_layout = false;
  // Per column (tree order): coefficients and evaluations with their log sizes; per sample: its
  // column. With the layout they fix the OODS evaluation's job tables (plan), which upload while
  // the device still computes the composition commitment.
  std::vector<const uint32_t*> polys, ceval;
  std::vector<uint32_t> plogs, clog, poly_of;
  EvalPlan plan;
  std::vector<QuotPlan> qplans;
  std::vector<uint32_t> qorder;
  struct PlanRelease {
    EvalPlan& p;
    std::vector<QuotPlan>& q;
    cudaStream_t s;
    ~PlanRelease() {
      eval_plan_free(p, s);
      for (QuotPlan& x : q) quot_plan_free(x, s);
    }
  } plan_release{plan, qplans, s};
  int32_t plan_st = STWO_OK;
  before_root_wait = [&] {
    lay = sample_layout(air, trees);
    have_layout = true;
    const size_t n_cols = lay.col_first.size() - 1;
    polys.assign(n_cols, nullptr);
    ceval.assign(n_cols, nullptr);
    plogs.assign(n_cols, 0);
    clog.assign(n_cols, 0);
    poly_of.assign(lay.sample_off.size(), 0);
    for (size_t t = 0; t < trees.size() && t + 1 < lay.tree_first.size(); t++)
      for (uint32_t c = lay.tree_first[t]; c < lay.tree_first[t + 1]; c++) {
        const uint32_t lc = c - lay.tree_first[t];
        polys[c] = trees[t].polys[lc];
        plogs[c] = trees[t].poly_logs[lc];
        ceval[c] = trees[t].evals[lc];
        clog[c] = trees[t].eval_logs[lc];
        for (uint32_t e = lay.col_first[c]; e < lay.col_first[c + 1]; e++) poly_of[e] = c;
      }
    if (!lay.sample_off.empty())
      plan_st = eval_plan_build(polys.data(), plogs.data(), (uint32_t)n_cols, poly_of.data(), lay.sample_off.data(),
                                (uint32_t)lay.sample_off.size(), (uint32_t)lay.offsets.size(), s, &plan);
    // The FRI quotient groups: columns by evaluation log size, descending (pcs/quotients.rs:76-101),
    // tree order within a size; each group's samples (local column, OODS evaluation, offset id).
    qorder.resize(n_cols);
    for (uint32_t c = 0; c < n_cols; c++) qorder[c] = (uint32_t)c;
    std::stable_sort(qorder.begin(), qorder.end(), [&](uint32_t a, uint32_t b) { return clog[a] > clog[b]; });
    for (size_t i = 0; i < n_cols && !plan_st;) {
      size_t j = i;
      while (j < n_cols && clog[qorder[j]] == clog[qorder[i]]) j++;
      std::vector<const uint32_t*> gc(j - i);
      std::vector<uint32_t> scol, seval, spt;
      for (size_t k = i; k < j; k++) {
        gc[k - i] = ceval[qorder[k]];
        for (uint32_t e = lay.col_first[qorder[k]]; e < lay.col_first[qorder[k] + 1]; e++) {
          scol.push_back((uint32_t)(k - i));
          seval.push_back(e);
          spt.push_back(lay.sample_off[e]);
        }
      }
      qplans.emplace_back();
      plan_st = quot_plan_build(clog[qorder[i]], gc.data(), (uint32_t)gc.size(), scol.data(), seval.data(), spt.data(),
                                (uint32_t)scol.size(), (uint32_t)lay.offsets.size(), cfg.log_blowup_factor, s,
                                &qplans.back());
      i = j;
    }
  };
  hq rc = ch.draw_felt();
  int32_t st = commit_composition(air, rc);
  before_root_wait = nullptr;
  if (st) return st;
  STWO_REQUIRE(have_layout && lay.tree_first.size() == trees.size() + 1, "sample layout not built");
  HPointQ oods = random_point(ch);

  // The point of each distinct mask offset; offsets that land on the same point share its id,
  // as the reference groups samples by point value (ColumnSampleBatch::new_vec).
  const uint32_t step = 1u << (31 - air.log_size());
  std::vector<HPointQ> upts;
  std::vector<uint32_t> pid(lay.offsets.size());
  for (size_t i = 0; i < lay.offsets.size(); i++) {
    const int off = lay.offsets[i];
    uint32_t idx = idx_reduce((uint64_t)step * (uint64_t)(off >= 0 ? off : -off));
    if (off < 0) idx = idx_reduce((1ull << 31) - idx);
    const HPointQ q = hpq_add_m31(oods, h_index_to_point(idx));
    uint32_t k = 0;
    while (k < upts.size() && !hpq_eq(upts[k], q)) k++;
    if (k == upts.size()) upts.push_back(q);
    pid[i] = k;
  }
  const size_t n_cols = lay.col_first.size() - 1;
  const size_t n_samples = lay.sample_off.size();
  if (plan_st) return plan_st;
  STWO_REQUIRE(n_samples > 0 && plan.d, "no OODS samples");

  // Batched OODS evaluation of every sampled polynomial (pcs/prover.rs:89-101): the plan's
  // evaluations take the point of their mask offset.
  std::vector<stwo_qm31_point> opts(lay.offsets.size());
  for (size_t i = 0; i < lay.offsets.size(); i++) opts[i] = {to_sq(upts[pid[i]].x), to_sq(upts[pid[i]].y)};
  std::vector<stwo_qm31> svals(n_samples);
  StageScope stage_oods("Evaluate columns out of domain", s);
  st = eval_plan_run(plan, opts.data(), svals.data(), s);
  if (st) return st;
  std::vector<hq> flat(n_samples);
  for (size_t e = 0; e < n_samples; e++) flat[e] = from_sq(svals[e]);
  ch.mix_felts(flat);

  // Sanity check of the composition at the OODS point (prover/mod.rs:70-76). It is host
  // arithmetic only, so it runs once every quotient and FRI kernel has been enqueued, just before
  // the host waits for the FRI results: the stream works meanwhile. Its verdict is checked before
  // the proof is written (the reference returns the same error earlier, with no proof either).
  struct OodsCheck {
    bool done = false, ok = true;
  } check;
  auto run_check = [&]() {
    if (check.done) return;
    std::vector<std::vector<std::vector<hq>>> mv(trees.size() - 1);
    for (size_t t = 0; t + 1 < trees.size(); t++) {
      mv[t].resize(lay.tree_first[t + 1] - lay.tree_first[t]);
      for (uint32_t c = lay.tree_first[t]; c < lay.tree_first[t + 1]; c++)
        mv[t][c - lay.tree_first[t]].assign(flat.begin() + lay.col_first[c], flat.begin() + lay.col_first[c + 1]);
    }
    const hq* comp = flat.data() + lay.col_first[lay.tree_first[trees.size() - 1]];
    const hq lhs = hq_add(hq_add(comp[0], hq_mul(comp[1], hq_make(0, 1, 0, 0))),
                          hq_add(hq_mul(comp[2], hq_make(0, 0, 1, 0)), hq_mul(comp[3], hq_make(0, 0, 0, 1))));
    // denom inverse 1 / coset_vanishing(CanonicCoset(log).coset, oods)
    stwo_coset tc = coset_new(1u << (31 - (air.log_size() + 1)), air.log_size());
    hpoint init = h_index_to_point(tc.initial_index);
    hpoint half = h_index_to_point(tc.step_size >> 1);
    hpoint shift = h_padd({init.x, h_sub(0, init.y)}, half);
    HPointQ q = hpq_add_m31(oods, shift);
    hq x = q.x;
    for (uint32_t i = 1; i < air.log_size(); i++) x = hq_sub(hq_add(hq_mul(x, x), hq_mul(x, x)), hq_make(1, 0, 0, 0));
    const hq rhs = air.eval_at_point(mv, rc, hq_inv(x));
    check.ok = std::memcmp(lhs.v, rhs.v, sizeof(rhs.v)) == 0;
    check.done = true;
  };

  // FRI quotients per log size, descending (pcs/quotients.rs:76-101); columns of one log size
  // keep their tree order.
  const std::vector<uint32_t>& order = qorder;
  hq qrc = ch.draw_felt();
  StageScope stage_q("Compute FRI quotients", s);
  std::vector<SecureCols> quotients;
  std::vector<uint32_t> qlogs;
  // The planned path needs each mask offset on its own point (always so in practice: offsets
  // are a few rows apart); otherwise offsets that share a point form one batch, as the reference
  // groups samples by point value, and the tables are built here.
  const bool planned = upts.size() == lay.offsets.size();
  for (size_t g = 0; planned && g < qplans.size(); g++) {
    const QuotPlan& qp = qplans[g];
    std::vector<uint32_t> bord;  // offset ids present in the group, in the order of their points
    for (uint32_t q = 0; q < qp.n_points; q++)
      if (qp.s_first[q + 1] > qp.s_first[q]) bord.push_back(q);
    std::sort(bord.begin(), bord.end(), [&](uint32_t a, uint32_t b) { return hpq_less(upts[pid[a]], upts[pid[b]]); });
    const uint32_t glog = qp.log_n;
    SecureCols q;
    for (int k = 0; k < 4; k++) {
      q.c[k] = arena.alloc((size_t)1 << glog);
      if (!q.c[k]) return STWO_ERR_OOM;
    }
    st = quot_plan_run(qp, eval_plan_values(plan), opts.data(), bord.data(), (uint32_t)bord.size(), to_sq(qrc), q.c, s);
    if (st) return st;
    quotients.push_back(q);
    qlogs.push_back(glog);
  }
  for (size_t i = 0; !planned && i < n_cols;) {
    size_t j = i;
    while (j < n_cols && clog[order[j]] == clog[order[i]]) j++;
    // ColumnSampleBatch::new_vec: group by point in CirclePoint<QM31> order.
    std::vector<uint32_t> points;
    for (size_t k = i; k < j; k++)
      for (uint32_t e = lay.col_first[order[k]]; e < lay.col_first[order[k] + 1]; e++) {
        const uint32_t p = pid[lay.sample_off[e]];
        if (std::find(points.begin(), points.end(), p) == points.end()) points.push_back(p);
      }
    std::sort(points.begin(), points.end(), [&](uint32_t a, uint32_t b) { return hpq_less(upts[a], upts[b]); });
    std::vector<std::vector<uint32_t>> bidx(points.size());
    std::vector<std::vector<stwo_qm31>> bval(points.size());
    for (size_t k = i; k < j; k++)
      for (uint32_t e = lay.col_first[order[k]]; e < lay.col_first[order[k] + 1]; e++) {
        const size_t b = std::find(points.begin(), points.end(), pid[lay.sample_off[e]]) - points.begin();
        bidx[b].push_back((uint32_t)(k - i));
        bval[b].push_back(svals[e]);
      }
    std::vector<stwo_sample_batch> batches(points.size());
    for (size_t b = 0; b < points.size(); b++)
      batches[b] = {{to_sq(upts[points[b]].x), to_sq(upts[points[b]].y)}, (uint32_t)bidx[b].size(), bidx[b].data(),
                    bval[b].data()};
    std::vector<const uint32_t*> gc(j - i);
    for (size_t k = i; k < j; k++) gc[k - i] = ceval[order[k]];
    const uint32_t glog = clog[order[i]];
    SecureCols q;
    for (int k = 0; k < 4; k++) {
      q.c[k] = arena.alloc((size_t)1 << glog);
      if (!q.c[k]) return STWO_ERR_OOM;
    }
    st = accumulate_quotients(glog, gc.data(), (uint32_t)gc.size(), to_sq(qrc), batches.data(),
                              (uint32_t)batches.size(), cfg.log_blowup_factor, q.c, s);
    if (st) return st;
    quotients.push_back(q);
    qlogs.push_back(glog);
    i = j;
  }

  StageScope stage_fri("FRI commitment", s);
  // FRI commitment (fri.rs:168-290).
  std::vector<ColRef> first_cols;
  for (size_t i = 0; i < quotients.size(); i++)
    for (int k = 0; k < 4; k++) first_cols.push_back({quotients[i].c[k], qlogs[i]});
  // The transcript of the commit phase runs on the device: each layer's root is mixed and its
  // alpha drawn by one thread on the stream, so the layers follow one another with no host round
  // trip; the roots, the channel state and the last layer come back together at the end.
  DevChannel* dch = reinterpret_cast<DevChannel*>(arena.alloc(sizeof(DevChannel) / 4));
  constexpr size_t FRI_MAX_STEPS = 40;
  uint32_t* alphas = arena.alloc(8 * FRI_MAX_STEPS);
  if (!dch || !alphas) return STWO_ERR_OOM;
  {
    uint32_t d[8];
    ch.digest.words(d);
    st = channel_set(dch, d, ch.n_sent, s);
    if (st) return st;
  }
  DevMerkle first_tree;
  size_t fstep = 0;
  st = first_tree.commit(first_cols, arena, s, false, dch, alphas + 8 * fstep);
  if (st) return st;
  if (!first_tree.channel_fused) st = fri_channel_step(dch, first_tree.layers[0], alphas + 8 * fstep, s);
  if (st) return st;
  struct Layer { SecureCols eval; stwo_coset dom; DevMerkle merkle; };
  std::vector<Layer> layers;
  stwo_coset dom = coset_new(1u << (31 - (qlogs[0] - 1 + 2)), qlogs[0] - 1);  // Coset::half_odds(log-1)
  SecureCols cur;
  for (int k = 0; k < 4; k++) {
    cur.c[k] = arena.alloc((size_t)1 << dom.log_size);
    if (!cur.c[k]) return STWO_ERR_OOM;
    STWO_CHECK_CUDA(cudaMemsetAsync(cur.c[k], 0, ((size_t)4) << dom.log_size, s));
  }
  const qm31 unused_alpha = {{0u, 0u}, {0u, 0u}};
  size_t last_size = (size_t)1 << (cfg.log_last_layer_degree_bound + cfg.log_blowup_factor);
  // A layer of 2^k points committed by the multi-block kernels (not the last layer, not in the
  // tail) gets its tree buffer before the fold that completes it, and that fold writes its leaves.
  auto tree_for = [&](uint32_t k, size_t next_after, uint32_t** out) -> int32_t {
    *out = nullptr;
    if (((size_t)1 << k) <= last_size) return STWO_OK;
    if (k <= FRI_TAIL_LOG && next_after == quotients.size()) return STWO_OK;
    *out = arena.alloc((size_t)8 * ((2ull << k) - 1));
    return *out ? STWO_OK : STWO_ERR_OOM;
  };
  auto leaves_of = [](uint32_t* tbuf, uint32_t k) { return tbuf ? tbuf + (size_t)8 * ((1ull << k) - 1) : nullptr; };
  size_t next = 0;
  uint32_t* pending_tree = nullptr;
  st = tree_for(dom.log_size, 1, &pending_tree);
  if (st) return st;
  st = fri_fold_circle(tree, canonic_half_coset(qlogs[0]), cur.c, const_cast<const uint32_t* const*>(quotients[0].c),
                       unused_alpha, s, alphas + 8 * fstep, leaves_of(pending_tree, dom.log_size));
  if (st) return st;
  next = 1;
  while (((size_t)1 << dom.log_size) > last_size) {
    if (dom.log_size <= FRI_TAIL_LOG && next == quotients.size()) {
      // The remaining small layers: buffers laid out as the per-kernel path would, one launch.
      std::vector<stwo_coset> doms;
      std::vector<std::array<uint32_t*, 4>> evals{{cur.c[0], cur.c[1], cur.c[2], cur.c[3]}};
      std::vector<uint32_t*> trees;
      const size_t first_step = fstep + 1;
      while (((size_t)1 << dom.log_size) > last_size) {
        STWO_REQUIRE(++fstep < FRI_MAX_STEPS, "too many FRI layers");
        const uint32_t k = dom.log_size;
        Layer L;
        L.eval = cur;
        L.dom = dom;
        uint32_t* tbuf = arena.alloc((size_t)8 * ((2ull << k) - 1));
        SecureCols nxt;
        for (int c = 0; c < 4; c++) nxt.c[c] = arena.alloc((size_t)1 << (k - 1));
        if (!tbuf || !nxt.c[0] || !nxt.c[1] || !nxt.c[2] || !nxt.c[3]) return STWO_ERR_OOM;
        L.merkle.layers.assign(k + 1, nullptr);
        for (uint32_t lg = 0; lg <= k; lg++) L.merkle.layers[lg] = tbuf + (size_t)8 * ((1ull << lg) - 1);
        for (int c = 0; c < 4; c++) L.merkle.sorted.push_back({cur.c[c], k});
        doms.push_back(dom);
        trees.push_back(tbuf);
        evals.push_back({nxt.c[0], nxt.c[1], nxt.c[2], nxt.c[3]});
        layers.push_back(L);
        cur = nxt;
        dom = coset_double(dom);
      }
      st = fri_tail(tree, doms, evals, trees, dch, alphas + 8 * first_step, s);
      if (st) return st;
      break;
    }
    Layer L;
    L.eval = cur;
    L.dom = dom;
    std::vector<ColRef> lc;
    for (int k = 0; k < 4; k++) lc.push_back({cur.c[k], dom.log_size});
    STWO_REQUIRE(++fstep < FRI_MAX_STEPS, "too many FRI layers");
    if (pending_tree) {
      st = L.merkle.commit_from_leaves(lc, pending_tree, s, dch, alphas + 8 * fstep);
      pending_tree = nullptr;
    } else {
      st = L.merkle.commit(lc, arena, s, false, dch, alphas + 8 * fstep);
    }
    if (st) return st;
    if (!L.merkle.channel_fused) st = fri_channel_step(dch, L.merkle.layers[0], alphas + 8 * fstep, s);
    if (st) return st;
    SecureCols nxt;
    for (int k = 0; k < 4; k++) {
      nxt.c[k] = arena.alloc((size_t)1 << (dom.log_size - 1));
      if (!nxt.c[k]) return STWO_ERR_OOM;
    }
    const uint32_t next_log = dom.log_size - 1;
    const bool inject = next < quotients.size() && qlogs[next] - 1 == next_log;
    uint32_t* next_tree = nullptr;
    st = tree_for(next_log, next + (inject ? 1 : 0), &next_tree);
    if (st) return st;
    uint32_t* next_leaves = leaves_of(next_tree, next_log);
    st = fri_fold_line(tree, dom, const_cast<const uint32_t* const*>(cur.c), unused_alpha, nxt.c, s,
                       alphas + 8 * fstep, inject ? nullptr : next_leaves);
    if (st) return st;
    dom = coset_double(dom);
    if (inject) {
      st = fri_fold_circle(tree, canonic_half_coset(qlogs[next]), nxt.c,
                           const_cast<const uint32_t* const*>(quotients[next].c), unused_alpha, s, alphas + 8 * fstep,
                           next_leaves);
      if (st) return st;
      next++;
    }
    pending_tree = next_tree;
    layers.push_back(L);
    cur = nxt;
  }
  STWO_REQUIRE(next == quotients.size(), "not all FRI columns consumed");
  STWO_REQUIRE(layers.size() + 1 + 5 <= (size_t)COLLECT_MAX, "too many FRI layers");
  // Roots, channel state and the last layer (fri.rs:272-290) in one copy to mapped host memory.
  std::vector<hq> last(last_size);
  {
    CollectList cl{};
    auto add = [&](const uint32_t* p, uint32_t n) {
      cl.src[cl.count] = p;
      cl.n[cl.count++] = n;
    };
    add(first_tree.layers[0], 8);
    for (auto& L : layers) add(L.merkle.layers[0], 8);
    add(reinterpret_cast<const uint32_t*>(dch), sizeof(DevChannel) / 4);
    for (int k = 0; k < 4; k++) add(cur.c[k], (uint32_t)last_size);
    size_t total = 8 * (1 + layers.size()) + sizeof(DevChannel) / 4 + 4 * last_size;
    Mapped mp;
    st = mapped_words(total, mp);
    if (st) return st;
    launch_pdl(k_collect, dim3(1), dim3(256), 0, s, cl, mp.dev);
    note_launch();
    STWO_LAUNCH_CHECK();
    run_check();
    STWO_CHECK_CUDA(cudaStreamSynchronize(s));
    const uint32_t* w = mp.host;
    first_tree.root = Digest::from_words(w);
    w += 8;
    for (auto& L : layers) {
      L.merkle.root = Digest::from_words(w);
      w += 8;
    }
    DevChannel dc;
    std::memcpy(&dc, w, sizeof(DevChannel));
    w += sizeof(DevChannel) / 4;
    if (dc.error) {
      set_error("FRI channel: felt draw exhausted its retries");
      return STWO_ERR_CUDA;
    }
    ch.digest = Digest::from_words(dc.digest);
    ch.n_sent = (uint64_t)dc.n_sent_lo | ((uint64_t)dc.n_sent_hi << 32);
    for (size_t i = 0; i < last_size; i++)
      last[i] = hq_make(w[i], w[last_size + i], w[2 * last_size + i], w[3 * last_size + i]);
  }
  std::vector<hq> coeffs = line_interpolate_host(dom, last);  // bit-reversed coefficient order
  bit_reverse_host(coeffs);                                   // natural order
  size_t bound = (size_t)1 << cfg.log_last_layer_degree_bound;
  for (size_t i = bound; i < coeffs.size(); i++)
    for (int k = 0; k < 4; k++)
      if (coeffs[i].v[k]) {
        set_error("invalid degree");
        return STWO_ERR_INVALID_ARG;
      }
  coeffs.resize(bound);
  bit_reverse_host(coeffs);
  ch.mix_felts(coeffs);

  // Proof of work (pcs/prover.rs:122-125).
  uint64_t nonce = 0;
  {
    StageScope stage_g("Grind", s);
    uint32_t d[8];
    ch.digest.words(d);
    st = stwo_grind_blake2s(d, cfg.pow_bits, &nonce, s);
    if (st) return st;
  }
  ch.mix_u64(nonce);

  StageScope stage_dec("Decommitment", s);
  // Decommitment (fri.rs:295-334, pcs/prover.rs:127-137): record every word to read, gather.
  Gather g;
  Queries q = generate_queries(ch, qlogs[0], cfg.n_queries);
  std::map<uint32_t, std::vector<size_t>> by_log;
  for (uint32_t l : std::set<uint32_t>(qlogs.begin(), qlogs.end())) by_log[l] = q.fold(qlogs[0] - l).pos;
  std::vector<size_t> first_witness;
  std::map<uint32_t, std::vector<size_t>> dpos;
  for (size_t c = 0; c < quotients.size(); c++) {
    Queries cq = q.fold(qlogs[0] - qlogs[c]);
    std::vector<size_t> pos;
    fri_positions_and_witness(quotients[c], cq.pos, g, pos, first_witness);
    dpos[qlogs[c]] = pos;
  }
  DecommitRecipe first_dec;
  first_tree.decommit(dpos, g, first_dec);
  std::vector<std::vector<size_t>> layer_witness(layers.size());
  std::vector<DecommitRecipe> layer_dec(layers.size());
  Queries lq = q.fold(1);
  for (size_t li = 0; li < layers.size(); li++) {
    std::vector<size_t> pos;
    fri_positions_and_witness(layers[li].eval, lq.pos, g, pos, layer_witness[li]);
    std::map<uint32_t, std::vector<size_t>> m;
    m[layers[li].dom.log_size] = pos;
    layers[li].merkle.decommit(m, g, layer_dec[li]);
    lq = lq.fold(1);
  }
  std::vector<DecommitRecipe> tree_dec(trees.size());
  for (size_t t = 0; t < trees.size(); t++) trees[t].merkle.decommit(by_log, g, tree_dec[t]);
  st = g.run(s);
  if (st) return st;

  // Canonical bytes: config, commitments, sampled values, decommitments, queried values, pow, FRI.
  StageScope stage_out("Proof assembly", s);
  ByteWriter w;
  write_config(w, cfg);
  w.u64(trees.size());
  for (auto& t : trees) w.digest(t.merkle.root);
  w.u64(trees.size());
  {
    for (size_t t = 0; t < trees.size(); t++) {
      w.u64(lay.tree_first[t + 1] - lay.tree_first[t]);
      for (uint32_t c = lay.tree_first[t]; c < lay.tree_first[t + 1]; c++) {
        w.u64(lay.col_first[c + 1] - lay.col_first[c]);
        for (uint32_t e = lay.col_first[c]; e < lay.col_first[c + 1]; e++) w.q(flat[e]);
      }
    }
  }
  w.u64(trees.size());
  for (auto& d : tree_dec) w.dec(d, g);
  w.u64(trees.size());
  for (auto& d : tree_dec) w.vals(d.queried, g);
  w.u64(nonce);
  auto write_witness = [&](const std::vector<size_t>& wi) {
    w.u64(wi.size() / 4);
    for (size_t i = 0; i < wi.size(); i++) w.u32(g.vres[wi[i]]);
  };
  write_witness(first_witness);
  w.dec(first_dec, g);
  w.digest(first_tree.root);
  w.u64(layers.size());
  for (size_t li = 0; li < layers.size(); li++) {
    write_witness(layer_witness[li]);
    w.dec(layer_dec[li], g);
    w.digest(layers[li].merkle.root);
  }
  w.u64(coeffs.size());
  for (auto& c : coeffs) w.q(c);
  run_check();
  if (!check.ok) {
    set_error("ConstraintsNotSatisfied");
    return STWO_ERR_INVALID_ARG;
  }
  out.swap(w.b);
  return arena.failed ? STWO_ERR_OOM : STWO_OK;
}

// Line polynomial coefficients from a bit-reversed evaluation on the line domain `dom`
// (poly/line.rs:225-290); the last FRI layer has 2^(log_last_layer + log_blowup) points.
std::vector<hq> line_interpolate_host(stwo_coset dom, std::vector<hq> v) {
  bit_reverse_host(v);
  stwo_coset d = dom;
  while (((size_t)1 << d.log_size) > 1) {
    size_t n = (size_t)1 << d.log_size, half = n / 2;
    for (size_t c = 0; c < v.size(); c += n)
      for (size_t i = 0; i < half; i++) {
        uint32_t x = h_index_to_point(idx_reduce((uint64_t)d.initial_index + (uint64_t)d.step_size * i)).x;
        uint32_t xi = h_inv(x);
        hq a = v[c + i], b = v[c + half + i];
        v[c + i] = hq_add(a, b);
        hq diff = hq_sub(a, b);
        for (int k = 0; k < 4; k++) diff.v[k] = h_mul(diff.v[k], xi);
        v[c + half + i] = diff;
      }
    d = coset_double(d);
  }
  uint32_t li = h_inv((uint32_t)(v.size() % P));
  for (auto& x : v)
    for (int k = 0; k < 4; k++) x.v[k] = h_mul(x.v[k], li);
  return v;
}

}  // namespace stwo
