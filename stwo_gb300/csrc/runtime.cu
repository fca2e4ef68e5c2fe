// Runtime: errors, device context, stream-ordered buffers and twiddle trees.
#include "common.cuh"
#include <array>
#include <cstdarg>
#include <atomic>
#include <chrono>

namespace stwo {

static thread_local char g_err[1024] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

static std::atomic<unsigned long long> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

struct StageRec {
  const char* name;
  cudaEvent_t a, b;
  std::chrono::steady_clock::time_point ha, hb;  // host clock at the stage's begin and end calls
};
static thread_local bool g_stage_on = false;
static thread_local std::vector<StageRec> g_stages;
static thread_local int g_stage_open = -1;

void stage_begin(const char* name, cudaStream_t s) {
  if (!g_stage_on) return;
  if (g_stage_open >= 0) stage_end(s);
  StageRec r{name, nullptr, nullptr, std::chrono::steady_clock::now(), {}};
  if (cudaEventCreate(&r.a) != cudaSuccess || cudaEventCreate(&r.b) != cudaSuccess) return;
  cudaEventRecord(r.a, s);
  g_stages.push_back(r);
  g_stage_open = (int)g_stages.size() - 1;
}
void stage_end(cudaStream_t s) {
  if (!g_stage_on || g_stage_open < 0) return;
  cudaEventRecord(g_stages[g_stage_open].b, s);
  g_stages[g_stage_open].hb = std::chrono::steady_clock::now();
  g_stage_open = -1;
}

DeviceContext& ctx() {
  static DeviceContext c;
  return c;
}

TuneState& tune_state() {
  static TuneState t;
  return t;
}
int tune_mode() { return tune_state().mode.load(); }
bool tune_lookup(uint32_t site, uint64_t key, uint32_t* choice) {
  TuneState& t = tune_state();
  std::lock_guard<std::mutex> g(t.mu);
  auto it = t.table.find({site, key});
  if (it == t.table.end()) return false;
  *choice = it->second;
  return true;
}
void tune_record(uint32_t site, uint64_t key, uint32_t choice) {
  TuneState& t = tune_state();
  std::lock_guard<std::mutex> g(t.mu);
  t.table[{site, key}] = choice;
}

int sm_count() {
  static const int n = [] {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    return v > 0 ? v : 152;
  }();
  return n;
}

// Keeps freed stream-ordered memory cached in the device's default pool instead of returning it
// at every synchronisation (the default release threshold is 0), so repeated proofs reuse their
// working set without re-mapping it.
static void keep_pool_memory() {
  static thread_local int done_dev = -1;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev == done_dev) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    uint64_t thr = ~0ull;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  done_dev = dev;
}

int32_t run_rate_probe(RateProbeKernel kern, uint32_t words, uint32_t rounds, cudaStream_t s, RateProbe* r) {
  int per_sm = 0;
  STWO_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, 0));
  r->blocks = (uint32_t)std::max(1, per_sm) * (uint32_t)sm_count();
  const size_t n = (size_t)r->blocks * 256 * words;
  uint32_t* d = nullptr;
  int32_t st = scratch_alloc((void**)&d, n * 8 + (size_t)r->blocks * 48, s);
  if (st) return st;
  unsigned long long* d_span = reinterpret_cast<unsigned long long*>(d + 2 * n);
  std::vector<unsigned long long> h(6 * (size_t)r->blocks);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t err = cudaMemsetAsync(d, 0x5a, n * 4, s);
  if (!err) err = cudaEventCreate(&e0);
  if (!err) err = cudaEventCreate(&e1);
  float ms = 0.f;
  if (!err) {
    kern<<<r->blocks, 256, 0, s>>>(d, d + n, d_span, rounds);  // warm-up
    cudaEventRecord(e0, s);
    kern<<<r->blocks, 256, 0, s>>>(d, d + n, d_span, rounds);
    cudaEventRecord(e1, s);
    note_launch();
    note_launch();
    err = cudaGetLastError();
    if (!err) err = cudaMemcpyAsync(h.data(), d_span, h.size() * 8, cudaMemcpyDeviceToHost, s);
    if (!err) err = cudaStreamSynchronize(s);
    if (!err) err = cudaEventElapsedTime(&ms, e0, e1);
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  scratch_free(d, s);
  if (err) {
    set_error("rate probe: %s", cudaGetErrorString(err));
    return STWO_ERR_CUDA;
  }
  // Per SM: busy cycles from its first block's start to its last block's end (the counter is the
  // SM's own), and the blocks it ran, whatever their residency; the median SM is reported.
  std::map<unsigned long long, std::array<unsigned long long, 3>> sm;  // min start, max end, blocks
  double sum_c = 0.0, sum_ns = 0.0;
  for (uint32_t b = 0; b < r->blocks; b++) {
    const unsigned long long* o = h.data() + 6 * (size_t)b;
    auto it = sm.find(o[0]);
    if (it == sm.end()) it = sm.emplace(o[0], std::array<unsigned long long, 3>{o[1], o[2], 0}).first;
    it->second[0] = std::min(it->second[0], o[1]);
    it->second[1] = std::max(it->second[1], o[2]);
    it->second[2]++;
    sum_c += (double)(o[2] - o[1]);
    sum_ns += (double)(o[4] - o[3]);
  }
  std::vector<std::pair<double, double>> per;  // (busy cycles per block, blocks) of each SM
  for (auto& kv : sm) per.push_back({(double)(kv.second[1] - kv.second[0]) / (double)kv.second[2],
                                     (double)kv.second[2]});
  std::sort(per.begin(), per.end());
  const auto& med = per[per.size() / 2];
  r->ms = ms;
  r->warps_per_sm = med.second * 8.0;
  r->sm_cycles = med.first * med.second;
  r->sm_mhz = sum_ns > 0.0 ? 1e3 * sum_c / sum_ns : 0.0;
  return STWO_OK;
}

int32_t scratch_alloc(void** p, size_t bytes, cudaStream_t s) {
  *p = nullptr;
  if (bytes == 0) return STWO_OK;
  keep_pool_memory();
  STWO_CHECK_CUDA(cudaMallocAsync(p, bytes, s));
  return STWO_OK;
}
void scratch_free(void* p, cudaStream_t s) {
  if (p) cudaFreeAsync(p, s);
}

// Pinned staging of one host thread. Buffers outlive their thread: a worker that exits hands
// them to a process-wide free list and the next new thread takes them over, so servers that
// start fresh workers do not call cudaHostAlloc (slow, and it can wait for running work) for
// every thread. A thread only exits between jobs, when nothing in flight still uses them.
namespace {
struct HostStaging {
  Mapped mapped;
  unsigned long long* small = nullptr;
};
std::mutex g_staging_mu;
std::vector<HostStaging*> g_staging_free;
struct StagingHolder {
  HostStaging* s = nullptr;
  ~StagingHolder() {
    if (!s) return;
    std::lock_guard<std::mutex> g(g_staging_mu);
    g_staging_free.push_back(s);
  }
};
HostStaging& staging() {
  thread_local StagingHolder h;
  if (!h.s) {
    std::lock_guard<std::mutex> g(g_staging_mu);
    if (!g_staging_free.empty()) {
      h.s = g_staging_free.back();
      g_staging_free.pop_back();
    } else {
      h.s = new HostStaging();
    }
  }
  return *h.s;
}
}  // namespace

unsigned long long* small_pinned() {
  HostStaging& st = staging();
  if (!st.small) {
    void* q = nullptr;
    if (cudaHostAlloc(&q, 64, cudaHostAllocDefault) != cudaSuccess) return nullptr;
    st.small = static_cast<unsigned long long*>(q);
  }
  return st.small;
}

int32_t mapped_words(size_t words, Mapped& m) {
  Mapped& tl = staging().mapped;
  if (tl.words < words) {
    if (tl.host) cudaFreeHost(tl.host);
    tl = Mapped{};
    size_t w = std::max<size_t>(words, 4096);
    STWO_CHECK_CUDA(cudaHostAlloc((void**)&tl.host, w * 4, cudaHostAllocMapped));
    STWO_CHECK_CUDA(cudaHostGetDevicePointer((void**)&tl.dev, tl.host, 0));
    tl.words = w;
  }
  m = tl;
  return STWO_OK;
}

hpoint h_index_to_point(uint32_t idx) {
  struct Tower {
    hpoint p[31];
    Tower() {
      p[0] = {2u, 1268011823u};  // M31_CIRCLE_GEN, crates/prover/src/core/circle.rs:203-206
      for (int b = 1; b < 31; b++) p[b] = h_padd(p[b - 1], p[b - 1]);
    }
  };
  static const Tower tw;  // thread-safe one-time initialisation
  const hpoint* tower = tw.p;
  hpoint r = {1u, 0u};
  idx &= IDX_MASK;
  for (int b = 0; b < 31; b++)
    if ((idx >> b) & 1) r = h_padd(r, tower[b]);
  return r;
}


// One thread per tree entry. Entry `pos` of level k (the root doubled k times, log R-k)
// lies at offset 2^R - 2^(R-k); it is the x-coordinate of the coset point with index
// bitrev_{R-k-1}(pos - offset). The final entry is the padding value 1.
__global__ void k_twiddle_tree(uint32_t init, uint32_t step, uint32_t R, uint32_t* tw, uint32_t* itw,
                               uint32_t* tw2, uint32_t* itw2, uint32_t* zero_flag) {
  uint32_t n = 1u << R;
  for (uint32_t pos = blockIdx.x * blockDim.x + threadIdx.x; pos < n; pos += gridDim.x * blockDim.x) {
    if (pos == n - 1) {
      tw[pos] = 1u;
      itw[pos] = 1u;
      tw2[pos] = 2u;
      itw2[pos] = 2u;
      continue;
    }
    uint32_t q = n - 1 - pos;              // = 2^(R-k) - 1 - j, in [2^(R-k-1), 2^(R-k) - 1]
    uint32_t k = R - 1 - (31 - __clz(q));  // floor(log2(q)) = R-k-1
    uint32_t lvl_log = R - k;                      // coset log size at this level
    uint32_t off = n - (1u << lvl_log);
    uint32_t j = pos - off;
    uint32_t ik = (uint32_t)(((uint64_t)init << k) & IDX_MASK);
    uint32_t sk = (uint32_t)(((uint64_t)step << k) & IDX_MASK);
    uint32_t idx = (uint32_t)(((uint64_t)ik + (uint64_t)sk * brev(j, lvl_log - 1)) & IDX_MASK);
    uint32_t x = index_to_point(idx).x;
    if (x == 0) atomicOr(zero_flag, 1u);  // "0 has no inverse" (fields/m31.rs:66)
    const uint32_t ix = m31_inv(x);
    tw[pos] = x;
    itw[pos] = ix;
    tw2[pos] = 2u * x;
    itw2[pos] = 2u * ix;
  }
}

int32_t build_tree(stwo_coset root, cudaStream_t stream, TwiddleTree* t) {
  STWO_REQUIRE(root.log_size <= 30, "twiddle root log_size %u > 30", root.log_size);
  t->root = root;
  t->size = (size_t)1 << root.log_size;
  STWO_CHECK_CUDA(cudaMalloc(&t->d_tw, t->size * 4 + 4));
  STWO_CHECK_CUDA(cudaMalloc(&t->d_itw, t->size * 4));
  STWO_CHECK_CUDA(cudaMalloc(&t->d_tw2, t->size * 8));
  t->d_itw2 = t->d_tw2 + t->size;
  // One word past the twiddles flags an x-coordinate equal to 0: such a coset has no inverse
  // twiddles and is rejected, as the reference panics on it.
  uint32_t* flag = t->d_tw + t->size;
  STWO_CHECK_CUDA(cudaMemsetAsync(flag, 0, 4, stream));
  uint32_t threads = 256;
  uint32_t blocks = (uint32_t)((t->size + threads - 1) / threads);
  if (blocks > 65535u) blocks = 65535u;
  k_twiddle_tree<<<blocks, threads, 0, stream>>>(root.initial_index, root.step_size, root.log_size, t->d_tw,
                                                 t->d_itw, t->d_tw2, t->d_itw2, flag);
  note_launch();
  STWO_LAUNCH_CHECK();
  uint32_t h_flag = 0;
  STWO_CHECK_CUDA(cudaMemcpyAsync(&h_flag, flag, 4, cudaMemcpyDeviceToHost, stream));
  STWO_CHECK_CUDA(cudaStreamSynchronize(stream));
  if (h_flag) {
    cudaFree(t->d_tw);
    cudaFree(t->d_itw);
    cudaFree(t->d_tw2);
    t->d_tw2 = t->d_itw2 = nullptr;
    t->d_tw = t->d_itw = nullptr;
    set_error("coset has a point with x = 0: 0 has no inverse");
    return STWO_ERR_INVALID_ARG;
  }
  return STWO_OK;
}

int32_t get_tree(stwo_coset root, cudaStream_t stream, TwiddleTree** out) {
  DeviceContext& c = ctx();
  std::lock_guard<std::mutex> g(c.mu);
  int dev = 0;
  cudaGetDevice(&dev);
  auto key = std::make_tuple(dev, root.initial_index, root.step_size, root.log_size);
  auto it = c.trees.find(key);
  if (it != c.trees.end()) {
    *out = it->second;
    return STWO_OK;
  }
  TwiddleTree* t = new TwiddleTree();
  int32_t st = build_tree(root, stream, t);
  if (st) {
    delete t;
    return st;
  }
  c.trees[key] = t;
  *out = t;
  return STWO_OK;
}

}  // namespace stwo

using namespace stwo;

struct stwo_twiddle_tree_s {
  TwiddleTree t;
};

extern "C" {

const char* stwo_status_string(stwo_status s) {
  switch (s) {
    case STWO_OK: return "ok";
    case STWO_ERR_INVALID_ARG: return "invalid argument";
    case STWO_ERR_OOM: return "out of device memory";
    case STWO_ERR_TIMEOUT: return "timeout";
    case STWO_ERR_CUDA: return "cuda error";
    case STWO_ERR_UNSUPPORTED: return "unsupported";
    default: return "unknown status";
  }
}

const char* stwo_last_error(void) { return g_err; }

uint64_t stwo_kernel_launches(void) { return g_launches.load(); }

stwo_status stwo_autotune_mode(int mode) {
  STWO_REQUIRE(mode >= 0 && mode <= 2, "autotune mode %d (0 off, 1 use, 2 tune)", mode);
  tune_state().mode.store(mode);
  return STWO_OK;
}
stwo_status stwo_autotune_set_entry(uint32_t site, uint64_t key, uint32_t choice) {
  tune_record(site, key, choice);
  return STWO_OK;
}
uint32_t stwo_autotune_entries(uint32_t* sites, uint64_t* keys, uint32_t* choices, uint32_t cap) {
  TuneState& t = tune_state();
  std::lock_guard<std::mutex> g(t.mu);
  uint32_t i = 0;
  for (const auto& kv : t.table) {
    if (i < cap && sites && keys && choices) {
      sites[i] = kv.first.first;
      keys[i] = kv.first.second;
      choices[i] = kv.second;
    }
    i++;
  }
  return i;
}
stwo_status stwo_autotune_clear(void) {
  TuneState& t = tune_state();
  std::lock_guard<std::mutex> g(t.mu);
  t.table.clear();
  return STWO_OK;
}

stwo_status stwo_set_stage_timing(int enable) {
  g_stage_on = enable != 0;
  for (auto& r : g_stages) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  g_stages.clear();
  g_stage_open = -1;
  return STWO_OK;
}

uint32_t stwo_stage_times(const char** names, float* ms, uint32_t cap) {
  // Stage durations (summed by name), then the stream time between consecutive stages, summed as
  // "gap before <stage>": device idle or unlabelled work while the host prepared the next stage.
  thread_local std::vector<std::string> gap_names;
  gap_names.clear();
  gap_names.reserve(2 * g_stages.size());
  std::vector<std::pair<const char*, float>> agg, gaps;
  auto add = [](std::vector<std::pair<const char*, float>>& v, const char* name, float t) {
    for (auto& a : v)
      if (strcmp(a.first, name) == 0) {
        a.second += t;
        return;
      }
    v.push_back({name, t});
  };
  for (size_t i = 0; i < g_stages.size(); i++) {
    const StageRec& r = g_stages[i];
    float t = 0;
    if (cudaEventSynchronize(r.b) != cudaSuccess || cudaEventElapsedTime(&t, r.a, r.b) != cudaSuccess) t = -1;
    add(agg, r.name, t);
    if (i > 0) {
      float g = 0;
      if (cudaEventElapsedTime(&g, g_stages[i - 1].b, r.a) != cudaSuccess) g = -1;
      std::string gn = std::string("gap before ") + r.name;
      const char* key = nullptr;
      for (auto& n : gap_names)
        if (n == gn) key = n.c_str();
      if (!key) {
        gap_names.push_back(gn);
        key = gap_names.back().c_str();
      }
      add(gaps, key, g);
    }
  }
  // Host time spent issuing each stage ("host: <stage>"): when it approaches the device time,
  // the stage is bound by host work or launch issue rather than by its kernels.
  std::vector<std::pair<const char*, float>> host;
  for (auto& r : g_stages) {
    std::string hn = std::string("host: ") + r.name;
    const char* key = nullptr;
    for (auto& n : gap_names)
      if (n == hn) key = n.c_str();
    if (!key) {
      gap_names.push_back(hn);
      key = gap_names.back().c_str();
    }
    add(host, key, std::chrono::duration<float, std::milli>(r.hb - r.ha).count());
  }
  for (auto& r : g_stages) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  for (auto& g : gaps) agg.push_back(g);
  for (auto& h : host) agg.push_back(h);
  g_stages.clear();
  g_stage_open = -1;
  uint32_t n = 0;
  for (auto& a : agg) {
    if (n < cap) {
      if (names) names[n] = a.first;
      if (ms) ms[n] = a.second;
    }
    n++;
  }
  return n;
}

stwo_status stwo_device_init(int device) {
  STWO_CHECK_CUDA(cudaSetDevice(device));
  STWO_CHECK_CUDA(cudaFree(nullptr));
  return STWO_OK;
}

stwo_status stwo_sync(void* stream) {
  STWO_CHECK_CUDA(cudaStreamSynchronize(as_stream(stream)));
  return STWO_OK;
}

stwo_status stwo_buf_alloc(void** d_ptr, size_t bytes, void* stream) {
  STWO_REQUIRE(d_ptr, "null out pointer");
  return scratch_alloc(d_ptr, bytes, as_stream(stream));
}
stwo_status stwo_buf_free(void* d_ptr, void* stream) {
  if (d_ptr) STWO_CHECK_CUDA(cudaFreeAsync(d_ptr, as_stream(stream)));
  return STWO_OK;
}
stwo_status stwo_buf_upload(void* d_dst, const void* h_src, size_t bytes, void* stream) {
  STWO_CHECK_CUDA(cudaMemcpyAsync(d_dst, h_src, bytes, cudaMemcpyHostToDevice, as_stream(stream)));
  STWO_CHECK_CUDA(cudaStreamSynchronize(as_stream(stream)));
  return STWO_OK;
}
stwo_status stwo_buf_download(void* h_dst, const void* d_src, size_t bytes, void* stream) {
  STWO_CHECK_CUDA(cudaMemcpyAsync(h_dst, d_src, bytes, cudaMemcpyDeviceToHost, as_stream(stream)));
  STWO_CHECK_CUDA(cudaStreamSynchronize(as_stream(stream)));
  return STWO_OK;
}
stwo_status stwo_buf_zero(void* d_dst, size_t bytes, void* stream) {
  STWO_CHECK_CUDA(cudaMemsetAsync(d_dst, 0, bytes, as_stream(stream)));
  return STWO_OK;
}

stwo_status stwo_twiddles_precompute(stwo_coset root, stwo_twiddle_tree* out, void* stream) {
  STWO_REQUIRE(out, "null out pointer");
  stwo_twiddle_tree_s* t = new stwo_twiddle_tree_s();
  int32_t st = build_tree(root, as_stream(stream), &t->t);
  if (st) {
    delete t;
    return st;
  }
  *out = t;
  return STWO_OK;
}

stwo_status stwo_twiddles_free(stwo_twiddle_tree tree) {
  if (!tree) return STWO_OK;
  cudaFree(tree->t.d_tw);
  cudaFree(tree->t.d_itw);
  cudaFree(tree->t.d_tw2);
  delete tree;
  return STWO_OK;
}

stwo_status stwo_twiddles_info(stwo_twiddle_tree tree, stwo_coset* root, const uint32_t** d_tw,
                               const uint32_t** d_itw, size_t* size) {
  STWO_REQUIRE(tree, "null tree");
  if (root) *root = tree->t.root;
  if (d_tw) *d_tw = tree->t.d_tw;
  if (d_itw) *d_itw = tree->t.d_itw;
  if (size) *size = tree->t.size;
  return STWO_OK;
}

}  // extern "C"

namespace stwo {
const TwiddleTree* tree_of(stwo_twiddle_tree t) { return t ? &t->t : nullptr; }
}
