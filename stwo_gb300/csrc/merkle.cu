// MerkleOps<Blake2sMerkleHasher>::commit_on_layer and GrindOps<Blake2sChannel>::grind.
//
// Node i of a layer = BLAKE2s-256( [prev[2i] || prev[2i+1]] || col_0[i] || ... || col_{k-1}[i] )
// with u32 little-endian column words (crates/prover/src/core/vcs/blake2_merkle.rs:14-30,
// backend/simd/blake2s.rs:60-145; the empty message when there is neither). One thread per node:
// a warp reads each column as one coalesced 128-byte line and streams 16 columns per
// compression, so a leaf costs ceil(k/16) compressions on the INT pipes.
#include "common.cuh"
#include "blake2s.cuh"
#include "dchannel.cuh"

namespace stwo {

constexpr int MERKLE_MAX_COLS = 3072;  // 24 KB of column pointers in the launch parameters
struct MerkleCols { const uint32_t* p[MERKLE_MAX_COLS]; };

// Hashes nodes [0, n_nodes) of a layer. When `n_cols` spans several launches the running
// chaining value and byte count persist in `state` (8 words + 1 per node); `first`/`last`
// mark the launch that starts / finishes the message. LAT: a layer too small to fill the GPU,
// whose threads each run their chain of compressions with little else to overlap, uses the
// latency-oriented compression (every addition on the FMA pipe).
template <bool LAT>
__global__ void __launch_bounds__(256) k_merkle_layer(uint32_t n_nodes, const uint32_t* __restrict__ prev,
                                                      MerkleCols cols, uint32_t n_cols, uint32_t* __restrict__ out,
                                                      uint32_t* __restrict__ state, uint32_t first, uint32_t last,
                                                      uint32_t one) {
  pdl_enter();
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_nodes) return;
  uint32_t h[8];
  uint32_t m[16];
  uint32_t t = 0;
  if (first) {
    b2s_init(h);
    if (prev) {
      const uint4* pp = reinterpret_cast<const uint4*>(prev + (size_t)16 * i);
#pragma unroll
      for (int q = 0; q < 4; q++) {
        uint4 w = pp[q];
        m[4 * q] = w.x;
        m[4 * q + 1] = w.y;
        m[4 * q + 2] = w.z;
        m[4 * q + 3] = w.w;
      }
      t = 64;
      bool fin = last && n_cols == 0;
      b2s_compress(h, m, t, fin);
    } else if (n_cols == 0 && last) {
#pragma unroll
      for (int q = 0; q < 16; q++) m[q] = 0;
      b2s_compress(h, m, 0, true);
    }
  } else {
#pragma unroll
    for (int q = 0; q < 8; q++) h[q] = state[(size_t)9 * i + q];
    t = state[(size_t)9 * i + 8];
  }
  uint32_t c = 0;
  if (LAT) {
    // Few threads: the next 16 column words are fetched while the current block compresses.
    uint32_t nx[16];
    auto fetch = [&](uint32_t c0) {
      const uint32_t kk = n_cols - c0 < 16 ? n_cols - c0 : 16;
#pragma unroll
      for (int q = 0; q < 16; q++) nx[q] = (uint32_t)q < kk ? __ldg(cols.p[c0 + q] + i) : 0u;
    };
    if (n_cols) fetch(0);
    while (c < n_cols) {
      const uint32_t k = n_cols - c < 16 ? n_cols - c : 16;
      const bool fin = last && (c + k == n_cols);
#pragma unroll
      for (int q = 0; q < 16; q++) m[q] = nx[q];
      if (c + k < n_cols) fetch(c + k);
      t += 4 * k;
      b2s_compress_lat(h, m, t, fin);
      c += k;
    }
  } else {
    while (c < n_cols) {
      uint32_t k = n_cols - c < 16 ? n_cols - c : 16;
      bool fin = last && (c + k == n_cols);
#pragma unroll
      for (int q = 0; q < 16; q++) m[q] = (uint32_t)q < k ? __ldg(cols.p[c + q] + i) : 0u;
      t += 4 * k;
      b2s_compress_fma(h, m, t, fin, one);
      c += k;
    }
  }
  if (last) {
    uint4* po = reinterpret_cast<uint4*>(out + (size_t)8 * i);
    po[0] = make_uint4(h[0], h[1], h[2], h[3]);
    po[1] = make_uint4(h[4], h[5], h[6], h[7]);
  } else {
#pragma unroll
    for (int q = 0; q < 8; q++) state[(size_t)9 * i + q] = h[q];
    state[(size_t)9 * i + 8] = t;
  }
}

// Layers of at most this many nodes (under two warps per SM) take the latency-oriented kernel.
constexpr uint32_t MERKLE_LAT_NODES = 8192;

int32_t merkle_commit_layer(uint32_t log_size, const uint32_t* prev, const uint32_t* const* cols, uint32_t n_cols,
                            uint32_t* out, cudaStream_t s) {
  STWO_REQUIRE(log_size <= 30, "layer log size %u > 30", log_size);
  STWO_REQUIRE(out, "null output");
  STWO_REQUIRE(n_cols == 0 || cols, "null column table");
  uint32_t n = 1u << log_size;
  // Columns are consumed 16 at a time; a launch takes a multiple of 16 so that only the last
  // launch sees a partial block.
  const uint32_t per_launch = (MERKLE_MAX_COLS / 16) * 16;
  uint32_t n_launch = n_cols <= per_launch ? 1 : (n_cols + per_launch - 1) / per_launch;
  uint32_t* state = nullptr;
  if (n_launch > 1) {
    int32_t st = scratch_alloc((void**)&state, (size_t)n * 9 * 4, s);
    if (st) return st;
  }
  // Built-in shape: a small layer goes out as one-warp blocks of the latency kernel, so that its
  // few warps land on different SMs instead of sharing the issue slots of one. Larger layers use
  // two-warp blocks: a layer of 2^17 nodes is then 2,048 blocks, 13-14 per SM, where 256-thread
  // blocks (3 or 4 per SM) left the SMs with three blocks idle for a quarter of the launch.
  // Shape c: 0 = latency kernel, 32 threads; 1..4 = throughput kernel, 32 << (c - 1) threads.
  auto launch_shape = [&](uint32_t shape, uint32_t l) -> int32_t {
    const uint32_t c0 = l * per_launch;
    const uint32_t nc = n_cols - c0 < per_launch ? n_cols - c0 : per_launch;
    MerkleCols mc;
    for (uint32_t q = 0; q < nc; q++) mc.p[q] = cols[c0 + q];
    const uint32_t threads = shape == 0 ? 32u : 32u << (shape - 1);
    const uint32_t blocks = (n + threads - 1) / threads;
    if (shape == 0)
      launch_pdl(k_merkle_layer<true>, dim3(blocks), dim3(threads), 0, s, n, prev, mc, nc, out, state, l == 0,
                 l + 1 == n_launch, 1u);
    else
      launch_pdl(k_merkle_layer<false>, dim3(blocks), dim3(threads), 0, s, n, prev, mc, nc, out, state, l == 0,
                 l + 1 == n_launch, 1u);
    note_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      set_error("merkle launch: %s", cudaGetErrorString(e));
      return STWO_ERR_CUDA;
    }
    return STWO_OK;
  };
  uint32_t shape = n <= MERKLE_LAT_NODES ? 0u : 2u;
  int32_t st = STWO_OK;
  if (n_launch == 1 && log_size >= 10) {
    // One launch recomputes the layer from its inputs, so it can be timed in place.
    static const uint32_t cands[] = {0, 1, 2, 3, 4};
    const uint64_t comps = (n_cols + 15) / 16 + (prev ? 1 : 0);
    st = tune_choice(TUNE_MERKLE_LAYER, ((uint64_t)log_size << 32) | comps, shape, cands, 5, s,
                     [&](uint32_t c) { return launch_shape(c, 0); }, &shape);
  }
  for (uint32_t l = 0; l < n_launch && !st; l++) st = launch_shape(shape, l);
  scratch_free(state, s);
  return st;
}

// ---------------------------------------------------------------- node subtrees
// Layers made only of child hashes (no columns of that size): each block hashes 2^k nodes of the
// first output layer from their children, then keeps halving in shared memory, writing every
// level, so one launch covers up to 8 levels of the tree (vcs/prover.rs:39-61 layer by layer).
constexpr int SUBTREE_LOG = 8;

struct LayerPtrs {
  uint32_t* p[SUBTREE_LOG + 1];
};

__device__ __forceinline__ void hash_children(const uint32_t* l, const uint32_t* r, uint32_t h[8]) {
  uint32_t m[16];
#pragma unroll
  for (int q = 0; q < 8; q++) {
    m[q] = l[q];
    m[8 + q] = r[q];
  }
  b2s_init(h);
  b2s_compress(h, m, 64, true);
}

// With `ch` set (on the launch that produces the root), thread 0 then runs one FRI transcript
// step on the device channel: mix the root, draw the folding alpha into alpha_out (alpha, alpha^2).
__global__ void __launch_bounds__(256) k_merkle_subtrees(const uint32_t* __restrict__ prev, uint32_t first_log,
                                                         uint32_t levels, LayerPtrs outs, DevChannel* ch,
                                                         uint32_t* alpha_out) {
  pdl_enter();
  __shared__ uint32_t sm[256 * 8];
  const uint32_t t = threadIdx.x;
  const uint32_t node = blockIdx.x * blockDim.x + t;  // node of layer first_log
  uint32_t h[8];
  if (node < (1u << first_log)) {
    const uint4* pp = reinterpret_cast<const uint4*>(prev + (size_t)16 * node);
    uint32_t m[16];
#pragma unroll
    for (int q = 0; q < 4; q++) {
      uint4 w = pp[q];
      m[4 * q] = w.x;
      m[4 * q + 1] = w.y;
      m[4 * q + 2] = w.z;
      m[4 * q + 3] = w.w;
    }
    b2s_init(h);
    b2s_compress(h, m, 64, true);
    uint4* po = reinterpret_cast<uint4*>(outs.p[0] + (size_t)8 * node);
    po[0] = make_uint4(h[0], h[1], h[2], h[3]);
    po[1] = make_uint4(h[4], h[5], h[6], h[7]);
#pragma unroll
    for (int q = 0; q < 8; q++) sm[t * 8 + q] = h[q];
  }
  __syncthreads();
  uint32_t width = blockDim.x;
  for (uint32_t lv = 1; lv < levels; lv++) {
    width >>= 1;
    uint32_t out_node = blockIdx.x * width + t;
    if (t < width) {
      hash_children(sm + (2 * t) * 8, sm + (2 * t + 1) * 8, h);
      uint4* po = reinterpret_cast<uint4*>(outs.p[lv] + (size_t)8 * out_node);
      po[0] = make_uint4(h[0], h[1], h[2], h[3]);
      po[1] = make_uint4(h[4], h[5], h[6], h[7]);
    }
    __syncthreads();
    if (t < width) {
#pragma unroll
      for (int q = 0; q < 8; q++) sm[t * 8 + q] = h[q];
    }
    __syncthreads();
  }
  if (ch && t == 0) {
    // This block's last level is the one-node root layer, written above by this thread.
    d_ch_mix_root(ch, outs.p[levels - 1]);
    const qm31 a = d_ch_draw_felt(ch);
    const qm31 a2 = qm31_mul(a, a);
    alpha_out[0] = a.a.a; alpha_out[1] = a.a.b; alpha_out[2] = a.b.a; alpha_out[3] = a.b.b;
    alpha_out[4] = a2.a.a; alpha_out[5] = a2.a.b; alpha_out[6] = a2.b.a; alpha_out[7] = a2.b.b;
  }
}

// Hashes the pure node layers first_log, first_log - 1, ..., first_log - n_levels + 1 from `prev`
// (layer first_log + 1). out[i] receives layer first_log - i.
int32_t merkle_node_layers(const uint32_t* prev, uint32_t first_log, uint32_t n_levels, uint32_t* const* out,
                           cudaStream_t s, DevChannel* ch, uint32_t* alpha_out) {
  uint32_t done = 0;
  while (done < n_levels) {
    uint32_t lg = first_log - done;
    uint32_t block_log = lg < (uint32_t)SUBTREE_LOG ? lg : (uint32_t)SUBTREE_LOG;
    uint32_t lv = std::min<uint32_t>(n_levels - done, block_log + 1);
    LayerPtrs lp;
    for (uint32_t i = 0; i < lv; i++) lp.p[i] = out[done + i];
    uint32_t threads = 1u << block_log;
    uint32_t blocks = 1u << (lg - block_log);
    // The channel step rides on the launch that ends at the root (one block, last level 0).
    const bool root_launch = blocks == 1 && lg + 1 == lv;
    launch_pdl(k_merkle_subtrees, dim3(blocks), dim3(threads), 0, s, prev, lg, lv, lp, root_launch ? ch : nullptr,
               root_launch ? alpha_out : nullptr);
    note_launch();
    STWO_LAUNCH_CHECK();
    prev = out[done + lv - 1];
    done += lv;
  }
  return STWO_OK;
}

// ---------------------------------------------------------------- grind
// Tests nonces [base, base + n): the smallest with >= pow_bits trailing zeros in word 0 of the
// raw compression (digest, [lo, hi, 0, ...], t = 0, f = 0) is folded into *best by atomicMin.
__global__ void k_grind(uint32_t d0, uint32_t d1, uint32_t d2, uint32_t d3, uint32_t d4, uint32_t d5, uint32_t d6,
                        uint32_t d7, uint64_t base, uint32_t n, uint32_t pow_bits,
                        unsigned long long* best) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t nonce = base + i;
  uint32_t h[8] = {d0, d1, d2, d3, d4, d5, d6, d7};
  uint32_t m[16];
#pragma unroll
  for (int q = 0; q < 16; q++) m[q] = 0;
  m[0] = (uint32_t)nonce;
  m[1] = (uint32_t)(nonce >> 32);
  b2s_compress(h, m, 0, false);
  uint32_t tz = h[0] == 0 ? 32u : (uint32_t)__ffs(h[0]) - 1;
  if (tz >= pow_bits) atomicMin(best, (unsigned long long)nonce);
}

// Register-only throughput of the compression that k_merkle_layer's many-node path runs
// (b2s_compress_fma): each thread chains `rounds` compressions of a 16-word message into its
// 8-word state, with no memory traffic in the loop. Its rate is the integer-datapath bound of the
// Merkle leaf layers on this device. Thread 0 of each block records its SM and the cycle counter
// and global timer around the loop.
__global__ void __launch_bounds__(256) k_blake2s_probe(const uint32_t* in, uint32_t* out, unsigned long long* span,
                                                       uint32_t rounds) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x, n = gridDim.x * blockDim.x;
  uint32_t h[8], m[16];
#pragma unroll
  for (int i = 0; i < 8; i++) h[i] = in[g + i * n];
#pragma unroll
  for (int i = 0; i < 16; i++) m[i] = in[g + (8 + i) * n];
  const uint32_t one = g_b2s_one;
  __syncthreads();
  const unsigned long long g0 = global_ns();
  const long long c0 = clock64();
  for (uint32_t it = 0; it < rounds; it++) b2s_compress_fma(h, m, 64u * (it + 1), false, one);
#pragma unroll
  for (int i = 0; i < 8; i++) out[g + i * n] = h[i];
  __syncthreads();
  if (threadIdx.x == 0) probe_record(span, c0, g0);
}

}  // namespace stwo

using namespace stwo;

extern "C" {

stwo_status stwo_blake2s_rate(uint32_t rounds, double* h_compressions_per_s, double* h_cycles_per_warp_compression,
                              double* h_probe_sm_mhz, void* stream) {
  STWO_REQUIRE(h_compressions_per_s && rounds >= 1 && rounds <= (1u << 16), "need 1 <= rounds <= 65536");
  RateProbe r;
  int32_t st = run_rate_probe(k_blake2s_probe, 24, rounds, as_stream(stream), &r);
  if (st) return st;
  *h_compressions_per_s = (double)r.blocks * 256.0 * rounds / (r.ms * 1e-3);
  // The SM's four schedulers shared its warps of `rounds` compressions each.
  if (h_cycles_per_warp_compression) *h_cycles_per_warp_compression = 4.0 * r.sm_cycles / (r.warps_per_sm * rounds);
  if (h_probe_sm_mhz) *h_probe_sm_mhz = r.sm_mhz;
  return STWO_OK;
}

stwo_status stwo_merkle_commit_layer(uint32_t log_size, const uint32_t* d_prev_layer, const uint32_t* const* d_cols,
                                     uint32_t n_cols, uint32_t* d_out, void* stream) {
  return merkle_commit_layer(log_size, d_prev_layer, d_cols, n_cols, d_out, as_stream(stream));
}

stwo_status stwo_grind_blake2s(const uint32_t h_digest[8], uint32_t pow_bits, uint64_t* h_nonce, void* stream) {
  STWO_REQUIRE(h_digest && h_nonce, "null argument");
  STWO_REQUIRE(pow_bits <= 32, "pow_bits > 32 is not supported");
  cudaStream_t s = as_stream(stream);
  unsigned long long* d_best = nullptr;
  int32_t st = scratch_alloc((void**)&d_best, sizeof(unsigned long long), s);
  if (st) return st;
  const unsigned long long none = ~0ull;
  // Batches grow geometrically: small proofs of work finish after one short launch.
  uint64_t base = 0;
  uint32_t batch = 1u << 14;
  unsigned long long best = none;
  stwo_status rc = STWO_OK;
  while (true) {
    if (cudaMemcpyAsync(d_best, &none, sizeof(none), cudaMemcpyHostToDevice, s) != cudaSuccess) { rc = STWO_ERR_CUDA; break; }
    uint32_t threads = 256;
    k_grind<<<(batch + threads - 1) / threads, threads, 0, s>>>(h_digest[0], h_digest[1], h_digest[2], h_digest[3],
                                                                 h_digest[4], h_digest[5], h_digest[6], h_digest[7],
                                                                 base, batch, pow_bits, d_best); note_launch();
    if (cudaGetLastError() != cudaSuccess) { rc = STWO_ERR_CUDA; break; }
    if (cudaMemcpyAsync(&best, d_best, sizeof(best), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) { rc = STWO_ERR_CUDA; break; }
    if (best != none) break;
    base += batch;
    if (batch < (1u << 26)) batch <<= 2;
    if (base >= (1ull << 44)) { rc = STWO_ERR_TIMEOUT; break; }
  }
  scratch_free(d_best, s);
  cudaStreamSynchronize(s);
  if (rc) {
    set_error("grind failed (status %d)", rc);
    return rc;
  }
  *h_nonce = best;
  return STWO_OK;
}

}  // extern "C"
