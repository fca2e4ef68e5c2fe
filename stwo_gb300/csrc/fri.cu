// FriOps: fold_line, fold_circle_into_line, decompose.
//
// fold_line (crates/prover/src/core/fri.rs:1132-1157): out[i] = f0 + alpha * f1 with
// (f0, f1) = ibutterfly(f(x), f(-x), 1/x), x = domain.at(bitrev(2i)).x. 1/x is entry i of the
// line domain's level of the inverse twiddle tree (backend/simd/fri.rs:24-59).
// fold_circle_into_line (fri.rs:1162-1189): dst[i] = dst[i] * alpha^2 + (f0 + alpha * f1) with
// (f0, f1) = ibutterfly(f(p), f(-p), 1/p.y); 1/p.y is the circle-layer twiddle derived from the
// half coset's level as [y, -y, -x, x] (backend/simd/fri.rs:61-109).
// decompose (backend/simd/fri.rs:111-161): lambda = (sum(first half) - sum(second half)) / N,
// g = f -+ lambda.
// Each kernel is one streaming pass over four coordinate columns: HBM-bound.
#include "common.cuh"
#include <array>
#include <mutex>
#include "blake2s.cuh"
#include "dchannel.cuh"

namespace stwo {

struct Secure4 { const uint32_t* p[4]; };
struct Secure4M { uint32_t* p[4]; };

__device__ __forceinline__ qm31 load_q(const Secure4& s, size_t i) {
  return qm31_from_u32(__ldg(s.p[0] + i), __ldg(s.p[1] + i), __ldg(s.p[2] + i), __ldg(s.p[3] + i));
}
__device__ __forceinline__ void store_q(const Secure4M& s, size_t i, qm31 v) {
  s.p[0][i] = v.a.a;
  s.p[1][i] = v.a.b;
  s.p[2][i] = v.b.a;
  s.p[3][i] = v.b.b;
}

__device__ __forceinline__ void ibfly_q(qm31& v0, qm31& v1, uint32_t it) {
  qm31 tmp = v0;
  v0 = qm31_add(tmp, v1);
  v1 = qm31_mul_m31(qm31_sub(tmp, v1), it);
}

// Two consecutive values of each coordinate are read as one 8-byte load.
__device__ __forceinline__ void load_pair(const Secure4& s, size_t i, qm31& a, qm31& b) {
  uint2 w0 = __ldg(reinterpret_cast<const uint2*>(s.p[0]) + i);
  uint2 w1 = __ldg(reinterpret_cast<const uint2*>(s.p[1]) + i);
  uint2 w2 = __ldg(reinterpret_cast<const uint2*>(s.p[2]) + i);
  uint2 w3 = __ldg(reinterpret_cast<const uint2*>(s.p[3]) + i);
  a = qm31_from_u32(w0.x, w1.x, w2.x, w3.x);
  b = qm31_from_u32(w0.y, w1.y, w2.y, w3.y);
}

// alpha (and alpha^2) from `alpha_dev` when it is set: the transcript then lives on the device.
__device__ __forceinline__ void load_alpha(const uint32_t* alpha_dev, qm31& alpha, qm31* alpha_sq) {
  if (!alpha_dev) return;
  alpha = qm31_from_u32(__ldg(alpha_dev), __ldg(alpha_dev + 1), __ldg(alpha_dev + 2), __ldg(alpha_dev + 3));
  if (alpha_sq) *alpha_sq = qm31_from_u32(__ldg(alpha_dev + 4), __ldg(alpha_dev + 5), __ldg(alpha_dev + 6), __ldg(alpha_dev + 7));
}

// Merkle leaf of one folded point for the next FRI layer's tree: BLAKE2s-256 of its four
// coordinates (16 bytes), the node k_merkle_layer computes for a layer of four columns and no
// children. `leaves` may be null (the next layer is hashed elsewhere).
__device__ __forceinline__ void fold_leaf(uint32_t* leaves, uint32_t i, const qm31& v) {
  if (!leaves) return;
  uint32_t h[8], m[16];
#pragma unroll
  for (int q = 0; q < 16; q++) m[q] = 0u;
  m[0] = v.a.a;
  m[1] = v.a.b;
  m[2] = v.b.a;
  m[3] = v.b.b;
  b2s_init(h);
  b2s_compress(h, m, 16, true);
  uint4* po = reinterpret_cast<uint4*>(leaves + (size_t)8 * i);
  po[0] = make_uint4(h[0], h[1], h[2], h[3]);
  po[1] = make_uint4(h[4], h[5], h[6], h[7]);
}

__global__ void k_fold_line(Secure4 src, Secure4M dst, uint32_t n_out, const uint32_t* __restrict__ itw_level,
                            qm31 alpha, const uint32_t* alpha_dev, uint32_t* leaves) {
  pdl_enter();
  load_alpha(alpha_dev, alpha, nullptr);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_out; i += gridDim.x * blockDim.x) {
    qm31 f0, f1;
    load_pair(src, i, f0, f1);
    ibfly_q(f0, f1, __ldg(itw_level + i));
    const qm31 r = qm31_add(f0, qm31_mul(alpha, f1));
    store_q(dst, i, r);
    fold_leaf(leaves, i, r);
  }
}

// `itw_level` = inverse twiddles of the half coset's level (2^(n-2) entries), used when
// n >= 3. For n <= 2 the y-coordinates come from the domain points directly.
__global__ void k_fold_circle(Secure4 src, Secure4M dst, uint32_t n_out, const uint32_t* __restrict__ itw_level,
                              uint32_t log_src, uint32_t half_init, uint32_t half_step, qm31 alpha, qm31 alpha_sq,
                              const uint32_t* alpha_dev, uint32_t* leaves) {
  pdl_enter();
  load_alpha(alpha_dev, alpha, &alpha_sq);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_out; i += gridDim.x * blockDim.x) {
    uint32_t yinv;
    if (log_src >= 3) {
      uint32_t t = __ldg(itw_level + ((i >> 1) ^ 1));
      yinv = ((i ^ (i >> 1)) & 1) ? m31_neg(t) : t;
    } else {
      // domain.at(bitrev(2i)): the half coset point bitrev(2i) when < half, else its conjugate.
      uint32_t k = brev(2 * i, log_src);
      uint32_t half = 1u << (log_src - 1);
      uint32_t idx = k < half ? half_init + half_step * k : (0u - (half_init + half_step * (k - half)));
      yinv = m31_inv(index_to_point(idx & 0x7fffffffu).y);
    }
    qm31 f0, f1;
    load_pair(src, i, f0, f1);
    ibfly_q(f0, f1, yinv);
    qm31 fp = qm31_add(qm31_mul(alpha, f1), f0);
    qm31 d = qm31_from_u32(dst.p[0][i], dst.p[1][i], dst.p[2][i], dst.p[3][i]);
    const qm31 r = qm31_add(qm31_mul(d, alpha_sq), fp);
    store_q(dst, i, r);
    fold_leaf(leaves, i, r);
  }
}

// One FRI transcript step on the device (fri.rs:198-214): mix the layer's Merkle root, draw the
// folding alpha; alpha and alpha^2 go to `alpha_out` (8 words).
__global__ void k_fri_channel_step(DevChannel* ch, const uint32_t* root, uint32_t* alpha_out) {
  pdl_enter();
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  d_ch_mix_root(ch, root);
  qm31 a = d_ch_draw_felt(ch);
  qm31 a2 = qm31_mul(a, a);
  alpha_out[0] = a.a.a; alpha_out[1] = a.a.b; alpha_out[2] = a.b.a; alpha_out[3] = a.b.b;
  alpha_out[4] = a2.a.a; alpha_out[5] = a2.a.b; alpha_out[6] = a2.b.a; alpha_out[7] = a2.b.b;
}

struct Digest8 { uint32_t w[8]; };
__global__ void k_channel_set(DevChannel* ch, Digest8 d, uint64_t n_sent) {
  pdl_enter();
  for (int i = 0; i < 8; i++) ch->digest[i] = d.w[i];
  ch->n_sent_lo = (uint32_t)n_sent;
  ch->n_sent_hi = (uint32_t)(n_sent >> 32);
  ch->error = 0u;
}

// Per-block partial sums of +f (first half) and -f (second half), four coordinates, reduced
// into 64-bit accumulators (each partial is < P, so 2^33 of them cannot overflow).
__global__ void k_decompose_sum(Secure4 src, uint32_t n, unsigned long long* acc) {
  __shared__ uint32_t part[4][32];
  uint32_t s[4] = {0, 0, 0, 0};
  uint32_t half = n >> 1;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
#pragma unroll
    for (int k = 0; k < 4; k++) {
      uint32_t v = __ldg(src.p[k] + i);
      s[k] = i < half ? m31_add(s[k], v) : m31_sub(s[k], v);
    }
  }
#pragma unroll
  for (int k = 0; k < 4; k++) {
    uint32_t v = s[k];
    for (int o = 16; o > 0; o >>= 1) v = m31_add(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) part[k][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    uint32_t v = 0;
    for (uint32_t w = 0; w < blockDim.x / 32; w++) v = m31_add(v, part[threadIdx.x][w]);
    atomicAdd(acc + threadIdx.x, (unsigned long long)v);
  }
}

__global__ void k_decompose_apply(Secure4 src, Secure4M dst, uint32_t n, const unsigned long long* acc,
                                  uint32_t inv_n, uint32_t* lambda_out) {
  qm31 lambda = qm31_mul_m31(qm31_from_u32(m31_reduce64(acc[0]), m31_reduce64(acc[1]), m31_reduce64(acc[2]),
                                           m31_reduce64(acc[3])),
                             inv_n);
  uint32_t half = n >> 1;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    lambda_out[0] = lambda.a.a;
    lambda_out[1] = lambda.a.b;
    lambda_out[2] = lambda.b.a;
    lambda_out[3] = lambda.b.b;
  }
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    qm31 v = load_q(src, i);
    store_q(dst, i, i < half ? qm31_sub(v, lambda) : qm31_add(v, lambda));
  }
}

static qm31 to_q(stwo_qm31 a) { return {{a.v[0], a.v[1]}, {a.v[2], a.v[3]}}; }
static uint32_t grid_for(size_t n, uint32_t threads) {
  size_t b = (n + threads - 1) / threads;
  size_t cap = (size_t)sm_count() * 16;
  return (uint32_t)std::max<size_t>(1, std::min(b, cap));
}

// Offset of the level of coset `c` in a tree whose root it is a doubling of.
static bool level_offset(const TwiddleTree* t, stwo_coset c, size_t* off) {
  if (!t || !coset_is_doubling_of(c, t->root)) return false;
  *off = t->size - ((size_t)1 << c.log_size);
  return true;
}

int32_t fri_fold_line(const TwiddleTree* tree, stwo_coset line_domain, const uint32_t* const src[4],
                      qm31 alpha, uint32_t* const out[4], cudaStream_t s, const uint32_t* alpha_dev,
                      uint32_t* leaves) {
  STWO_REQUIRE(line_domain.log_size >= 1, "Evaluation too small");
  size_t off;
  STWO_REQUIRE(level_offset(tree, line_domain, &off), "line domain is not a doubling of the twiddle root");
  uint32_t n_out = 1u << (line_domain.log_size - 1);
  Secure4 sp{{src[0], src[1], src[2], src[3]}};
  Secure4M dp{{out[0], out[1], out[2], out[3]}};
  launch_pdl(k_fold_line, dim3(grid_for(n_out, 256)), dim3(256), 0, s, sp, dp, n_out, tree->d_itw + off, alpha,
             alpha_dev, leaves);
  note_launch();
  STWO_LAUNCH_CHECK();
  return STWO_OK;
}

int32_t fri_fold_circle(const TwiddleTree* tree, stwo_coset half, uint32_t* const dst[4],
                        const uint32_t* const src[4], qm31 alpha, cudaStream_t s, const uint32_t* alpha_dev,
                        uint32_t* leaves) {
  uint32_t log_src = half.log_size + 1;
  size_t off = 0;
  const uint32_t* lvl = nullptr;
  if (log_src >= 3) {
    STWO_REQUIRE(level_offset(tree, half, &off), "domain is not a doubling of the twiddle root");
    lvl = tree->d_itw + off;
  }
  uint32_t n_out = 1u << (log_src - 1);
  Secure4 sp{{src[0], src[1], src[2], src[3]}};
  Secure4M dp{{dst[0], dst[1], dst[2], dst[3]}};
  // alpha^2 computed on the device side of the arithmetic is identical; do it on the host once.
  uint32_t a[4] = {alpha.a.a, alpha.a.b, alpha.b.a, alpha.b.b};
  // (a + bu)^2 = a^2 + (2+i) b^2 + 2ab u over CM31.
  auto cmul = [](uint32_t x0, uint32_t x1, uint32_t y0, uint32_t y1, uint32_t* r0, uint32_t* r1) {
    *r0 = h_sub(h_mul(x0, y0), h_mul(x1, y1));
    *r1 = h_add(h_mul(x0, y1), h_mul(x1, y0));
  };
  uint32_t aa0, aa1, bb0, bb1, ab0, ab1;
  cmul(a[0], a[1], a[0], a[1], &aa0, &aa1);
  cmul(a[2], a[3], a[2], a[3], &bb0, &bb1);
  cmul(a[0], a[1], a[2], a[3], &ab0, &ab1);
  uint32_t rb0 = h_sub(h_add(bb0, bb0), bb1), rb1 = h_add(bb0, h_add(bb1, bb1));
  qm31 a2 = {{h_add(aa0, rb0), h_add(aa1, rb1)}, {h_add(ab0, ab0), h_add(ab1, ab1)}};
  launch_pdl(k_fold_circle, dim3(grid_for(n_out, 256)), dim3(256), 0, s, sp, dp, n_out, lvl, log_src,
             half.initial_index, half.step_size, alpha, a2, alpha_dev, leaves);
  note_launch();
  STWO_LAUNCH_CHECK();
  return STWO_OK;
}

int32_t fri_decompose(const uint32_t* const src[4], uint32_t log_size, uint32_t* const g[4], stwo_qm31* lambda,
                      cudaStream_t s) {
  STWO_REQUIRE(log_size >= 1 && log_size <= 30, "bad log size %u", log_size);
  uint32_t n = 1u << log_size;
  unsigned long long* acc = nullptr;
  int32_t st = scratch_alloc((void**)&acc, 4 * sizeof(unsigned long long) + 16, s);
  if (st) return st;
  uint32_t* lam = reinterpret_cast<uint32_t*>(acc + 4);
  cudaMemsetAsync(acc, 0, 4 * sizeof(unsigned long long), s);
  Secure4 sp{{src[0], src[1], src[2], src[3]}};
  Secure4M dp{{g[0], g[1], g[2], g[3]}};
  k_decompose_sum<<<grid_for(n, 256), 256, 0, s>>>(sp, n, acc); note_launch();
  k_decompose_apply<<<grid_for(n, 256), 256, 0, s>>>(sp, dp, n, acc, h_inv(n % P), lam); note_launch();
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(lambda->v, lam, 16, cudaMemcpyDeviceToHost, s);
  scratch_free(acc, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    set_error("decompose: %s", cudaGetErrorString(e));
    return STWO_ERR_CUDA;
  }
  return STWO_OK;
}

// ---------------------------------------------------------------- small-layer tail
// The FRI layers of at most 2^FRI_TAIL_MAX_LOG points, in one single-block launch. Per layer:
// Blake2s leaves of its four coordinate columns, the node levels up to the root, the transcript
// step (mix the root, draw alpha) on the device channel, and the line fold into the next layer.
// The results are the ones of the per-kernel path (the same Merkle layout as DevMerkle, the same
// fold as k_fold_line, the same channel as dchannel.cuh); only the schedule differs:
//   - node levels read their children from shared memory (ping-pong buffers) and write each
//     level to the tree in HBM for the decommitment; levels of at most 32 nodes run in warp 0
//     with warp barriers only;
//   - the fold of layer j hashes, in the same thread, the leaf of layer j + 1 it produced;
//   - the transcript step uses the unrolled compression.
constexpr uint32_t FRI_TAIL_MAX_LAYERS = 16;
constexpr uint32_t FRI_TAIL_MAX_LOG = 10;
constexpr uint32_t FRI_TAIL_THREADS = 1024;
constexpr size_t FRI_TAIL_SMEM = (size_t)8 * 4 * ((1u << FRI_TAIL_MAX_LOG) + (1u << (FRI_TAIL_MAX_LOG - 1)));
struct FriTailParams {
  uint32_t n_layers;
  uint32_t log[FRI_TAIL_MAX_LAYERS];           // layer j has 2^log[j] points
  const uint32_t* eval[FRI_TAIL_MAX_LAYERS + 1][4];  // eval[j + 1] receives the fold of layer j
  uint32_t* tree[FRI_TAIL_MAX_LAYERS];         // all Merkle layers of layer j (root at offset 0)
  const uint32_t* itw[FRI_TAIL_MAX_LAYERS];    // inverse twiddles of layer j's line domain level
  DevChannel* ch;
  uint32_t* alphas;                            // 8 words per layer: alpha, alpha^2
};

// Blake2s-256 of a message of `bytes` <= 64 bytes given as 16 words (zero padded): one final
// compression. Out of line, so that the single thread or warp that runs the upper levels and the
// transcript step executes one copy of the unrolled rounds and keeps it in the instruction cache.
static __device__ __noinline__ void tail_hash(const uint32_t* w, uint32_t bytes, uint32_t* out) {
  uint32_t h[8], m[16];
#pragma unroll
  for (int q = 0; q < 16; q++) m[q] = w[q];
  b2s_init(h);
  b2s_compress_lat(h, m, bytes, true);
#pragma unroll
  for (int q = 0; q < 8; q++) out[q] = h[q];
}
__device__ __forceinline__ void tail_hash64(const uint32_t w[16], uint32_t out[8]) { tail_hash(w, 64, out); }

// Leaf hash of one point: its four coordinates as a 16-byte message.
__device__ __forceinline__ void tail_leaf(const qm31& v, uint32_t* tree_leaf, uint32_t* s_leaf) {
  uint32_t h[8], m[16];
#pragma unroll
  for (int q = 0; q < 16; q++) m[q] = 0u;
  m[0] = v.a.a;
  m[1] = v.a.b;
  m[2] = v.b.a;
  m[3] = v.b.b;
  tail_hash(m, 16, h);
#pragma unroll
  for (int q = 0; q < 8; q++) {
    tree_leaf[q] = h[q];
    s_leaf[q] = h[q];
  }
}

// One node of level `out` from its children in shared memory `src`.
__device__ __forceinline__ void tail_node(const uint32_t* src, uint32_t i, uint32_t* dst, uint32_t* tree_level) {
  uint32_t m[16], h[8];
#pragma unroll
  for (int q = 0; q < 16; q++) m[q] = src[16 * i + q];
  tail_hash64(m, h);
#pragma unroll
  for (int q = 0; q < 8; q++) {
    dst[8 * i + q] = h[q];
    tree_level[8 * i + q] = h[q];
  }
}

// mix_root then draw_felt of dchannel.cuh (d_ch_mix_root, d_ch_draw_base8), unrolled.
__device__ qm31 tail_channel_step(DevChannel* c, const uint32_t* root) {
  uint32_t w[16], d[8];
#pragma unroll
  for (int i = 0; i < 8; i++) {
    w[i] = c->digest[i];
    w[8 + i] = root[i];
  }
  tail_hash64(w, d);
  uint32_t nlo = 0, nhi = 0;
  uint32_t f[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  bool ok = false;
  for (int attempt = 0; attempt < 64 && !ok; attempt++) {
#pragma unroll
    for (int i = 0; i < 8; i++) w[i] = d[i];
    w[8] = nlo;
    w[9] = nhi;
#pragma unroll
    for (int i = 10; i < 16; i++) w[i] = 0u;
    if (++nlo == 0) nhi++;
    uint32_t h[8];
    tail_hash64(w, h);
    ok = true;
#pragma unroll
    for (int i = 0; i < 8; i++) ok = ok && h[i] < 2u * P;
    if (ok) {
#pragma unroll
      for (int i = 0; i < 8; i++) f[i] = h[i] >= P ? h[i] - P : h[i];
    }
  }
#pragma unroll
  for (int i = 0; i < 8; i++) c->digest[i] = d[i];
  c->n_sent_lo = nlo;
  c->n_sent_hi = nhi;
  if (!ok) c->error = 1u;
  return qm31_from_u32(f[0], f[1], f[2], f[3]);
}

__global__ void __launch_bounds__(FRI_TAIL_THREADS) k_fri_tail(FriTailParams p) {
  pdl_enter();
  extern __shared__ uint32_t s_nodes[];
  uint32_t* const s_a = s_nodes;                                    // levels k, k - 2, ...
  uint32_t* const s_b = s_nodes + 8 * (1u << FRI_TAIL_MAX_LOG);     // levels k - 1, k - 3, ...
  __shared__ qm31 s_alpha;
  const uint32_t tid = threadIdx.x;
  // Leaves of the first layer, from its evaluation in HBM.
  {
    const uint32_t n = 1u << p.log[0];
    const uint32_t* const* c = p.eval[0];
    uint32_t* leaves = p.tree[0] + (size_t)8 * (n - 1);
    for (uint32_t i = tid; i < n; i += blockDim.x)
      tail_leaf(qm31_from_u32(c[0][i], c[1][i], c[2][i], c[3][i]), leaves + 8 * i, s_a + 8 * i);
  }
  __syncthreads();
  for (uint32_t j = 0; j < p.n_layers; j++) {
    const uint32_t k = p.log[j], n = 1u << k;
    uint32_t* tree = p.tree[j];
    uint32_t* src = s_a;
    uint32_t* dst = s_b;
    int lg = (int)k - 1;
    for (; lg >= 5; lg--) {
      const uint32_t w = 1u << lg;
      for (uint32_t i = tid; i < w; i += blockDim.x) tail_node(src, i, dst, tree + (size_t)8 * (w - 1));
      __syncthreads();
      uint32_t* t = src;
      src = dst;
      dst = t;
    }
    if (tid < 32) {
      for (; lg >= 0; lg--) {
        const uint32_t w = 1u << lg;
        if (tid < w) tail_node(src, tid, dst, tree + (size_t)8 * (w - 1));
        __syncwarp();
        uint32_t* t = src;
        src = dst;
        dst = t;
      }
      if (tid == 0) {
        const qm31 a = tail_channel_step(p.ch, src);
        const qm31 a2 = qm31_mul(a, a);
        uint32_t* o = p.alphas + 8 * j;
        o[0] = a.a.a; o[1] = a.a.b; o[2] = a.b.a; o[3] = a.b.b;
        o[4] = a2.a.a; o[5] = a2.a.b; o[6] = a2.b.a; o[7] = a2.b.b;
        s_alpha = a;
      }
    }
    __syncthreads();
    const qm31 alpha = s_alpha;
    const uint32_t* const* c = p.eval[j];
    uint32_t* const* nxt = const_cast<uint32_t* const*>(p.eval[j + 1]);
    const bool next_in_tail = j + 1 < p.n_layers;
    uint32_t* next_leaves = next_in_tail ? p.tree[j + 1] + (size_t)8 * (n / 2 - 1) : nullptr;
    for (uint32_t i = tid; i < n / 2; i += blockDim.x) {
      qm31 f0 = qm31_from_u32(c[0][2 * i], c[1][2 * i], c[2][2 * i], c[3][2 * i]);
      qm31 f1 = qm31_from_u32(c[0][2 * i + 1], c[1][2 * i + 1], c[2][2 * i + 1], c[3][2 * i + 1]);
      ibfly_q(f0, f1, p.itw[j][i]);
      const qm31 r = qm31_add(f0, qm31_mul(alpha, f1));
      nxt[0][i] = r.a.a;
      nxt[1][i] = r.a.b;
      nxt[2][i] = r.b.a;
      nxt[3][i] = r.b.b;
      if (next_in_tail) tail_leaf(r, next_leaves + 8 * i, s_a + 8 * i);
    }
    __syncthreads();
  }
}

// Launches the tail over layers whose line domains are `doms` (each the doubling of the last);
// eval[0] holds the first layer, eval[j + 1] receives each fold.
int32_t fri_tail(const TwiddleTree* tree, const std::vector<stwo_coset>& doms,
                 const std::vector<std::array<uint32_t*, 4>>& evals, const std::vector<uint32_t*>& trees,
                 DevChannel* ch, uint32_t* alphas, cudaStream_t s) {
  STWO_REQUIRE(!doms.empty() && doms.size() <= FRI_TAIL_MAX_LAYERS, "FRI tail of %zu layers", doms.size());
  STWO_REQUIRE(evals.size() == doms.size() + 1 && trees.size() == doms.size(), "FRI tail buffers");
  FriTailParams p{};
  p.n_layers = (uint32_t)doms.size();
  for (size_t j = 0; j < doms.size(); j++) {
    STWO_REQUIRE(doms[j].log_size >= 1, "Evaluation too small");
    STWO_REQUIRE(doms[j].log_size <= FRI_TAIL_MAX_LOG, "FRI tail layer of 2^%u points", doms[j].log_size);
    STWO_REQUIRE(j == 0 || doms[j].log_size + 1 == doms[j - 1].log_size, "FRI tail layers must halve");
    size_t off;
    STWO_REQUIRE(level_offset(tree, doms[j], &off), "line domain is not a doubling of the twiddle root");
    p.log[j] = doms[j].log_size;
    p.itw[j] = tree->d_itw + off;
    p.tree[j] = trees[j];
  }
  for (size_t j = 0; j < evals.size(); j++)
    for (int k = 0; k < 4; k++) p.eval[j][k] = evals[j][k];
  p.ch = ch;
  p.alphas = alphas;
  // The 48 KB of dynamic shared memory needs the opt-in attribute, once per device.
  {
    static std::mutex mu;
    static bool done[256] = {};
    int dev = 0;
    STWO_CHECK_CUDA(cudaGetDevice(&dev));
    STWO_REQUIRE(dev >= 0 && dev < 256, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> g(mu);
    if (!done[dev]) {
      STWO_CHECK_CUDA(
          cudaFuncSetAttribute(k_fri_tail, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FRI_TAIL_SMEM));
      done[dev] = true;
    }
  }
  launch_pdl(k_fri_tail, dim3(1), dim3(FRI_TAIL_THREADS), FRI_TAIL_SMEM, s, p);
  note_launch();
  STWO_LAUNCH_CHECK();
  return STWO_OK;
}

int32_t fri_channel_step(DevChannel* ch, const uint32_t* root, uint32_t* alpha_out, cudaStream_t s) {
  launch_pdl(k_fri_channel_step, dim3(1), dim3(32), 0, s, ch, root, alpha_out);
  note_launch();
  STWO_LAUNCH_CHECK();
  return STWO_OK;
}

int32_t channel_set(DevChannel* ch, const uint32_t digest[8], uint64_t n_sent, cudaStream_t s) {
  Digest8 d;
  for (int i = 0; i < 8; i++) d.w[i] = digest[i];
  launch_pdl(k_channel_set, dim3(1), dim3(1), 0, s, ch, d, n_sent);
  note_launch();
  STWO_LAUNCH_CHECK();
  return STWO_OK;
}

}  // namespace stwo

using namespace stwo;

extern "C" {

stwo_status stwo_fri_fold_line(stwo_twiddle_tree tree, stwo_coset line_domain, const uint32_t* const d_eval[4],
                               stwo_qm31 alpha, uint32_t* const d_out[4], void* stream) {
  return fri_fold_line(tree_of(tree), line_domain, d_eval, to_q(alpha), d_out, as_stream(stream), nullptr, nullptr);
}

stwo_status stwo_fri_fold_circle_into_line(stwo_twiddle_tree tree, stwo_coset src_half_coset,
                                           uint32_t* const d_dst[4], const uint32_t* const d_src[4],
                                           stwo_qm31 alpha, void* stream) {
  return fri_fold_circle(tree_of(tree), src_half_coset, d_dst, d_src, to_q(alpha), as_stream(stream), nullptr,
                         nullptr);
}

stwo_status stwo_fri_decompose(const uint32_t* const d_eval[4], uint32_t log_size, uint32_t* const d_g[4],
                               stwo_qm31* h_lambda, void* stream) {
  STWO_REQUIRE(h_lambda, "null lambda");
  return fri_decompose(d_eval, log_size, d_g, h_lambda, as_stream(stream));
}

}  // extern "C"
