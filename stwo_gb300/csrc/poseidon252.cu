// Poseidon252 Merkle hashing and grinding on the device: the second BackendForChannel
// instantiation of the reference (backend/simd/mod.rs:34-35), MerkleOps<Poseidon252MerkleHasher>
// and GrindOps<Poseidon252Channel>.
//
// Hasher (crates/prover/src/core/vcs/poseidon252_merkle.rs:17-45): a node hashes, with the
// Starknet poseidon_hash_many, its two children (when it has a previous layer) followed by its
// column values packed eight per field element (value k of a block times 2^(31 (7 - k))). The hash
// is the Hades permutation over the STARK field p = 2^251 + 17 * 2^192 + 1: width 3, 4 full
// rounds, 83 partial rounds, 4 full rounds; x^3 S-boxes (all words in full rounds, the last word in
// partial rounds); MDS [[3, 1, 1], [1, -1, 1], [1, 1, -2]]. hash_many is a sponge of rate 2 from
// [0, 0, 0] with a 1 added to word (values left over) before the final permutation. Grinding
// (backend/simd/grind.rs:65-79) looks for the smallest nonce whose poseidon_hash(digest, nonce)
// has pow_bits trailing zeros as channel/poseidon252.rs:59-62 counts them: the first 16 bytes of
// the big-endian encoding read as a little-endian u128.
//
// GB300 formulation: one thread per node (or nonce). Field elements are 8 little-endian 32-bit
// limbs in Montgomery form (radix 2^256); the product is CIOS with the sparse modulus (limbs 0, 6
// and 7 nonzero, -p^-1 = -1 mod 2^32), so each reduction step is three multiply-adds. Round
// constants sit in constant memory, read uniformly by a warp. This is integer-multiply work on
// the FMA pipe: about 214 field products per permutation.
#include "common.cuh"
#include "poseidon252_constants.cuh"

namespace stwo {

struct f252 {
  uint32_t w[8];
};

__device__ __forceinline__ bool f252_geq_p(const uint32_t* t) {
  // p = [1, 0, 0, 0, 0, 0, 17, 2^27]
  if (t[7] != 0x08000000u) return t[7] > 0x08000000u;
  if (t[6] != 17u) return t[6] > 17u;
  if (t[5] | t[4] | t[3] | t[2] | t[1]) return true;
  return t[0] >= 1u;
}
__device__ __forceinline__ void f252_sub_p(uint32_t* t) {
  uint64_t c = (uint64_t)t[0] - 1u;
  t[0] = (uint32_t)c;
  int64_t b = (int64_t)(c >> 63);  // borrow 0 or 1
#pragma unroll
  for (int j = 1; j < 6; j++) {
    uint64_t d = (uint64_t)t[j] - (uint64_t)b;
    t[j] = (uint32_t)d;
    b = (int64_t)(d >> 63);
  }
  uint64_t d6 = (uint64_t)t[6] - 17u - (uint64_t)b;
  t[6] = (uint32_t)d6;
  b = (int64_t)(d6 >> 63);
  t[7] = t[7] - 0x08000000u - (uint32_t)b;
}

// Montgomery product a * b / 2^256 mod p for a, b < 2^256 with a * b < 2^256 p; result < p.
__device__ __forceinline__ f252 f252_mul(const f252& a, const f252& b) {
  uint32_t t[10];
#pragma unroll
  for (int j = 0; j < 10; j++) t[j] = 0;
#pragma unroll
  for (int i = 0; i < 8; i++) {
    uint64_t c = 0;
#pragma unroll
    for (int j = 0; j < 8; j++) {
      c += (uint64_t)a.w[j] * b.w[i] + t[j];
      t[j] = (uint32_t)c;
      c >>= 32;
    }
    c += t[8];
    t[8] = (uint32_t)c;
    t[9] = (uint32_t)(c >> 32);
    // m = -t0 mod 2^32; t += m p, then drop the (zero) low limb.
    const uint32_t m = 0u - t[0];
    c = ((uint64_t)t[0] + m) >> 32;
#pragma unroll
    for (int j = 1; j < 6; j++) {
      c += t[j];
      t[j - 1] = (uint32_t)c;
      c >>= 32;
    }
    c += (uint64_t)m * 17u + t[6];
    t[5] = (uint32_t)c;
    c >>= 32;
    c += (uint64_t)m * 0x08000000u + t[7];
    t[6] = (uint32_t)c;
    c >>= 32;
    c += t[8];
    t[7] = (uint32_t)c;
    t[8] = t[9] + (uint32_t)(c >> 32);
  }
  if (f252_geq_p(t)) f252_sub_p(t);  // t < 2p and t[8] = 0
  f252 r;
#pragma unroll
  for (int j = 0; j < 8; j++) r.w[j] = t[j];
  return r;
}

__device__ __forceinline__ f252 f252_add(const f252& a, const f252& b) {
  f252 r;
  uint64_t c = 0;
#pragma unroll
  for (int j = 0; j < 8; j++) {
    c += (uint64_t)a.w[j] + b.w[j];
    r.w[j] = (uint32_t)c;
    c >>= 32;
  }
  if (f252_geq_p(r.w)) f252_sub_p(r.w);  // a + b < 2p < 2^253: no carry out
  return r;
}
__device__ __forceinline__ f252 f252_sub(const f252& a, const f252& b) {
  f252 r;
  int64_t br = 0;
#pragma unroll
  for (int j = 0; j < 8; j++) {
    const uint64_t d = (uint64_t)a.w[j] - b.w[j] - (uint64_t)br;
    r.w[j] = (uint32_t)d;
    br = (int64_t)(d >> 63);
  }
  if (br) {  // add p back
    uint64_t c = (uint64_t)r.w[0] + 1u;
    r.w[0] = (uint32_t)c;
    c >>= 32;
#pragma unroll
    for (int j = 1; j < 6; j++) {
      c += r.w[j];
      r.w[j] = (uint32_t)c;
      c >>= 32;
    }
    c += (uint64_t)r.w[6] + 17u;
    r.w[6] = (uint32_t)c;
    c >>= 32;
    r.w[7] = (uint32_t)(c + r.w[7] + 0x08000000u);
  }
  return r;
}
__device__ __forceinline__ f252 f252_const(const uint32_t (&c)[8]) {
  f252 r;
#pragma unroll
  for (int j = 0; j < 8; j++) r.w[j] = c[j];
  return r;
}
__device__ __forceinline__ f252 to_mont(const f252& x) { return f252_mul(x, f252_const(c_p252_r2)); }
__device__ __forceinline__ f252 from_mont(const f252& x) {
  f252 one{};
  one.w[0] = 1u;
  return f252_mul(x, one);
}
__device__ __forceinline__ f252 cube(const f252& x) { return f252_mul(f252_mul(x, x), x); }

__device__ void hades(f252& s0, f252& s1, f252& s2) {
#pragma unroll 1
  for (int r = 0; r < P252_ROUNDS; r++) {
    s0 = f252_add(s0, f252_const(c_p252_ark[3 * r]));
    s1 = f252_add(s1, f252_const(c_p252_ark[3 * r + 1]));
    s2 = f252_add(s2, f252_const(c_p252_ark[3 * r + 2]));
    if (r < 4 || r >= P252_ROUNDS - 4) {
      s0 = cube(s0);
      s1 = cube(s1);
    }
    s2 = cube(s2);
    // [[3, 1, 1], [1, -1, 1], [1, 1, -2]]
    const f252 t = f252_add(s0, s1);       // a + b
    const f252 u = f252_add(s0, s2);       // a + c
    const f252 n0 = f252_add(f252_add(t, u), s0);  // 3a + b + c
    const f252 n1 = f252_sub(u, s1);       // a - b + c
    const f252 n2 = f252_sub(f252_sub(t, s2), s2);  // a + b - 2c
    s0 = n0;
    s1 = n1;
    s2 = n2;
  }
}

// Canonical 8-limb words -> Montgomery form.
__device__ __forceinline__ f252 load_felt(const uint32_t* p) {
  f252 x;
#pragma unroll
  for (int j = 0; j < 8; j++) x.w[j] = p[j];
  return to_mont(x);
}

// One Merkle node per thread: poseidon_hash_many over [left, right]? + packed column blocks.
__global__ void __launch_bounds__(128) k_p252_merkle_layer(uint32_t n_nodes, const uint32_t* __restrict__ prev,
                                                           const uint32_t* const* __restrict__ cols,
                                                           uint32_t n_cols, uint32_t* __restrict__ out) {
  pdl_enter();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_nodes) return;
  const uint32_t n_children = prev ? 2u : 0u;
  const uint32_t n_in = n_children + (n_cols + 7) / 8;
  auto input = [&](uint32_t k) -> f252 {
    if (k < n_children) return load_felt(prev + (2 * (size_t)i + k) * 8);
    const uint32_t b = k - n_children;
    f252 w{};
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const uint32_t idx = 8 * b + q;
      const uint32_t x = idx < n_cols ? __ldg(cols[idx] + i) : 0u;
      const uint32_t off = 31u * (7u - q);
      const uint32_t limb = off >> 5, sh = off & 31u;
      w.w[limb] |= x << sh;
      if (sh > 1u) w.w[limb + 1] |= x >> (32u - sh);
    }
    return to_mont(w);  // an integer below 2^248 < p
  };
  f252 s0{}, s1{}, s2{};
  uint32_t k = 0;
  for (; k + 2 <= n_in; k += 2) {
    s0 = f252_add(s0, input(k));
    s1 = f252_add(s1, input(k + 1));
    hades(s0, s1, s2);
  }
  const uint32_t rem = n_in - k;
  if (rem == 1) s0 = f252_add(s0, input(k));
  if (rem == 0) s0 = f252_add(s0, f252_const(c_p252_one));
  else s1 = f252_add(s1, f252_const(c_p252_one));
  hades(s0, s1, s2);
  const f252 h = from_mont(s0);
#pragma unroll
  for (int j = 0; j < 8; j++) out[(size_t)i * 8 + j] = h.w[j];
}

// Trailing zeros as channel/poseidon252.rs:59-62 counts them on the canonical value.
__device__ __forceinline__ uint32_t p252_trailing_zeros(const f252& v) {
#pragma unroll 1
  for (int i = 0; i < 16; i++) {
    const int byte = 31 - i;  // big-endian byte i = little-endian byte 31 - i
    const uint32_t b = (v.w[byte >> 2] >> (8 * (byte & 3))) & 0xFFu;
    if (b) return 8u * i + (uint32_t)(__ffs(b) - 1);
  }
  return 128u;
}

__global__ void __launch_bounds__(128) k_p252_grind(f252 digest_m, uint32_t pow_bits, unsigned long long base,
                                                    unsigned long long* best) {
  const unsigned long long nonce = base + blockIdx.x * blockDim.x + threadIdx.x;
  f252 n{};
  n.w[0] = (uint32_t)nonce;
  n.w[1] = (uint32_t)(nonce >> 32);
  f252 s0 = digest_m, s1 = to_mont(n), s2 = f252_const(c_p252_two);
  hades(s0, s1, s2);
  if (p252_trailing_zeros(from_mont(s0)) >= pow_bits) atomicMin(best, nonce);
}

__global__ void k_p252_to_mont(f252 x, f252* out) { *out = to_mont(x); }

}  // namespace stwo

using namespace stwo;

extern "C" {

stwo_status stwo_merkle_commit_layer_poseidon252(uint32_t log_size, const uint32_t* d_prev_layer,
                                                 const uint32_t* const* d_cols, uint32_t n_cols, uint32_t* d_out,
                                                 void* stream) {
  STWO_REQUIRE(log_size <= 30, "log_size %u > 30", log_size);
  STWO_REQUIRE(d_out, "null output layer");
  STWO_REQUIRE(n_cols == 0 || d_cols, "null column table");
  cudaStream_t s = as_stream(stream);
  const uint32_t n = 1u << log_size;
  const uint32_t** d_tab = nullptr;
  if (n_cols) {
    for (uint32_t c = 0; c < n_cols; c++) STWO_REQUIRE(d_cols[c], "null column %u", c);
    int32_t st = scratch_alloc((void**)&d_tab, (size_t)n_cols * sizeof(void*), s);
    if (st) return st;
    cudaError_t e = cudaMemcpyAsync(d_tab, d_cols, (size_t)n_cols * sizeof(void*), cudaMemcpyHostToDevice, s);
    if (e) {
      scratch_free(d_tab, s);
      set_error("poseidon252 layer: %s", cudaGetErrorString(e));
      return STWO_ERR_CUDA;
    }
  }
  launch_pdl(k_p252_merkle_layer, dim3((n + 127) / 128), dim3(128), 0, s, n, d_prev_layer, d_tab, n_cols, d_out);
  note_launch();
  cudaError_t e = cudaGetLastError();
  if (d_tab) scratch_free(d_tab, s);
  if (e) {
    set_error("poseidon252 layer: %s", cudaGetErrorString(e));
    return STWO_ERR_CUDA;
  }
  return STWO_OK;
}

stwo_status stwo_grind_poseidon252(const uint32_t h_digest[8], uint32_t pow_bits, uint64_t* h_nonce, void* stream) {
  STWO_REQUIRE(h_digest && h_nonce, "null argument");
  STWO_REQUIRE(pow_bits <= 32, "pow_bits %u > 32", pow_bits);
  cudaStream_t s = as_stream(stream);
  f252 d;
  for (int j = 0; j < 8; j++) d.w[j] = h_digest[j];
  unsigned long long* buf = nullptr;  // [0] best nonce, [1..5) the digest in Montgomery form
  int32_t st = scratch_alloc((void**)&buf, 64, s);
  if (st) return st;
  unsigned long long h_buf[5];
  cudaError_t e = cudaSuccess;
  k_p252_to_mont<<<1, 1, 0, s>>>(d, reinterpret_cast<f252*>(buf + 1));
  note_launch();
  e = cudaGetLastError();
  if (!e) e = cudaMemcpyAsync(h_buf, buf, 40, cudaMemcpyDeviceToHost, s);
  if (!e) e = cudaStreamSynchronize(s);
  f252 dm;
  std::memcpy(dm.w, h_buf + 1, 32);
  // Batches of nonces in increasing order; the first batch with a hit holds the minimum.
  const unsigned long long batch = 1ull << 17;
  unsigned long long found = ~0ull;
  for (unsigned long long base = 0; !e && found == ~0ull; base += batch) {
    if (base > (1ull << 36)) {
      scratch_free(buf, s);
      set_error("poseidon252 grind: no nonce below 2^36");
      return STWO_ERR_TIMEOUT;
    }
    unsigned long long init = ~0ull;
    e = cudaMemcpyAsync(buf, &init, 8, cudaMemcpyHostToDevice, s);
    if (!e) {
      k_p252_grind<<<(uint32_t)(batch / 128), 128, 0, s>>>(dm, pow_bits, base, buf);
      note_launch();
      e = cudaGetLastError();
    }
    if (!e) e = cudaMemcpyAsync(&found, buf, 8, cudaMemcpyDeviceToHost, s);
    if (!e) e = cudaStreamSynchronize(s);
  }
  scratch_free(buf, s);
  if (e) {
    set_error("poseidon252 grind: %s", cudaGetErrorString(e));
    return STWO_ERR_CUDA;
  }
  *h_nonce = found;
  return STWO_OK;
}

}  // extern "C"
