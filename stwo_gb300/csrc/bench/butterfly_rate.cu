// Register-only throughput of the circle-FFT butterfly over M31 (a standalone measurement program,
// not part of the library). Each thread holds 16 words and 15 doubled twiddles in registers and
// runs ITERS rounds of 4 forward butterfly layers (32 butterflies per round), the shape of one
// register round of the FFT tile kernels, with no memory traffic in the loop. The variants differ
// only in how sums and products are reduced mod P = 2^31 - 1:
//   0  min(x, x - P) after the product, the sum and the difference (the library's butterfly)
//   1  the sum and the difference reduced with a multiply: x - P * (x >> 31), the shift done as
//      a high-half product by a run-time 2 so that it stays on the multiply path
//   2  every reduction with the multiply form
//   3  the add-and-min instruction (__viaddmin_u32) for every reduction
// Every variant is checked word for word against variant 0. Build and run:
//   nvcc -O3 -std=c++17 -gencode arch=compute_103a,code=sm_103a butterfly_rate.cu -o butterfly_rate
//   ./butterfly_rate            (BF_ONCE=1: one launch per variant, for counter captures)
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

constexpr uint32_t P = 0x7fffffffu;
struct Consts { uint32_t two, neg_p; };

__device__ __forceinline__ uint32_t red_min(uint32_t s) { return min(s, s - P); }
__device__ __forceinline__ uint32_t red_mul(uint32_t s, const Consts& k) {
  uint32_t q, r;
  asm("mul.hi.u32 %0, %1, %2;" : "=r"(q) : "r"(s), "r"(k.two));
  asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(q), "r"(k.neg_p), "r"(s));
  return r;
}
// a * t mod P (up to one P) with the doubled twiddle t2 = 2t: the 64-bit product splits at bit 32
// into floor(at / 2^31) and (at mod 2^31).
__device__ __forceinline__ uint32_t mul_raw(uint32_t a, uint32_t t2) {
  const uint64_t p = (uint64_t)a * t2;
  return (uint32_t)(p >> 32) + ((uint32_t)p >> 1);
}
template <int V>
__device__ __forceinline__ void bfly(uint32_t& v0, uint32_t& v1, uint32_t t2, const Consts& k) {
  if constexpr (V == 0) {
    const uint32_t t = red_min(mul_raw(v1, t2));
    const uint32_t d = v0 - t;
    v1 = min(d, d + P);
    v0 = red_min(v0 + t);
  } else if constexpr (V == 1) {
    const uint32_t t = red_min(mul_raw(v1, t2));
    v1 = red_mul(v0 + P - t, k);
    v0 = red_mul(v0 + t, k);
  } else if constexpr (V == 2) {
    const uint32_t t = red_mul(mul_raw(v1, t2), k);
    v1 = red_mul(v0 + P - t, k);
    v0 = red_mul(v0 + t, k);
  } else {
    const uint32_t s = mul_raw(v1, t2);
    const uint32_t t = __viaddmin_u32(s, 0x80000001u, s);
    const uint32_t d = v0 - t;
    v1 = __viaddmin_u32(d, P, d);
    const uint32_t a = v0 + t;
    v0 = __viaddmin_u32(a, 0x80000001u, a);
  }
}
template <int V>
__global__ void __launch_bounds__(256) k_bfly(const uint32_t* in, const uint32_t* tw, uint32_t* out, Consts k,
                                               int iters) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x, n = gridDim.x * blockDim.x;
  uint32_t v[16], t[15];
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = in[g + i * n];
#pragma unroll
  for (int i = 0; i < 15; i++) t[i] = tw[(g * 15 + i) & 4095];
  for (int it = 0; it < iters; it++) {
    int ti = 0;
#pragma unroll
    for (int j = 3; j >= 0; j--)
#pragma unroll
      for (int kh = 0; kh < (1 << (3 - j)); kh++) {
        const uint32_t tt = t[ti++];
#pragma unroll
        for (int kl = 0; kl < (1 << j); kl++) bfly<V>(v[(kh << (j + 1)) | kl], v[(kh << (j + 1)) | kl | (1 << j)], tt, k);
      }
  }
#pragma unroll
  for (int i = 0; i < 16; i++) out[g + i * n] = red_min(v[i] == P ? 0u : v[i]);
}

template <int V>
static float run(const uint32_t* din, const uint32_t* dtw, uint32_t* dout, Consts k, int blocks, int iters, bool once) {
  if (once) {
    k_bfly<V><<<blocks, 256>>>(din, dtw, dout, k, iters);
    cudaDeviceSynchronize();
    return 0.f;
  }
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  for (int w = 0; w < 3; w++) k_bfly<V><<<blocks, 256>>>(din, dtw, dout, k, iters);
  cudaEventRecord(a);
  for (int r = 0; r < 5; r++) k_bfly<V><<<blocks, 256>>>(din, dtw, dout, k, iters);
  cudaEventRecord(b);
  cudaEventSynchronize(b);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  return ms / 5;
}

int main() {
  const bool once = getenv("BF_ONCE") != nullptr;
  int sms = 0, clk_khz = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  cudaDeviceGetAttribute(&clk_khz, cudaDevAttrClockRate, 0);
  const int blocks = sms * 8, iters = 256;
  const size_t n = (size_t)blocks * 256 * 16;
  std::vector<uint32_t> h(n), htw(4096), ref(n), got(n);
  uint64_t x = 12345;
  auto rnd = [&]() { x ^= x << 13; x ^= x >> 7; x ^= x << 17; return (uint32_t)(x % P); };
  for (auto& e : h) e = rnd();
  for (auto& e : htw) e = 2 * (rnd() % (P - 1));
  uint32_t *din, *dtw, *dout;
  if (cudaMalloc(&din, n * 4) || cudaMalloc(&dtw, 4096 * 4) || cudaMalloc(&dout, n * 4)) return 1;
  cudaMemcpy(din, h.data(), n * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(dtw, htw.data(), 4096 * 4, cudaMemcpyHostToDevice);
  const Consts k{2u, 0x80000001u};
  float ms[4];
  ms[0] = run<0>(din, dtw, dout, k, blocks, iters, once);
  cudaMemcpy(ref.data(), dout, n * 4, cudaMemcpyDeviceToHost);
  bool ok = true;
#define VARIANT(I)                                                    \
  ms[I] = run<I>(din, dtw, dout, k, blocks, iters, once);             \
  cudaMemcpy(got.data(), dout, n * 4, cudaMemcpyDeviceToHost);         \
  if (got != ref) { printf("variant %d differs from variant 0\n", I); ok = false; }
  VARIANT(1) VARIANT(2) VARIANT(3)
  const double bf = (double)blocks * 256 * iters * 32;  // butterflies per launch
  for (int i = 0; i < 4 && !once; i++)
    printf("variant %d: %.3f ms  %.3f T butterflies/s  %.2f SM cycles per warp-butterfly per SMSP at %d MHz\n", i,
           ms[i], bf / ms[i] / 1e9, ms[i] * 1e-3 * clk_khz * 1e3 * sms * 4 / (bf / 32), clk_khz / 1000);
  cudaError_t e = cudaGetLastError();
  printf("%s %s\n", ok ? "all variants equal" : "MISMATCH", cudaGetErrorString(e));
  return (ok && e == cudaSuccess) ? 0 : 1;
}
