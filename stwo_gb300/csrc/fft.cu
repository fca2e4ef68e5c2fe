// Circle FFT / IFFT over M31 (PolyOps::interpolate_columns / evaluate_polynomials).
//
// Transform: the reference CPU backend's layer order (crates/prover/src/core/backend/cpu/
// circle.rs:18-135): evaluate runs line layers L-1..1 with the twiddle-tree slices of
// poly/utils.rs:62-77 and then the circle layer 0 whose twiddles are derived from the first
// line layer as [y, -y, -x, x] (cpu/circle.rs:209-229); interpolate runs them in reverse with
// inverse twiddles and scales by 1/2^L. Any correct schedule gives identical words because
// every operation is exact in the field.
//
// GB300 schedule: a column of 2^L words is processed in passes. Each pass moves tiles of
// 2^T words (T <= 13) HBM -> shared memory -> HBM; inside a tile, each thread holds 2^4
// words in registers and applies 4 butterfly layers per round, exchanging through shared
// memory between rounds. A contiguous pass covers layers [0, 13); strided passes cover
// higher layers with the 2^c lowest address bits kept contiguous for coalesced access.
// Evaluation on a larger domain (blowup) fuses the zero-extension into the first pass: each
// of the 2^(L-F) sub-domain chunks reads the 2^F coefficients and applies the big domain's
// twiddles, exactly as the reference SIMD backend's sub-domain evaluation
// (backend/simd/circle.rs:230-294).
#include "common.cuh"

namespace stwo {

// Butterflies with doubled twiddles t2 = 2t (a 32-bit word): the 64-bit product a * t2 = 2at
// splits at bit 32 into floor(at / 2^31) (the high word) and (at mod 2^31) (the low word shifted
// right once), whose sum is at mod P up to one subtraction. The results equal those of
// bfly / ibfly (crates/prover/src/core/fft.rs:5-21) with t.
__device__ __forceinline__ uint32_t mul_tw2(uint32_t a, uint32_t t2) {
  const uint64_t p = (uint64_t)a * t2;
  const uint32_t s = (uint32_t)(p >> 32) + ((uint32_t)p >> 1);  // < 2P
  return min(s, s - P);
}
__device__ __forceinline__ uint32_t neg_tw2(uint32_t t2) { return t2 ? 0xFFFFFFFEu - t2 : 0u; }  // 2(P - t)
__device__ __forceinline__ void bfly2(uint32_t& v0, uint32_t& v1, uint32_t t2) {
  const uint32_t tmp = mul_tw2(v1, t2);
  v1 = m31_sub(v0, tmp);
  v0 = m31_add(v0, tmp);
}
__device__ __forceinline__ void ibfly2(uint32_t& v0, uint32_t& v1, uint32_t it2) {
  const uint32_t tmp = v0;
  v0 = m31_add(tmp, v1);
  v1 = mul_tw2(m31_sub(tmp, v1), it2);
}

constexpr uint32_t FFT_TMAX = 12;   // contiguous tile: 2^12 words = 16 KB (+ padding)
constexpr uint32_t FFT_R = 4;        // 2^4 words per thread, 4 layers per register round

struct FftPass {
  uint32_t L;        // log size of the destination column (domain log size)
  uint32_t F;        // number of FFT layers = log size of the source column
  uint32_t lo, nl;   // this pass covers layers [lo, lo + nl)
  uint32_t c;        // number of low address bits kept contiguous in a tile
  uint32_t T;        // tile log size = c + nl
  const uint32_t* tw;  // twiddles (forward) or inverse twiddles
  uint32_t tw_size;    // tree size 2^root.log_size
  uint32_t small_y;    // circle-layer twiddle when L <= 2 (inverted for interpolate), doubled
  uint32_t scale;      // output multiplier (1 = none)
  uint32_t read_src;   // read from src (masked to 2^F) instead of dst
};

__device__ __forceinline__ uint32_t pad_idx(uint32_t e) { return e + (e >> 5); }

__device__ __forceinline__ uint32_t fft_twiddle(const FftPass& p, uint32_t layer, uint32_t idx0) {
  if (layer >= 1) {
    uint32_t off = p.tw_size - (1u << (p.L - layer));
    return __ldg(&p.tw[off + (idx0 >> (layer + 1))]);
  }
  uint32_t h = idx0 >> 1;
  if (p.L <= 2) return (h & 1) ? neg_tw2(p.small_y) : p.small_y;
  uint32_t off = p.tw_size - (1u << (p.L - 1));
  uint32_t t = __ldg(&p.tw[off + ((h >> 1) ^ 1)]);
  return ((h ^ (h >> 1)) & 1) ? neg_tw2(t) : t;
}

// Global index of tile element e: its low c bits are global bits [0, c), the next nl bits are
// the layer bits [lo, lo + nl); `fixed` carries every other bit of the tile.
__device__ __forceinline__ uint32_t tile_to_global(const FftPass& p, uint32_t e, uint32_t fixed) {
  return (e & ((1u << p.c) - 1)) | ((e >> p.c) << p.lo) | fixed;
}

// Bits of the tile id, lowest first: the sub-domain chunk bits [F, L) (so that the chunks that
// read the same source tile run back to back and share it through L2), then [c, lo), then
// [lo + nl, F).
__device__ __forceinline__ uint32_t tile_fixed_bits(const FftPass& p, uint32_t tile) {
  uint32_t nchunk = p.L - p.F;
  uint32_t chunk = tile & ((1u << nchunk) - 1);
  tile >>= nchunk;
  uint32_t mid_bits = p.lo - p.c;
  uint32_t mid = tile & ((1u << mid_bits) - 1);
  uint32_t top = tile >> mid_bits;
  return (chunk << p.F) | (mid << p.c) | (top << (p.lo + p.nl));
}

// One register round over tile bits [a, a + RB): each thread owns groups of 2^RB words differing
// in those bits, applies RB butterfly layers in registers (one twiddle load per distinct
// twiddle), and writes the group back.
template <bool INV, int RB>
__device__ __forceinline__ void fft_round(const FftPass& p, uint32_t* sm, uint32_t a, uint32_t fixed) {
  const uint32_t G = (1u << p.T) >> RB;
  for (uint32_t grp = threadIdx.x; grp < G; grp += blockDim.x) {
    const uint32_t base = (grp & ((1u << a) - 1)) | ((grp >> a) << (a + RB));
    uint32_t v[1 << RB];
#pragma unroll
    for (int k = 0; k < (1 << RB); k++) v[k] = sm[pad_idx(base | ((uint32_t)k << a))];
#pragma unroll
    for (int jj = 0; jj < RB; jj++) {
      const int j = INV ? jj : (RB - 1 - jj);
      const uint32_t layer = p.lo + (a + j - p.c);
#pragma unroll
      for (int kh = 0; kh < (1 << (RB - 1 - j)); kh++) {
        const int k0 = kh << (j + 1);
        const uint32_t g0 = tile_to_global(p, base | ((uint32_t)k0 << a), fixed);
        const uint32_t t = fft_twiddle(p, layer, g0);
#pragma unroll
        for (int kl = 0; kl < (1 << j); kl++) {
          if (INV) ibfly2(v[k0 | kl], v[k0 | kl | (1 << j)], t);
          else bfly2(v[k0 | kl], v[k0 | kl | (1 << j)], t);
        }
      }
    }
#pragma unroll
    for (int k = 0; k < (1 << RB); k++) sm[pad_idx(base | ((uint32_t)k << a))] = v[k];
  }
  __syncthreads();
}

template <bool INV>
__device__ __forceinline__ void fft_round_dispatch(const FftPass& p, uint32_t* sm, uint32_t a, uint32_t rb,
                                                   uint32_t fixed) {
  switch (rb) {
    case 4: fft_round<INV, 4>(p, sm, a, fixed); break;
    case 3: fft_round<INV, 3>(p, sm, a, fixed); break;
    case 2: fft_round<INV, 2>(p, sm, a, fixed); break;
    default: fft_round<INV, 1>(p, sm, a, fixed); break;
  }
}

template <bool INV, int MAXT>
__global__ void __launch_bounds__(MAXT) k_fft_pass(FftPass p, ConstColPtrs src, ColPtrs dst) {
  extern __shared__ uint32_t sm[];
  pdl_enter();
  const uint32_t col = blockIdx.y;
  const uint32_t n_tile = 1u << p.T;
  const uint32_t fixed = tile_fixed_bits(p, blockIdx.x);
  const uint32_t* s = p.read_src ? src.p[col] : dst.p[col];
  const uint32_t smask = p.read_src ? ((1u << p.F) - 1) : 0xffffffffu;
  uint32_t* d = dst.p[col];

  for (uint32_t e = threadIdx.x; e < n_tile; e += blockDim.x)
    sm[pad_idx(e)] = __ldg(&s[tile_to_global(p, e, fixed) & smask]);
  __syncthreads();

  if (!INV) {
    uint32_t top = p.c + p.nl;
    while (top > p.c) {
      uint32_t rb = min(FFT_R, top - p.c);
      uint32_t a = top - rb;
      fft_round_dispatch<INV>(p, sm, a, rb, fixed);
      top = a;
    }
  } else {
    uint32_t bot = p.c;
    while (bot < p.c + p.nl) {
      uint32_t rb = min(FFT_R, p.c + p.nl - bot);
      fft_round_dispatch<INV>(p, sm, bot, rb, fixed);
      bot += rb;
    }
  }

  for (uint32_t e = threadIdx.x; e < n_tile; e += blockDim.x) {
    uint32_t v = sm[pad_idx(e)];
    if (p.scale != 1u) v = m31_mul(v, p.scale);
    d[tile_to_global(p, e, fixed)] = v;
  }
}

// ---------------------------------------------------------------------------------------------
// Specialised pass kernel: the tile shape (C contiguous low bits, NL layer bits) is a template
// parameter, so every shared-memory offset and twiddle offset is an immediate and each
// butterfly costs the field arithmetic plus ~1 issue slot of addressing. Requires L >= 3 (the
// circle layer's twiddles come from the tree) and a tile of >= 2^4 words; other shapes use the
// generic kernel above.

template <bool INV, int C, int NL, int A, int RB>
__device__ __forceinline__ void fft_round_ct(const FftPass& p, uint32_t* sm, uint32_t fixed_hi, uint32_t llo) {
  constexpr int T = C + NL;
  constexpr int THREADS = 1 << (T - 4);
  constexpr int G = 1 << (T - RB);
#pragma unroll
  for (int it = 0; it < G / THREADS; it++) {
    const uint32_t grp = threadIdx.x + it * THREADS;
    const uint32_t base = (grp & ((1u << A) - 1)) | ((grp >> A) << (A + RB));
    const uint32_t pb = base + (base >> 5);
    uint32_t v[1 << RB];
#pragma unroll
    for (int k = 0; k < (1 << RB); k++) v[k] = sm[pb + (k << A) + ((k << A) >> 5)];
#pragma unroll
    for (int jj = 0; jj < RB; jj++) {
      const int j = INV ? jj : (RB - 1 - jj);
      const int lt = A + j - C;  // layer - lo
      // Twiddle index of the pair group: (tile bits above the layer) | (fixed bits above the tile).
      const uint32_t hb = (base >> (A + j + 1)) | (fixed_hi << (T - A - j - 1));
      const bool circle = (lt == 0) && (C == 0) && (p.lo == 0);
      const uint32_t* twp;
      if (circle) twp = p.tw + (p.tw_size - (llo >> 1)) + (hb >> 1);
      else twp = p.tw + (p.tw_size - (llo >> lt)) + hb;
#pragma unroll
      for (int kh = 0; kh < (1 << (RB - 1 - j)); kh++) {
        uint32_t t;
        if (circle) {
          // [y, -y, -x, x] from the first line layer (cpu/circle.rs:209-229). In a round of >= 3
          // bits the low two bits of the pair index are those of kh: entry and sign are
          // compile-time; otherwise they come from the full index.
          if (RB - 1 - j >= 2) {
            uint32_t raw = __ldg(twp + ((kh >> 1) ^ 1));
            t = ((kh ^ (kh >> 1)) & 1) ? neg_tw2(raw) : raw;
          } else {
            const uint32_t h = hb + kh;
            uint32_t raw = __ldg(p.tw + (p.tw_size - (llo >> 1)) + ((h >> 1) ^ 1));
            t = ((h ^ (h >> 1)) & 1) ? neg_tw2(raw) : raw;
          }
        } else {
          t = __ldg(twp + kh);
        }
        const int k0 = kh << (j + 1);
#pragma unroll
        for (int kl = 0; kl < (1 << j); kl++) {
          if (INV) ibfly2(v[k0 | kl], v[k0 | kl | (1 << j)], t);
          else bfly2(v[k0 | kl], v[k0 | kl | (1 << j)], t);
        }
      }
    }
#pragma unroll
    for (int k = 0; k < (1 << RB); k++) sm[pb + (k << A) + ((k << A) >> 5)] = v[k];
  }
  __syncthreads();
}

template <bool INV, int C, int NL, int TOP>
__device__ __forceinline__ void fft_rounds_fwd(const FftPass& p, uint32_t* sm, uint32_t fixed_hi, uint32_t llo) {
  if constexpr (TOP > C) {
    // The partial round (if NL is not a multiple of 4) goes first, at the top, so that the
    // lowest round is always a full 4-layer one.
    constexpr int RB = ((TOP - C - 1) % 4) + 1;
    fft_round_ct<INV, C, NL, TOP - RB, RB>(p, sm, fixed_hi, llo);
    fft_rounds_fwd<INV, C, NL, TOP - RB>(p, sm, fixed_hi, llo);
  }
}
template <bool INV, int C, int NL, int BOT>
__device__ __forceinline__ void fft_rounds_inv(const FftPass& p, uint32_t* sm, uint32_t fixed_hi, uint32_t llo) {
  if constexpr (BOT < C + NL) {
    constexpr int RB = (C + NL - BOT) < 4 ? (C + NL - BOT) : 4;
    fft_round_ct<INV, C, NL, BOT, RB>(p, sm, fixed_hi, llo);
    fft_rounds_inv<INV, C, NL, BOT + RB>(p, sm, fixed_hi, llo);
  }
}

// At least 5 resident blocks per SM: the 2^12-word tiles of 256 threads otherwise take 63-80
// registers and 4 blocks, and the kernel is bound by issue latency with too few warps (0.64
// instructions issued per cycle per scheduler). Capping at 48 registers (a 12-byte spill) gives
// 40 warps per SM and 6-7% shorter FFT passes on 1,296 columns of 2^16-2^18 words.
template <bool INV, int C, int NL>
__global__ void __launch_bounds__(1 << (C + NL - 4), 5) k_fft_tile(FftPass p, ConstColPtrs src, ColPtrs dst) {
  constexpr int T = C + NL;
  constexpr int THREADS = 1 << (T - 4);
  constexpr int PADW = THREADS + THREADS / 32;  // padded stride of consecutive thread rows
  __shared__ uint32_t sm[(1 << T) + (1 << T) / 32 + 1];
  pdl_enter();
  const uint32_t col = blockIdx.y;
  const uint32_t fixed = tile_fixed_bits(p, blockIdx.x);
  const uint32_t fixed_hi = fixed >> (p.lo + NL);
  const uint32_t llo = 1u << (p.L - p.lo);
  const uint32_t* s = p.read_src ? src.p[col] : dst.p[col];
  const uint32_t smask = p.read_src ? ((1u << p.F) - 1) : 0xffffffffu;
  uint32_t* d = dst.p[col];
  const uint32_t t = threadIdx.x;
  const uint32_t pt = t + (t >> 5);
  // Global index of element e = t + i * THREADS. When THREADS is a multiple of 2^C it is
  // g_t + i * gstep; otherwise it is computed per element.
  constexpr bool kStep = C <= T - 4;
  const uint32_t gt = (t & ((1u << C) - 1)) | ((t >> C) << p.lo) | fixed;
  const uint32_t gstep = kStep ? ((uint32_t)(THREADS >> C) << p.lo) : 0u;
  auto gidx = [&](int i) -> uint32_t {
    if constexpr (kStep) {
      return gt + i * gstep;
    } else {
      uint32_t e = t + i * THREADS;
      return (e & ((1u << C) - 1)) | ((e >> C) << p.lo) | fixed;
    }
  };
  // Padded shared-memory slot of element t + i * THREADS.
  auto sidx = [&](int i) -> uint32_t {
    if constexpr (THREADS >= 32) return pt + i * PADW;
    else return pad_idx(t + i * THREADS);
  };
#pragma unroll
  for (int i = 0; i < 16; i++) sm[sidx(i)] = __ldg(&s[gidx(i) & smask]);
  __syncthreads();
  if (!INV) fft_rounds_fwd<INV, C, NL, C + NL>(p, sm, fixed_hi, llo);
  else fft_rounds_inv<INV, C, NL, C>(p, sm, fixed_hi, llo);
#pragma unroll
  for (int i = 0; i < 16; i++) {
    uint32_t v = sm[sidx(i)];
    if (p.scale != 1u) v = m31_mul(v, p.scale);
    d[gidx(i)] = v;
  }
}

// Strided pass of RB <= 4 layers [lo, lo + RB) straight from HBM to registers: each thread owns
// the 2^RB words g0 + k * 2^lo (k < 2^RB) where g0 has zero layer bits; consecutive threads take
// consecutive low bits, so every load and store of a warp is one 128-byte line. No shared memory
// and no barrier. Requires lo >= 5.
template <bool INV, int RB>
__global__ void __launch_bounds__(256) k_fft_reg(FftPass p, ConstColPtrs src, ColPtrs dst) {
  pdl_enter();
  const uint32_t col = blockIdx.y;
  const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;  // < 2^(L - RB)
  // Insert RB zero bits at position lo.
  const uint32_t g0 = (gid & ((1u << p.lo) - 1)) | ((gid >> p.lo) << (p.lo + RB));
  const uint32_t* s = p.read_src ? src.p[col] : dst.p[col];
  const uint32_t smask = p.read_src ? ((1u << p.F) - 1) : 0xffffffffu;
  uint32_t* d = dst.p[col];
  uint32_t v[1 << RB];
#pragma unroll
  for (int k = 0; k < (1 << RB); k++) v[k] = __ldg(&s[(g0 + ((uint32_t)k << p.lo)) & smask]);
#pragma unroll
  for (int jj = 0; jj < RB; jj++) {
    const int j = INV ? jj : (RB - 1 - jj);
    const uint32_t layer = p.lo + j;
    const uint32_t* twp = p.tw + (p.tw_size - (1u << (p.L - layer))) + (g0 >> (layer + 1));
#pragma unroll
    for (int kh = 0; kh < (1 << (RB - 1 - j)); kh++) {
      const uint32_t t = __ldg(twp + kh);
      const int k0 = kh << (j + 1);
#pragma unroll
      for (int kl = 0; kl < (1 << j); kl++) {
        if (INV) ibfly2(v[k0 | kl], v[k0 | kl | (1 << j)], t);
        else bfly2(v[k0 | kl], v[k0 | kl | (1 << j)], t);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < (1 << RB); k++) {
    uint32_t x = v[k];
    if (p.scale != 1u) x = m31_mul(x, p.scale);
    d[g0 + ((uint32_t)k << p.lo)] = x;
  }
}

// Launches the specialised kernel when one exists for (c, nl); returns false otherwise.
template <bool INV>
static bool launch_tile(const FftPass& p, dim3 grid, cudaStream_t s, const ConstColPtrs& sp, const ColPtrs& dp) {
#define STWO_FFT_CASE(CC, NN)                                                          \
  if (p.c == CC && p.nl == NN) {                                                       \
    launch_pdl(k_fft_tile<INV, CC, NN>, grid, dim3(1 << (CC + NN - 4)), 0, s, p, sp, dp); \
    return true;                                                                       \
  }
  STWO_FFT_CASE(0, 4) STWO_FFT_CASE(0, 5) STWO_FFT_CASE(0, 6) STWO_FFT_CASE(0, 7) STWO_FFT_CASE(0, 8)
  STWO_FFT_CASE(0, 9) STWO_FFT_CASE(0, 10) STWO_FFT_CASE(0, 11) STWO_FFT_CASE(0, 12)
  STWO_FFT_CASE(11, 1) STWO_FFT_CASE(10, 2) STWO_FFT_CASE(9, 3) STWO_FFT_CASE(8, 4) STWO_FFT_CASE(7, 5)
  STWO_FFT_CASE(6, 6) STWO_FFT_CASE(5, 7) STWO_FFT_CASE(4, 8)
#undef STWO_FFT_CASE
  return false;
}

struct PassPlan {
  uint32_t lo, nl, c;
};

// A contiguous pass over [0, min(F, 12)); strided passes above it with tiles of <= 2^13 words
// whose rows keep >= 8 contiguous words (32 bytes).
static std::vector<PassPlan> plan_passes(uint32_t F) {
  std::vector<PassPlan> v;
  if (F == 0) return v;
  uint32_t low = F < FFT_TMAX ? F : FFT_TMAX;
  v.push_back({0, low, 0});
  uint32_t lo = low;
  while (lo < F) {
    uint32_t rem = F - lo;
    uint32_t max_nl = FFT_TMAX - 4;  // rows of >= 16 contiguous words (64 bytes)
    uint32_t n_passes = (rem + max_nl - 1) / max_nl;
    uint32_t nl = (rem + n_passes - 1) / n_passes;
    uint32_t c = FFT_TMAX - nl;
    if (c > lo) c = lo;
    v.push_back({lo, nl, c});
    lo += nl;
  }
  return v;
}

// Runs the layers [0, F) of a 2^L-point circle FFT (F == L for interpolation): the passes
// [pass_begin, pass_end) of its plan, in execution order (all of them by default).
static int32_t run_fft(const TwiddleTree* tree, stwo_coset half, bool inverse, const uint32_t* const* src,
                       uint32_t F, uint32_t* const* dst, uint32_t n_cols, cudaStream_t s, size_t pass_begin = 0,
                       size_t pass_end = SIZE_MAX) {
  const uint32_t L = half.log_size + 1;
  STWO_REQUIRE(tree, "null twiddle tree");
  STWO_REQUIRE(L <= 30, "domain log size %u > 30", L);
  STWO_REQUIRE(F <= L, "Can only evaluate on larger domains");
  if (!coset_is_doubling_of(half, tree->root)) {
    // Domains below 2^5 take their own twiddles, as the reference SIMD backend's CPU path for
    // them does (backend/simd/circle.rs:137-140, 247-255); larger ones must match the tree.
    STWO_REQUIRE(L < 5, "domain half coset is not a doubling of the twiddle root");
    TwiddleTree* own = nullptr;
    int32_t st = get_tree(half, s, &own);
    if (st) return st;
    tree = own;
  }
  if (n_cols == 0) return STWO_OK;

  FftPass base{};
  base.L = L;
  base.F = F;
  base.tw = inverse ? tree->d_itw2 : tree->d_tw2;
  base.tw_size = (uint32_t)tree->size;
  base.scale = 1u;
  base.small_y = 0;
  if (L <= 2) {
    uint32_t y = h_index_to_point(half.initial_index).y;
    base.small_y = 2u * (inverse ? h_inv(y) : y);  // doubled, as every twiddle here
  }

  std::vector<PassPlan> plan = plan_passes(F);
  if (!inverse) std::reverse(plan.begin(), plan.end());
  if (F == 0) {
    // A single coefficient: the constant polynomial, evaluated everywhere to that value.
    STWO_REQUIRE(!inverse, "empty interpolation");
    plan.push_back({0, 0, 0});
  }

  for (uint32_t c0 = 0; c0 < n_cols; c0 += MAX_PARAM_COLS) {
    uint32_t nc = std::min<uint32_t>(MAX_PARAM_COLS, n_cols - c0);
    ConstColPtrs sp;
    ColPtrs dp;
    for (uint32_t i = 0; i < nc; i++) {
      sp.p[i] = src ? src[c0 + i] : dst[c0 + i];
      dp.p[i] = dst[c0 + i];
    }
    for (size_t pi = pass_begin; pi < std::min(pass_end, plan.size()); pi++) {
      FftPass p = base;
      p.lo = plan[pi].lo;
      p.nl = plan[pi].nl;
      p.c = plan[pi].c;
      p.T = p.c + p.nl;
      p.read_src = (pi == 0 && src) ? 1u : 0u;
      if (inverse && pi + 1 == plan.size()) p.scale = h_inv((uint32_t)((1ull << L) % P));
      uint32_t tiles_log = L - p.T;
      STWO_REQUIRE(tiles_log < 31, "too many tiles");
      dim3 grid(1u << tiles_log, nc);
      uint32_t groups = (1u << p.T) >> std::min(FFT_R, p.T);
      uint32_t threads = std::max<uint32_t>(32, groups);
      size_t smem = ((size_t)(1u << p.T) + ((1u << p.T) >> 5) + 1) * 4;
      bool done = false;
      if (p.lo >= 5 && p.nl >= 1 && p.nl <= 4 && L - p.nl >= 8) {
        // Register-only strided pass.
        dim3 g2(1u << (L - p.nl - 8), nc);
#define STWO_REG_CASE(RB)                                                       \
  if (p.nl == RB) {                                                             \
    if (inverse) launch_pdl(k_fft_reg<true, RB>, g2, dim3(256), 0, s, p, sp, dp);  \
    else launch_pdl(k_fft_reg<false, RB>, g2, dim3(256), 0, s, p, sp, dp);         \
  }
        STWO_REG_CASE(1) STWO_REG_CASE(2) STWO_REG_CASE(3) STWO_REG_CASE(4)
#undef STWO_REG_CASE
        done = true;
      }
      if (!done && L >= 3 && p.T >= 4) done = inverse ? launch_tile<true>(p, grid, s, sp, dp) : launch_tile<false>(p, grid, s, sp, dp);
      if (done) {
      } else if (threads <= 256) {
        if (inverse) launch_pdl(k_fft_pass<true, 256>, grid, dim3(threads), smem, s, p, sp, dp);
        else launch_pdl(k_fft_pass<false, 256>, grid, dim3(threads), smem, s, p, sp, dp);
      } else {
        if (inverse) launch_pdl(k_fft_pass<true, 512>, grid, dim3(threads), smem, s, p, sp, dp);
        else launch_pdl(k_fft_pass<false, 512>, grid, dim3(threads), smem, s, p, sp, dp);
      }
      note_launch();
      STWO_LAUNCH_CHECK();
    }
  }
  return STWO_OK;
}

int32_t fft_interpolate(const TwiddleTree* tree, stwo_coset half, uint32_t* const* cols, uint32_t n, cudaStream_t s) {
  return run_fft(tree, half, true, nullptr, half.log_size + 1, cols, n, s);
}
int32_t fft_evaluate(const TwiddleTree* tree, stwo_coset half, const uint32_t* const* coeffs, uint32_t coeff_log,
                     uint32_t* const* out, uint32_t n, cudaStream_t s) {
  return run_fft(tree, half, false, coeffs, coeff_log, out, n, s);
}

// The last interpolation pass and the first evaluation pass in one kernel, for 2^13..2^16-point
// columns, where both are register passes over the same layers [12, F): a thread loads the 2^RB
// evaluations g0 + k 2^12, applies the inverse layers and the 1/2^F scale, stores the 2^RB
// coefficients in place, then for each sub-domain of the evaluation domain applies the forward
// layers to them and stores that sub-domain's 2^RB words. The coefficients are read from HBM once
// instead of twice (written by the interpolation, read back by the evaluation).
template <int RB>
__global__ void __launch_bounds__(256) k_fft_reg_ie(FftPass pi, FftPass pe, ColPtrs cols, ColPtrs out) {
  pdl_enter();
  const uint32_t col = blockIdx.y;
  const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;  // < 2^(F - RB)
  const uint32_t lo = pi.lo;
  const uint32_t g0 = (gid & ((1u << lo) - 1)) | ((gid >> lo) << (lo + RB));
  uint32_t* c = cols.p[col];
  uint32_t v[1 << RB];
#pragma unroll
  for (int k = 0; k < (1 << RB); k++) v[k] = c[g0 + ((uint32_t)k << lo)];
#pragma unroll
  for (int j = 0; j < RB; j++) {
    const uint32_t layer = lo + j;
    const uint32_t* twp = pi.tw + (pi.tw_size - (1u << (pi.L - layer))) + (g0 >> (layer + 1));
#pragma unroll
    for (int kh = 0; kh < (1 << (RB - 1 - j)); kh++) {
      const uint32_t t = __ldg(twp + kh);
      const int k0 = kh << (j + 1);
#pragma unroll
      for (int kl = 0; kl < (1 << j); kl++) ibfly2(v[k0 | kl], v[k0 | kl | (1 << j)], t);
    }
  }
#pragma unroll
  for (int k = 0; k < (1 << RB); k++) {
    v[k] = m31_mul(v[k], pi.scale);
    c[g0 + ((uint32_t)k << lo)] = v[k];
  }
  uint32_t* o = out.p[col];
  for (uint32_t sub = 0; sub < (1u << (pe.L - pe.F)); sub++) {
    const uint32_t gs = g0 | (sub << pe.F);
    uint32_t w[1 << RB];
#pragma unroll
    for (int k = 0; k < (1 << RB); k++) w[k] = v[k];
#pragma unroll
    for (int jj = 0; jj < RB; jj++) {
      const int j = RB - 1 - jj;
      const uint32_t layer = lo + j;
      const uint32_t* twp = pe.tw + (pe.tw_size - (1u << (pe.L - layer))) + (gs >> (layer + 1));
#pragma unroll
      for (int kh = 0; kh < (1 << (RB - 1 - j)); kh++) {
        const uint32_t t = __ldg(twp + kh);
        const int k0 = kh << (j + 1);
#pragma unroll
        for (int kl = 0; kl < (1 << j); kl++) bfly2(w[k0 | kl], w[k0 | kl | (1 << j)], t);
      }
    }
#pragma unroll
    for (int k = 0; k < (1 << RB); k++) o[gs + ((uint32_t)k << lo)] = w[k];
  }
}

// Interpolates n columns of 2^F evaluations on the domain of `src_half` in place (coefficients
// left in `cols`) and evaluates them on the larger domain of `dst_half` into `out`: the same words
// as fft_interpolate followed by fft_evaluate. For F in [13, 16] the pass both transforms share
// runs fused (k_fft_reg_ie). In two steps, so that a caller can time them apart: the first runs
// the interpolation (up to and including the fused pass, where there is one; `*fused` says which),
// the second the rest of the evaluation.
int32_t fft_interpolate_extend_begin(const TwiddleTree* tree_src, stwo_coset src_half, uint32_t* const* cols,
                                     uint32_t n, const TwiddleTree* tree_dst, stwo_coset dst_half,
                                     uint32_t* const* out, cudaStream_t s, bool* fused) {
  const uint32_t F = src_half.log_size + 1, L = dst_half.log_size + 1;
  STWO_REQUIRE(tree_src && tree_dst && fused, "null argument");
  STWO_REQUIRE(L >= F && L <= 30, "evaluation domain 2^%u smaller than 2^%u", L, F);
  *fused = n > 0 && F >= 13 && F <= 16 && coset_is_doubling_of(src_half, tree_src->root) &&
           coset_is_doubling_of(dst_half, tree_dst->root);
  if (!*fused) return run_fft(tree_src, src_half, true, nullptr, F, cols, n, s);
  // Interpolation plan: [0, 12) then [12, F); evaluation plan: [12, F) then [0, 12).
  int32_t st = run_fft(tree_src, src_half, true, nullptr, F, cols, n, s, 0, 1);
  if (st) return st;
  const uint32_t RB = F - 12;
  FftPass pi{}, pe{};
  pi.L = F;
  pi.F = F;
  pi.lo = 12;
  pi.nl = RB;
  pi.tw = tree_src->d_itw2;
  pi.tw_size = (uint32_t)tree_src->size;
  pi.scale = h_inv((uint32_t)((1ull << F) % P));
  pe.L = L;
  pe.F = F;
  pe.lo = 12;
  pe.nl = RB;
  pe.tw = tree_dst->d_tw2;
  pe.tw_size = (uint32_t)tree_dst->size;
  pe.scale = 1u;
  for (uint32_t c0 = 0; c0 < n; c0 += MAX_PARAM_COLS) {
    const uint32_t nc = std::min<uint32_t>(MAX_PARAM_COLS, n - c0);
    ColPtrs cp, op;
    for (uint32_t i = 0; i < nc; i++) {
      cp.p[i] = cols[c0 + i];
      op.p[i] = out[c0 + i];
    }
    const dim3 grid(1u << (F - RB - 8), nc);  // one thread per 2^RB-word group: 2^12 per column
    switch (RB) {
      case 1: launch_pdl(k_fft_reg_ie<1>, grid, dim3(256), 0, s, pi, pe, cp, op); break;
      case 2: launch_pdl(k_fft_reg_ie<2>, grid, dim3(256), 0, s, pi, pe, cp, op); break;
      case 3: launch_pdl(k_fft_reg_ie<3>, grid, dim3(256), 0, s, pi, pe, cp, op); break;
      default: launch_pdl(k_fft_reg_ie<4>, grid, dim3(256), 0, s, pi, pe, cp, op); break;
    }
    note_launch();
    STWO_LAUNCH_CHECK();
  }
  return STWO_OK;
}
int32_t fft_interpolate_extend_end(const TwiddleTree* tree_dst, stwo_coset dst_half, uint32_t coeff_log,
                                   uint32_t* const* cols, uint32_t n, uint32_t* const* out, bool fused,
                                   cudaStream_t s) {
  if (fused) return run_fft(tree_dst, dst_half, false, nullptr, coeff_log, out, n, s, 1);
  std::vector<const uint32_t*> co(cols, cols + n);
  return run_fft(tree_dst, dst_half, false, co.data(), coeff_log, out, n, s);
}
int32_t fft_interpolate_evaluate(const TwiddleTree* tree_src, stwo_coset src_half, uint32_t* const* cols, uint32_t n,
                                 const TwiddleTree* tree_dst, stwo_coset dst_half, uint32_t* const* out,
                                 cudaStream_t s) {
  bool fused = false;
  int32_t st = fft_interpolate_extend_begin(tree_src, src_half, cols, n, tree_dst, dst_half, out, s, &fused);
  if (st) return st;
  return fft_interpolate_extend_end(tree_dst, dst_half, src_half.log_size + 1, cols, n, out, fused, s);
}

// Register-only throughput of the butterfly above: each thread keeps 16 words and 15 doubled
// twiddles in registers and runs `rounds` rounds of 4 forward layers (the shape of one register
// round of k_fft_tile), with no memory traffic in the loop. Its rate is the integer-datapath
// bound of the circle FFT on this device. Compiled for 4 to 6 resident blocks per SM (the register
// budget decides how many warps hide the butterflies' dependency chains); the best is reported.
// Thread 0 of each block records its SM and the cycle counter and global timer around the loop
// (between two barriers).
template <int MINB>
__global__ void __launch_bounds__(256, MINB)
    k_butterfly_probe(const uint32_t* in, uint32_t* out, unsigned long long* span, uint32_t rounds) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x, n = gridDim.x * blockDim.x;
  uint32_t v[16], t[15];
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = in[g + i * n];
#pragma unroll
  for (int i = 0; i < 15; i++) t[i] = 2u * (in[(g * 15 + i) % (16 * n)] % (P - 1));
  __syncthreads();
  const unsigned long long g0 = global_ns();
  const long long c0 = clock64();
  for (uint32_t it = 0; it < rounds; it++) {
    int ti = 0;
#pragma unroll
    for (int j = 3; j >= 0; j--)
#pragma unroll
      for (int kh = 0; kh < (1 << (3 - j)); kh++) {
        const uint32_t tt = t[ti++];
#pragma unroll
        for (int kl = 0; kl < (1 << j); kl++) bfly2(v[(kh << (j + 1)) | kl], v[(kh << (j + 1)) | kl | (1 << j)], tt);
      }
  }
#pragma unroll
  for (int i = 0; i < 16; i++) out[g + i * n] = v[i];
  __syncthreads();
  if (threadIdx.x == 0) probe_record(span, c0, g0);
}

}  // namespace stwo

using namespace stwo;

extern "C" {

stwo_status stwo_butterfly_rate(uint32_t rounds, double* h_butterflies_per_s, double* h_cycles_per_warp_butterfly,
                                double* h_probe_sm_mhz, void* stream) {
  STWO_REQUIRE(h_butterflies_per_s && rounds >= 1 && rounds <= (1u << 16), "need 1 <= rounds <= 65536");
  double best = 0.0, best_cycles = 0.0, best_mhz = 0.0;
  for (int variant = 0; variant < 3; variant++) {
    RateProbeKernel kern =
        variant == 0 ? k_butterfly_probe<4> : variant == 1 ? k_butterfly_probe<5> : k_butterfly_probe<6>;
    RateProbe r;
    int32_t st = run_rate_probe(kern, 16, rounds, as_stream(stream), &r);
    if (st) return st;
    best = std::max(best, (double)r.blocks * 256.0 * rounds * 32.0 / (r.ms * 1e-3));
    // The SM's four schedulers shared its warps of rounds * 32 butterflies each.
    const double c = 4.0 * r.sm_cycles / (r.warps_per_sm * rounds * 32.0);
    if (best_cycles == 0.0 || c < best_cycles) {
      best_cycles = c;
      best_mhz = r.sm_mhz;
    }
  }
  *h_butterflies_per_s = best;
  if (h_cycles_per_warp_butterfly) *h_cycles_per_warp_butterfly = best_cycles;
  if (h_probe_sm_mhz) *h_probe_sm_mhz = best_mhz;
  return STWO_OK;
}

stwo_status stwo_interpolate_columns(stwo_twiddle_tree tree, stwo_coset domain_half_coset, uint32_t* const* d_cols,
                                     uint32_t n_cols, void* stream) {
  STWO_REQUIRE(n_cols == 0 || d_cols, "null column table");
  return fft_interpolate(tree_of(tree), domain_half_coset, d_cols, n_cols, as_stream(stream));
}

stwo_status stwo_evaluate_columns(stwo_twiddle_tree tree, stwo_coset domain_half_coset,
                                  const uint32_t* const* d_coeffs, uint32_t coeff_log_size, uint32_t* const* d_out,
                                  uint32_t n_cols, void* stream) {
  STWO_REQUIRE(n_cols == 0 || (d_coeffs && d_out), "null column table");
  return fft_evaluate(tree_of(tree), domain_half_coset, d_coeffs, coeff_log_size, d_out, n_cols, as_stream(stream));
}

}  // extern "C"
