// Split-BF16 tensor-core GEMM machinery shared by VdaggerV and the diluted
// traces (tcgen05, sm_103a).
//
// A complex product sum_k x_k y_k (or sum_k conj(x_k) y_k) with FP64 inputs is
// computed to FP64 accuracy from BF16 tensor-core products:
//
// * Complex -> real.  With K' = 2K interleaved (re, im), rows
//   A'(2i) = (Re v_i, Im v_i), A'(2i+1) = (-Im v_i, Re v_i) and
//   B(j) = (Re w_j, Im w_j), one real GEMM D = A' B^T gives
//   D(2i, j) = Re(v_i^H w_j) and D(2i+1, j) = Im(v_i^H w_j).  Feeding
//   v = conj(x) gives the unconjugated sum_k x_k w_k.
// * Exact split.  Every row (column) is scaled by 2^-e (e: exponent of its
//   largest |entry|) and cut into 6 signed slices of at most 8 bits:
//   x = sum_p a_p 2^(-7-8(p-1)), a_p integer in [-128, 128], exact in BF16
//   (balanced base-256 digits of the 55-bit fixed-point value, digits6).
//   47 bits are kept.
// * FP32 accumulation.  Slice products a_p b_q (|.| <= 2^14) of the same
//   scale level l = p + q are accumulated in one TMEM accumulator.  Over a chunk
//   of 512 K' values the levels 2 and 3 (one and two slice pairs) stay within
//   2^24 and are exact; the lower levels (scale <= 2^-16) can round only by
//   2^-24 of their own magnitude, at most 2^-40 of the row scale.  21 pairs
//   (p + q <= 7), 6 accumulators.
// * Promotion.  After every chunk the 6 accumulators are read from TMEM and
//   added, scaled by 2^-8l, into a double-float (two FP32) accumulator in
//   registers; FP64 units are not used in the loop.  The result of a tile
//   entry is (hi + lo) 2^(e_row + e_col - 14).
//
// Slices live in global memory already in the tcgen05 K-major core-matrix
// layout, one contiguous block of kStageA (kStageB) bytes per (tile, k-tile),
// and are moved to shared memory by bulk asynchronous copies (cp.async.bulk)
// completing on mbarriers.  Warp roles (ozaki_tiles): one warp issues the
// copies, one issues tcgen05.mma, eight promote and hand the result to the
// epilogue; CTAs are persistent over the tiles of a launch.
// Every mbarrier wait is bounded; on timeout the kernel records an error code
// in *err and winds down, and TMEM is always released.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace slaph {
namespace dev {
namespace tc {

constexpr int kSlices = 6;
constexpr int kTM = 128;       // rows of A' per tile (64 complex rows x re/im)
constexpr int kTN = 80;        // columns of B per tile
constexpr int kTK = 32;        // K' per k-tile (bf16 elements)
constexpr int kChunkKT = 16;   // k-tiles per chunk (512 K') between promotions
constexpr int kStages = 2;     // (a 5-stage pipeline of 16-wide k-tiles measured slower)
constexpr uint32_t kABlk = kTM * kTK * 2;            // 8192 B
constexpr uint32_t kBBlk = kTN * kTK * 2;            // 5120 B
constexpr uint32_t kStageA = kSlices * kABlk;        // 49152 B
constexpr uint32_t kStageB = kSlices * kBBlk;        // 30720 B
constexpr uint32_t kStageBytes = kStageA + kStageB;  // 79872 B
constexpr uint32_t kSmemBytes = kStages * kStageBytes;
constexpr uint32_t kTmemCols = 512;
constexpr int kLevels = 6;  // p + q = 2..7
constexpr long long kWaitCycles = 4000000000LL;  // ~2 s at 2 GHz

// byte offset of element (r, k) in a K-major, no-swizzle core-matrix tile with
// 32 bf16 per row: core matrices of 8 rows x 16 B, adjacent along K at 128 B,
// 8-row groups at 512 B.
__host__ __device__ __forceinline__ uint32_t core_off(int r, int k) {
  return ((r >> 3) * 4 + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

__device__ __forceinline__ uint32_t smem_u32(void const *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: false (and *err = code) when the phase did not complete
// within `limit` clock cycles.
__device__ __forceinline__ bool mbar_wait_for(uint64_t *bar, uint32_t parity, int *err, int code,
                                              long long limit) {
  long long const t0 = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (clock64() - t0 > limit) {
      atomicCAS(err, 0, code);
      return false;
    }
  }
  return true;
}
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, int *err, int code) {
  return mbar_wait_for(bar, parity, err, code, kWaitCycles);
}
__device__ __forceinline__ void bulk_g2s(void *dst, void const *src, uint32_t bytes,
                                         uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Shared-memory matrix descriptor, K-major, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((addr >> 4) & 0x3FFFu);
  d |= static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16;
  d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32;
  d |= static_cast<uint64_t>(1) << 46;  // descriptor version (tcgen05)
  return d;                             // base offset 0, no swizzle
}
// Instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, M = kTM, N = n (a multiple of 16 up to 256).
__host__ __device__ constexpr uint32_t idesc_n(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(n >> 3) << 17) |
         (static_cast<uint32_t>(kTM >> 4) << 24);
}
// Level blocks (kTN columns each) one MMA covers: the accumulators of levels
// l .. l + kLevelGroup - 1 sit side by side in TMEM, and the B slices
// q .. q + kLevelGroup - 1 side by side in shared memory with a uniform
// 8-row-group stride, so A_p against [B_q; ...] is one MMA of N = 3 kTN into
// the accumulators p + q onwards.
constexpr int kLevelGroup = 256 / kTN;
static_assert(kLevelGroup >= 1 && (kLevelGroup * kTN) % 16 == 0, "MMA N");

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b,
                                         uint32_t accumulate, uint32_t idesc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}
// Error-free x + y into (s, e) (Knuth's two-sum).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  float const bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// ---------------------------------------------------------------- slicing
// 64-bit fixed point of v relative to 2^e: F = round(v 2^(55-e)), |F| <= 2^55.
__device__ __forceinline__ long long fixed55(double v, int e) {
  long long const bits = __double_as_longlong(v);
  int const ex = static_cast<int>((bits >> 52) & 0x7FF);
  if (ex == 0) return 0;  // zero or subnormal: below 2^-1022, negligible here
  long long m = (bits & 0xFFFFFFFFFFFFFLL) | (1LL << 52);
  // v = m 2^(ex - 1075); F = m 2^(ex - 1075 + 55 - e)
  int const sh = ex - 1075 + 55 - e;
  long long F;
  if (sh >= 0) {
    F = sh < 11 ? (m << sh) : (1LL << 62);  // sh >= 11 cannot occur for |v| <= 2^e
  } else if (sh > -63) {
    F = (m + (1LL << (-sh - 1))) >> (-sh);
  } else {
    F = 0;
  }
  return bits < 0 ? -F : F;
}

// The 6 balanced base-256 digits of a 64-bit fixed-point value F (|F| <= 2^55)
// at 2^48, 2^40, ..., 2^8, as floats: F = sum_p d_p 2^(48-8p) + r with
// |r| <= 2^7, d_0 in [-128, 128] and d_1..d_5 in [-128, 127] (all exact in
// BF16).  With G = F + C, C = 0x808080808080 (2^7 in every byte below the
// top), the lower digits are the bytes 5..1 of G minus 128 and the top digit is
// G >> 48: the sum of the digits is G - C + 2^7 - (G mod 2^8).  Each lower
// digit is one byte permutation into the mantissa of 2^23 and one FP32
// subtraction.
__device__ __forceinline__ void digits6(long long F, float (&d)[kSlices]) {
  long long const G = F + 0x808080808080LL;
  uint32_t const lo = static_cast<uint32_t>(G);
  uint32_t const hi = static_cast<uint32_t>(static_cast<unsigned long long>(G) >> 32);
  float const bias = 8388736.0f;  // 2^23 + 128
  d[0] = static_cast<float>(static_cast<int>(G >> 48));
  d[1] = __int_as_float(__byte_perm(hi, 0x4B000000u, 0x7441)) - bias;
  d[2] = __int_as_float(__byte_perm(hi, 0x4B000000u, 0x7440)) - bias;
  d[3] = __int_as_float(__byte_perm(lo, 0x4B000000u, 0x7443)) - bias;
  d[4] = __int_as_float(__byte_perm(lo, 0x4B000000u, 0x7442)) - bias;
  d[5] = __int_as_float(__byte_perm(lo, 0x4B000000u, 0x7441)) - bias;
}

// Two small integers held exactly in floats to a BF16 pair (a in the low half).
__device__ __forceinline__ uint32_t bf16x2(float a, float b) {
  uint32_t r;
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(b), "f"(a));
  return r;
}

// The same for a float, with integer operations only: round(v 2^(55-e)) for
// |v| < 2^e (then the shift below is at most 31 and |F| < 2^55).
__device__ __forceinline__ long long fixed55f(float v, int e) {
  int const bits = __float_as_int(v);
  int const ex = (bits >> 23) & 0xFF;
  if (ex == 0) return 0;  // zero or subnormal: below 2^-126 2^e, negligible here
  long long const m = (bits & 0x7FFFFF) | 0x800000;  // v = m 2^(ex - 150)
  int const sh = ex - 150 + 55 - e;
  long long F;
  if (sh >= 0) {
    F = m << (sh < 31 ? sh : 31);
  } else if (sh > -40) {
    F = (m + (1LL << (-sh - 1))) >> (-sh);
  } else {
    F = 0;
  }
  return bits < 0 ? -F : F;
}

// Exponent e with max |x| < 2^e, from the largest |x| given as the bit
// pattern of a float (0 for a zero maximum).
__device__ __forceinline__ int expo_of_absbits(unsigned int b) {
  if (b == 0) return 0;
  int const ex = static_cast<int>(b >> 23);
  return ex == 0 ? -125 : ex - 126;
}
// The same for a double bit pattern.
__device__ __forceinline__ int expo_of_absbits64(unsigned long long b) {
  if (b == 0) return 0;
  int const ex = static_cast<int>(b >> 52);
  return ex == 0 ? -1021 : ex - 1022;
}

// Writes the slices of complex element x = (fr, fi) 2^(e-55) (K index m,
// K' = 2m, 2m+1) of A row `row` of a tile stream laid out
// [m_tile][k_tile][slice][kTM x kTK]: row 2r gets (Re x, Im x), row 2r+1 gets
// (-Im x, Re x) (the negated digits of Im x).
__device__ __forceinline__ void put_a_fx(uint8_t *region, int64_t k_tiles, int row, int64_t m,
                                         long long fr, long long fi) {
  float dre[kSlices], dim[kSlices];
  digits6(fr, dre);
  digits6(fi, dim);
  int const mt = row / (kTM / 2), r0 = 2 * (row % (kTM / 2));
  int64_t const kt = m / (kTK / 2);
  int const k = 2 * static_cast<int>(m % (kTK / 2));
  uint8_t *blk = region + (static_cast<int64_t>(mt) * k_tiles + kt) * kStageA;
#pragma unroll
  for (int p = 0; p < kSlices; ++p) {
    uint8_t *b = blk + p * kABlk;
    *reinterpret_cast<uint32_t *>(b + core_off(r0, k)) = bf16x2(dre[p], dim[p]);
    *reinterpret_cast<uint32_t *>(b + core_off(r0 + 1, k)) = bf16x2(-dim[p], dre[p]);
  }
}

// The same for B column `col` of a stream laid out [n_tile][k_tile][slice][kTN x kTK]:
// (Re y, Im y).
__device__ __forceinline__ void put_b_fx(uint8_t *region, int64_t k_tiles, int col, int64_t m,
                                         long long fr, long long fi) {
  float dre[kSlices], dim[kSlices];
  digits6(fr, dre);
  digits6(fi, dim);
  int const nt = col / kTN, r = col % kTN;
  int64_t const kt = m / (kTK / 2);
  int const k = 2 * static_cast<int>(m % (kTK / 2));
  uint8_t *blk = region + (static_cast<int64_t>(nt) * k_tiles + kt) * kStageB;
#pragma unroll
  for (int p = 0; p < kSlices; ++p)
    *reinterpret_cast<uint32_t *>(blk + p * kBBlk + core_off(r, k)) = bf16x2(dre[p], dim[p]);
}

__device__ __forceinline__ void put_a(uint8_t *region, int64_t k_tiles, int row, int64_t m,
                                      double2 x, int e) {
  put_a_fx(region, k_tiles, row, m, fixed55(x.x, e), fixed55(x.y, e));
}
__device__ __forceinline__ void put_b(uint8_t *region, int64_t k_tiles, int col, int64_t m,
                                      double2 y, int e) {
  put_b_fx(region, k_tiles, col, m, fixed55(y.x, e), fixed55(y.y, e));
}

// Exponent e with max |x| < 2^e for a positive maximum (0 for m == 0).
__device__ __forceinline__ int expo_of_max(double m) {
  int e = 0;
  if (m > 0) frexp(m * (1.0 + 1e-15), &e);
  return e;
}

// The tiles of one launch, each a 128 x 80 output tile of D = A' B^T over
// k_tiles k-tiles, computed by a persistent CTA: CTA b takes tiles b, b + G,
// b + 2G, ... (G = gridDim.x, at most one CTA per SM).  The operands:
// src.context(i, lane) fetches what the copies of tile i need (called one tile
// ahead by the producer warp), src.load(ctx, kt, dst, bar, lane), called by all
// lanes of the producer warp, issues the copies of k-tile kt into the stage at
// dst and announces their bytes on bar (load_contiguous for operands whose
// kStageA / kStageB blocks are consecutive per k-tile).  The results:
// epi.prepare(i, row, col0) fetches the epilogue's data of tile i before its
// first chunk is promoted, epi(pre, i, row, col0, hi, lo) writes them.  Must be
// called by all kThreads threads with kSmemBytes of dynamic shared memory.
//
// Roles: warp kProducerWarp issues the bulk copies, running ahead across tile
// boundaries; warp kMmaWarp issues tcgen05.mma; promotion warps 0..7 read the
// level accumulators after every chunk.  A promotion warp w owns TMEM lane
// quadrant w % 4 (rows 32 (w % 4) + lane) and the kColsW columns from
// kColsW (w / 4) on.  Once the last chunk of a tile is promoted the
// accumulators are released, so the MMAs of the next tile run while the
// promotion warps hand the previous tile to the epilogue, with the
// double-float (hi, lo) of the row's kColsW columns; the result is
// (hi + lo) 2^(e_row + e_col - 14).
//
// Chunk value of one column, sum_l E_l 2^-8l: levels 0 and 1 are exact
// integers in FP32; levels 3..5 (at most 2^-24 of the row scale) are summed in
// FP32 first, rounding by at most 2^-24 of their own magnitude, then levels 1,
// 2 and that sum enter through error-free two-sums.
constexpr int kPromoWarps = 8;
constexpr int kProducerWarp = kPromoWarps, kMmaWarp = kPromoWarps + 1;
constexpr int kThreads = 32 * (kPromoWarps + 2);
constexpr int kColsW = kTN / (kPromoWarps / 4);  // 40
static_assert(kColsW % 8 == 0, "promotion loads 8 columns at a time");

__device__ __forceinline__ void tmem_ld8_issue(uint32_t taddr, uint32_t (&r)[8]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7])
      : "r"(taddr));
}
// Waits for the TMEM loads of this thread; the loaded registers pass through
// the wait (and through empty asm statements after it), so that no use of
// them can be scheduled before the data has arrived.
template <int N>
__device__ __forceinline__ void tmem_ld_wait(uint32_t (&r)[N][8]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(r[0][0]), "+r"(r[0][1]), "+r"(r[0][2]), "+r"(r[0][3]), "+r"(r[0][4]),
                 "+r"(r[0][5]), "+r"(r[0][6]), "+r"(r[0][7])
               :
               : "memory");
#pragma unroll
  for (int l = 1; l < N; ++l)
    asm volatile(""
                 : "+r"(r[l][0]), "+r"(r[l][1]), "+r"(r[l][2]), "+r"(r[l][3]), "+r"(r[l][4]),
                   "+r"(r[l][5]), "+r"(r[l][6]), "+r"(r[l][7]));
}

// Stage loader for tiles whose A and B k-tile blocks are contiguous: lane 0
// copies block kt of a (kStageA bytes) and of b (kStageB bytes).
__device__ __forceinline__ void load_contiguous(uint8_t const *a, uint8_t const *b, int kt,
                                                uint8_t *dst, uint64_t *bar, int lane) {
  if (lane != 0) return;
  mbar_expect_tx(bar, kStageBytes);
  bulk_g2s(dst, a + static_cast<int64_t>(kt) * kStageA, kStageA, bar);
  bulk_g2s(dst + kStageA, b + static_cast<int64_t>(kt) * kStageB, kStageB, bar);
}

template <typename Src, typename Epilogue>
__device__ __forceinline__ void ozaki_tiles(uint8_t *smem, int n_tiles, int k_tiles,
                                            Src const &src, int *err, Epilogue const &epi) {
  __shared__ __align__(8) uint64_t full_bar[kStages], empty_bar[kStages];
  __shared__ __align__(8) uint64_t acc_full, acc_empty, done_bar;
  __shared__ uint32_t tmem_slot;

  int const warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  int const n_chunks = (k_tiles + kChunkKT - 1) / kChunkKT;
  int const first_tile = blockIdx.x, tile_step = gridDim.x;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    mbar_init(&acc_full, 1);
    mbar_init(&acc_empty, kPromoWarps * 32);
    mbar_init(&done_bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  uint32_t const tmem = tmem_slot;

  if (warp == kProducerWarp) {
    int64_t g = 0;  // k-tiles issued over all tiles of this CTA
    bool ok = true;
    // per-tile operand addresses, fetched one tile ahead
    auto cur = src.context(first_tile < n_tiles ? first_tile : 0, lane);
    for (int i = first_tile; i < n_tiles && ok; i += tile_step) {
      auto const nxt = src.context(i + tile_step < n_tiles ? i + tile_step : i, lane);
      for (int kt = 0; kt < k_tiles; ++kt, ++g) {
        int const s = static_cast<int>(g % kStages);
        uint32_t const use = static_cast<uint32_t>(g / kStages);
        bool free_ok = true;
        if (lane == 0 && g >= kStages) free_ok = mbar_wait(&empty_bar[s], (use - 1) & 1, err, 1);
        if (!__shfl_sync(0xffffffffu, free_ok, 0)) {
          ok = false;
          break;
        }
        src.load(cur, kt, smem + s * kStageBytes, &full_bar[s], lane);
      }
      cur = nxt;
    }
    // The copies of the last stages have landed before shared memory is
    // released (immediate when the MMA warp consumed them).
    if (lane == 0)
      for (int64_t q = g > kStages ? g - kStages : 0; q < g; ++q)
        mbar_wait(&full_bar[q % kStages], static_cast<uint32_t>(q / kStages) & 1, err, 6);
  } else if (warp == kMmaWarp) {
    if (lane == 0) {  // MMA issuer
      bool ok = true;
      int64_t g = 0, c_all = 0;  // k-tiles and chunks consumed over all tiles
      for (int i = first_tile; i < n_tiles && ok; i += tile_step) {
        for (int c = 0; c < n_chunks && ok; ++c, ++c_all) {
          // accumulators free: the previous chunk (of this or the last tile) promoted
          if (c_all > 0 &&
              !mbar_wait(&acc_empty, static_cast<uint32_t>(c_all - 1) & 1, err, 2)) {
            ok = false;
            break;
          }
          tc_fence_after();
          bool first = true;  // the chunk's first k-step starts every accumulator
          int const kt_end = min(k_tiles, (c + 1) * kChunkKT);
          for (int kt = c * kChunkKT; kt < kt_end; ++kt, ++g) {
            int const s = static_cast<int>(g % kStages);
            uint32_t const use = static_cast<uint32_t>(g / kStages);
            if (!mbar_wait(&full_bar[s], use & 1, err, 3)) {
              ok = false;
              break;
            }
            tc_fence_after();
            uint32_t const base = smem_u32(smem + s * kStageBytes);
#pragma unroll
            for (int ks = 0; ks < kTK / 16; ++ks) {
              // The 21 slice pairs p + q <= 5 (0-based; 1-based p + q <= 7), as
              // 9 MMAs: A_p against the B slices q0 .. q0 + nb - 1 into the
              // level accumulators p + q0 onwards.  Per level the slice pairs
              // still arrive in increasing p, and the p = 0 MMAs of a chunk's
              // first k-step (levels 0..5) overwrite instead of accumulating.
#pragma unroll
              for (int p = 0; p < kSlices; ++p) {
#pragma unroll
                for (int q0 = 0; q0 < kSlices - p; q0 += kLevelGroup) {
                  int const nb = min(kLevelGroup, kSlices - p - q0);
                  uint64_t const ad = smem_desc(base + p * kABlk + ks * 256, 128, 512);
                  uint64_t const bd =
                      smem_desc(base + kStageA + q0 * kBBlk + ks * 256, 128, 512);
                  uint32_t const acc = (first && p == 0) ? 0u : 1u;
                  mma_bf16(tmem + static_cast<uint32_t>((p + q0) * kTN), ad, bd, acc,
                           idesc_n(nb * kTN));
                }
              }
              first = false;
            }
            mma_commit(&empty_bar[s]);  // stage s free once these MMAs complete
          }
          if (ok) mma_commit(&acc_full);
        }
      }
      mma_commit(&done_bar);
      mbar_wait(&done_bar, 0, err, 4);
    }
  } else {
    // Promotion warps: lane row = 32 (warp % 4) + lane, columns col0 .. col0 + kColsW.
    int const row = 32 * (warp % 4) + lane;
    int const col0 = kColsW * (warp / 4);
    uint32_t const lane_addr =
        tmem + (static_cast<uint32_t>(32 * (warp % 4)) << 16) + static_cast<uint32_t>(col0);
    int64_t c_all = 0;
    bool ok = true;
    for (int i = first_tile; i < n_tiles && ok; i += tile_step) {
      // the tile's epilogue data, loaded while its first chunk is multiplied
      auto const pre = epi.prepare(i, row, col0);
      float hi[kColsW], lo[kColsW];
#pragma unroll
      for (int j = 0; j < kColsW; ++j) hi[j] = lo[j] = 0.f;
      for (int c = 0; c < n_chunks; ++c, ++c_all) {
        // Waits are decided warp-uniformly: the TMEM loads below must be
        // reached by all lanes of a warp or by none.
        if (!__all_sync(0xffffffffu,
                        mbar_wait(&acc_full, static_cast<uint32_t>(c_all) & 1, err, 5))) {
          ok = false;
          break;
        }
        tc_fence_after();
#pragma unroll
        for (int cb = 0; cb < kColsW / 8; ++cb) {
          // Levels 0..2, then 3..5, eight columns at a time (the registers of
          // three warps on one SM sub-partition share its 16K).
          uint32_t const ca = lane_addr + static_cast<uint32_t>(cb * 8);
          uint32_t r[3][8];
#pragma unroll
          for (int l = 0; l < 3; ++l) tmem_ld8_issue(ca + static_cast<uint32_t>(l * kTN), r[l]);
          tmem_ld_wait(r);
          float s2[8], xs[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            float s1, x1, x2;
            two_sum(__uint_as_float(r[0][u]), __uint_as_float(r[1][u]) * 0x1p-8f, s1, x1);
            two_sum(s1, __uint_as_float(r[2][u]) * 0x1p-16f, s2[u], x2);
            xs[u] = x1 + x2;
          }
#pragma unroll
          for (int l = 0; l < 3; ++l)
            tmem_ld8_issue(ca + static_cast<uint32_t>((3 + l) * kTN), r[l]);
          tmem_ld_wait(r);
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            float const low =
                fmaf(__uint_as_float(r[2][u]), 0x1p-16f,
                     fmaf(__uint_as_float(r[1][u]), 0x1p-8f, __uint_as_float(r[0][u]))) *
                0x1p-24f;
            float s3, x3;
            two_sum(s2[u], low, s3, x3);
            // Running (hi, lo) += (s3, xs + x3), renormalised so that
            // |lo| <= ulp(hi)/2.
            int const j = cb * 8 + u;
            float s, e;
            two_sum(hi[j], s3, s, e);
            e += lo[j] + (xs[u] + x3);
            float const h = s + e;
            lo[j] = e - (h - s);
            hi[j] = h;
          }
        }
        tc_fence_before();
        mbar_arrive(&acc_empty);
      }
      // After a timeout the values are incomplete; *err makes the host discard them.
      if (ok) epi(pre, i, row, col0, hi, lo);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTmemCols)
                 : "memory");
  }
}

// Persistent grid of a launch of n_tiles tiles: at most one CTA per SM.
inline int persistent_grid(int64_t n_tiles) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      sms < 1)
    sms = 1;
  return static_cast<int>(n_tiles < sms ? n_tiles : sms);
}

}  // namespace tc
}  // namespace dev
}  // namespace slaph
