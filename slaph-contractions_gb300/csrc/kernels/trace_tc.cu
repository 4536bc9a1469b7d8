// Dense diluted-trace groups on the tensor cores (tcgen05, sm_103a).
//
// factor_to_trace (src/DilutedTrace.cpp:84-138) computes tr(L R) =
// sum_k L_k (R^T)_k over the (4 dilE)^2 entries k of the two factor matrices.
// When the lists of one trace shape pair every A group with every B group, the
// values of entry (i, j) of all lists are the complex matrix product
//   T(ia, ib) = sum_k A[a_ia + i]_k B[b_ib + j]^T_k,
// a GEMM with K = (4 dilE)^2.  It runs with the split-BF16 scheme of
// tc_common.cuh: A rows are conj(A) (so that the conjugating form gives the
// plain product), B columns are the transposed B matrices.
//
// Operands are double-float matrices (float4 (re_hi, re_lo, im_hi, im_lo)) in
// the natural (A) and transposed (B) layouts.  trace_slice_kernel cuts the
// matrices of one 8-row core-matrix group per CTA into the operand stream of
// their GEMM region, with each matrix's exponent; trace_gemm_kernel computes 64 x 80 complex output tiles
// (persistent CTAs, one per SM) and writes FP64 trace values: the 32 lanes of
// a warp hold 16 consecutive A groups (re, im) of one output column, so the
// stores of each column are 256 contiguous bytes.
#include <cuda_runtime.h>

#include <cstdint>

#include "kernels.cuh"
#include "tc_common.cuh"

namespace slaph {
namespace dev {

namespace {

using namespace tc;

constexpr int kSliceThreads = 256;  // eight warps per row group

// Largest |re|, |im| of every matrix slot first..first+n, as the bit pattern
// of the float (from the high words; |hi + lo| < 2^e whenever |hi| < 2^e, as
// |lo| <= ulp(hi) / 2).  One warp per slot.
__global__ void __launch_bounds__(256)
    slot_maxbits_kernel(unsigned int *bits, float4 const *slots, int64_t first, int64_t n,
                        int32_t eds) {
  int64_t const w = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) / 32;
  int const lane = threadIdx.x % 32;
  if (w >= n) return;
  int64_t const ms = static_cast<int64_t>(eds) * eds;
  float4 const *src = slots + (first + w) * ms;
  unsigned int mx = 0;
#pragma unroll 4
  for (int64_t m = lane; m < ms; m += 32) {
    float4 const v = src[m];
    mx = max(mx, max(__float_as_uint(v.x) & 0x7FFFFFFFu, __float_as_uint(v.z) & 0x7FFFFFFFu));
  }
  mx = __reduce_max_sync(0xffffffffu, mx);
  if (lane == 0) bits[first + w] = mx;
}

// One row group per CTA (TrSliceGroup), one pass over its matrices with the
// largest entries of their slots (slot_maxbits): the warps take k-tiles in
// turn.  In a k-tile, lane (r, kc) = (lane / 4, lane % 4) converts the four
// complex entries 4 kc .. 4 kc + 3 of core-matrix row r (B: matrix r; A:
// matrix r / 2, A' row parity r % 2) into one 16-byte row segment per slice,
// so that each slice store of a warp writes 512 contiguous bytes.  Integer
// and FP32 operations only: the fixed-point value of a double-float entry is
// the sum of those of its two words.  Rows past the group's n are not written
// (the GEMM tiles mask them).
template <bool kIsA>
__global__ void __launch_bounds__(kSliceThreads)
    trace_slice_kernel(uint8_t *scratch, int32_t *expo, TrSliceGroup const *groups,
                       float4 const *slots, unsigned int const *slot_bits, int32_t eds) {
  TrSliceGroup const gr = groups[blockIdx.x];
  int64_t const ms = static_cast<int64_t>(eds) * eds;
  int32_t const k_tiles = static_cast<int32_t>(ms / (kTK / 2));
  int const warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  if (threadIdx.x < gr.n)
    expo[gr.expo0 + threadIdx.x] =
        expo_of_absbits(slot_bits[groups[blockIdx.x].slot[threadIdx.x]]);
  int const r = lane / 4, kc = lane % 4;
  int const mi = kIsA ? r / 2 : r;  // matrix of this lane
  if (mi >= gr.n) return;
  int const slot = groups[blockIdx.x].slot[mi];
  int const e = expo_of_absbits(slot_bits[slot]);
  float4 const *src = slots + static_cast<int64_t>(slot) * ms + 4 * kc;
  uint8_t *region = scratch + gr.dst;
  uint8_t *base;
  uint32_t blk;
  if (kIsA) {
    int const cr = gr.row0 + mi, arow = 2 * (cr % (kTM / 2)) + (r & 1);
    base = region + static_cast<int64_t>(cr / (kTM / 2)) * k_tiles * kStageA +
           ((arow >> 3) * 4 + kc) * 128 + (arow & 7) * 16;
    blk = kABlk;
  } else {
    int const c = gr.row0 + mi, rr = c % kTN;
    base = region + static_cast<int64_t>(c / kTN) * k_tiles * kStageB +
           ((rr >> 3) * 4 + kc) * 128 + (rr & 7) * 16;
    blk = kBBlk;
  }
  for (int kt = warp; kt < k_tiles; kt += kSliceThreads / 32) {
    uint32_t w[kSlices][4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      float4 const v = src[kt * (kTK / 2) + q];
      long long const fr = fixed55f(v.x, e) + fixed55f(v.y, e);
      long long const fi = fixed55f(v.z, e) + fixed55f(v.w, e);
      float dre[kSlices], dim[kSlices];
      digits6(fr, dre);
      if (kIsA) {
        // conj: A' rows (Re x, Im x) and (-Im x, Re x) of x = conj(v)
        digits6(-fi, dim);
#pragma unroll
        for (int s = 0; s < kSlices; ++s)
          w[s][q] = (r & 1) ? bf16x2(-dim[s], dre[s]) : bf16x2(dre[s], dim[s]);
      } else {
        digits6(fi, dim);
#pragma unroll
        for (int s = 0; s < kSlices; ++s) w[s][q] = bf16x2(dre[s], dim[s]);
      }
    }
    uint8_t *dst = base + static_cast<int64_t>(kt) * (kIsA ? kStageA : kStageB);
#pragma unroll
    for (int s = 0; s < kSlices; ++s)
      *reinterpret_cast<uint4 *>(dst + s * blk) = make_uint4(w[s][0], w[s][1], w[s][2], w[s][3]);
  }
}

// FP64 trace values of one tile: value (r, c) = (hi + lo) 2^(e_r + e_c - 14)
// at values[out + c * ld + r], component row & 1 (re, im).
struct TraceEpilogue {
  double *values;
  int32_t const *expo;
  TrTile const *tiles;
  // Lane k holds the exponents of the warp's columns k and 32 + k; the column
  // loop takes them by warp shuffles.
  struct Pre {
    TrTile t;
    int e0, e1, er;
  };
  __device__ __forceinline__ Pre prepare(int i, int row, int col0) const {
    Pre p;
    p.t = tiles[i];
    int const lane = threadIdx.x % 32;
    p.e0 = col0 + lane < p.t.cols ? expo[p.t.eb + col0 + lane] : 0;
    p.e1 = lane < kColsW - 32 && col0 + 32 + lane < p.t.cols ? expo[p.t.eb + col0 + 32 + lane] : 0;
    p.er = row / 2 < p.t.rows ? expo[p.t.ea + row / 2] : 0;
    return p;
  }
  __device__ __forceinline__ void operator()(Pre const &p, int i, int row, int col0,
                                             float const (&hi)[kColsW],
                                             float const (&lo)[kColsW]) const {
    TrTile const &t = p.t;
    int const r = row / 2;
    bool const row_ok = r < t.rows;
    double *dst = values + 2 * (t.out + r) + (row & 1);
#pragma unroll
    for (int c = 0; c < kColsW; ++c) {
      int const ec = __shfl_sync(0xffffffffu, c < 32 ? p.e0 : p.e1, c % 32);
      int const col = col0 + c;
      if (row_ok && col < t.cols)
        dst[2 * static_cast<int64_t>(col) * t.ld] =
            ldexp(static_cast<double>(hi[c]) + static_cast<double>(lo[c]), p.er + ec - 14);
    }
  }
};

struct TraceSrc {
  uint8_t const *scratch;
  TrTile const *tiles;
  struct Ctx {
    uint8_t const *a, *b;
  };
  __device__ __forceinline__ Ctx context(int i, int lane) const {
    return Ctx{scratch + tiles[i].a_src, scratch + tiles[i].b_src};
  }
  __device__ __forceinline__ void load(Ctx const &c, int kt, uint8_t *dst, uint64_t *bar,
                                       int lane) const {
    if (lane == 0) load_contiguous(c.a, c.b, kt, dst, bar, 0);
  }
};

__global__ void __launch_bounds__(kThreads, 1)
    trace_gemm_kernel(double2 *values, uint8_t const *scratch, int32_t const *expo,
                      TrTile const *tiles, int32_t n_tiles, int32_t k_tiles, int *err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  TraceEpilogue epi{reinterpret_cast<double *>(values), expo, tiles};
  ozaki_tiles(smem, n_tiles, k_tiles, TraceSrc{scratch, tiles}, err, epi);
}

}  // namespace

int64_t trace_tc_k_tiles(int32_t eds) {
  return static_cast<int64_t>(eds) * eds / (kTK / 2);
}
size_t trace_tc_a_bytes(int32_t rows, int32_t eds) {
  return static_cast<size_t>((rows + kTM / 2 - 1) / (kTM / 2)) * trace_tc_k_tiles(eds) * kStageA;
}
size_t trace_tc_b_bytes(int32_t cols, int32_t eds) {
  return static_cast<size_t>((cols + kTN - 1) / kTN) * trace_tc_k_tiles(eds) * kStageB;
}

cudaError_t slot_maxbits(unsigned int *bits, float4 const *slots, int64_t first, int64_t n,
                         int32_t eds, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  slot_maxbits_kernel<<<static_cast<unsigned>((n * 32 + 255) / 256), 256, 0, stream>>>(
      bits, slots, first, n, eds);
  return cudaGetLastError();
}

cudaError_t trace_tc_slice(uint8_t *scratch, int32_t *expo, TrSliceGroup const *a_groups,
                           int64_t n_a, TrSliceGroup const *b_groups, int64_t n_b,
                           float4 const *slots_n, float4 const *slots_t,
                           unsigned int const *slot_bits, int32_t eds, cudaStream_t stream) {
  if ((static_cast<int64_t>(eds) * eds) % (kTK / 2) != 0) return cudaErrorInvalidValue;
  if (n_a > 0)
    trace_slice_kernel<true><<<static_cast<unsigned>(n_a), kSliceThreads, 0, stream>>>(
        scratch, expo, a_groups, slots_n, slot_bits, eds);
  if (n_b > 0)
    trace_slice_kernel<false><<<static_cast<unsigned>(n_b), kSliceThreads, 0, stream>>>(
        scratch, expo, b_groups, slots_t, slot_bits, eds);
  return cudaGetLastError();
}

size_t tc_a_bytes(int32_t rows, int32_t k_tiles) {
  return static_cast<size_t>((rows + kTM / 2 - 1) / (kTM / 2)) * k_tiles * kStageA;
}
size_t tc_b_bytes(int32_t cols, int32_t k_tiles) {
  return static_cast<size_t>((cols + kTN - 1) / kTN) * k_tiles * kStageB;
}

cudaError_t tc_gemm(double2 *out, uint8_t const *scratch, int32_t const *expo,
                    TrTile const *tiles, int64_t n_tiles, int32_t k_tiles, int *err,
                    cudaStream_t stream) {
  if (n_tiles == 0) return cudaSuccess;
  if (k_tiles < 1) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(trace_gemm_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(kSmemBytes));
  if (e != cudaSuccess) return e;
  for (int64_t t0 = 0; t0 < n_tiles; t0 += 0x7fffffffLL) {
    int64_t const n = n_tiles - t0 < 0x7fffffffLL ? n_tiles - t0 : 0x7fffffffLL;
    trace_gemm_kernel<<<static_cast<unsigned>(persistent_grid(n)), kThreads, kSmemBytes,
                        stream>>>(out, scratch, expo, tiles + t0, static_cast<int32_t>(n),
                                  k_tiles, err);
  }
  return cudaGetLastError();
}

cudaError_t trace_tc_gemm(double2 *values, uint8_t const *scratch, int32_t const *expo,
                          TrTile const *tiles, int64_t n_tiles, int32_t eds, int *err,
                          cudaStream_t stream) {
  return tc_gemm(values, scratch, expo, tiles, n_tiles,
                 static_cast<int32_t>(trace_tc_k_tiles(eds)), err, stream);
}

}  // namespace dev
}  // namespace slaph
