// Diluted-factor products on the tensor cores (tcgen05, sm_103a).
//
// operator* (src/DilutedFactor.cpp:6-51) and multiply<1,1>
// (include/DilutedFactor.hpp:164-187) form C = L R for every compatible pair of
// left and right factor matrices (eds x eds, eds = 4 dilE).  Within one
// dependency level each left matrix meets dozens of right matrices, every one
// with its own set, so the products of a level are grouped by left matrix:
// a group holds 64 / eds left matrices (one 64-row M tile of stacked rows) and
// the union U of their right matrices (eds columns each), and one GEMM
//   D(group row (l, i), column (u, j)) = sum_k L_l(i, k) R_u(k, j)
// gives every product of the group; the epilogue keeps the entries of the
// pairs the level asks for and writes them as double-float matrices into the
// product slots, in the natural and the transposed layout, together with the
// largest entry of every slot (for the slicing of the trace operands).
//
// Operands, in the split-BF16 scheme of tc_common.cuh: A rows are the rows of
// the left matrices (conjugated, so that the conjugating form gives the plain
// product), one exponent per row; each distinct right matrix of the level is
// sliced once into a stream of its own, [k-tile][slice][8-column group][512
// bytes] with one exponent per column, and the producer of the GEMM gathers a
// tile's B stage from those streams with one bulk copy per (slice, right
// matrix).
#include <cuda_runtime.h>

#include <cstdint>

#include "kernels.cuh"
#include "tc_common.cuh"

namespace slaph {
namespace dev {

namespace {

using namespace tc;

constexpr int kPSliceThreads = 256;

// Row group (A: four complex rows = eight A' rows; B: eight columns) of one
// k-tile: lane (r, kc) = (lane / 4, lane % 4) converts the four complex
// entries 4 kc .. 4 kc + 3 of its row into one 16-byte row segment per slice.
// v: the entries, e: the row's exponent; A rows are conjugated.
template <bool kIsA>
__device__ __forceinline__ void slice_row_segment(float4 const (&v)[4], int e, int r,
                                                  uint8_t *dst, uint32_t blk) {
  uint32_t w[kSlices][4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    long long const fr = fixed55f(v[q].x, e) + fixed55f(v[q].y, e);
    long long const fi = fixed55f(v[q].z, e) + fixed55f(v[q].w, e);
    float dre[kSlices], dim[kSlices];
    digits6(fr, dre);
    if (kIsA) {
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
#pragma unroll
  for (int s = 0; s < kSlices; ++s)
    *reinterpret_cast<uint4 *>(dst + s * blk) = make_uint4(w[s][0], w[s][1], w[s][2], w[s][3]);
}

// Largest |re|, |im| (high words) of the lanes' entries, over the lanes whose
// bits `mask` differ (the lanes of one row).
__device__ __forceinline__ unsigned int row_max(float4 const (&v)[4], unsigned int mx,
                                                int mask) {
#pragma unroll
  for (int q = 0; q < 4; ++q)
    mx = max(mx, max(__float_as_uint(v[q].x) & 0x7FFFFFFFu, __float_as_uint(v[q].z) & 0x7FFFFFFFu));
#pragma unroll
  for (int o = 1; o <= 4; o <<= 1)
    if (mask & o) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  return mx;
}

// A regions: one CTA per group; the group's 64 rows (left matrix l = row /
// eds, row i = row % eds, read from the transposed layout where rows are
// contiguous) in quads of four rows, warp w taking quads w, w + 8.  Rows of
// absent left matrices are not written (the epilogue skips them).
__global__ void __launch_bounds__(kPSliceThreads)
    prod_slice_a_kernel(uint8_t *scratch, int32_t *expo, ProdGroup const *groups,
                        float4 const *slots_t, int32_t eds, int64_t a_bytes) {
  ProdGroup const gr = groups[blockIdx.x];
  int64_t const ms = static_cast<int64_t>(eds) * eds;
  int const k_tiles = eds / (kTK / 2);
  int const warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  int const r = lane / 4, kc = lane % 4;
  uint8_t *region = scratch + static_cast<int64_t>(blockIdx.x) * a_bytes;
  for (int quad = warp; quad < (kTM / 2) / 4; quad += kPSliceThreads / 32) {
    int const cr = 4 * quad + r / 2;  // complex row of the M tile
    int const l = cr / eds, i = cr % eds;
    if (l >= gr.n_l) continue;  // warp-uniform: a quad lies inside one matrix
    float4 const *src =
        slots_t + static_cast<int64_t>(groups[blockIdx.x].l[l]) * ms + static_cast<int64_t>(i) * eds;
    unsigned int mx = 0;
    for (int kt = 0; kt < k_tiles; ++kt) {
      float4 v[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) v[q] = src[kt * (kTK / 2) + 4 * kc + q];
      mx = row_max(v, mx, 1 | 2 | 4);
    }
    // |hi + lo| < 2^e whenever |hi| < 2^e (|lo| <= ulp(hi) / 2).
    int const e = expo_of_absbits(mx);
    if (lane % 8 == 0) expo[gr.ea + cr] = e;
    int const arow = 2 * cr + (r & 1);
    uint8_t *base = region + ((arow >> 3) * 4 + kc) * 128 + (arow & 7) * 16;
    for (int kt = 0; kt < k_tiles; ++kt) {
      float4 v[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) v[q] = src[kt * (kTK / 2) + 4 * kc + q];
      slice_row_segment<true>(v, e, r, base + static_cast<int64_t>(kt) * kStageA, kABlk);
    }
  }
}

// Right-matrix streams: one CTA per distinct right matrix of the level, warp w
// taking the 8-column groups w, w + 8, ... (columns read from the natural
// layout, where they are contiguous).
__global__ void __launch_bounds__(kPSliceThreads)
    prod_slice_r_kernel(uint8_t *streams, int32_t *expo, int32_t const *r_slots,
                        float4 const *slots_n, int32_t eds) {
  int64_t const ms = static_cast<int64_t>(eds) * eds;
  int const k_tiles = eds / (kTK / 2), n_cg = eds / 8;
  int const warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  int const r = lane / 4, kc = lane % 4;
  uint8_t *stream = streams + static_cast<int64_t>(blockIdx.x) * prod_tc_r_bytes(eds);
  float4 const *mat = slots_n + static_cast<int64_t>(r_slots[blockIdx.x]) * ms;
  for (int cg = warp; cg < n_cg; cg += kPSliceThreads / 32) {
    int const j = 8 * cg + r;
    float4 const *src = mat + static_cast<int64_t>(j) * eds;
    unsigned int mx = 0;
    for (int kt = 0; kt < k_tiles; ++kt) {
      float4 v[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) v[q] = src[kt * (kTK / 2) + 4 * kc + q];
      mx = row_max(v, mx, 1 | 2);
    }
    int const e = expo_of_absbits(mx);
    if (kc == 0) expo[static_cast<int64_t>(blockIdx.x) * eds + j] = e;
    for (int kt = 0; kt < k_tiles; ++kt) {
      float4 v[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) v[q] = src[kt * (kTK / 2) + 4 * kc + q];
      // [k-tile][slice][8-column group][512 B]: a slice step is n_cg groups
      uint8_t *dst = stream + ((static_cast<int64_t>(kt) * kSlices * n_cg + cg) * 4 + kc) * 128 +
                     r * 16;
      slice_row_segment<false>(v, e, r, dst, static_cast<uint32_t>(n_cg) * 512u);
    }
  }
}

// Stage loader of the product GEMM: the group's A block (lane 0) and the B
// stage gathered from the right-matrix streams, one copy per (slice, right
// matrix) spread over the lanes; padding columns of a group's last tile are not
// copied (the epilogue skips them).
struct ProdTiles {
  uint8_t const *scratch;  // A regions from 0, right-matrix streams from r_off
  int64_t a_bytes, r_off;
  ProdTile const *tiles;
  ProdGroup const *groups;
  int32_t const *u_list;  // right-matrix index of each group column block
  int32_t eds, k_tiles;
  // One tile's copies: the A block, and per lane up to two B copies (one per
  // (slice, right matrix overlapping the tile): its columns are contiguous
  // both in its stream and in the stage), addresses of k-tile 0.
  struct Ctx {
    uint8_t const *a;
    uint8_t const *src[2];
    uint32_t dst[2], bytes[2];
    uint32_t tx;
  };
  __device__ __forceinline__ Ctx context(int i, int lane) const {
    ProdTile const t = tiles[i];
    ProdGroup const gr = groups[t.group];
    Ctx c;
    c.a = scratch + t.group * a_bytes;
    int const c0 = t.nt * kTN;
    int const cols = min(kTN, eds * gr.n_u - c0);  // a multiple of 8
    c.tx = kStageA + static_cast<uint32_t>(kSlices * cols) * 64u;
    int64_t const r_bytes = prod_tc_r_bytes(eds);
    int const r_cg = eds / 8, u0 = c0 / eds, n_blk = (c0 + cols - 1) / eds - u0 + 1;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      int const q = lane + 32 * h;
      c.bytes[h] = 0;
      c.src[h] = scratch;
      c.dst[h] = 0;
      if (q < kSlices * n_blk) {
        int const s = q / n_blk, u = u0 + q % n_blk;
        int const cs = max(c0, u * eds), ce = min(c0 + cols, (u + 1) * eds);
        c.src[h] = scratch + r_off + u_list[gr.u_off + u] * r_bytes +
                   (static_cast<int64_t>(s) * r_cg + (cs - u * eds) / 8) * 512;
        c.dst[h] = kStageA + s * kBBlk + ((cs - c0) / 8) * 512;
        c.bytes[h] = static_cast<uint32_t>(ce - cs) * 64u;
      }
    }
    return c;
  }
  __device__ __forceinline__ void load(Ctx const &c, int kt, uint8_t *dst, uint64_t *bar,
                                       int lane) const {
    if (lane == 0) {
      mbar_expect_tx(bar, c.tx);
      bulk_g2s(dst, c.a + static_cast<int64_t>(kt) * kStageA, kStageA, bar);
    }
    __syncwarp();
    // k-tile step of a stream: kSlices x eds columns x 64 bytes
    int64_t const kt_off = static_cast<int64_t>(kt) * kSlices * eds * 64;
#pragma unroll
    for (int h = 0; h < 2; ++h)
      if (c.bytes[h]) bulk_g2s(dst + c.dst[h], c.src[h] + kt_off, c.bytes[h], bar);
  }
};

// x 2^sh for |sh| <= 252, as two multiplications by powers of two (each exact
// for a normal result).
__device__ __forceinline__ float scale2(float x, int sh) {
  int const s1 = sh / 2, s2 = sh - s1;
  return (x * __int_as_float((s1 + 127) << 23)) * __int_as_float((s2 + 127) << 23);
}

// Epilogue: A' row 2 cr + (re | im), cr = l eds + i; column c = u eds + j.
// A warp's 32 rows lie in one left matrix l.  Before the tile is promoted,
// lane k fetches the product slot and the column exponent of the warp's
// columns k and 32 + k; the column loop takes them by warp shuffles.
// The even lane of each row pair holds Re, the odd one Im; after one exchange
// the even lane writes the natural layout and the odd lane the transposed one.
struct ProdEpilogue {
  ProdTiles tl;
  int32_t const *expo;    // A rows from 0 (64 per group), right columns from r_expo
  int64_t r_expo;
  int32_t const *out_tab;  // [group column block][4]: product slot per left matrix
  float4 *slots_n, *slots_t;
  unsigned int *slot_bits;  // largest |re|, |im| per slot (float bits), by atomicMax
  struct Pre {
    int ok, er, cbase;
    int slot0, ec0, slot1, ec1;
  };
  __device__ __forceinline__ Pre prepare(int it, int row, int col0) const {
    Pre p{0, 0, 0, -1, 0, -1, 0};
    ProdTile const t = tl.tiles[it];
    ProdGroup const gr = tl.groups[t.group];
    int const eds = tl.eds, lane = threadIdx.x % 32;
    int const cr = row / 2, l = cr / eds;
    p.cbase = t.nt * kTN + col0;
    if (l >= gr.n_l) return p;  // warp-uniform
    p.ok = 1;
    p.er = expo[gr.ea + cr];
    int const ncols = eds * gr.n_u;
    auto meta = [&](int c, int &slot, int &ec) {
      if (c >= ncols) return;
      int const u = c / eds;
      slot = out_tab[4 * (gr.u_off + u) + l];
      ec = expo[r_expo + static_cast<int64_t>(tl.u_list[gr.u_off + u]) * eds + c % eds];
    };
    meta(p.cbase + lane, p.slot0, p.ec0);
    if (lane < kColsW - 32) meta(p.cbase + 32 + lane, p.slot1, p.ec1);
    return p;
  }
  __device__ __forceinline__ void operator()(Pre const &p, int, int row, int,
                                             float const (&hi)[kColsW],
                                             float const (&lo)[kColsW]) const {
    if (!p.ok) return;  // warp-uniform
    int const eds = tl.eds;
    int64_t const ms = static_cast<int64_t>(eds) * eds;
    int const i = (row / 2) % eds;
    // The slot of a column is the same for the whole warp (one left matrix):
    // the largest |hi| of a run of columns of one slot goes to slot_bits by
    // one warp reduction and one atomic.
    int run_slot = -1;
    unsigned int run_max = 0;
    auto flush = [&] {
      unsigned int const m = __reduce_max_sync(0xffffffffu, run_max);
      if (run_slot >= 0 && (threadIdx.x % 32) == 0) atomicMax(slot_bits + run_slot, m);
    };
#pragma unroll
    for (int cc = 0; cc < kColsW; ++cc) {
      int const slot = __shfl_sync(0xffffffffu, cc < 32 ? p.slot0 : p.slot1, cc % 32);
      int const ec = __shfl_sync(0xffffffffu, cc < 32 ? p.ec0 : p.ec1, cc % 32);
      int const sh = max(p.er + ec - 14, -252);
      float const h = scale2(hi[cc], sh), lw = scale2(lo[cc], sh);
      float const oh = __shfl_xor_sync(0xffffffffu, h, 1);
      float const ol = __shfl_xor_sync(0xffffffffu, lw, 1);
      if (slot != run_slot) {  // warp-uniform
        flush();
        run_slot = slot;
        run_max = 0;
      }
      if (slot < 0) continue;
      run_max = max(run_max, __float_as_uint(h) & 0x7FFFFFFFu);
      int const j = (p.cbase + cc) % eds;
      if ((row & 1) == 0)
        slots_n[slot * ms + i + static_cast<int64_t>(eds) * j] = make_float4(h, lw, oh, ol);
      else
        slots_t[slot * ms + j + static_cast<int64_t>(eds) * i] = make_float4(oh, ol, h, lw);
    }
    flush();
  }
};

__global__ void __launch_bounds__(kThreads, 1)
    product_gemm_kernel(ProdTiles tl, int32_t n_tiles, int32_t const *expo, int64_t r_expo,
                        int32_t const *out_tab, float4 *slots_n, float4 *slots_t,
                        unsigned int *slot_bits, int *err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  ProdEpilogue epi{tl, expo, r_expo, out_tab, slots_n, slots_t, slot_bits};
  ozaki_tiles(smem, n_tiles, tl.k_tiles, tl, err, epi);
}

}  // namespace

bool prod_tc_supported(int32_t eds) { return eds == 16 || eds == 32 || eds == 64; }
int64_t prod_tc_a_bytes(int32_t eds) {
  return static_cast<int64_t>(eds / (kTK / 2)) * kStageA;
}

cudaError_t products_tc(float4 *slots_n, float4 *slots_t, uint8_t *scratch, int64_t r_off,
                        int32_t *expo, int64_t r_expo, ProdGroup const *groups, int64_t n_groups,
                        int32_t const *r_slots, int64_t n_r, int32_t const *u_list,
                        int32_t const *out_tab, ProdTile const *tiles, int64_t n_tiles,
                        int32_t eds, unsigned int *slot_bits, int *err, cudaStream_t stream) {
  if (n_tiles == 0) return cudaSuccess;
  if (!prod_tc_supported(eds) || n_groups > 0x7fffffffLL || n_r > 0x7fffffffLL ||
      n_tiles > 0x7fffffffLL)
    return cudaErrorInvalidValue;
  int64_t const a_bytes = prod_tc_a_bytes(eds);
  prod_slice_a_kernel<<<static_cast<unsigned>(n_groups), kPSliceThreads, 0, stream>>>(
      scratch, expo, groups, slots_t, eds, a_bytes);
  if (n_r > 0)
    prod_slice_r_kernel<<<static_cast<unsigned>(n_r), kPSliceThreads, 0, stream>>>(
        scratch + r_off, expo + r_expo, r_slots, slots_n, eds);
  cudaError_t e = cudaFuncSetAttribute(product_gemm_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(kSmemBytes));
  if (e != cudaSuccess) return e;
  ProdTiles const tl{scratch, a_bytes, r_off, tiles, groups, u_list, eds, eds / (kTK / 2)};
  product_gemm_kernel<<<static_cast<unsigned>(persistent_grid(n_tiles)), kThreads, kSmemBytes,
                        stream>>>(tl, static_cast<int32_t>(n_tiles), expo, r_expo, out_tab,
                                  slots_n, slots_t, slot_bits, err);
  return cudaGetLastError();
}

}  // namespace dev
}  // namespace slaph
