// Split-BF16 tensor-core VdaggerV (tcgen05, sm_103a).
//
// VdaggerV = V^H diag(phase) V (src/OperatorFactory.cpp:292-300) with FP64
// inputs and an FP64-accurate result from BF16 tensor-core products, by the
// split-BF16 scheme of tc_common.cuh: A' rows are the eigenvectors V_i, B
// columns W_j = diag(phase) V_j, K' = 2 * 3L^3; rows are scaled by the
// exponent of the eigenvector's largest |entry| (the same for W, |phase| = 1).
//
// Data path: slices are written once per timeslice (A) and per timeslice and
// operator (B) to HBM, already in the tcgen05 core-matrix layout, and streamed
// into shared memory by the GEMM.  The B columns of all operators of a
// timeslice form one N dimension (column o nev + j: operator o, eigenvector
// j), cut into tiles of kTN without padding between operators; the tiles of a
// batch of timeslices (m tiles x n tiles x timeslices) go to persistent CTAs.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "kernels.cuh"
#include "tc_common.cuh"

namespace slaph {
namespace dev {

namespace {

using namespace tc;

// Exponent e_i with max_x |V(x, i)| < 2^e_i per eigenvector (one block per i).
__global__ void colmax_kernel(int32_t *expo, double2 const *Vt, Geometry g) {
  int const i = blockIdx.x;
  double2 const *col = Vt + static_cast<int64_t>(i) * g.dim_row;
  double m = 0;
  for (int64_t x = threadIdx.x; x < g.dim_row; x += blockDim.x) {
    double2 const v = col[x];
    m = fmax(m, v.x * v.x + v.y * v.y);
  }
  __shared__ double red[256];
  red[threadIdx.x] = m;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    int e = 0;
    double const mx = sqrt(red[0]);
    if (mx > 0) frexp(mx * (1.0 + 1e-15), &e);
    expo[i] = e;
  }
}

// A slices of one timeslice: [m_tile][k_tile][slice][kTM x kTK core layout].
// Thread per (eigenvector i, site-colour x).
__global__ void slice_a_kernel(uint16_t *out, double2 const *Vt, int32_t const *expo,
                               int32_t k_tiles, Geometry g) {
  int64_t const x = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  int const i = blockIdx.y;
  if (x >= static_cast<int64_t>(k_tiles) * (kTK / 2)) return;
  double2 v = make_double2(0, 0);
  if (x < g.dim_row) v = Vt[static_cast<int64_t>(i) * g.dim_row + x];
  put_a(reinterpret_cast<uint8_t *>(out), k_tiles, i, x, v, expo[i]);
}

// B slices of W = diag(phase_op) V for the operators ops[0..n_ops) of the
// call, at global B columns col0 + o nev + j: [n_tile][k_tile][slice][kTN x kTK]
// over the columns of all operators.  A warp covers one 8-column group of one
// operator's eigenvectors in one k-tile: lane (r, kg) = (lane % 8, lane / 8)
// takes eigenvector 8 rg + r and the 4 complex K entries 4 kg .. 4 kg + 3, i.e.
// one 16-byte row of a core matrix, so that the slice stores of the warp cover
// one or two 8-row core-matrix columns.  V is read and put in fixed point once
// for all operators; the phase product is taken in fixed point with integer
// operations only: with V = F_v 2^(e-55) and phase = P 2^-62 (|P| <= 2^62),
// W = ((F_v 4) P / 2^64) 2^(e-55), the high word of a 128-bit product.  K
// entries x >= dim_row are written as zero; columns past the last operator's
// stay as the per-build clear of the scratch left them (zero).
__global__ void __launch_bounds__(256)
    slice_b_kernel(uint8_t *out, double2 const *Vt, longlong2 const *phase_fx,
                   int32_t const *ops, int32_t n_ops, int32_t const *expo, int32_t k_tiles,
                   int64_t col0, Geometry g) {
  int64_t const wid = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) / 32;
  int const lane = threadIdx.x % 32;
  int64_t const groups = (g.nev + 7) / 8;
  if (wid >= groups * k_tiles) return;
  int64_t const kt = wid / groups;
  int const rg = static_cast<int>(wid % groups);
  int const r = lane % 8, kg = lane / 8;
  int const j = rg * 8 + r;
  if (j >= g.nev) return;
  int64_t const x0 = kt * (kTK / 2) + 4 * kg;
  int64_t const sites = g.dim_row / 3;
  long long vr[4], vi[4];
  int64_t site[4];
  int const e = expo[j];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    int64_t const x = x0 + q;
    bool const in = x < g.dim_row;
    double2 const v = in ? Vt[static_cast<int64_t>(j) * g.dim_row + x] : make_double2(0, 0);
    vr[q] = fixed55(v.x, e) * 4;
    vi[q] = fixed55(v.y, e) * 4;
    site[q] = in ? x / 3 : 0;
  }
  for (int o = 0; o < n_ops; ++o) {
    longlong2 const *ph = phase_fx + static_cast<int64_t>(ops[o]) * sites;
    uint32_t w[kSlices][4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      longlong2 const p = ph[site[q]];
      long long const wr = __mul64hi(vr[q], p.x) - __mul64hi(vi[q], p.y);
      long long const wi = __mul64hi(vr[q], p.y) + __mul64hi(vi[q], p.x);
      float dre[kSlices], dim[kSlices];
      digits6(wr, dre);
      digits6(wi, dim);
#pragma unroll
      for (int s = 0; s < kSlices; ++s) w[s][q] = bf16x2(dre[s], dim[s]);
    }
    int64_t const gc = col0 + static_cast<int64_t>(o) * g.nev + j;
    int64_t const nt = gc / kTN;
    int const rr = static_cast<int>(gc % kTN);
    uint8_t *dst = out + (nt * k_tiles + kt) * kStageB + ((rr >> 3) * 4 + kg) * 128 + (rr & 7) * 16;
#pragma unroll
    for (int s = 0; s < kSlices; ++s)
      *reinterpret_cast<uint4 *>(dst + s * kBBlk) = make_uint4(w[s][0], w[s][1], w[s][2], w[s][3]);
  }
}

__global__ void phase_fixed_kernel(longlong2 *dst, double2 const *src, int64_t n) {
  int64_t const k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (k >= n) return;
  double2 const v = src[k];
  dst[k] = make_longlong2(__double2ll_rn(ldexp(v.x, 62)), __double2ll_rn(ldexp(v.y, 62)));
}

// Tile i of a launch: m tile i % m_tiles, n tile (i / m_tiles) % n_tiles,
// batch slot i / (m_tiles n_tiles) (timeslice t0 + slot).  Slot b has its own A
// slices, B slices and exponents at stride slot_bytes in the scratch buffer:
// the eigenvectors' exponents, then per operator o >= n_comp (displaced) the
// exponents of its B columns at (1 + o) nev.
struct VdvTiles {
  uint8_t const *scratch;
  size_t slot_bytes, b_off, e_off;
  int32_t m_tiles, n_tiles, k_tiles;
  __device__ __forceinline__ void decode(int i, int &mt, int &nt, int &slot) const {
    mt = i % m_tiles;
    nt = (i / m_tiles) % n_tiles;
    slot = i / (m_tiles * n_tiles);
  }
  struct Ctx {
    uint8_t const *a, *b;
  };
  __device__ __forceinline__ Ctx context(int i, int lane) const {
    int mt, nt, slot;
    decode(i, mt, nt, slot);
    uint8_t const *sbase = scratch + slot * slot_bytes;
    return Ctx{sbase + static_cast<int64_t>(mt) * k_tiles * kStageA,
               sbase + b_off + static_cast<int64_t>(nt) * k_tiles * kStageB};
  }
  __device__ __forceinline__ void load(Ctx const &c, int kt, uint8_t *dst, uint64_t *bar,
                                       int lane) const {
    if (lane == 0) load_contiguous(c.a, c.b, kt, dst, bar, 0);
  }
};

// Epilogue of one VdaggerV tile: D = (hi + lo) 2^(e_i + f_c - 14), rows
// (2i, 2i+1) = (Re, Im) of VdaggerV_o(i, j) for the tile's B columns c = o nev
// + j, written to operator o's column-major nev x nev block of timeslice t; e:
// exponents of the eigenvectors (A rows), f: those of the B columns (the
// eigenvectors' for momentum operators, |phase| = 1; those of D(V) for the
// displaced ones, o >= n_comp, at (1 + o) nev).
struct VdvEpilogue {
  VdvTiles tl;
  double2 *vdv;
  int32_t const *ops;
  int nev, n_comp, n_cols, Lt, t0;
  struct Pre {};
  __device__ __forceinline__ Pre prepare(int, int, int) const { return Pre{}; }
  __device__ __forceinline__ void operator()(Pre const &, int it, int row, int col0,
                                             float const (&hi)[kColsW],
                                             float const (&lo)[kColsW]) const {
    int mt, nt, slot;
    tl.decode(it, mt, nt, slot);
    int const i = mt * (kTM / 2) + row / 2;
    if (i >= nev) return;
    int32_t const *expo =
        reinterpret_cast<int32_t const *>(tl.scratch + slot * tl.slot_bytes + tl.e_off);
    int const t = t0 + slot;
    int const ei = expo[i];
#pragma unroll
    for (int jj = 0; jj < kColsW; ++jj) {
      int const c = nt * kTN + col0 + jj;
      if (c < n_cols) {
        int const o = c / nev, j = c - o * nev;
        int const ec = o < n_comp ? expo[j] : expo[(1 + o) * nev + j];
        double *outd = reinterpret_cast<double *>(
            vdv + (static_cast<int64_t>(2 * ops[o]) * Lt + t) * nev * nev);
        double const val = ldexp(static_cast<double>(hi[jj]) + static_cast<double>(lo[jj]),
                                 ei + ec - 14);
        outd[2 * (i + static_cast<int64_t>(nev) * j) + (row & 1)] = val;
      }
    }
  }
};

// The GEMM: m_tiles x n_tiles x batch tiles over persistent CTAs, kThreads
// threads each.
__global__ void __launch_bounds__(kThreads, 1)
    ozaki_gemm_kernel(VdvTiles tl, int32_t n_tiles, double2 *vdv, int32_t const *ops,
                      int32_t n_ops, int32_t n_comp, int32_t t0, Geometry g, int *err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  VdvEpilogue epi{tl, vdv, ops, g.nev, n_comp, n_ops * g.nev, g.Lt, t0};
  ozaki_tiles(smem, n_tiles, tl.k_tiles, tl, err, epi);
}

}  // namespace

namespace {
struct TcLayout {
  int64_t k_tiles, m_tiles, n_tiles;
  size_t a_bytes, b_bytes, e_off, slot_bytes;
};
TcLayout tc_layout(Geometry const &g, int32_t n_ops) {
  TcLayout L{};
  L.k_tiles = (g.dim_row + kTK / 2 - 1) / (kTK / 2);
  L.m_tiles = (2LL * g.nev + kTM - 1) / kTM;
  L.n_tiles = (static_cast<int64_t>(n_ops) * g.nev + kTN - 1) / kTN;  // all operators
  L.a_bytes = static_cast<size_t>(L.m_tiles * L.k_tiles) * kStageA;
  L.b_bytes = static_cast<size_t>(L.n_tiles * L.k_tiles) * kStageB;
  L.e_off = L.a_bytes + L.b_bytes;
  // exponents: the eigenvectors', then room for one set per operator
  L.slot_bytes =
      (L.e_off + static_cast<size_t>(1 + n_ops) * g.nev * sizeof(int32_t) + 1023) / 1024 * 1024;
  return L;
}
}  // namespace

size_t vdaggerv_tc_scratch_bytes(Geometry g, int32_t n_ops, int32_t batch) {
  return tc_layout(g, n_ops).slot_bytes * static_cast<size_t>(batch > 0 ? batch : 1);
}

int32_t vdaggerv_tc_batch(Geometry g, int32_t n_ops, int32_t sm_count, size_t max_bytes,
                          int32_t n_t) {
  TcLayout const L = tc_layout(g, n_ops);
  int64_t const per_t = L.m_tiles * L.n_tiles;  // tiles of one timeslice
  int64_t const sms = sm_count > 0 ? sm_count : 1;
  int64_t const nt = n_t > 0 ? n_t : 1;
  int64_t fit = static_cast<int64_t>(max_bytes / L.slot_bytes);
  if (fit > nt) fit = nt;
  if (fit < 1) fit = 1;
  // Persistent CTAs take the tiles of a launch in rounds of one tile per SM;
  // the batch with the fewest rounds over all nt timeslices wastes the least
  // of the last round of each launch (the smaller batch on a tie).
  int64_t best = 1, best_rounds = -1;
  for (int64_t b = 1; b <= fit; ++b) {
    int64_t const launches = (nt + b - 1) / b, last = nt - (launches - 1) * b;
    int64_t const rounds = (launches - 1) * ((per_t * b + sms - 1) / sms) +
                           (per_t * last + sms - 1) / sms;
    if (best_rounds < 0 || rounds < best_rounds) {
      best = b;
      best_rounds = rounds;
    }
  }
  return static_cast<int32_t>(best);
}

cudaError_t phase_fixed(longlong2 *phase_fx, double2 const *phase, int64_t n,
                        cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  phase_fixed_kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, stream>>>(phase_fx,
                                                                              phase, n);
  return cudaGetLastError();
}

cudaError_t vdaggerv_tc(double2 *vdv, double2 const *V, longlong2 const *phase_fx,
                        int32_t const *ops, int32_t n_comp, int32_t t0, int32_t nt, Geometry g,
                        void *scratch, size_t scratch_bytes, int *err, cudaStream_t stream,
                        cudaEvent_t const *t_ready, VdvDisplaced const *disp,
                        cudaEvent_t const *gemm_ev, int32_t n_gemm_ev, int32_t v_t0,
                        bool clear_scratch) {
  int32_t const n_disp = disp ? disp->n : 0;
  int32_t const n = n_comp + n_disp;
  if (n == 0 || nt == 0) return cudaSuccess;
  if (n_disp > 0 && (!disp->n_steps || !disp->steps || !disp->U || !disp->W ||
                     !disp->unit_phase || !disp->unit_op))
    return cudaErrorInvalidValue;
  TcLayout const L = tc_layout(g, n);
  if (L.k_tiles > 0x7fffffffLL / kTK) return cudaErrorInvalidValue;
  int64_t const batch = static_cast<int64_t>(scratch_bytes / L.slot_bytes);
  if (batch < 1) return cudaErrorInvalidValue;
  uint8_t *base = static_cast<uint8_t *>(scratch);
  cudaError_t e = cudaFuncSetAttribute(ozaki_gemm_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(kSmemBytes));
  if (e != cudaSuccess) return e;
  // Padding rows of the last tiles are never written by the slicing: clear
  // the slots once per build.
  if (clear_scratch) {
    e = cudaMemsetAsync(base, 0,
                        L.slot_bytes * static_cast<size_t>(std::min<int64_t>(batch, nt)), stream);
    if (e != cudaSuccess) return e;
  }
  int64_t const xs = L.k_tiles * (kTK / 2);
  unsigned const xb = static_cast<unsigned>((xs + 255) / 256);
  // slice_b_kernel: one warp per (k-tile, group of 8 eigenvectors)
  unsigned const bb =
      static_cast<unsigned>((L.k_tiles * ((g.nev + 7) / 8) * 32 + 255) / 256);
  size_t const links = static_cast<size_t>(g.dim_row / 3) * 27;  // of one timeslice
  int32_t gemm_k = 0;
  for (int32_t tb = t0; tb < t0 + nt; tb += static_cast<int32_t>(batch)) {
    int32_t const nb = static_cast<int32_t>(std::min<int64_t>(batch, t0 + nt - tb));
    for (int32_t b = 0; b < nb; ++b) {
      int32_t const t = tb + b;
      if (t_ready && t_ready[t]) {
        e = cudaStreamWaitEvent(stream, t_ready[t], 0);
        if (e != cudaSuccess) return e;
      }
      double2 const *Vt = V + static_cast<int64_t>(t - v_t0) * g.nev * g.dim_row;
      uint8_t *slot = base + b * L.slot_bytes;
      int32_t *expo = reinterpret_cast<int32_t *>(slot + L.e_off);
      colmax_kernel<<<g.nev, 256, 0, stream>>>(expo, Vt, g);
      slice_a_kernel<<<dim3(xb, g.nev), 256, 0, stream>>>(
          reinterpret_cast<uint16_t *>(slot), Vt, expo, static_cast<int32_t>(L.k_tiles), g);
      if (n_comp > 0)
        slice_b_kernel<<<bb, 256, 0, stream>>>(slot + L.a_bytes, Vt, phase_fx, ops, n_comp, expo,
                                                static_cast<int32_t>(L.k_tiles), 0, g);
      // Displaced operators: W = D(V_t) in the reference's in-place sweep
      // order, B = W with phase 1 and W's own column exponents.
      for (int32_t d = 0; d < n_disp; ++d) {
        int32_t const o = n_comp + d;
        e = cudaMemcpyAsync(disp->W, Vt, sizeof(double2) * g.nev * g.dim_row,
                            cudaMemcpyDeviceToDevice, stream);
        if (e != cudaSuccess) return e;
        for (int32_t k = 0; k < disp->n_steps[d]; ++k) {
          int32_t const *st = disp->steps + 2 * (static_cast<int64_t>(d) * kMaxDispSteps + k);
          e = displace(disp->W, disp->U + links * t, st[0], st[1], g, stream);
          if (e != cudaSuccess) return e;
        }
        int32_t *expo_w = expo + static_cast<int64_t>(1 + o) * g.nev;
        colmax_kernel<<<g.nev, 256, 0, stream>>>(expo_w, disp->W, g);
        slice_b_kernel<<<bb, 256, 0, stream>>>(slot + L.a_bytes, disp->W, disp->unit_phase,
                                                disp->unit_op, 1, expo_w,
                                                static_cast<int32_t>(L.k_tiles),
                                                static_cast<int64_t>(o) * g.nev, g);
      }
    }
    bool const timed = gemm_ev && 2 * gemm_k + 1 < n_gemm_ev;
    if (timed) {
      e = cudaEventRecord(gemm_ev[2 * gemm_k], stream);
      if (e != cudaSuccess) return e;
    }
    VdvTiles const tl{base, L.slot_bytes, L.a_bytes, L.e_off, static_cast<int32_t>(L.m_tiles),
                      static_cast<int32_t>(L.n_tiles), static_cast<int32_t>(L.k_tiles)};
    int64_t const n_tiles = L.m_tiles * L.n_tiles * nb;
    ozaki_gemm_kernel<<<static_cast<unsigned>(persistent_grid(n_tiles)), kThreads, kSmemBytes,
                        stream>>>(tl, static_cast<int32_t>(n_tiles), vdv, ops, n, n_comp, tb, g,
                                  err);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (timed) {
      e = cudaEventRecord(gemm_ev[2 * gemm_k + 1], stream);
      if (e != cudaSuccess) return e;
    }
    ++gemm_k;
  }
  return cudaSuccess;
}

int32_t vdaggerv_tc_gemm_launches(int32_t nt, int32_t batch) {
  return batch > 0 ? (nt + batch - 1) / batch : 0;
}

}  // namespace dev
}  // namespace slaph
