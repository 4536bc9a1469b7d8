// Diluted factors Q1 and Q2 on the tensor cores (tcgen05, sm_103a).
//
// The factor builders of src/DilutedFactorFactory.cpp are products over the
// eigenvector index with K = nev:
//   Q2M[t,b1,r1,vdv](a, bd nev + v) = sum_w conj(P_r1((4t+bd) nev + w, b1 eds + a)) VdV_t(w, v)
//     (:200-218; one dense GEMM per timeslice: perambulator rows x VdaggerV columns)
//   X1[t](r a, (r2 b d) c) = sum_v Q1R_r(a, v) P_r2((4t+d) nev + v, b eds + c)
//     (:146-164 for all four Dirac blocks d at once; Q1 picks one block per row
//      block and scales it by the gamma phase)
//   Q2(a, c) = sum_bd sum_v s(bd, a) Gval[bd] Q2M_m(a, bd nev + v) P_r2((4t+Grow[bd]) nev + v, b2 eds + c)
//     (:221-243 with K = (bd, v), the gamma_5 signs s folded into the rows and
//      the gamma phases into the columns)
// They run on the split-BF16 tile pipeline of tc_common.cuh (the GEMM kernel
// of trace_tc.cu, whose epilogue writes dense FP64 complex outputs).  Operand
// rows and columns are gathered from up to four strided segments of a source
// array, each with an exact factor +-1, +-i, and cut into slices here; K is
// padded with zeros to whole k-tiles.
#include <cuda_runtime.h>

#include <cstdint>

#include "kernels.cuh"
#include "tc_common.cuh"

namespace slaph {
namespace dev {

__constant__ int32_t c_gamma_row_tc[16][4];
__constant__ int32_t c_gamma_phase_tc[16][4];

namespace {

using namespace tc;

constexpr int kGThreads = 128;

__device__ __forceinline__ unsigned long long absbits(double2 v) {
  unsigned long long const a = __double_as_longlong(v.x) & 0x7FFFFFFFFFFFFFFFULL;
  unsigned long long const b = __double_as_longlong(v.y) & 0x7FFFFFFFFFFFFFFFULL;
  return a > b ? a : b;
}
__device__ __forceinline__ unsigned long long absbits(float4 v) {
  unsigned int const a = __float_as_uint(v.x) & 0x7FFFFFFFu;
  unsigned int const b = __float_as_uint(v.z) & 0x7FFFFFFFu;
  return a > b ? a : b;
}
__device__ __forceinline__ int expo_of(unsigned long long b, double2 const *) {
  return expo_of_absbits64(b);
}
__device__ __forceinline__ int expo_of(unsigned long long b, float4 const *) {
  return expo_of_absbits(static_cast<unsigned int>(b));
}
__device__ __forceinline__ void to_fixed(double2 v, int e, long long &fr, long long &fi) {
  fr = fixed55(v.x, e);
  fi = fixed55(v.y, e);
}
__device__ __forceinline__ void to_fixed(float4 v, int e, long long &fr, long long &fi) {
  fr = fixed55f(v.x, e) + fixed55f(v.y, e);
  fi = fixed55f(v.z, e) + fixed55f(v.w, e);
}

// One operand row (A) or column (B) per CTA.  Exponent of its largest |re|,
// |im| over all segments, then the slices of (conj?)(factor x value).
template <bool kIsA, typename T>
__global__ void __launch_bounds__(kGThreads)
    gvec_slice_kernel(uint8_t *scratch, int32_t *expo, GVec const *items, T const *src,
                      int32_t k_tiles, int32_t conj) {
  GVec const it = items[blockIdx.x];
  int64_t const K = static_cast<int64_t>(it.n_seg) * it.seg_len;
  int64_t const Kp = static_cast<int64_t>(k_tiles) * (kTK / 2);
  unsigned long long mx = 0;
  for (int64_t k = threadIdx.x; k < K; k += kGThreads) {
    int const s = static_cast<int>(k / it.seg_len);
    int64_t const j = k - static_cast<int64_t>(s) * it.seg_len;
    T const v = src[it.seg[s].src + j * it.stride];
    unsigned long long const b = absbits(v);
    mx = b > mx ? b : mx;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long const y = __shfl_xor_sync(0xffffffffu, mx, o);
    mx = y > mx ? y : mx;
  }
  __shared__ unsigned long long red[kGThreads / 32];
  if (threadIdx.x % 32 == 0) red[threadIdx.x / 32] = mx;
  __syncthreads();
  mx = red[0];
#pragma unroll
  for (int w = 1; w < kGThreads / 32; ++w) mx = red[w] > mx ? red[w] : mx;
  int const e = expo_of(mx, src);
  if (threadIdx.x == 0) expo[it.expo] = e;
  uint8_t *region = scratch + it.dst;
  for (int64_t k = threadIdx.x; k < Kp; k += kGThreads) {
    long long fr = 0, fi = 0;
    if (k < K) {
      int const s = static_cast<int>(k / it.seg_len);
      int64_t const j = k - static_cast<int64_t>(s) * it.seg_len;
      to_fixed(src[it.seg[s].src + j * it.stride], e, fr, fi);
      long long const r = fr, i = fi;
      switch (it.seg[s].factor & 3) {
        case 1: fr = -i; fi = r; break;   // x i
        case 2: fr = -r; fi = -i; break;  // x -1
        case 3: fr = i; fi = -r; break;   // x -i
        default: break;
      }
      if (conj) fi = -fi;
    }
    if (kIsA)
      put_a_fx(region, k_tiles, it.row, k, fr, fi);
    else
      put_b_fx(region, k_tiles, it.row, k, fr, fi);
  }
}

__device__ __forceinline__ float4 df_of(double2 v) {
  float const rh = static_cast<float>(v.x), ih = static_cast<float>(v.y);
  return make_float4(rh, static_cast<float>(v.x - static_cast<double>(rh)), ih,
                     static_cast<float>(v.y - static_cast<double>(ih)));
}
__device__ __forceinline__ double2 phase_mul(int code, double2 v) {
  switch (code & 3) {
    case 1: return make_double2(-v.y, v.x);
    case 2: return make_double2(-v.x, -v.y);
    case 3: return make_double2(v.y, -v.x);
    default: return v;
  }
}

// Q1 (src/DilutedFactorFactory.cpp:146-164) from X1: entry (a, c) of the
// factor is gamma_phase[row] X1[row0 + a, col0 + Grow[row] eds + c] with
// row = a / dilE; written double-float in both layouts.
__global__ void q1_gather_kernel(float4 *sn, float4 *st, Q1Gather const *g, double2 const *x,
                                 int32_t dilE) {
  Q1Gather const q = g[blockIdx.y];
  int const eds = 4 * dilE;
  int const k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= eds * eds) return;
  int const a = k % eds, c = k / eds;
  int const row = a / dilE;
  double2 const v = x[q.x_off + (q.row0 + a) +
                      static_cast<int64_t>(q.ld) *
                          (q.col0 + c_gamma_row_tc[q.gamma][row] * eds + c)];
  float4 const f = df_of(phase_mul(c_gamma_phase_tc[q.gamma][row], v));
  int64_t const ms = static_cast<int64_t>(eds) * eds;
  sn[q.slot * ms + k] = f;
  st[q.slot * ms + c + static_cast<int64_t>(eds) * a] = f;
}

// Q2 from its GEMM output: entry (a, c) at y[off + a + ld c].
__global__ void q2_gather_kernel(float4 *sn, float4 *st, Q2Gather const *g, double2 const *y,
                                 int32_t eds) {
  Q2Gather const q = g[blockIdx.y];
  int const k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= eds * eds) return;
  int const a = k % eds, c = k / eds;
  float4 const f = df_of(y[q.off + a + static_cast<int64_t>(q.ld) * c]);
  int64_t const ms = static_cast<int64_t>(eds) * eds;
  sn[q.slot * ms + k] = f;
  st[q.slot * ms + c + static_cast<int64_t>(eds) * a] = f;
}

template <typename I, typename F>
cudaError_t in_chunks(I const *p, int64_t n, F &&launch) {
  for (int64_t s = 0; s < n; s += 65535) {
    int const c = static_cast<int>(n - s < 65535 ? n - s : 65535);
    launch(p + s, c);
    cudaError_t const e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace

cudaError_t upload_gamma_tc(cudaStream_t stream) {
  int32_t row[16][4], ph[16][4];
  for (int m = 0; m < 16; ++m)
    for (int c = 0; c < 4; ++c) {
      row[m][c] = gamma_row_host(m, c);
      ph[m][c] = gamma_phase_host(m, c);
    }
  cudaError_t e = cudaMemcpyToSymbolAsync(c_gamma_row_tc, row, sizeof row, 0,
                                          cudaMemcpyHostToDevice, stream);
  if (e != cudaSuccess) return e;
  return cudaMemcpyToSymbolAsync(c_gamma_phase_tc, ph, sizeof ph, 0, cudaMemcpyHostToDevice,
                                 stream);
}

cudaError_t gvec_slice_f64(uint8_t *scratch, int32_t *expo, GVec const *items, int64_t n,
                           bool is_a, bool conj, double2 const *src, int32_t k_tiles,
                           cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  if (is_a)
    gvec_slice_kernel<true, double2><<<static_cast<unsigned>(n), kGThreads, 0, stream>>>(
        scratch, expo, items, src, k_tiles, conj ? 1 : 0);
  else
    gvec_slice_kernel<false, double2><<<static_cast<unsigned>(n), kGThreads, 0, stream>>>(
        scratch, expo, items, src, k_tiles, conj ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t gvec_slice_df(uint8_t *scratch, int32_t *expo, GVec const *items, int64_t n,
                          bool is_a, bool conj, float4 const *src, int32_t k_tiles,
                          cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  if (is_a)
    gvec_slice_kernel<true, float4><<<static_cast<unsigned>(n), kGThreads, 0, stream>>>(
        scratch, expo, items, src, k_tiles, conj ? 1 : 0);
  else
    gvec_slice_kernel<false, float4><<<static_cast<unsigned>(n), kGThreads, 0, stream>>>(
        scratch, expo, items, src, k_tiles, conj ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t q1_gather(float4 *sn, float4 *st, Q1Gather const *g, int64_t n, double2 const *x,
                      int32_t dilE, cudaStream_t stream) {
  int const eds = 4 * dilE;
  unsigned const bx = static_cast<unsigned>((eds * eds + 255) / 256);
  return in_chunks(g, n, [&](Q1Gather const *p, int c) {
    q1_gather_kernel<<<dim3(bx, c), 256, 0, stream>>>(sn, st, p, x, dilE);
  });
}

cudaError_t q2_gather(float4 *sn, float4 *st, Q2Gather const *g, int64_t n, double2 const *y,
                      int32_t eds, cudaStream_t stream) {
  unsigned const bx = static_cast<unsigned>((eds * eds + 255) / 256);
  return in_chunks(g, n, [&](Q2Gather const *p, int c) {
    q2_gather_kernel<<<dim3(bx, c), 256, 0, stream>>>(sn, st, p, y, eds);
  });
}

int32_t gemm_k_tiles(int64_t K) { return static_cast<int32_t>((K + kTK / 2 - 1) / (kTK / 2)); }

}  // namespace dev
}  // namespace slaph
