// FP64 kernels of the contraction engine (sm_103a).
//
// Each kernel restates one step of the reference path on the device; the
// reference file:line is given per kernel.  Complex values are double2,
// matrices column-major.
#include <cuda_runtime.h>

#include <cstdint>

#include "kernels.cuh"

namespace slaph {
namespace dev {

namespace {

__constant__ int32_t c_gamma_row[16][4];
__constant__ double2 c_gamma_val[16][4];

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 conjd(double2 a) { return make_double2(a.x, -a.y); }
// acc += a * b
__device__ __forceinline__ void cfma(double2 &acc, double2 a, double2 b) {
  acc.x = fma(a.x, b.x, fma(-a.y, b.y, acc.x));
  acc.y = fma(a.x, b.y, fma(a.y, b.x, acc.y));
}
// acc += conj(a) * b
__device__ __forceinline__ void cfmac(double2 &acc, double2 a, double2 b) {
  acc.x = fma(a.x, b.x, fma(a.y, b.y, acc.x));
  acc.y = fma(a.x, b.y, fma(-a.y, b.x, acc.y));
}

// Neumaier accumulator on complex values, include/KahanAccumulator.hpp:14-48;
// with kahan == 0 it is NativeAccumulator (:50-72).
struct Acc {
  double2 s, c;
  int kahan;
  __device__ explicit Acc(int k) : s(make_double2(0, 0)), c(make_double2(0, 0)), kahan(k) {}
  __device__ void add(double2 x) {
    if (!kahan) {
      s.x += x.x;
      s.y += x.y;
      return;
    }
    double2 const t = make_double2(s.x + x.x, s.y + x.y);
    if (hypot(s.x, s.y) >= hypot(x.x, x.y)) {
      c.x += (s.x - t.x) + x.x;
      c.y += (s.y - t.y) + x.y;
    } else {
      c.x += (x.x - t.x) + s.x;
      c.y += (x.y - t.y) + s.y;
    }
    s = t;
  }
  __device__ double2 value() const { return kahan ? make_double2(s.x + c.x, s.y + c.y) : s; }
};

__device__ __forceinline__ int64_t gidx() {
  return blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
}

// ---------------------------------------------------------------- momenta
// create_momenta, src/OperatorFactory.cpp:64-95: exp(-i (px x + py y + pz z)
// 2pi/L) with site index x*Ly*Lz + y*Lz + z.
__global__ void momenta_kernel(double2 *phase, int32_t const *mom, int32_t n_ops, Geometry g) {
  int64_t const vol = static_cast<int64_t>(g.Lx) * g.Ly * g.Lz;
  int64_t const k = gidx();
  if (k >= vol * n_ops) return;
  int const op = static_cast<int>(k / vol);
  int64_t const site = k % vol;
  int const x = static_cast<int>(site / (static_cast<int64_t>(g.Ly) * g.Lz));
  int const y = static_cast<int>((site / g.Lz) % g.Ly);
  int const z = static_cast<int>(site % g.Lz);
  double const ipx = mom[3 * op] * 2. * M_PI / static_cast<double>(g.Lx);
  double const ipy = mom[3 * op + 1] * 2. * M_PI / static_cast<double>(g.Ly);
  double const ipz = mom[3 * op + 2] * 2. * M_PI / static_cast<double>(g.Lz);
  double const arg = (ipx * x + ipy * y) + ipz * z;
  double s, c;
  sincos(arg, &s, &c);
  phase[k] = make_double2(c, -s);
}

// ---------------------------------------------------------------- VdaggerV
// OperatorFactory::build_vdaggerv, src/OperatorFactory.cpp:292-300:
// vdv = V^H (diag(mom) V), mom(x) = phase[x / 3].  64 x 64 output tile per
// CTA, 16 rows of V per step, 4 x 4 outputs per thread.
constexpr int VT = 64, VK = 16;

// kW: B = W (a displaced copy of V_t, one operator and timeslice per launch:
// ops[0] is the operator, t0 the timeslice) instead of diag(phase) V_t.
template <bool kW>
__global__ void __launch_bounds__(256) vdv_fp64_kernel(double2 *vdv, double2 const *V,
                                                       double2 const *phase,
                                                       int32_t const *ops, int32_t t0,
                                                       Geometry g, double2 const *W,
                                                       int32_t v_t0) {
  __shared__ double2 As[VK][VT];
  __shared__ double2 Bs[VK][VT];
  int const nev = g.nev;
  int64_t const dim_row = g.dim_row;
  int64_t const vol = dim_row / 3;
  int const tiles = (nev + VT - 1) / VT;
  int const i0 = (blockIdx.x % tiles) * VT, j0 = (blockIdx.x / tiles) * VT;
  int const op = ops[blockIdx.y];
  int const t = t0 + blockIdx.z;
  int const tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
  double2 const *Vt = V + static_cast<int64_t>(t - v_t0) * nev * dim_row;
  double2 const *ph = kW ? nullptr : phase + static_cast<int64_t>(op) * vol;
  double2 acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = make_double2(0, 0);

  for (int64_t x0 = 0; x0 < dim_row; x0 += VK) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      int const k = tid + 256 * q;
      int const xx = k % VK, ii = k / VK;
      int64_t const x = x0 + xx;
      int const i = i0 + ii, j = j0 + ii;
      double2 a = make_double2(0, 0), b = make_double2(0, 0);
      if (x < dim_row) {
        if (i < nev) a = Vt[static_cast<int64_t>(i) * dim_row + x];
        if (j < nev)
          b = kW ? W[static_cast<int64_t>(j) * dim_row + x]
                 : cmul(ph[x / 3], Vt[static_cast<int64_t>(j) * dim_row + x]);
      }
      As[xx][ii] = a;
      Bs[xx][ii] = b;
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < VK; ++kk) {
      double2 a[4], b[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        a[q] = As[kk][ty + 16 * q];
        b[q] = Bs[kk][tx + 16 * q];
      }
#pragma unroll
      for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) cfmac(acc[p][q], a[p], b[q]);
    }
    __syncthreads();
  }
  double2 *out = vdv + (static_cast<int64_t>(2 * op) * g.Lt + t) * nev * nev;
#pragma unroll
  for (int p = 0; p < 4; ++p)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      int const i = i0 + ty + 16 * p, j = j0 + tx + 16 * q;
      if (i < nev && j < nev) out[i + static_cast<int64_t>(nev) * j] = acc[p][q];
    }
}

__global__ void vdv_identity_kernel(double2 *vdv, int32_t op, Geometry g) {
  int64_t const blk = static_cast<int64_t>(g.nev) * g.nev;
  int64_t const k = gidx();
  if (k >= blk * g.Lt) return;
  int64_t const e = k % blk;
  int64_t const t = k / blk;
  double2 const v = make_double2((e % g.nev) == (e / g.nev) ? 1.0 : 0.0, 0.0);
  vdv[(static_cast<int64_t>(2 * op) * g.Lt + t) * blk + e] = v;
  vdv[(static_cast<int64_t>(2 * op + 1) * g.Lt + t) * blk + e] = v;
}

// return_vdaggerv(...).adjoint(), src/DilutedFactorFactory.cpp:53-54.
__global__ void vdv_dagger_kernel(double2 *vdv, int32_t n_ops, Geometry g) {
  int64_t const blk = static_cast<int64_t>(g.nev) * g.nev;
  int64_t const k = gidx();
  if (k >= blk * g.Lt * n_ops) return;
  int64_t const e = k % blk;
  int64_t const rest = k / blk;
  int64_t const t = rest % g.Lt, op = rest / g.Lt;
  int64_t const i = e % g.nev, j = e / g.nev;
  double2 const src = vdv[(2 * op * g.Lt + t) * blk + j + g.nev * i];
  vdv[((2 * op + 1) * g.Lt + t) * blk + e] = conjd(src);
}

// ---------------------------------------------------------------- factors
__device__ __forceinline__ double2 const *vdv_block(double2 const *vdv, int code, int t,
                                                    Geometry const &g) {
  return vdv + (static_cast<int64_t>(code) * g.Lt + t) * g.nev * static_cast<int64_t>(g.nev);
}
__device__ __forceinline__ double2 rnd(double2 const *noise, int r, int64_t blk,
                                       Geometry const &g) {
  return noise[static_cast<int64_t>(r) * g.Lt * 4 * g.nev + blk];
}
__device__ __forceinline__ int64_t peram_rows(Geometry const &g) {
  return 4LL * g.nev * g.Lt;
}
__device__ __forceinline__ double2 const *peram_of(double2 const *peram, int r,
                                                   Geometry const &g) {
  return peram + static_cast<int64_t>(r) * peram_rows(g) * g.nb * 4 * g.dilE;
}

// Q0 intermediate, src/DilutedFactorFactory.cpp:66-78:
// M[v, e + dilE d] = sum_{w = e mod dilE} rho_r2[d + 4(w + nev t)] vdv[v, w].
__global__ void q0m_kernel(double2 *out, Q0MInst const *inst, double2 const *vdv,
                           double2 const *noise, Geometry g) {
  Q0MInst const in = inst[blockIdx.y];
  int const nev = g.nev, eds = 4 * g.dilE;
  int const k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nev * eds) return;
  int const v = k % nev, c = k / nev;
  int const e = c % g.dilE, d = c / g.dilE;
  double2 const *m = vdv_block(vdv, in.vdv, in.t, g);
  double2 acc = make_double2(0, 0);
  for (int w = e; w < nev; w += g.dilE)
    cfma(acc, rnd(noise, in.r2, d + 4 * (w + static_cast<int64_t>(nev) * in.t), g),
         m[v + static_cast<int64_t>(nev) * w]);
  out[static_cast<int64_t>(blockIdx.y) * nev * eds + k] = acc;
}

// Q1 intermediate, src/DilutedFactorFactory.cpp:134-144:
// R[e + dilE d, j] = sum_{v = e mod dilE} conj(rho_r1[d + 4 v + 4 nev t]) vdv[v, j].
__global__ void q1r_kernel(double2 *out, Q1RInst const *inst, double2 const *vdv,
                           double2 const *noise, Geometry g) {
  Q1RInst const in = inst[blockIdx.y];
  int const nev = g.nev, eds = 4 * g.dilE;
  int const k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nev * eds) return;
  int const a = k % eds, j = k / eds;
  int const e = a % g.dilE, d = a / g.dilE;
  double2 const *m = vdv_block(vdv, in.vdv, in.t, g);
  double2 acc = make_double2(0, 0);
  for (int v = e; v < nev; v += g.dilE)
    cfmac(acc, rnd(noise, in.r1, d + 4 * (v + static_cast<int64_t>(nev) * in.t), g),
          m[v + static_cast<int64_t>(nev) * j]);
  out[static_cast<int64_t>(blockIdx.y) * nev * eds + k] = acc;
}

// Q2 intermediate, src/DilutedFactorFactory.cpp:203-218 (without the gamma_5
// signs, applied in q2_kernel):
// M[col dilE + e, row nev + v] = sum_w conj(P_r1[(4t + row) nev + w,
//                                               (4 b1 + col) dilE + e]) vdv[w, v].
// Per CTA a 32 x 64 tile of one dirac row; 16 w per step.
constexpr int MT = 32, NT = 64, KT = 16;
__global__ void __launch_bounds__(256) q2m_kernel(double2 *out, Q2MInst const *inst,
                                                  double2 const *vdv, double2 const *peram,
                                                  Geometry g) {
  __shared__ double2 As[KT][MT + 1];
  __shared__ double2 Bs[KT][NT];
  Q2MInst const in = inst[blockIdx.z];
  int const nev = g.nev, eds = 4 * g.dilE;
  int const ntile = (nev + NT - 1) / NT, mtile = (eds + MT - 1) / MT;
  int const row = blockIdx.y;  // dirac row of the perambulator block
  int const v0 = (blockIdx.x % ntile) * NT;
  int const a0 = (blockIdx.x / ntile) * MT;
  if (a0 >= mtile * MT) return;
  int const tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
  int64_t const rows = peram_rows(g);
  double2 const *P = peram_of(peram, in.r1, g) +
                     (static_cast<int64_t>(4 * in.t + row) * nev) +
                     rows * (static_cast<int64_t>(in.b1) * eds);
  double2 const *m = vdv_block(vdv, in.vdv, in.t, g);
  double2 acc[2][4];
#pragma unroll
  for (int p = 0; p < 2; ++p)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[p][q] = make_double2(0, 0);
  for (int w0 = 0; w0 < nev; w0 += KT) {
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      int const k = tid + 256 * q;
      int const ww = k % KT, aa = k / KT;
      int const w = w0 + ww, a = a0 + aa;
      As[ww][aa] = (w < nev && a < eds) ? P[w + rows * a] : make_double2(0, 0);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      int const k = tid + 256 * q;
      int const ww = k % KT, vv = k / KT;
      int const w = w0 + ww, v = v0 + vv;
      Bs[ww][vv] = (w < nev && v < nev) ? m[w + static_cast<int64_t>(nev) * v]
                                        : make_double2(0, 0);
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < KT; ++kk) {
      double2 a[2], b[4];
#pragma unroll
      for (int p = 0; p < 2; ++p) a[p] = As[kk][ty + 16 * p];
#pragma unroll
      for (int q = 0; q < 4; ++q) b[q] = Bs[kk][tx + 16 * q];
#pragma unroll
      for (int p = 0; p < 2; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) cfmac(acc[p][q], a[p], b[q]);
    }
    __syncthreads();
  }
  double2 *o = out + static_cast<int64_t>(blockIdx.z) * eds * 4 * nev;
#pragma unroll
  for (int p = 0; p < 2; ++p)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      int const a = a0 + ty + 16 * p, v = v0 + tx + 16 * q;
      if (a < eds && v < nev) o[a + static_cast<int64_t>(eds) * (row * nev + v)] = acc[p][q];
    }
}

// Q0 factor, src/DilutedFactorFactory.cpp:80-98:
// Q0[e1 + dilE g, d dilE + e2] = val[d] sum_{v = e1} M[v, d dilE + e2]
//                                conj(rho_r1[g + 4(v + nev t)]),  g = row[d].
__global__ void q0_kernel(double2 *slots, Q0Inst const *inst, double2 const *q0m,
                          double2 const *noise, Geometry g) {
  Q0Inst const in = inst[blockIdx.y];
  int const nev = g.nev, dilE = g.dilE, eds = 4 * dilE;
  int const k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= eds * eds) return;
  int const a = k % eds, b = k / eds;
  int const d = b / dilE;
  int const gr = c_gamma_row[in.gamma][d];
  double2 acc = make_double2(0, 0);
  if (a / dilE == gr) {
    int const e1 = a % dilE;
    double2 const *M = q0m + static_cast<int64_t>(in.m) * nev * eds;
    double2 const val = c_gamma_val[in.gamma][d];
    for (int v = e1; v < nev; v += dilE) {
      double2 const vm = cmul(val, M[v + static_cast<int64_t>(nev) * b]);
      double2 const cr =
          conjd(rnd(noise, in.r1, gr + 4 * (v + static_cast<int64_t>(nev) * in.t), g));
      cfma(acc, vm, cr);
    }
  }
  slots[static_cast<int64_t>(in.slot) * eds * eds + k] = acc;
}

// Q1 factor, src/DilutedFactorFactory.cpp:146-164:
// Q1[row dilE + e, col dilE + f] = val[row] sum_v R[row dilE + e, v]
//        P_r2[(4t + grow[row]) nev + v, (4b + col) dilE + f].
__global__ void q1_kernel(double2 *slots, Q1Inst const *inst, double2 const *q1r,
                          double2 const *peram, Geometry g) {
  Q1Inst const in = inst[blockIdx.y];
  int const nev = g.nev, dilE = g.dilE, eds = 4 * dilE;
  int const k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= eds * eds) return;
  int const a = k % eds, c = k / eds;
  int const row = a / dilE;
  int64_t const rows = peram_rows(g);
  double2 const *R = q1r + static_cast<int64_t>(in.r) * nev * eds;
  double2 const *P = peram_of(peram, in.r2, g) +
                     static_cast<int64_t>(4 * in.t + c_gamma_row[in.gamma][row]) * nev +
                     rows * (static_cast<int64_t>(in.b) * eds + c);
  double2 acc = make_double2(0, 0);
  for (int v = 0; v < nev; ++v) cfma(acc, R[a + static_cast<int64_t>(eds) * v], P[v]);
  slots[static_cast<int64_t>(in.slot) * eds * eds + k] = cmul(c_gamma_val[in.gamma][row], acc);
}

// Q2 factor, src/DilutedFactorFactory.cpp:214-243:
// Q2[r dilE + e, col dilE + f] = sum_bd val[bd] s(bd, r)
//     sum_v M[r dilE + e, bd nev + v] P_r2[(4t + grow[bd]) nev + v, (4 b2 + col) dilE + f]
// with the gamma_5 sign s = -1 when bd + r == 3 or |bd - r| > 1 (:215-216).
__global__ void q2_kernel(double2 *slots, Q2Inst const *inst, double2 const *q2m,
                          double2 const *peram, Geometry g) {
  Q2Inst const in = inst[blockIdx.y];
  int const nev = g.nev, dilE = g.dilE, eds = 4 * dilE;
  int const k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= eds * eds) return;
  int const a = k % eds, c = k / eds;
  int const r = a / dilE;
  int64_t const rows = peram_rows(g);
  double2 const *M = q2m + static_cast<int64_t>(in.m) * eds * 4 * nev;
  double2 const *Pr = peram_of(peram, in.r2, g) + rows * (static_cast<int64_t>(in.b2) * eds + c);
  double2 total = make_double2(0, 0);
  for (int bd = 0; bd < 4; ++bd) {
    double2 const *P = Pr + static_cast<int64_t>(4 * in.t + c_gamma_row[in.gamma][bd]) * nev;
    double2 const *Mb = M + a + static_cast<int64_t>(eds) * bd * nev;
    double2 acc = make_double2(0, 0);
    for (int v = 0; v < nev; ++v) cfma(acc, Mb[static_cast<int64_t>(eds) * v], P[v]);
    bool const flip = (bd + r == 3) || (bd - r > 1) || (r - bd > 1);
    double2 const val = c_gamma_val[in.gamma][bd];
    double2 const s = flip ? make_double2(-val.x, -val.y) : val;
    double2 const pr = cmul(s, acc);
    total.x += pr.x;
    total.y += pr.y;
  }
  slots[static_cast<int64_t>(in.slot) * eds * eds + k] = total;
}

// ---------------------------------------------------------------- products
// operator*(vector<DF>, vector<DF>) data part, src/DilutedFactor.cpp:40-41:
// C = A * B for eds x eds matrices; one CTA per product, operands in smem.
__global__ void __launch_bounds__(256) product_kernel(double2 *slots, ProdInst const *p,
                                                      int32_t eds) {
  extern __shared__ double2 sm[];
  ProdInst const in = p[blockIdx.x];
  int64_t const ms = static_cast<int64_t>(eds) * eds;
  double2 *As = sm, *Bs = sm + ms;
  double2 const *A = slots + in.a * ms;
  double2 const *B = slots + in.b * ms;
  for (int k = threadIdx.x; k < ms; k += blockDim.x) {
    As[k] = A[k];
    Bs[k] = B[k];
  }
  __syncthreads();
  double2 *C = slots + in.c * ms;
  for (int k = threadIdx.x; k < ms; k += blockDim.x) {
    int const i = k % eds, j = k / eds;
    double2 acc = make_double2(0, 0);
    for (int q = 0; q < eds; ++q) cfma(acc, As[i + eds * q], Bs[q + eds * j]);
    C[k] = acc;
  }
}

// ---------------------------------------------------------------- traces
// factor_to_trace, src/DilutedTrace.cpp:84-165: tr(L R) per entry (or tr(F)).
// One CTA per list, one warp per entry, one lane per row.
__global__ void __launch_bounds__(256) trace_kernel(double2 *values, TraceList const *lists,
                                                    int32_t const *which,
                                                    int32_t const *shape_i,
                                                    int32_t const *shape_j,
                                                    int64_t const *shape_off,
                                                    double2 const *slots, int32_t eds) {
  TraceList const L = lists[which[blockIdx.x]];
  int64_t const off = shape_off[L.shape];
  int const n = static_cast<int>(shape_off[L.shape + 1] - off);
  int const warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  int64_t const ms = static_cast<int64_t>(eds) * eds;
  for (int e = warp; e < n; e += blockDim.x / 32) {
    int const ia = shape_i[off + e], jb = shape_j[off + e];
    double2 const *A = slots + (static_cast<int64_t>(L.a_base) + ia) * ms;
    double2 acc = make_double2(0, 0);
    if (jb >= 0) {
      double2 const *B = slots + (static_cast<int64_t>(L.b_base) + jb) * ms;
      for (int i = lane; i < eds; i += 32) {
        double2 row = make_double2(0, 0);
        for (int j = 0; j < eds; ++j) cfma(row, A[i + eds * j], B[j + eds * i]);
        acc.x += row.x;
        acc.y += row.y;
      }
    } else {
      for (int i = lane; i < eds; i += 32) {
        acc.x += A[i + eds * i].x;
        acc.y += A[i + eds * i].y;
      }
    }
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
      acc.x += __shfl_down_sync(0xffffffffu, acc.x, s);
      acc.y += __shfl_down_sync(0xffffffffu, acc.y, s);
    }
    if (lane == 0) values[L.val_off + static_cast<int64_t>(e) * L.stride] = acc;
  }
}

// ---------------------------------------------------------------- terms
// resolve_request1/2/3 (src/Diagram.cpp:9-94) with inner_product
// (src/DilutedTrace.cpp:5-82): one thread per (request, slice pair), the
// reference's loop order and accumulator.
__global__ void term_kernel(double2 *term_val, Term const *terms, int64_t n,
                            TraceList const *lists, double2 const *values,
                            uint16_t const *shape_mask, int64_t const *shape_off,
                            int32_t kahan) {
  int64_t const k = gidx();
  if (k >= n) return;
  Term const t = terms[k];
  TraceList const L0 = lists[t.list[0]];
  int64_t const o0 = shape_off[L0.shape];
  int64_t const n0 = shape_off[L0.shape + 1] - o0;
  double2 const *x0 = values + L0.val_off;
  int64_t const s0 = L0.stride;
  uint16_t const *m0 = shape_mask + o0;
  double2 res;
  if (t.n == 1) {
    Acc a(kahan);
    for (int64_t e = 0; e < n0; ++e) a.add(x0[e * s0]);
    double2 const v = a.value();
    res = make_double2(v.x / static_cast<double>(n0), v.y / static_cast<double>(n0));
  } else {
    TraceList const L1 = lists[t.list[1]];
    int64_t const o1 = shape_off[L1.shape];
    int64_t const n1 = shape_off[L1.shape + 1] - o1;
    double2 const *x1 = values + L1.val_off;
    int64_t const s1 = L1.stride;
    uint16_t const *m1 = shape_mask + o1;
    int64_t num = 0;
    Acc result(kahan);
    if (t.n == 2) {
      for (int64_t l = 0; l < n0; ++l) {
        Acc rs(kahan);
        for (int64_t r = 0; r < n1; ++r) {
          if ((m0[l] & m1[r]) != 0u) continue;
          rs.add(x1[r * s1]);
          ++num;
        }
        result.add(cmul(x0[l * s0], rs.value()));
      }
    } else {
      TraceList const L2 = lists[t.list[2]];
      int64_t const o2 = shape_off[L2.shape];
      int64_t const n2 = shape_off[L2.shape + 1] - o2;
      double2 const *x2 = values + L2.val_off;
      int64_t const s2 = L2.stride;
      uint16_t const *m2 = shape_mask + o2;
      for (int64_t l = 0; l < n0; ++l)
        for (int64_t m = 0; m < n1; ++m) {
          Acc rs(kahan);
          for (int64_t r = 0; r < n2; ++r) {
            if ((m0[l] & m1[m] & m2[r]) != 0u) continue;
            rs.add(x2[r * s2]);
            ++num;
          }
          result.add(cmul(cmul(x0[l * s0], x1[m * s1]), rs.value()));
        }
    }
    double2 const v = result.value();
    double const dn = static_cast<double>(num);
    res = num ? make_double2(v.x / dn, v.y / dn) : make_double2(0, 0);
  }
  term_val[k] = res;
}

// Diagram::assemble (src/Diagram.cpp:96-114): correlator[dt][i] += c in the
// order the terms were produced.
__global__ void accumulate_kernel(double2 *running, int32_t const *seg_out,
                                  int64_t const *seg_off, int64_t n_seg, int32_t const *idx,
                                  double2 const *term_val) {
  int64_t const s = gidx();
  if (s >= n_seg) return;
  double2 acc = running[seg_out[s]];
  for (int64_t k = seg_off[s]; k < seg_off[s + 1]; ++k) {
    double2 const v = term_val[idx[k]];
    acc.x += v.x;
    acc.y += v.y;
  }
  running[seg_out[s]] = acc;
}

int blocks_for(int64_t n, int threads) {
  return static_cast<int>((n + threads - 1) / threads);
}

}  // namespace

// The gamma table of src/Gamma.cpp:18-246 (tmLQCD basis): for matrix m and
// column c the non-zero row and its value (+-1, +-i).
namespace {
// Gamma table (the data of src/Gamma.cpp:18-246): Gamma_m has, in column c, its
// single nonzero at row kGammaRow[m][c] with value kGammaVal[m][c] (re, im).
int32_t const kGammaRow[16][4] = {{2, 3, 0, 1}, {3, 2, 1, 0}, {3, 2, 1, 0}, {2, 3, 0, 1},
                                  {0, 1, 2, 3}, {0, 1, 2, 3}, {2, 3, 0, 1}, {3, 2, 1, 0},
                                  {3, 2, 1, 0}, {2, 3, 0, 1}, {1, 0, 3, 2}, {1, 0, 3, 2},
                                  {0, 1, 2, 3}, {1, 0, 3, 2}, {1, 0, 3, 2}, {0, 1, 2, 3}};
double const kGammaVal[16][4][2] = {
    {{1, 0}, {1, 0}, {1, 0}, {1, 0}},      {{0, -1}, {0, -1}, {0, 1}, {0, 1}},
    {{1, 0}, {-1, 0}, {-1, 0}, {1, 0}},    {{0, -1}, {0, 1}, {0, 1}, {0, -1}},
    {{1, 0}, {1, 0}, {1, 0}, {1, 0}},      {{1, 0}, {1, 0}, {-1, 0}, {-1, 0}},
    {{1, 0}, {1, 0}, {-1, 0}, {-1, 0}},    {{0, -1}, {0, -1}, {0, -1}, {0, -1}},
    {{1, 0}, {-1, 0}, {1, 0}, {-1, 0}},    {{0, -1}, {0, 1}, {0, -1}, {0, 1}},
    {{0, -1}, {0, -1}, {0, 1}, {0, 1}},    {{1, 0}, {-1, 0}, {-1, 0}, {1, 0}},
    {{0, -1}, {0, 1}, {0, 1}, {0, -1}},    {{0, -1}, {0, -1}, {0, -1}, {0, -1}},
    {{1, 0}, {-1, 0}, {1, 0}, {-1, 0}},    {{0, -1}, {0, 1}, {0, -1}, {0, 1}}};
}  // namespace

int32_t gamma_row_host(int32_t m, int32_t c) { return kGammaRow[m][c]; }
int32_t gamma_phase_host(int32_t m, int32_t c) {
  double const re = kGammaVal[m][c][0], im = kGammaVal[m][c][1];
  return re > 0 ? 0 : im > 0 ? 1 : re < 0 ? 2 : 3;
}

cudaError_t upload_gamma(cudaStream_t stream) {
  double2 v[16][4];
  for (int m = 0; m < 16; ++m)
    for (int c = 0; c < 4; ++c) v[m][c] = make_double2(kGammaVal[m][c][0], kGammaVal[m][c][1]);
  cudaError_t e = cudaMemcpyToSymbolAsync(c_gamma_row, kGammaRow, sizeof kGammaRow, 0,
                                          cudaMemcpyHostToDevice, stream);
  if (e != cudaSuccess) return e;
  return cudaMemcpyToSymbolAsync(c_gamma_val, v, sizeof v, 0, cudaMemcpyHostToDevice, stream);
}

cudaError_t momenta(double2 *phase, int32_t const *mom, int32_t n_ops, Geometry g,
                    cudaStream_t stream) {
  int64_t const n = static_cast<int64_t>(g.Lx) * g.Ly * g.Lz * n_ops;
  if (n == 0) return cudaSuccess;
  momenta_kernel<<<blocks_for(n, 256), 256, 0, stream>>>(phase, mom, n_ops, g);
  return cudaGetLastError();
}

cudaError_t vdaggerv_fp64(double2 *vdv, double2 const *V, double2 const *phase,
                          int32_t const *ops, int32_t n, int32_t t0, int32_t nt, Geometry g,
                          cudaStream_t stream, int32_t v_t0) {
  if (n == 0 || nt == 0) return cudaSuccess;
  int const tiles = (g.nev + VT - 1) / VT;
  dim3 grid(tiles * tiles, n, nt);
  vdv_fp64_kernel<false><<<grid, 256, 0, stream>>>(vdv, V, phase, ops, t0, g, nullptr, v_t0);
  return cudaGetLastError();
}

// displace_eigenvectors (src/OperatorFactory.cpp:33-55) for one step on a
// cubic lattice: W (a copy of V_t) is updated in place line by line, each line
// of the step's direction in increasing site index as the reference sweeps
// it, so a site reads the already-displaced value of a preceding neighbour.
// Forward: W(s) = U(s, d) W(s + d); backward: W(s) = U(s - d, d)^H W(s - d)
// (forward_uv / backward_uv, src/GaugeField.cpp:543-560).  U: links of the
// timeslice, [site][dir][a + 3 b].  One thread per (eigenvector, line).
__global__ void displace_kernel(double2 *W, double2 const *U, int32_t dir, int32_t forward,
                                Geometry g) {
  int const L = g.Lx;
  int64_t const lines = static_cast<int64_t>(L) * L;
  int64_t const k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (k >= lines * g.nev) return;
  int64_t const ev = k / lines, l = k % lines;
  int64_t stride, base;
  if (dir == 0) {
    stride = lines;
    base = l;
  } else if (dir == 1) {
    stride = L;
    base = (l / L) * lines + (l % L);
  } else {
    stride = 1;
    base = l * L;
  }
  double2 *col = W + ev * g.dim_row;
  double2 carry[3];  // forward: updated first site; backward: updated previous site
  for (int c = 0; c < L; ++c) {
    int64_t const s = base + c * stride;
    double2 v[3], out[3];
    double2 const *u;
    if (forward) {
      int64_t const up = base + ((c + 1) % L) * stride;
      bool const updated = c + 1 == L && c > 0;  // the wrap reads the updated first site
#pragma unroll
      for (int b = 0; b < 3; ++b) v[b] = updated ? carry[b] : col[3 * up + b];
      u = U + (s * 3 + dir) * 9;
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        double2 acc = make_double2(0, 0);
#pragma unroll
        for (int b = 0; b < 3; ++b) cfma(acc, u[a + 3 * b], v[b]);
        out[a] = acc;
      }
      if (c == 0)
#pragma unroll
        for (int a = 0; a < 3; ++a) carry[a] = out[a];
    } else {
      int64_t const dn = base + ((c + L - 1) % L) * stride;
#pragma unroll
      for (int b = 0; b < 3; ++b) v[b] = c == 0 ? col[3 * dn + b] : carry[b];
      u = U + (dn * 3 + dir) * 9;
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        double2 acc = make_double2(0, 0);
#pragma unroll
        for (int b = 0; b < 3; ++b) {
          double2 const ub = u[b + 3 * a];
          cfma(acc, make_double2(ub.x, -ub.y), v[b]);
        }
        out[a] = acc;
      }
#pragma unroll
      for (int a = 0; a < 3; ++a) carry[a] = out[a];
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) col[3 * s + a] = out[a];
  }
}

cudaError_t displace(double2 *W, double2 const *U, int32_t dir, int32_t forward, Geometry g,
                     cudaStream_t stream) {
  if (dir < 0 || dir > 2 || g.Lx != g.Ly || g.Lx != g.Lz) return cudaErrorInvalidValue;
  int64_t const n = static_cast<int64_t>(g.Lx) * g.Lx * g.nev;
  displace_kernel<<<blocks_for(n, 128), 128, 0, stream>>>(W, U, dir, forward, g);
  return cudaGetLastError();
}

cudaError_t vdaggerv_fp64_w(double2 *vdv, double2 const *V, double2 const *W,
                            int32_t const *op, int32_t t, Geometry g, cudaStream_t stream,
                            int32_t v_t0) {
  int const tiles = (g.nev + VT - 1) / VT;
  vdv_fp64_kernel<true><<<dim3(tiles * tiles, 1, 1), 256, 0, stream>>>(vdv, V, nullptr, op, t,
                                                                       g, W, v_t0);
  return cudaGetLastError();
}

cudaError_t vdaggerv_identity(double2 *vdv, int32_t op, Geometry g, cudaStream_t stream) {
  int64_t const n = static_cast<int64_t>(g.nev) * g.nev * g.Lt;
  vdv_identity_kernel<<<blocks_for(n, 256), 256, 0, stream>>>(vdv, op, g);
  return cudaGetLastError();
}

cudaError_t vdaggerv_daggers(double2 *vdv, int32_t n_ops, Geometry g, cudaStream_t stream) {
  int64_t const n = static_cast<int64_t>(g.nev) * g.nev * g.Lt * n_ops;
  if (n == 0) return cudaSuccess;
  vdv_dagger_kernel<<<blocks_for(n, 256), 256, 0, stream>>>(vdv, n_ops, g);
  return cudaGetLastError();
}

// Grids over instances are split in chunks of 65535 (gridDim.y limit).
template <typename Inst, typename F>
cudaError_t chunked(Inst const *inst, int64_t n, F &&launch) {
  for (int64_t s = 0; s < n; s += 65535) {
    int const c = static_cast<int>(n - s < 65535 ? n - s : 65535);
    launch(inst + s, c, s);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t q0m(double2 *out, Q0MInst const *inst, int64_t n, double2 const *vdv,
                double2 const *noise, Geometry g, cudaStream_t stream) {
  int64_t const per = static_cast<int64_t>(g.nev) * 4 * g.dilE;
  return chunked(inst, n, [&](Q0MInst const *p, int c, int64_t s) {
    q0m_kernel<<<dim3(blocks_for(per, 256), c), 256, 0, stream>>>(out + s * per, p, vdv, noise, g);
  });
}

cudaError_t q1r(double2 *out, Q1RInst const *inst, int64_t n, double2 const *vdv,
                double2 const *noise, Geometry g, cudaStream_t stream) {
  int64_t const per = static_cast<int64_t>(g.nev) * 4 * g.dilE;
  return chunked(inst, n, [&](Q1RInst const *p, int c, int64_t s) {
    q1r_kernel<<<dim3(blocks_for(per, 256), c), 256, 0, stream>>>(out + s * per, p, vdv, noise, g);
  });
}

cudaError_t q2m(double2 *out, Q2MInst const *inst, int64_t n, double2 const *vdv,
                double2 const *peram, Geometry g, cudaStream_t stream) {
  int const eds = 4 * g.dilE;
  int64_t const per = static_cast<int64_t>(eds) * 4 * g.nev;
  int const ntile = (g.nev + NT - 1) / NT, mtile = (eds + MT - 1) / MT;
  return chunked(inst, n, [&](Q2MInst const *p, int c, int64_t s) {
    q2m_kernel<<<dim3(ntile * mtile, 4, c), 256, 0, stream>>>(out + s * per, p, vdv, peram, g);
  });
}

cudaError_t q0(double2 *slots, Q0Inst const *inst, int64_t n, double2 const *q0m_,
               double2 const *noise, Geometry g, cudaStream_t stream) {
  int64_t const per = 16LL * g.dilE * g.dilE;
  return chunked(inst, n, [&](Q0Inst const *p, int c, int64_t) {
    q0_kernel<<<dim3(blocks_for(per, 256), c), 256, 0, stream>>>(slots, p, q0m_, noise, g);
  });
}

cudaError_t q1(double2 *slots, Q1Inst const *inst, int64_t n, double2 const *q1r_,
               double2 const *peram, Geometry g, cudaStream_t stream) {
  int64_t const per = 16LL * g.dilE * g.dilE;
  return chunked(inst, n, [&](Q1Inst const *p, int c, int64_t) {
    q1_kernel<<<dim3(blocks_for(per, 256), c), 256, 0, stream>>>(slots, p, q1r_, peram, g);
  });
}

cudaError_t q2(double2 *slots, Q2Inst const *inst, int64_t n, double2 const *q2m_,
               double2 const *peram, Geometry g, cudaStream_t stream) {
  int64_t const per = 16LL * g.dilE * g.dilE;
  return chunked(inst, n, [&](Q2Inst const *p, int c, int64_t) {
    q2_kernel<<<dim3(blocks_for(per, 256), c), 256, 0, stream>>>(slots, p, q2m_, peram, g);
  });
}

cudaError_t products(double2 *slots, ProdInst const *p, int64_t n, int32_t eds,
                     cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  size_t const smem = 2 * sizeof(double2) * eds * eds;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(product_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return e;
  }
  for (int64_t s = 0; s < n; s += 0x7fffffffLL) {
    int64_t const c = n - s < 0x7fffffffLL ? n - s : 0x7fffffffLL;
    product_kernel<<<static_cast<unsigned>(c), 256, smem, stream>>>(slots, p + s, eds);
  }
  return cudaGetLastError();
}

cudaError_t traces(double2 *values, TraceList const *lists, int32_t const *which,
                   int64_t n_which, int32_t const *shape_i, int32_t const *shape_j,
                   int64_t const *shape_off, double2 const *slots, int32_t eds,
                   cudaStream_t stream) {
  if (n_which == 0) return cudaSuccess;
  trace_kernel<<<static_cast<unsigned>(n_which), 256, 0, stream>>>(
      values, lists, which, shape_i, shape_j, shape_off, slots, eds);
  return cudaGetLastError();
}

cudaError_t terms(double2 *term_val, Term const *t, int64_t n, TraceList const *lists,
                  double2 const *values, uint16_t const *shape_mask,
                  int64_t const *shape_off, int32_t kahan, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  term_kernel<<<blocks_for(n, 128), 128, 0, stream>>>(term_val, t, n, lists, values,
                                                      shape_mask, shape_off, kahan);
  return cudaGetLastError();
}

cudaError_t accumulate(double2 *running, int32_t const *seg_out, int64_t const *seg_off,
                       int64_t n_seg, int32_t const *idx, double2 const *term_val,
                       cudaStream_t stream) {
  if (n_seg == 0) return cudaSuccess;
  accumulate_kernel<<<blocks_for(n_seg, 128), 128, 0, stream>>>(running, seg_out, seg_off,
                                                               n_seg, idx, term_val);
  return cudaGetLastError();
}

}  // namespace dev
}  // namespace slaph

// ---------------------------------------------------------------- double-float
// Split-precision traces for the mixed path.  Matrices are converted once to
// double-float form (hi = fl32(x), lo = fl32(x - hi)), 16 bytes per complex
// like the FP64 layout; tr(L R) is then a compensated dot product on the FP32
// units (error-free products via FMA, Knuth two-sum accumulation, the cross
// terms hi*lo added to the compensation), summed in FP64 across the warp.
// GB300's FP32 units are ~60x faster than its FP64 units.
namespace slaph {
namespace dev {
namespace {

// Each matrix in both layouts: dst_n[k] as stored (column-major), dst_t the
// transpose, so that tr(L R) = sum_k L[k] R^T[k] reads both operands with
// unit stride.
__global__ void split_df_kernel(float4 *dst_n, float4 *dst_t, double2 const *src, int64_t n,
                                int32_t eds) {
  int64_t const k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (k >= n) return;
  double2 const v = src[k];
  float const rh = static_cast<float>(v.x), ih = static_cast<float>(v.y);
  float const rl = static_cast<float>(v.x - static_cast<double>(rh));
  float const il = static_cast<float>(v.y - static_cast<double>(ih));
  float4 const f = make_float4(rh, rl, ih, il);
  int64_t const ms = static_cast<int64_t>(eds) * eds;
  int64_t const slot = k / ms;
  int const e = static_cast<int>(k % ms);
  int const i = e % eds, j = e / eds;
  dst_n[k] = f;
  dst_t[slot * ms + j + static_cast<int64_t>(eds) * i] = f;
}

struct DfAcc {
  float s, c;
};
// acc += (xh + xl)(yh + yl), dropping xl*yl (relative 2^-48): error-free
// product by FMA, Knuth two-sum into s, all low-order parts into c.
__device__ __forceinline__ void df_mac(DfAcc &a, float xh, float xl, float yh, float yl) {
  float const p = xh * yh;
  float const e = fmaf(xh, yh, -p);
  float const s = a.s + p;
  float const bb = s - a.s;
  float const err = (a.s - (s - bb)) + (p - bb);
  a.s = s;
  a.c += err + e + fmaf(xh, yl, xl * yh);
}

// Warp sum of (s, c) pairs with error-free two-sums (FP32 units only).
__device__ __forceinline__ void df_warp_sum(DfAcc &a) {
#pragma unroll
  for (int sh = 16; sh > 0; sh >>= 1) {
    float const os = __shfl_down_sync(0xffffffffu, a.s, sh);
    float const oc = __shfl_down_sync(0xffffffffu, a.c, sh);
    float const s = a.s + os;
    float const bb = s - a.s;
    float const err = (a.s - (s - bb)) + (os - bb);
    a.s = s;
    a.c += oc + err;
  }
}

__global__ void __launch_bounds__(256) trace_df_kernel(float4 *values, TraceList const *lists,
                                                       int32_t const *which,
                                                       int32_t const *shape_i,
                                                       int32_t const *shape_j,
                                                       int64_t const *shape_off,
                                                       float4 const *slots_n,
                                                       float4 const *slots_t, int32_t eds) {
  TraceList const L = lists[which[blockIdx.x]];
  int64_t const off = shape_off[L.shape];
  int const n = static_cast<int>(shape_off[L.shape + 1] - off);
  int const warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  int64_t const ms = static_cast<int64_t>(eds) * eds;
  for (int e = warp; e < n; e += blockDim.x / 32) {
    int const ia = shape_i[off + e], jb = shape_j[off + e];
    float4 const *A = slots_n + (static_cast<int64_t>(L.a_base) + ia) * ms;
    DfAcc ar{0.f, 0.f}, ai{0.f, 0.f};
    if (jb >= 0) {
      float4 const *B = slots_t + (static_cast<int64_t>(L.b_base) + jb) * ms;
      DfAcc br{0.f, 0.f}, bi{0.f, 0.f};  // second accumulator set (ILP)
      int64_t k = lane;
      for (; k + 32 < ms; k += 64) {
        float4 const x0 = A[k], y0 = B[k];
        float4 const x1 = A[k + 32], y1 = B[k + 32];
        df_mac(ar, x0.x, x0.y, y0.x, y0.y);
        df_mac(br, x1.x, x1.y, y1.x, y1.y);
        df_mac(ar, -x0.z, -x0.w, y0.z, y0.w);
        df_mac(br, -x1.z, -x1.w, y1.z, y1.w);
        df_mac(ai, x0.x, x0.y, y0.z, y0.w);
        df_mac(bi, x1.x, x1.y, y1.z, y1.w);
        df_mac(ai, x0.z, x0.w, y0.x, y0.y);
        df_mac(bi, x1.z, x1.w, y1.x, y1.y);
      }
      for (; k < ms; k += 32) {
        float4 const x = A[k], y = B[k];
        df_mac(ar, x.x, x.y, y.x, y.y);
        df_mac(ar, -x.z, -x.w, y.z, y.w);
        df_mac(ai, x.x, x.y, y.z, y.w);
        df_mac(ai, x.z, x.w, y.x, y.y);
      }
      df_mac(ar, br.s, br.c, 1.f, 0.f);
      df_mac(ai, bi.s, bi.c, 1.f, 0.f);
    } else {
      for (int i = lane; i < eds; i += 32) {
        float4 const x = A[i + static_cast<int64_t>(eds) * i];
        df_mac(ar, x.x, x.y, 1.f, 0.f);
        df_mac(ai, x.z, x.w, 1.f, 0.f);
      }
    }
    df_warp_sum(ar);
    df_warp_sum(ai);
    if (lane == 0)
      values[L.val_off + static_cast<int64_t>(e) * L.stride] =
          make_float4(ar.s, ar.c, ai.s, ai.c);
  }
}

// Double-float (s, c) pairs to FP64: values[k] = (s_re + c_re, s_im + c_im).
__global__ void df_to_fp64_kernel(double2 *dst, float4 const *src, int64_t n) {
  int64_t const k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (k >= n) return;
  float4 const v = src[k];
  dst[k] = make_double2(static_cast<double>(v.x) + static_cast<double>(v.y),
                        static_cast<double>(v.z) + static_cast<double>(v.w));
}

// Mixed path: C = A B in double-float arithmetic (operator*,
// src/DilutedFactor.cpp:40-41).  Both operands are staged in shared memory as
// stored (column-major): consecutive threads read consecutive rows of A and a
// broadcast element of B.  The result is written in both layouts, so products
// never pass through FP64.
__global__ void __launch_bounds__(256) product_df_kernel(float4 *slots_n, float4 *slots_t,
                                                         ProdInst const *p, int32_t eds) {
  extern __shared__ float4 sdf[];
  ProdInst const in = p[blockIdx.x];
  int64_t const ms = static_cast<int64_t>(eds) * eds;
  float4 *As = sdf, *Bs = sdf + ms;  // As[i + eds k] = A(i, k); Bs[k + eds j] = B(k, j)
  float4 const *A = slots_n + in.a * ms;
  float4 const *B = slots_n + in.b * ms;
  for (int k = threadIdx.x; k < ms; k += blockDim.x) {
    As[k] = A[k];
    Bs[k] = B[k];
  }
  __syncthreads();
  // Thread (i, c) computes the four entries (i, jb + c + u per), u = 0..3, of
  // each pass: one load of A(i, q) serves four multiply-adds, and the B loads
  // of a warp (one column per warp when eds >= 32) are broadcasts.
  int const per = blockDim.x / eds;
  int const i = threadIdx.x % eds, c = threadIdx.x / eds;
  if (c >= per) return;
  for (int jb = 0; jb < eds; jb += 4 * per) {
    DfAcc ar[4], ai[4];
    int jj[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      ar[u] = ai[u] = DfAcc{0.f, 0.f};
      jj[u] = min(jb + c + u * per, eds - 1);  // clamped: computed, not stored
    }
    for (int q = 0; q < eds; ++q) {
      float4 const x = As[i + eds * q];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        float4 const y = Bs[q + eds * jj[u]];
        df_mac(ar[u], x.x, x.y, y.x, y.y);
        df_mac(ar[u], -x.z, -x.w, y.z, y.w);
        df_mac(ai[u], x.x, x.y, y.z, y.w);
        df_mac(ai[u], x.z, x.w, y.x, y.y);
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      int const j = jb + c + u * per;
      if (j >= eds) break;
      float const rh = ar[u].s + ar[u].c, ih = ai[u].s + ai[u].c;
      float4 const f =
          make_float4(rh, ar[u].c - (rh - ar[u].s), ih, ai[u].c - (ih - ai[u].s));
      slots_n[in.c * ms + i + static_cast<int64_t>(eds) * j] = f;
      slots_t[in.c * ms + j + static_cast<int64_t>(eds) * i] = f;
    }
  }
}

}  // namespace

cudaError_t split_df(float4 *dst_n, float4 *dst_t, double2 const *src, int64_t n, int32_t eds,
                     cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  split_df_kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, stream>>>(dst_n, dst_t, src,
                                                                              n, eds);
  return cudaGetLastError();
}

cudaError_t products_df(float4 *slots_n, float4 *slots_t, ProdInst const *p, int64_t n,
                        int32_t eds, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  if (eds < 1 || eds > 256) return cudaErrorInvalidValue;  // one row per thread of 256
  size_t const smem = 2 * sizeof(float4) * eds * eds;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(product_df_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return e;
  }
  for (int64_t s0 = 0; s0 < n; s0 += 0x7fffffffLL) {
    int64_t const c = n - s0 < 0x7fffffffLL ? n - s0 : 0x7fffffffLL;
    product_df_kernel<<<static_cast<unsigned>(c), 256, smem, stream>>>(slots_n, slots_t, p + s0,
                                                                        eds);
  }
  return cudaGetLastError();
}

cudaError_t traces_df(float4 *values_df, TraceList const *lists, int32_t const *which,
                      int64_t n_which, int32_t const *shape_i, int32_t const *shape_j,
                      int64_t const *shape_off, float4 const *slots_n, float4 const *slots_t,
                      int32_t eds, cudaStream_t stream) {
  if (n_which == 0) return cudaSuccess;
  trace_df_kernel<<<static_cast<unsigned>(n_which), 256, 0, stream>>>(
      values_df, lists, which, shape_i, shape_j, shape_off, slots_n, slots_t, eds);
  return cudaGetLastError();
}

cudaError_t df_values_to_fp64(double2 *values, float4 const *values_df, int64_t n_values,
                              cudaStream_t stream) {
  if (n_values <= 0) return cudaSuccess;
  df_to_fp64_kernel<<<static_cast<unsigned>((n_values + 255) / 256), 256, 0, stream>>>(
      values, values_df, n_values);
  return cudaGetLastError();
}

}  // namespace dev
}  // namespace slaph

// ---------------------------------------------------------------- df factors
// Mixed path: the diluted-factor kernels above in double-float arithmetic.
// Inputs (VdaggerV, perambulators, noise) are converted once per
// configuration; the factors are written in both layouts for the products and
// traces.  Same formulas and reference lines as the FP64 kernels.
namespace slaph {
namespace dev {
namespace {

struct CDf {
  DfAcc r, i;
};
__device__ __forceinline__ CDf cdf_zero() { return CDf{{0.f, 0.f}, {0.f, 0.f}}; }
// acc += x * y
__device__ __forceinline__ void cdf_mac(CDf &a, float4 x, float4 y) {
  df_mac(a.r, x.x, x.y, y.x, y.y);
  df_mac(a.r, -x.z, -x.w, y.z, y.w);
  df_mac(a.i, x.x, x.y, y.z, y.w);
  df_mac(a.i, x.z, x.w, y.x, y.y);
}
// acc += conj(x) * y
__device__ __forceinline__ void cdf_macc(CDf &a, float4 x, float4 y) {
  df_mac(a.r, x.x, x.y, y.x, y.y);
  df_mac(a.r, x.z, x.w, y.z, y.w);
  df_mac(a.i, x.x, x.y, y.z, y.w);
  df_mac(a.i, -x.z, -x.w, y.x, y.y);
}
__device__ __forceinline__ float4 cdf_value(CDf const &a) {
  float const rh = a.r.s + a.r.c, ih = a.i.s + a.i.c;
  return make_float4(rh, a.r.c - (rh - a.r.s), ih, a.i.c - (ih - a.i.s));
}
// exact for the gamma values +-1, +-i
__device__ __forceinline__ float4 gamma_mul(double2 g, float4 v) {
  if (g.y == 0.0) return g.x > 0 ? v : make_float4(-v.x, -v.y, -v.z, -v.w);
  return g.y > 0 ? make_float4(-v.z, -v.w, v.x, v.y) : make_float4(v.z, v.w, -v.x, -v.y);
}
__device__ __forceinline__ float4 conj_df(float4 v) { return make_float4(v.x, v.y, -v.z, -v.w); }

__global__ void to_df_kernel(float4 *dst, double2 const *src, int64_t n) {
  int64_t const k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (k >= n) return;
  double2 const v = src[k];
  float const rh = static_cast<float>(v.x), ih = static_cast<float>(v.y);
  dst[k] = make_float4(rh, static_cast<float>(v.x - static_cast<double>(rh)), ih,
                       static_cast<float>(v.y - static_cast<double>(ih)));
}

__device__ __forceinline__ float4 const *vdv_block_df(float4 const *vdv, int code, int t,
                                                      Geometry const &g) {
  return vdv + (static_cast<int64_t>(code) * g.Lt + t) * g.nev * static_cast<int64_t>(g.nev);
}

__global__ void q0m_df_kernel(float4 *out, Q0MInst const *inst, float4 const *vdv,
                              float4 const *noise, Geometry g) {
  Q0MInst const in = inst[blockIdx.y];
  int const nev = g.nev, eds = 4 * g.dilE;
  int const k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nev * eds) return;
  int const v = k % nev, c = k / nev;
  int const e = c % g.dilE, d = c / g.dilE;
  float4 const *m = vdv_block_df(vdv, in.vdv, in.t, g);
  float4 const *rho = noise + static_cast<int64_t>(in.r2) * g.Lt * 4 * nev;
  CDf acc = cdf_zero();
  for (int w = e; w < nev; w += g.dilE)
    cdf_mac(acc, rho[d + 4 * (w + static_cast<int64_t>(nev) * in.t)],
            m[v + static_cast<int64_t>(nev) * w]);
  out[static_cast<int64_t>(blockIdx.y) * nev * eds + k] = cdf_value(acc);
}

__global__ void q1r_df_kernel(float4 *out, Q1RInst const *inst, float4 const *vdv,
                              float4 const *noise, Geometry g) {
  Q1RInst const in = inst[blockIdx.y];
  int const nev = g.nev, eds = 4 * g.dilE;
  int const k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nev * eds) return;
  int const a = k % eds, j = k / eds;
  int const e = a % g.dilE, d = a / g.dilE;
  float4 const *m = vdv_block_df(vdv, in.vdv, in.t, g);
  float4 const *rho = noise + static_cast<int64_t>(in.r1) * g.Lt * 4 * nev;
  CDf acc = cdf_zero();
  for (int v = e; v < nev; v += g.dilE)
    cdf_macc(acc, rho[d + 4 * (v + static_cast<int64_t>(nev) * in.t)],
             m[v + static_cast<int64_t>(nev) * j]);
  out[static_cast<int64_t>(blockIdx.y) * nev * eds + k] = cdf_value(acc);
}

__global__ void __launch_bounds__(256) q2m_df_kernel(float4 *out, Q2MInst const *inst,
                                                     float4 const *vdv, float4 const *peram,
                                                     Geometry g) {
  __shared__ float4 As[KT][MT + 1];
  __shared__ float4 Bs[KT][NT];
  Q2MInst const in = inst[blockIdx.z];
  int const nev = g.nev, eds = 4 * g.dilE;
  int const ntile = (nev + NT - 1) / NT, mtile = (eds + MT - 1) / MT;
  int const row = blockIdx.y;
  int const v0 = (blockIdx.x % ntile) * NT;
  int const a0 = (blockIdx.x / ntile) * MT;
  if (a0 >= mtile * MT) return;
  int const tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
  int64_t const rows = peram_rows(g);
  float4 const *P = peram + static_cast<int64_t>(in.r1) * rows * g.nb * 4 * g.dilE +
                    (static_cast<int64_t>(4 * in.t + row) * nev) +
                    rows * (static_cast<int64_t>(in.b1) * eds);
  float4 const *m = vdv_block_df(vdv, in.vdv, in.t, g);
  CDf acc[2][4];
#pragma unroll
  for (int p = 0; p < 2; ++p)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[p][q] = cdf_zero();
  float4 const z = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int w0 = 0; w0 < nev; w0 += KT) {
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      int const k = tid + 256 * q;
      int const ww = k % KT, aa = k / KT;
      int const w = w0 + ww, a = a0 + aa;
      As[ww][aa] = (w < nev && a < eds) ? P[w + rows * a] : z;
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      int const k = tid + 256 * q;
      int const ww = k % KT, vv = k / KT;
      int const w = w0 + ww, v = v0 + vv;
      Bs[ww][vv] = (w < nev && v < nev) ? m[w + static_cast<int64_t>(nev) * v] : z;
    }
    __syncthreads();
    for (int kk = 0; kk < KT; ++kk) {
      float4 a[2], b[4];
#pragma unroll
      for (int p = 0; p < 2; ++p) a[p] = As[kk][ty + 16 * p];
#pragma unroll
      for (int q = 0; q < 4; ++q) b[q] = Bs[kk][tx + 16 * q];
#pragma unroll
      for (int p = 0; p < 2; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) cdf_macc(acc[p][q], a[p], b[q]);
    }
    __syncthreads();
  }
  float4 *o = out + static_cast<int64_t>(blockIdx.z) * eds * 4 * nev;
#pragma unroll
  for (int p = 0; p < 2; ++p)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      int const a = a0 + ty + 16 * p, v = v0 + tx + 16 * q;
      if (a < eds && v < nev)
        o[a + static_cast<int64_t>(eds) * (row * nev + v)] = cdf_value(acc[p][q]);
    }
}

__device__ __forceinline__ void store_factor_df(float4 *sn, float4 *st, int slot, int k, int eds,
                                                float4 v) {
  int64_t const ms = static_cast<int64_t>(eds) * eds;
  int const i = k % eds, j = k / eds;
  sn[slot * ms + k] = v;
  st[slot * ms + j + static_cast<int64_t>(eds) * i] = v;
}

__global__ void q0_df_kernel(float4 *sn, float4 *st, Q0Inst const *inst, float4 const *q0m,
                             float4 const *noise, Geometry g) {
  Q0Inst const in = inst[blockIdx.y];
  int const nev = g.nev, dilE = g.dilE, eds = 4 * dilE;
  int const k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= eds * eds) return;
  int const a = k % eds, b = k / eds;
  int const d = b / dilE;
  int const gr = c_gamma_row[in.gamma][d];
  CDf acc = cdf_zero();
  if (a / dilE == gr) {
    int const e1 = a % dilE;
    float4 const *M = q0m + static_cast<int64_t>(in.m) * nev * eds;
    float4 const *rho = noise + static_cast<int64_t>(in.r1) * g.Lt * 4 * nev;
    double2 const val = c_gamma_val[in.gamma][d];
    for (int v = e1; v < nev; v += dilE)
      cdf_mac(acc, gamma_mul(val, M[v + static_cast<int64_t>(nev) * b]),
              conj_df(rho[gr + 4 * (v + static_cast<int64_t>(nev) * in.t)]));
  }
  store_factor_df(sn, st, in.slot, k, eds, cdf_value(acc));
}

__global__ void q1_df_kernel(float4 *sn, float4 *st, Q1Inst const *inst, float4 const *q1r,
                             float4 const *peram, Geometry g) {
  Q1Inst const in = inst[blockIdx.y];
  int const nev = g.nev, dilE = g.dilE, eds = 4 * dilE;
  int const k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= eds * eds) return;
  int const a = k % eds, c = k / eds;
  int const row = a / dilE;
  int64_t const rows = peram_rows(g);
  float4 const *R = q1r + static_cast<int64_t>(in.r) * nev * eds;
  float4 const *P = peram + static_cast<int64_t>(in.r2) * rows * g.nb * 4 * g.dilE +
                    static_cast<int64_t>(4 * in.t + c_gamma_row[in.gamma][row]) * nev +
                    rows * (static_cast<int64_t>(in.b) * eds + c);
  CDf acc = cdf_zero();
  for (int v = 0; v < nev; ++v) cdf_mac(acc, R[a + static_cast<int64_t>(eds) * v], P[v]);
  store_factor_df(sn, st, in.slot, k, eds, gamma_mul(c_gamma_val[in.gamma][row], cdf_value(acc)));
}

__global__ void q2_df_kernel(float4 *sn, float4 *st, Q2Inst const *inst, float4 const *q2m,
                             float4 const *peram, Geometry g) {
  Q2Inst const in = inst[blockIdx.y];
  int const nev = g.nev, dilE = g.dilE, eds = 4 * dilE;
  int const k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= eds * eds) return;
  int const a = k % eds, c = k / eds;
  int const r = a / dilE;
  int64_t const rows = peram_rows(g);
  float4 const *M = q2m + static_cast<int64_t>(in.m) * eds * 4 * nev;
  float4 const *Pr = peram + static_cast<int64_t>(in.r2) * rows * g.nb * 4 * g.dilE +
                     rows * (static_cast<int64_t>(in.b2) * eds + c);
  CDf total = cdf_zero();
  for (int bd = 0; bd < 4; ++bd) {
    float4 const *P = Pr + static_cast<int64_t>(4 * in.t + c_gamma_row[in.gamma][bd]) * nev;
    float4 const *Mb = M + a + static_cast<int64_t>(eds) * bd * nev;
    bool const flip = (bd + r == 3) || (bd - r > 1) || (r - bd > 1);
    double2 const val = c_gamma_val[in.gamma][bd];
    double2 const s = flip ? make_double2(-val.x, -val.y) : val;
    for (int v = 0; v < nev; ++v)
      cdf_mac(total, gamma_mul(s, Mb[static_cast<int64_t>(eds) * v]), P[v]);
  }
  store_factor_df(sn, st, in.slot, k, eds, cdf_value(total));
}

int blocks256(int64_t n) { return static_cast<int>((n + 255) / 256); }

}  // namespace

cudaError_t to_df(float4 *dst, double2 const *src, int64_t n, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  to_df_kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, stream>>>(dst, src, n);
  return cudaGetLastError();
}

cudaError_t factors_df(float4 *sn, float4 *st, float4 *q0m_buf, float4 *q1r_buf,
                       float4 *q2m_buf, Q0MInst const *q0m_i, int64_t n_q0m,
                       Q1RInst const *q1r_i, int64_t n_q1r, Q2MInst const *q2m_i, int64_t n_q2m,
                       Q0Inst const *q0_i, int64_t n_q0, Q1Inst const *q1_i, int64_t n_q1,
                       Q2Inst const *q2_i, int64_t n_q2, float4 const *vdv,
                       float4 const *noise, float4 const *peram, Geometry g,
                       cudaStream_t stream) {
  int const eds = 4 * g.dilE;
  int64_t const per_m = static_cast<int64_t>(g.nev) * eds;
  int64_t const per_f = static_cast<int64_t>(eds) * eds;
  cudaError_t e;
  e = chunked(q0m_i, n_q0m, [&](Q0MInst const *p, int c, int64_t s) {
    q0m_df_kernel<<<dim3(blocks256(per_m), c), 256, 0, stream>>>(q0m_buf + s * per_m, p, vdv,
                                                                 noise, g);
  });
  if (e != cudaSuccess) return e;
  e = chunked(q1r_i, n_q1r, [&](Q1RInst const *p, int c, int64_t s) {
    q1r_df_kernel<<<dim3(blocks256(per_m), c), 256, 0, stream>>>(q1r_buf + s * per_m, p, vdv,
                                                                 noise, g);
  });
  if (e != cudaSuccess) return e;
  int const ntile = (g.nev + NT - 1) / NT, mtile = (eds + MT - 1) / MT;
  int64_t const per_q2m = static_cast<int64_t>(eds) * 4 * g.nev;
  e = chunked(q2m_i, n_q2m, [&](Q2MInst const *p, int c, int64_t s) {
    q2m_df_kernel<<<dim3(ntile * mtile, 4, c), 256, 0, stream>>>(q2m_buf + s * per_q2m, p, vdv,
                                                                 peram, g);
  });
  if (e != cudaSuccess) return e;
  e = chunked(q0_i, n_q0, [&](Q0Inst const *p, int c, int64_t) {
    q0_df_kernel<<<dim3(blocks256(per_f), c), 256, 0, stream>>>(sn, st, p, q0m_buf, noise, g);
  });
  if (e != cudaSuccess) return e;
  e = chunked(q1_i, n_q1, [&](Q1Inst const *p, int c, int64_t) {
    q1_df_kernel<<<dim3(blocks256(per_f), c), 256, 0, stream>>>(sn, st, p, q1r_buf, peram, g);
  });
  if (e != cudaSuccess) return e;
  return chunked(q2_i, n_q2, [&](Q2Inst const *p, int c, int64_t) {
    q2_df_kernel<<<dim3(blocks256(per_f), c), 256, 0, stream>>>(sn, st, p, q2m_buf, peram, g);
  });
}

}  // namespace dev
}  // namespace slaph
