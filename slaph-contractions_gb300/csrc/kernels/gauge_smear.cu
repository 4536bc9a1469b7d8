// HYP smearing of the spatial gauge links (GaugeField::smearing_hyp,
// src/GaugeField.cpp:322-427), FP64, every timeslice of a chunk at once.
//
// One iteration is two launches:
//   inner: one thread per (timeslice, site, direction, perpendicular n) builds
//          the decorated link  P(U(s,d) (1 - a2) + (a2 / 2) staple_p)  where
//          staple_p is the up and down staple of U in direction p = get_dirs(d)[n]
//          (:336-376), stored at slot d + 3 n;
//   outer: one thread per (timeslice, site, direction) sums the staples of the
//          decorated links in both other directions, each taken from the slot
//          decor(., plane) of the plane that excludes it (:380-416), and
//          replaces U(s,d) by P(U(s,d) (1 - a1) + (a1 / 4) outer).
// Only a thread's own link is read from U in the outer launch, so it updates U
// in place.  P is proj_to_su3_imp (:203-210): M (M^H M)^(-1/2) scaled by the
// principal cube root of 1/det, with (M^H M)^(-1/2) from a cyclic complex
// Jacobi eigen-decomposition (the principal square root of a Hermitian
// positive-definite matrix is V diag(sqrt(lambda)) V^H).
//
// Sites and neighbours follow GaugeField::init (src/GaugeField.cpp:39-98) on a
// cubic lattice: s = (x0 L + x1) L + x2, direction d steps x_d periodically.
// Links: [site][dir][a + 3 b] (column-major 3x3), 9 complex per link.
#include <cuda_runtime.h>

#include <cstdint>

#include "kernels.cuh"

namespace slaph {
namespace dev {
namespace {

struct M3 {
  double2 e[9];  // (a, b) at a + 3 b
};

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) {
  return make_double2(a.x + b.x, a.y + b.y);
}
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double cnorm(double2 a) { return a.x * a.x + a.y * a.y; }

__device__ __forceinline__ double2 csub(double2 a, double2 b) {
  return make_double2(a.x - b.x, a.y - b.y);
}
__device__ __forceinline__ double2 det3(M3 const &m) {
  double2 const c0 = csub(cmul(m.e[4], m.e[8]), cmul(m.e[7], m.e[5]));
  double2 const c1 = csub(cmul(m.e[1], m.e[8]), cmul(m.e[7], m.e[2]));
  double2 const c2 = csub(cmul(m.e[1], m.e[5]), cmul(m.e[4], m.e[2]));
  return cadd(csub(cmul(m.e[0], c0), cmul(m.e[3], c1)), cmul(m.e[6], c2));
}

__device__ __forceinline__ M3 load(double2 const *p) {
  M3 m;
#pragma unroll
  for (int i = 0; i < 9; ++i) m.e[i] = p[i];
  return m;
}
__device__ __forceinline__ void store(double2 *p, M3 const &m) {
#pragma unroll
  for (int i = 0; i < 9; ++i) p[i] = m.e[i];
}

// x y, x^H y, x y^H
__device__ __forceinline__ M3 mul(M3 const &x, M3 const &y) {
  M3 r;
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      double2 acc = cmul(x.e[a], y.e[3 * b]);
      acc = cadd(acc, cmul(x.e[a + 3], y.e[1 + 3 * b]));
      r.e[a + 3 * b] = cadd(acc, cmul(x.e[a + 6], y.e[2 + 3 * b]));
    }
  return r;
}
__device__ __forceinline__ M3 mul_hn(M3 const &x, M3 const &y) {
  M3 r;
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      double2 acc = cmul(cconj(x.e[3 * a]), y.e[3 * b]);
      acc = cadd(acc, cmul(cconj(x.e[1 + 3 * a]), y.e[1 + 3 * b]));
      r.e[a + 3 * b] = cadd(acc, cmul(cconj(x.e[2 + 3 * a]), y.e[2 + 3 * b]));
    }
  return r;
}
__device__ __forceinline__ M3 mul_nh(M3 const &x, M3 const &y) {
  M3 r;
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      double2 acc = cmul(x.e[a], cconj(y.e[b]));
      acc = cadd(acc, cmul(x.e[a + 3], cconj(y.e[b + 3])));
      r.e[a + 3 * b] = cadd(acc, cmul(x.e[a + 6], cconj(y.e[b + 6])));
    }
  return r;
}

// G^H H G and V G for the Jacobi rotation of the pair (p, q): G is the
// identity but for G(p,p) = c, G(p,q) = s, G(q,p) = -s conj(ph),
// G(q,q) = c conj(ph), with ph the phase of H(p,q).
__device__ __forceinline__ void rotate(M3 &h, M3 &v, int p, int q, double c, double s,
                                       double2 ph) {
  double2 const phc = cconj(ph);
#pragma unroll
  for (int i = 0; i < 3; ++i) {  // columns p, q of H G and V G
    double2 const hp = h.e[i + 3 * p], hq = cmul(phc, h.e[i + 3 * q]);
    h.e[i + 3 * p] = make_double2(c * hp.x - s * hq.x, c * hp.y - s * hq.y);
    h.e[i + 3 * q] = make_double2(s * hp.x + c * hq.x, s * hp.y + c * hq.y);
    double2 const vp = v.e[i + 3 * p], vq = cmul(phc, v.e[i + 3 * q]);
    v.e[i + 3 * p] = make_double2(c * vp.x - s * vq.x, c * vp.y - s * vq.y);
    v.e[i + 3 * q] = make_double2(s * vp.x + c * vq.x, s * vp.y + c * vq.y);
  }
#pragma unroll
  for (int j = 0; j < 3; ++j) {  // rows p, q of G^H (H G)
    double2 const hp = h.e[p + 3 * j], hq = cmul(ph, h.e[q + 3 * j]);
    h.e[p + 3 * j] = make_double2(c * hp.x - s * hq.x, c * hp.y - s * hq.y);
    h.e[q + 3 * j] = make_double2(s * hp.x + c * hq.x, s * hp.y + c * hq.y);
  }
  h.e[p + 3 * q] = h.e[q + 3 * p] = make_double2(0, 0);
}

__device__ __forceinline__ void jacobi_pair(M3 &h, M3 &v, int p, int q) {
  double2 const apq = h.e[p + 3 * q];
  double const r = hypot(apq.x, apq.y);
  if (r == 0) return;
  double2 const ph = make_double2(apq.x / r, apq.y / r);
  double const th = (h.e[q + 3 * q].x - h.e[p + 3 * p].x) / (2 * r);
  double const t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1));
  double const c = 1 / sqrt(t * t + 1);
  rotate(h, v, p, q, c, t * c, ph);
}

// proj_to_su3_imp (src/GaugeField.cpp:203-210).
__device__ M3 proj_su3(M3 const &m) {
  M3 h = mul_hn(m, m), v;
#pragma unroll
  for (int i = 0; i < 9; ++i) v.e[i] = make_double2(i % 4 == 0 ? 1.0 : 0.0, 0.0);
  for (int sweep = 0; sweep < 30; ++sweep) {
    double const off = cnorm(h.e[3]) + cnorm(h.e[6]) + cnorm(h.e[7]);
    double const diag = cnorm(h.e[0]) + cnorm(h.e[4]) + cnorm(h.e[8]);
    if (off <= 1e-32 * diag) break;
    jacobi_pair(h, v, 0, 1);
    jacobi_pair(h, v, 0, 2);
    jacobi_pair(h, v, 1, 2);
  }
  // X = V diag(lambda^-1/2) V^H, out = M X
  double d[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) d[i] = 1 / sqrt(h.e[4 * i].x);
  M3 vd;
#pragma unroll
  for (int i = 0; i < 9; ++i) vd.e[i] = make_double2(v.e[i].x * d[i / 3], v.e[i].y * d[i / 3]);
  M3 out = mul(m, mul_nh(vd, v));
  // det^(-1/3) on the principal branch
  double2 const det = det3(out);
  double const mag = pow(hypot(det.x, det.y), -1.0 / 3.0);
  double sn, cs;
  sincos(-atan2(det.y, det.x) / 3.0, &sn, &cs);
  double2 const f = make_double2(mag * cs, mag * sn);
#pragma unroll
  for (int i = 0; i < 9; ++i) out.e[i] = cmul(out.e[i], f);
  return out;
}

__device__ __forceinline__ int64_t step(int64_t s, int dir, int L, int delta) {
  int64_t const stride = dir == 0 ? static_cast<int64_t>(L) * L : (dir == 1 ? L : 1);
  int const c = static_cast<int>((s / stride) % L);
  int const nc = (c + delta + L) % L;
  return s + (nc - c) * stride;
}

__device__ __forceinline__ double2 const *link(double2 const *U, int64_t s, int dir) {
  return U + (3 * s + dir) * 9;
}

// Decorated links of one chunk: dec[(t V3 + s) 6 + d + 3 n].
__global__ void hyp_inner_kernel(double2 *dec, double2 const *U, int32_t L, int64_t V3,
                                 int64_t n_items, double alpha2) {
  int64_t const k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (k >= n_items) return;
  int64_t const ts = k / 6;  // t V3 + s
  int const slot = static_cast<int>(k % 6);
  int const dir = slot % 3, n = slot / 3;
  int const perp = n == 0 ? (dir == 0 ? 1 : 0) : (dir == 2 ? 1 : 2);
  int64_t const t = ts / V3, s = ts % V3;
  double2 const *Ut = U + t * V3 * 27;
  int64_t const s_up = step(s, perp, L, 1), s_dir = step(s, dir, L, 1);
  int64_t const s_dn = step(s, perp, L, -1), s_dn_dir = step(s_dn, dir, L, 1);
  M3 st = mul(load(link(Ut, s, perp)), mul_nh(load(link(Ut, s_up, dir)), load(link(Ut, s_dir, perp))));
  M3 const dn = mul_hn(load(link(Ut, s_dn, perp)),
                       mul(load(link(Ut, s_dn, dir)), load(link(Ut, s_dn_dir, perp))));
  M3 const u = load(link(Ut, s, dir));
  double const w = 1 - alpha2, a = alpha2 / 2.;
#pragma unroll
  for (int i = 0; i < 9; ++i)
    st.e[i] = make_double2(u.e[i].x * w + (st.e[i].x + dn.e[i].x) * a,
                           u.e[i].y * w + (st.e[i].y + dn.e[i].y) * a);
  store(dec + k * 9, proj_su3(st));
}

// decor (src/GaugeField.cpp:170-190): slot of the link in direction d that
// was smeared with the third direction `plane`.
__device__ __forceinline__ int decor(int d, int plane) {
  if (d == 0) return plane == 1 ? 0 : 3;
  if (d == 1) return plane == 0 ? 1 : 4;
  return plane == 0 ? 2 : 5;
}

__global__ void hyp_outer_kernel(double2 *U, double2 const *dec, int32_t L, int64_t V3,
                                 int64_t n_items, double alpha1) {
  int64_t const k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (k >= n_items) return;
  int64_t const ts = k / 3;
  int const dir = static_cast<int>(k % 3);
  int64_t const t = ts / V3, s = ts % V3;
  double2 const *Dt = dec + t * V3 * 54;
  M3 outer;
#pragma unroll
  for (int i = 0; i < 9; ++i) outer.e[i] = make_double2(0, 0);
#pragma unroll
  for (int nd = 0; nd < 3; ++nd) {
    if (nd == dir) continue;
    int const plane = 3 - dir - nd;
    int const a = decor(nd, plane), b = decor(dir, plane);
    int64_t const s_up = step(s, nd, L, 1), s_dir = step(s, dir, L, 1);
    int64_t const s_dn = step(s, nd, L, -1), s_dn_dir = step(s_dn, dir, L, 1);
    M3 const up = mul(load(Dt + (6 * s + a) * 9),
                      mul_nh(load(Dt + (6 * s_up + b) * 9), load(Dt + (6 * s_dir + a) * 9)));
    M3 const dn = mul_hn(load(Dt + (6 * s_dn + a) * 9),
                         mul(load(Dt + (6 * s_dn + b) * 9), load(Dt + (6 * s_dn_dir + a) * 9)));
#pragma unroll
    for (int i = 0; i < 9; ++i) outer.e[i] = cadd(outer.e[i], cadd(up.e[i], dn.e[i]));
  }
  double2 *u = U + (t * V3 * 3 + 3 * s + dir) * 9;
  M3 const m = load(u);
  double const w = 1 - alpha1, c = alpha1 / 4.;
#pragma unroll
  for (int i = 0; i < 9; ++i)
    outer.e[i] = make_double2(m.e[i].x * w + outer.e[i].x * c, m.e[i].y * w + outer.e[i].y * c);
  store(u, proj_su3(outer));
}

inline unsigned blocks_of(int64_t n, int threads) {
  return static_cast<unsigned>((n + threads - 1) / threads);
}

}  // namespace

int64_t hyp_scratch_doubles_per_timeslice(int32_t L) {
  return static_cast<int64_t>(L) * L * L * 6 * 9 * 2;
}

cudaError_t hyp_smear(double2 *U, double2 *dec, int32_t L, int32_t n_t, double alpha1,
                      double alpha2, cudaStream_t stream) {
  if (L < 1 || n_t < 1) return cudaErrorInvalidValue;
  int64_t const V3 = static_cast<int64_t>(L) * L * L;
  int64_t const n_inner = n_t * V3 * 6, n_outer = n_t * V3 * 3;
  hyp_inner_kernel<<<blocks_of(n_inner, 128), 128, 0, stream>>>(dec, U, L, V3, n_inner, alpha2);
  cudaError_t const e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  hyp_outer_kernel<<<blocks_of(n_outer, 128), 128, 0, stream>>>(U, dec, L, V3, n_outer, alpha1);
  return cudaGetLastError();
}

}  // namespace dev
}  // namespace slaph
