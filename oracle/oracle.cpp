// FP64 CPU oracle for the sLapH contraction hot path — TEST INFRASTRUCTURE.
//
// A restatement of the reference algorithm in plain C++17 + OpenMP, written to
// follow the reference's own control flow (memoised factor and trace maps per
// OpenMP thread, cleared per block pair) so that it reproduces the reference
// outputs.  Each function names the reference file:line it follows.  Only the
// tests, the smoke check and the CPU-baseline leg of bench.py use it.
#include "oracle.h"

#include <omp.h>

#include <array>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <functional>
#include <algorithm>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace {

thread_local std::string g_err;
int g_threads = 0;

using cd = std::complex<double>;

inline cd mul(cd a, cd b) {
  return {a.real() * b.real() - a.imag() * b.imag(),
          a.real() * b.imag() + a.imag() * b.real()};
}

// Column-major complex matrix (the Eigen::MatrixXcd layout).
struct Mat {
  int r = 0, c = 0;
  std::vector<cd> d;
  Mat() = default;
  Mat(int r_, int c_) : r(r_), c(c_), d(static_cast<size_t>(r_) * c_) {}
  cd &operator()(int i, int j) { return d[i + static_cast<size_t>(r) * j]; }
  cd operator()(int i, int j) const { return d[i + static_cast<size_t>(r) * j]; }
  static Mat identity(int n) {
    Mat m(n, n);
    for (int i = 0; i < n; ++i) m(i, i) = 1.0;
    return m;
  }
  Mat adjoint() const {
    Mat m(c, r);
    for (int j = 0; j < c; ++j)
      for (int i = 0; i < r; ++i) m(j, i) = std::conj((*this)(i, j));
    return m;
  }
};

// C = A * B.
Mat matmul(Mat const &A, Mat const &B) {
  Mat C(A.r, B.c);
  for (int j = 0; j < B.c; ++j)
    for (int k = 0; k < A.c; ++k) {
      cd const b = B(k, j);
      cd const *a = &A.d[static_cast<size_t>(A.r) * k];
      cd *cc = &C.d[static_cast<size_t>(C.r) * j];
      for (int i = 0; i < A.r; ++i) cc[i] += mul(a[i], b);
    }
  return C;
}

// tr(L * R) = sum_i sum_k L(i,k) R(k,i).
cd trace_of_product(Mat const &L, Mat const &R) {
  cd s = 0;
  for (int i = 0; i < L.r; ++i) {
    cd row = 0;
    for (int k = 0; k < L.c; ++k) row += mul(L(i, k), R(k, i));
    s += row;
  }
  return s;
}

cd trace(Mat const &F) {
  cd s = 0;
  for (int i = 0; i < F.r; ++i) s += F(i, i);
  return s;
}

// Neumaier / native accumulators, include/KahanAccumulator.hpp:14-72.
struct Acc {
  bool kahan = false;
  cd sum = 0, c = 0;
  explicit Acc(bool k) : kahan(k) {}
  void add(cd x) {
    if (!kahan) {
      sum += x;
      return;
    }
    cd const t = sum + x;
    if (std::abs(sum) >= std::abs(x))
      c += (sum - t) + x;
    else
      c += (x - t) + sum;
    sum = t;
  }
  cd value() const { return kahan ? sum + c : sum; }
};

// ---------------------------------------------------------------- gamma
// Dense tmLQCD basis (tests/gtest/gamma.cpp:22-40); the sparse table of
// src/Gamma.cpp:18-246 is derived from it by products.
struct GammaSparse {
  int row[4];
  cd value[4];
};

std::vector<GammaSparse> make_gamma_table() {
  cd const I(0, 1);
  using D = std::array<std::array<cd, 4>, 4>;
  D g[4] = {};
  g[0] = {{{0, 0, 1, 0}, {0, 0, 0, 1}, {1, 0, 0, 0}, {0, 1, 0, 0}}};
  g[1] = {{{0, 0, 0, I}, {0, 0, I, 0}, {0, -I, 0, 0}, {-I, 0, 0, 0}}};
  g[2] = {{{0, 0, 0, 1}, {0, 0, -1, 0}, {0, -1, 0, 0}, {1, 0, 0, 0}}};
  g[3] = {{{0, 0, I, 0}, {0, 0, 0, -I}, {-I, 0, 0, 0}, {0, I, 0, 0}}};
  auto prod = [](D const &a, D const &b) {
    D c{};
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j)
        for (int k = 0; k < 4; ++k) c[i][j] += a[i][k] * b[k][j];
    return c;
  };
  D one{};
  for (int i = 0; i < 4; ++i) one[i][i] = 1;
  D g5 = prod(prod(prod(g[0], g[1]), g[2]), g[3]);
  std::vector<D> dense = {g[0],
                          g[1],
                          g[2],
                          g[3],
                          one,
                          g5,
                          prod(g[0], g5),
                          prod(g[1], g5),
                          prod(g[2], g5),
                          prod(g[3], g5),
                          prod(g[0], g[1]),
                          prod(g[0], g[2]),
                          prod(g[0], g[3]),
                          prod(prod(g[0], g[1]), g5),
                          prod(prod(g[0], g[2]), g5),
                          prod(prod(g[0], g[3]), g5)};
  std::vector<GammaSparse> out(16);
  for (int m = 0; m < 16; ++m)
    for (int col = 0; col < 4; ++col) {
      int nz = -1;
      for (int row = 0; row < 4; ++row)
        if (std::abs(dense[m][row][col]) > 0.5) nz = row;
      out[m].row[col] = nz;
      out[m].value[col] = dense[m][nz][col];
    }
  return out;
}

std::vector<GammaSparse> const &gamma_table() {
  static std::vector<GammaSparse> const t = make_gamma_table();
  return t;
}

// ---------------------------------------------------------------- momenta
// create_momenta, src/OperatorFactory.cpp:64-95.
void create_momentum(int Lx, int Ly, int Lz, const int p[3], cd *out) {
  static const cd I(0.0, 1.0);
  double const ipx = p[0] * 2. * M_PI / static_cast<double>(Lx);
  double const ipy = p[1] * 2. * M_PI / static_cast<double>(Ly);
  double const ipz = p[2] * 2. * M_PI / static_cast<double>(Lz);
  for (int x = 0; x < Lx; ++x) {
    int const xH = x * Ly * Lz;
    double const ipxH = ipx * x;
    for (int y = 0; y < Ly; ++y) {
      int const xHyH = xH + y * Lz;
      double const ipxHipyH = ipxH + ipy * y;
      for (int z = 0; z < Lz; ++z) out[xHyH + z] = std::exp(-I * (ipxHipyH + ipz * z));
    }
  }
}

// C (n x n) = A^H B for A, B of K x n (column-major), blocked over K.
void gemm_ah_b(cd const *A, cd const *B, long K, int n, cd *C) {
  for (long i = 0; i < static_cast<long>(n) * n; ++i) C[i] = 0;
  long const KB = 96;
  for (long k0 = 0; k0 < K; k0 += KB) {
    long const kb = std::min(KB, K - k0);
    for (int j = 0; j < n; j += 2) {
      int const nj = std::min(2, n - j);
      for (int i = 0; i < n; i += 2) {
        int const ni = std::min(2, n - i);
        double acc[2][2][2] = {};
        for (int jj = 0; jj < nj; ++jj)
          for (int ii = 0; ii < ni; ++ii) {
            double const *a = reinterpret_cast<double const *>(A + K * (i + ii) + k0);
            double const *b = reinterpret_cast<double const *>(B + K * (j + jj) + k0);
            double sr = 0, si = 0;
            for (long k = 0; k < kb; ++k) {
              double const ar = a[2 * k], ai = a[2 * k + 1];
              double const br = b[2 * k], bi = b[2 * k + 1];
              sr += ar * br + ai * bi;
              si += ar * bi - ai * br;
            }
            acc[ii][jj][0] = sr;
            acc[ii][jj][1] = si;
          }
        for (int jj = 0; jj < nj; ++jj)
          for (int ii = 0; ii < ni; ++ii)
            C[(i + ii) + static_cast<long>(n) * (j + jj)] +=
                cd(acc[ii][jj][0], acc[ii][jj][1]);
      }
    }
  }
}

// ---------------------------------------------------------------- dilution
enum class DilType { block, interlace };

// BlockIterator, include/dilution-iterator.hpp:21-191.
struct BlockIter {
  int slice_source, slice_sink, block_source, block_sink, num_slice, num_block, pass;
  DilType type;
  void next() {
    int const bs = num_slice / num_block;
    if (type == DilType::block) {
      int const src_begin = block_source * bs, src_end = (block_source + 1) * bs;
      int const snk_begin = block_sink * bs, snk_end = (block_sink + 1) * bs;
      ++slice_sink;
      if (slice_sink == snk_end) {
        slice_sink = snk_begin;
        ++slice_source;
      }
      if (slice_source == src_end) {
        slice_source = snk_begin;
        slice_sink = src_begin;
        ++pass;
        if (block_source == block_sink) ++pass;
        std::swap(block_source, block_sink);
      }
    } else {
      int const src_begin = block_source, snk_begin = block_sink;
      slice_sink += bs;
      if (slice_sink >= num_slice) {
        slice_sink = snk_begin;
        slice_source += bs;
      }
      if (slice_source >= num_slice) {
        slice_source = snk_begin;
        slice_sink = src_begin;
        ++pass;
        if (block_source == block_sink) ++pass;
        std::swap(block_source, block_sink);
      }
    }
  }
};

// DilutionScheme, include/dilution-iterator.hpp:306-356 (block size = dilT).
struct DilScheme {
  int num_slice, num_block;
  DilType type;
  DilScheme(int ns, int block_size, DilType t)
      : num_slice(ns), num_block(ns / block_size), type(t) {}
  int size() const { return num_block * (num_block + 1) / 2; }
  std::pair<int, int> blocks(int i) const {
    int bsnk = 0, bsrc = 0;
    for (int j = 0; j < i; ++j) {
      ++bsnk;
      if (bsnk == num_block) {
        ++bsrc;
        bsnk = bsrc;
      }
    }
    return {bsrc, bsnk};
  }
  std::vector<std::pair<int, int>> slices(int i) const {
    auto b = blocks(i);
    int const bs = num_slice / num_block;
    BlockIter it{};
    if (type == DilType::block)
      it = {b.first * bs, b.second * bs, b.first, b.second, num_slice, num_block, 0, type};
    else
      it = {b.first, b.second, b.first, b.second, num_slice, num_block, 0, type};
    std::vector<std::pair<int, int>> out;
    // end(): same blocks/sizes, pass 2; comparison ignores slices
    // (include/dilution-iterator.hpp:126-130).
    int const b0 = b.first, b1 = b.second;
    while (!((it.block_source == b0 && it.block_sink == b1 && it.pass == 2))) {
      out.emplace_back(it.slice_source, it.slice_sink);
      it.next();
      if (out.size() > static_cast<size_t>(4 * num_slice * num_slice))
        throw std::runtime_error("dilution iterator did not terminate");
    }
    return out;
  }
  int time_to_block(int t) const {
    int const bs = num_slice / num_block;
    return type == DilType::block ? t / bs : t % bs;
  }
};

// ---------------------------------------------------------------- factors
struct DF {  // DilutedFactor, include/DilutedFactor.hpp:19-25
  Mat data;
  int r1, r2;
  uint16_t used;
};
using DFList = std::vector<DF>;
using DFMap = std::map<long, DFList>;  // operator key -> factors

struct DT {  // DilutedTrace, include/DilutedTrace.hpp:7-12
  cd data;
  uint16_t used;
};
using DTMap = std::map<long, std::vector<DT>>;

struct Inputs {
  slaph_dims dims;
  slaph_plan const *plan;
  double const *vdv;            // [n_ops][Lt][nev][nev]
  double const *const *peram;   // [n_rnd]
  double const *noise;          // [n_rnd][Lt*4*nev]
  int n_ops;
  bool kahan;

  long peram_rows() const { return 4L * dims.nev * dims.Lt; }
  cd P(int r, long row, long col) const {
    double const *p = peram[r] + 2 * (row + peram_rows() * col);
    return {p[0], p[1]};
  }
  cd rnd(int r, long blk) const {
    double const *p = noise + 2 * (static_cast<long>(r) * dims.Lt * 4 * dims.nev + blk);
    return {p[0], p[1]};
  }
  // return_vdaggerv + optional adjoint (src/DilutedFactorFactory.cpp:49-58).
  Mat vdaggerv(slaph_factor_index const &op, int t) const {
    int const n = dims.nev;
    if (op.id_vdaggerv < 0 || op.id_vdaggerv >= n_ops)
      throw std::runtime_error("VdaggerV id out of range");
    Mat m(n, n);
    double const *src =
        vdv + 2 * (static_cast<long>(op.id_vdaggerv) * dims.Lt + t) * n * static_cast<long>(n);
    std::memcpy(static_cast<void *>(m.d.data()), src, sizeof(cd) * n * static_cast<size_t>(n));
    return op.need_vdaggerv_daggering ? m.adjoint() : m;
  }
  // peram[r].block(row0, col0, nr, nc)
  Mat peram_block(int r, long row0, long col0, int nr, int nc) const {
    Mat m(nr, nc);
    for (int j = 0; j < nc; ++j)
      for (int i = 0; i < nr; ++i) m(i, j) = P(r, row0 + i, col0 + j);
    return m;
  }
};

constexpr int dilD = 4;

// DilutedFactorFactory<Q0>::build, src/DilutedFactorFactory.cpp:34-101.
void build_q0(Inputs const &in, int t1, std::map<std::array<int, 1>, DFMap> &Ql) {
  int const nev = in.dims.nev, dilE = in.dims.dilE, eds = dilD * dilE;
  auto const &gam = gamma_table();
  auto &dst = Ql[{t1}];
  for (int opk = 0; opk < in.plan->n_factors[0]; ++opk) {
    auto const &op = in.plan->factors[0][opk];
    Mat const vdv = in.vdaggerv(op, t1);
    int check = -1;
    Mat M;
    for (int k = 0; k < op.n_rnd_pairs; ++k) {
      int const r1 = op.rnd_pairs[2 * k], r2 = op.rnd_pairs[2 * k + 1];
      if (check != r2) {
        M = Mat(nev, 4 * dilE);
        for (int v = 0; v < nev; ++v)
          for (int block = 0; block < 4; ++block) {
            long const blk = block + (v + static_cast<long>(nev) * t1) * 4;
            cd const rr = in.rnd(r2, blk);
            int const col = v % dilE + dilE * block;
            for (int i = 0; i < nev; ++i) M(i, col) += mul(rr, vdv(i, v));
          }
      }
      Mat matrix(eds, eds);
      for (int block = 0; block < 4; ++block) {
        cd const value = gam[op.gamma].value[block];
        int const gi = gam[op.gamma].row[block];
        for (int v = 0; v < nev; ++v) {
          long const blk = gi + (v + static_cast<long>(nev) * t1) * dilD;
          cd const cr = std::conj(in.rnd(r1, blk));
          for (int e = 0; e < dilE; ++e)
            matrix(v % dilE + dilE * gi, block * dilE + e) +=
                mul(mul(value, M(v, block * dilE + e)), cr);
        }
      }
      check = r2;
      dst[opk].push_back({std::move(matrix), r1, r2, 0});
    }
  }
}

// DilutedFactorFactory<Q1>::build, src/DilutedFactorFactory.cpp:104-170.
void build_q1(Inputs const &in, int t1, int b2, std::map<std::array<int, 2>, DFMap> &Ql) {
  int const nev = in.dims.nev, dilE = in.dims.dilE, eds = dilD * dilE;
  auto const &gam = gamma_table();
  auto &dst = Ql[{t1, b2}];
  for (int opk = 0; opk < in.plan->n_factors[1]; ++opk) {
    auto const &op = in.plan->factors[1][opk];
    Mat const vdv = in.vdaggerv(op, t1);
    for (int k = 0; k < op.n_rnd_pairs; ++k) {
      int const r1 = op.rnd_pairs[2 * k], r2 = op.rnd_pairs[2 * k + 1];
      Mat rvdv(eds, nev);
      for (int v = 0; v < nev; ++v)
        for (int block = 0; block < dilD; ++block) {
          long const blk = block + v * dilD + static_cast<long>(dilD) * nev * t1;
          cd const cr = std::conj(in.rnd(r1, blk));
          int const row = v % dilE + dilE * block;
          for (int j = 0; j < nev; ++j) rvdv(row, j) += mul(cr, vdv(v, j));
        }
      Mat matrix(eds, eds);
      for (int row = 0; row < dilD; ++row) {
        cd const value = gam[op.gamma].value[row];
        Mat A(dilE, nev);
        for (int j = 0; j < nev; ++j)
          for (int i = 0; i < dilE; ++i) A(i, j) = rvdv(row * dilE + i, j);
        for (int col = 0; col < dilD; ++col) {
          Mat const B = in.peram_block(r2, (static_cast<long>(t1) * dilD + gam[op.gamma].row[row]) * nev,
                                       (static_cast<long>(b2) * dilD + col) * dilE, nev, dilE);
          Mat const AB = matmul(A, B);
          for (int j = 0; j < dilE; ++j)
            for (int i = 0; i < dilE; ++i)
              matrix(row * dilE + i, col * dilE + j) = mul(value, AB(i, j));
        }
      }
      dst[opk].push_back({std::move(matrix), r1, r2, 0});
    }
  }
}

// DilutedFactorFactory<Q2>::build, src/DilutedFactorFactory.cpp:173-253.
void build_q2(Inputs const &in, int b1, int t1, int b2,
              std::map<std::array<int, 3>, DFMap> &Ql) {
  int const nev = in.dims.nev, dilE = in.dims.dilE, eds = dilD * dilE;
  auto const &gam = gamma_table();
  auto &dst = Ql[{b1, t1, b2}];
  for (int opk = 0; opk < in.plan->n_factors[2]; ++opk) {
    auto const &op = in.plan->factors[2][opk];
    Mat const vdv = in.vdaggerv(op, t1);
    Mat M(dilD * dilE, 4 * nev);
    int check = -1;
    for (int k = 0; k < op.n_rnd_pairs; ++k) {
      int const r1 = op.rnd_pairs[2 * k], r2 = op.rnd_pairs[2 * k + 1];
      if (check != r1) {
        for (int row = 0; row < dilD; ++row)
          for (int col = 0; col < 4; ++col) {
            Mat const Pb = in.peram_block(r1, (static_cast<long>(t1) * 4 + row) * nev,
                                          (static_cast<long>(b1) * dilD + col) * dilE, nev,
                                          dilE);
            Mat const blk = matmul(Pb.adjoint(), vdv);
            bool const flip = ((row + col) == 3) || (std::abs(row - col) > 1);
            for (int j = 0; j < nev; ++j)
              for (int i = 0; i < dilE; ++i)
                M(col * dilE + i, row * nev + j) = flip ? -blk(i, j) : blk(i, j);
          }
      }
      Mat matrix(eds, eds);
      for (int bd = 0; bd < dilD; ++bd) {
        cd const value = gam[op.gamma].value[bd];
        int const gi = gam[op.gamma].row[bd];
        for (int row = 0; row < dilD; ++row) {
          Mat A(dilE, nev);
          for (int j = 0; j < nev; ++j)
            for (int i = 0; i < dilE; ++i) A(i, j) = mul(value, M(row * dilE + i, bd * nev + j));
          for (int col = 0; col < dilD; ++col) {
            Mat const B = in.peram_block(r2, (static_cast<long>(t1) * 4 + gi) * nev,
                                         (static_cast<long>(b2) * dilD + col) * dilE, nev, dilE);
            Mat const AB = matmul(A, B);
            for (int j = 0; j < dilE; ++j)
              for (int i = 0; i < dilE; ++i) matrix(row * dilE + i, col * dilE + j) += AB(i, j);
          }
        }
      }
      check = r1;
      dst[opk].push_back({std::move(matrix), r1, r2, 0});
    }
  }
}

template <int N, typename BuildFn>
struct FactorFactory {
  std::map<std::array<int, N>, DFMap> Ql;
  BuildFn fn;
  explicit FactorFactory(BuildFn f) : fn(f) {}
  DFMap const &operator[](std::array<int, N> const &key) {
    if (Ql.count(key) == 0) fn(key, Ql);
    return Ql.at(key);
  }
  void clear() { Ql.clear(); }
};

// operator*(vector<DF>, vector<DF>), src/DilutedFactor.cpp:6-51.
DFList operator*(DFList const &L, DFList const &R) {
  DFList out;
  for (auto const &l : L) {
    int const inner = l.r2;
    for (auto const &r : R) {
      if (!(inner == r.r1 && l.r1 != r.r2)) continue;
      if ((l.used & r.used) != 0u) continue;
      uint16_t const used = l.used | r.used | static_cast<uint16_t>(1u << inner);
      out.push_back({matmul(l.data, r.data), l.r1, r.r2, used});
    }
  }
  if (out.empty())
    throw std::runtime_error(
        "vector<DilutedFactor> operator*(vector<DilutedFactor>, vector<DilutedFactor>) "
        "has an empty result.");
  return out;
}

// factor_to_trace(L, R), src/DilutedTrace.cpp:84-138.
std::vector<DT> factor_to_trace(DFList const &L, DFList const &R) {
  std::vector<DT> out;
  for (auto const &l : L) {
    int const outer = l.r1, inner = l.r2;
    for (auto const &r : R) {
      if (!(inner == r.r1 && outer == r.r2)) continue;
      if ((l.used & r.used) != 0u) continue;
      uint16_t const used = l.used | r.used | static_cast<uint16_t>(1u << inner) |
                            static_cast<uint16_t>(1u << outer);
      out.push_back({trace_of_product(l.data, r.data), used});
    }
  }
  if (out.empty())
    throw std::runtime_error(
        "vector<DilutedTrace> factor_to_trace(vector<DilutedFactor>, "
        "vector<DilutedFactor>) has an empty result. Not enough random vectors?");
  return out;
}

// factor_to_trace(vec), src/DilutedTrace.cpp:140-165.
std::vector<DT> factor_to_trace(DFList const &v) {
  std::vector<DT> out;
  for (auto const &e : v) {
    if (e.r1 != e.r2) continue;
    out.push_back({trace(e.data), static_cast<uint16_t>(e.used | (1u << e.r1))});
  }
  if (out.empty())
    throw std::runtime_error(
        "vector<DilutedTrace> factor_to_trace(vector<DilutedFactor>) has an empty "
        "result.");
  return out;
}

// multiply<1,1>, include/DilutedFactor.hpp:164-187.
void multiply(std::map<std::array<long, 2>, DFList> &L, std::array<long, 2> const &key,
              DFMap const &f0, DFMap const &f1) {
  if (L.count(key) == 0) L[key] = f0.at(key[0]) * f1.at(key[1]);
}

// ---------------------------------------------------------------- parts
struct Parts {  // DiagramParts, include/Diagram.hpp:12-107
  Inputs const &in;
  DilScheme const &ds;
  std::function<void(std::array<int, 1> const &, std::map<std::array<int, 1>, DFMap> &)> f0;
  std::function<void(std::array<int, 2> const &, std::map<std::array<int, 2>, DFMap> &)> f1;
  std::function<void(std::array<int, 3> const &, std::map<std::array<int, 3>, DFMap> &)> f2;
  FactorFactory<1, decltype(f0)> q0;
  FactorFactory<2, decltype(f1)> q1;
  FactorFactory<3, decltype(f2)> q2;
  std::map<std::vector<int>, DTMap> tr[SLAPH_TR_KINDS];

  Parts(Inputs const &in_, DilScheme const &ds_)
      : in(in_),
        ds(ds_),
        f0([this](std::array<int, 1> const &k, std::map<std::array<int, 1>, DFMap> &m) {
          build_q0(in, k[0], m);
        }),
        f1([this](std::array<int, 2> const &k, std::map<std::array<int, 2>, DFMap> &m) {
          build_q1(in, k[0], k[1], m);
        }),
        f2([this](std::array<int, 3> const &k, std::map<std::array<int, 3>, DFMap> &m) {
          build_q2(in, k[0], k[1], k[2], m);
        }),
        q0(f0),
        q1(f1),
        q2(f2) {}

  void clear() {
    q0.clear();
    q1.clear();
    q2.clear();
    // DilutedTrace1Factory::clear() keeps its cache
    // (include/DilutedTraceFactory.hpp:61).
    for (int k = 1; k < SLAPH_TR_KINDS; ++k) tr[k].clear();
  }

  int const *ids(int kind, long i) const {
    static int const arity[SLAPH_TR_KINDS] = {1, 2, 2, 3, 3, 4, 4, 6};
    return in.plan->trace_ql_ids[kind] + i * arity[kind];
  }
  long n_ids(int kind) const { return in.plan->n_trace_ids[kind]; }
  int blk(int t) const { return ds.time_to_block(t); }

  // DilutedTrace*Factory::build, src/DilutedTraceFactory.cpp:13-245.
  void build(int kind, std::vector<int> const &t, DTMap &out) {
    using K2 = std::array<long, 2>;
    switch (kind) {
      case SLAPH_TR_Q1: {
        int const b = blk(t[0]);
        for (long i = 0; i < n_ids(kind); ++i)
          out[i] = factor_to_trace(q1[{t[0], b}].at(ids(kind, i)[0]));
        break;
      }
      case SLAPH_TR_Q1Q1: {
        int const b1 = blk(t[0]), b2 = blk(t[1]);
        for (long i = 0; i < n_ids(kind); ++i) {
          auto c = ids(kind, i);
          DFList const &l = q1[{t[0], b2}].at(c[0]);
          DFList const &r = q1[{t[1], b1}].at(c[1]);
          out[i] = factor_to_trace(l, r);
        }
        break;
      }
      case SLAPH_TR_Q0Q2: {
        int const b2 = blk(t[1]);
        for (long i = 0; i < n_ids(kind); ++i) {
          auto c = ids(kind, i);
          DFList const &l = q0[{t[1]}].at(c[1]);
          DFList const &r = q2[{b2, t[0], b2}].at(c[0]);
          out[i] = factor_to_trace(l, r);
        }
        break;
      }
      case SLAPH_TR_Q1Q1Q1: {
        int const b1 = blk(t[0]), b2 = blk(t[1]), b3 = blk(t[2]);
        std::map<K2, DFList> L1;
        for (long i = 0; i < n_ids(kind); ++i) {
          auto c = ids(kind, i);
          DFMap const &a = q1[{t[0], b2}];
          DFMap const &b = q1[{t[1], b3}];
          multiply(L1, {c[0], c[1]}, a, b);
        }
        for (long i = 0; i < n_ids(kind); ++i) {
          auto c = ids(kind, i);
          DFList const &r = q1[{t[2], b1}].at(c[2]);
          out[i] = factor_to_trace(L1[{c[0], c[1]}], r);
        }
        break;
      }
      case SLAPH_TR_Q1Q0Q2: {
        int const b1 = blk(t[0]), b2 = blk(t[1]), b3 = blk(t[2]);
        std::map<K2, DFList> L1;
        for (long i = 0; i < n_ids(kind); ++i) {
          auto c = ids(kind, i);
          DFMap const &a = q0[{t[0]}];
          DFMap const &b = q2[{b1, t[0], b2}];
          multiply(L1, {c[2], c[0]}, a, b);
        }
        for (long i = 0; i < n_ids(kind); ++i) {
          auto c = ids(kind, i);
          DFList const &r = q1[{t[1], b3}].at(c[1]);
          out[i] = factor_to_trace(L1[{c[2], c[0]}], r);
        }
        break;
      }
      case SLAPH_TR_Q1Q1Q1Q1: {
        int const b0 = blk(t[0]), b1 = blk(t[1]), b2 = blk(t[2]), b3 = blk(t[3]);
        std::map<K2, DFList> L1, L2;
        for (long i = 0; i < n_ids(kind); ++i) {
          auto c = ids(kind, i);
          {
            DFMap const &a = q1[{t[0], b1}];
            DFMap const &b = q1[{t[1], b2}];
            multiply(L1, {c[0], c[1]}, a, b);
          }
          {
            DFMap const &a = q1[{t[2], b3}];
            DFMap const &b = q1[{t[3], b0}];
            multiply(L2, {c[2], c[3]}, a, b);
          }
        }
        for (long i = 0; i < n_ids(kind); ++i) {
          auto c = ids(kind, i);
          out[i] = factor_to_trace(L1[{c[0], c[1]}], L2[{c[2], c[3]}]);
        }
        break;
      }
      case SLAPH_TR_Q2Q0Q2Q0: {
        int const b0 = blk(t[0]), b2 = blk(t[2]);
        std::map<K2, DFList> L1, L2;
        for (long i = 0; i < n_ids(kind); ++i) {
          auto c = ids(kind, i);
          {
            DFMap const &a = q0[{t[0]}];
            DFMap const &b = q2[{b0, t[1], b2}];
            multiply(L1, {c[0], c[1]}, a, b);
          }
          {
            DFMap const &a = q0[{t[2]}];
            DFMap const &b = q2[{b2, t[3], b0}];
            multiply(L2, {c[2], c[3]}, a, b);
          }
        }
        for (long i = 0; i < n_ids(kind); ++i) {
          auto c = ids(kind, i);
          out[i] = factor_to_trace(L1[{c[0], c[1]}], L2[{c[2], c[3]}]);
        }
        break;
      }
      case SLAPH_TR_Q2Q0Q2Q0Q2Q0: {
        int const b1 = blk(t[1]), b3 = blk(t[3]), b5 = blk(t[5]);
        for (long i = 0; i < n_ids(kind); ++i) {
          auto c = ids(kind, i);
          DFMap const &m0 = q2[{b5, t[0], b1}];
          DFMap const &m1 = q0[{t[1]}];
          DFMap const &m2 = q2[{b1, t[2], b3}];
          DFMap const &m3 = q0[{t[3]}];
          DFMap const &m4 = q2[{b3, t[4], b5}];
          DFMap const &m5 = q0[{t[5]}];
          DFList const p = (((m0.at(c[1]) * m1.at(c[2])) * m2.at(c[3])) * m3.at(c[4])) *
                           m4.at(c[5]);
          out[i] = factor_to_trace(p, m5.at(c[0]));
        }
        break;
      }
      default:
        throw std::runtime_error("unknown trace kind");
    }
  }

  // AbstractDilutedTraceFactory::get, include/DilutedTraceFactory.hpp:52-57.
  std::vector<DT> const &get(slaph_trace_request const &r, int src, int snk) {
    std::vector<int> key(r.n_loc);
    for (int l = 0; l < r.n_loc; ++l) key[l] = r.loc[l] == 0 ? src : snk;
    auto &m = tr[r.kind];
    auto it = m.find(key);
    if (it == m.end()) {
      DTMap built;
      build(r.kind, key, built);
      it = m.emplace(key, std::move(built)).first;
    }
    return it->second.at(r.tr_id);
  }
};

// inner_product, src/DilutedTrace.cpp:5-82.
cd inner_product(std::vector<DT> const &L, std::vector<DT> const &R, bool kahan) {
  long num = 0;
  Acc result(kahan);
  for (auto const &l : L) {
    Acc right_sum(kahan);
    for (auto const &r : R) {
      if ((l.used & r.used) != 0u) continue;
      right_sum.add(r.data);
      ++num;
    }
    result.add(l.data * right_sum.value());
  }
  if (num == 0)
    throw std::runtime_error(
        "compcomp_t inner_product(vector<DilutedTrace>, vector<DilutedTrace>) has an empty "
        "result. Not enough random vectors?");
  return result.value() / static_cast<double>(num);
}

cd inner_product(std::vector<DT> const &L, std::vector<DT> const &M, std::vector<DT> const &R,
                 bool kahan) {
  long num = 0;
  Acc result(kahan);
  for (auto const &l : L)
    for (auto const &m : M) {
      Acc right_sum(kahan);
      for (auto const &r : R) {
        if ((l.used & m.used & r.used) != 0u) continue;
        right_sum.add(r.data);
        ++num;
      }
      result.add(l.data * m.data * right_sum.value());
    }
  if (num == 0)
    throw std::runtime_error(
        "compcomp_t inner_product(vector<DilutedTrace>, vector<DilutedTrace>) has an empty "
        "result. Not enough random vectors?");
  return result.value() / static_cast<double>(num);
}

// resolve_request{1,2,3}, src/Diagram.cpp:9-94.
cd resolve(slaph_correlator_request const &req, int src, int snk, Parts &q, bool kahan) {
  if (req.n_traces == 1) {
    auto const &x = q.get(req.traces[0], src, snk);
    Acc a(kahan);
    for (auto const &e : x) a.add(e.data);
    return a.value() / static_cast<double>(x.size());
  }
  if (req.n_traces == 2) {
    auto const &x0 = q.get(req.traces[0], src, snk);
    auto const &x1 = q.get(req.traces[1], src, snk);
    return inner_product(x0, x1, kahan);
  }
  if (req.n_traces == 3) {
    auto const &x0 = q.get(req.traces[0], src, snk);
    auto const &x1 = q.get(req.traces[1], src, snk);
    auto const &x2 = q.get(req.traces[2], src, snk);
    return inner_product(x0, x1, x2, kahan);
  }
  throw std::runtime_error("This many traces are not implemented yet.");
}

void check_dims(slaph_dims const *d) {
  if (!d || d->Lt < 1 || d->Lx < 1 || d->Ly < 1 || d->Lz < 1 || d->nev < 1 || d->dilT < 1 ||
      d->dilE < 1 || d->Lt % d->dilT != 0)
    throw std::runtime_error("invalid dims");
}

template <typename F>
int guarded(F &&f) {
  try {
    f();
    return SLAPH_OK;
  } catch (std::exception const &e) {
    g_err = e.what();
    return SLAPH_ERR_ARG;
  }
}

// GaugeField::init (src/GaugeField.cpp:39-98): neighbour tables of the
// spatial index, restated with the same arguments (L1 = Lx, L2 = Ly).
void gauge_neighbours(int L1, int L2, std::vector<int> &iup, std::vector<int> &idown) {
  long const V3 = static_cast<long>(L1) * L1 * L2;
  iup.assign(3 * V3, 0);
  idown.assign(3 * V3, 0);
  int const L0_h = L1 * L2;
  int x0_h[3], x1_h[3], x2_h[3];
  for (int x0 = 0; x0 < L1; ++x0) {
    x0_h[2] = x0 * L0_h;
    x0_h[0] = x0 - 1 < 0 ? L0_h * (L1 - 1) : (x0 - 1) * L0_h;
    x0_h[1] = x0 + 1 == L1 ? 0 : (x0 + 1) * L0_h;
    for (int x1 = 0; x1 < L1; ++x1) {
      x1_h[2] = x1 * L2;
      x1_h[0] = x1 - 1 < 0 ? L2 * (L1 - 1) : (x1 - 1) * L2;
      x1_h[1] = x1 + 1 == L1 ? 0 : (x1 + 1) * L2;
      for (int x2 = 0; x2 < L2; ++x2) {
        x2_h[2] = x2;
        x2_h[0] = x2 - 1 < 0 ? L2 - 1 : x2 - 1;
        x2_h[1] = x2 + 1 == L2 ? 0 : x2 + 1;
        long const i = x0_h[2] + x1_h[2] + x2_h[2];
        iup[3 * i + 0] = x0_h[1] + x1_h[2] + x2_h[2];
        iup[3 * i + 1] = x0_h[2] + x1_h[1] + x2_h[2];
        iup[3 * i + 2] = x0_h[2] + x1_h[2] + x2_h[1];
        idown[3 * i + 0] = x0_h[0] + x1_h[2] + x2_h[2];
        idown[3 * i + 1] = x0_h[2] + x1_h[0] + x2_h[2];
        idown[3 * i + 2] = x0_h[2] + x1_h[2] + x2_h[0];
      }
    }
  }
}

// displace_eigenvectors (src/OperatorFactory.cpp:33-55) with forward_uv /
// backward_uv (src/GaugeField.cpp:543-560): every step sweeps the sites in
// index order and updates the eigenvector in place, so a site reads the
// already-displaced value of a neighbour that precedes it.  U points to the
// timeslice's links [site][dir][a + 3 b].
void displace(Mat &res, cd const *U, slaph_vdv_op const &op, std::vector<int> const &iup,
              std::vector<int> const &idown) {
  long const V3 = res.r / 3;
  for (int k = 0; k < op.n_disp; ++k) {
    char const fb = op.disp[2 * k], axis = op.disp[2 * k + 1];
    int const dir = axis == 'x' ? 0 : axis == 'y' ? 1 : 2;
    for (int ev = 0; ev < res.c; ++ev) {
      cd *v = &res.d[static_cast<size_t>(res.r) * ev];
      for (long s = 0; s < V3; ++s) {
        cd out[3];
        if (fb == '>') {
          long const up = iup[3 * s + dir];
          cd const *u = U + (3 * s + dir) * 9;
          for (int a = 0; a < 3; ++a) {
            out[a] = 0;
            for (int b = 0; b < 3; ++b) out[a] += mul(u[a + 3 * b], v[3 * up + b]);
          }
        } else {
          long const dn = idown[3 * s + dir];
          cd const *u = U + (3 * dn + dir) * 9;
          for (int a = 0; a < 3; ++a) {
            out[a] = 0;
            for (int b = 0; b < 3; ++b) out[a] += mul(std::conj(u[b + 3 * a]), v[3 * dn + b]);
          }
        }
        for (int a = 0; a < 3; ++a) v[3 * s + a] = out[a];
      }
    }
  }
}

// ---------------------------------------------------------------- HYP smearing
using M3 = std::array<cd, 9>;  // 3x3, element (a, b) at a + 3 b
M3 m3_mul(M3 const &x, M3 const &y) {
  M3 r{};
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b)
      for (int k = 0; k < 3; ++k) r[a + 3 * b] += x[a + 3 * k] * y[k + 3 * b];
  return r;
}
M3 m3_adj(M3 const &x) {
  M3 r{};
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) r[a + 3 * b] = std::conj(x[b + 3 * a]);
  return r;
}
M3 m3_axpy(M3 const &x, double ax, M3 const &y, double ay) {
  M3 r{};
  for (int i = 0; i < 9; ++i) r[i] = x[i] * ax + y[i] * ay;
  return r;
}
cd m3_det(M3 const &m) {
  return m[0] * (m[4] * m[8] - m[7] * m[5]) - m[3] * (m[1] * m[8] - m[7] * m[2]) +
         m[6] * (m[1] * m[5] - m[4] * m[2]);
}
// H^(-1/2) of a Hermitian positive-definite 3x3 matrix from its eigen-
// decomposition by cyclic complex Jacobi rotations (pairs (0,1), (0,2), (1,2);
// stop when the off-diagonal norm is below 1e-16 of the diagonal's, at most
// 30 sweeps).  Eigen's principal matrix square root used by the reference
// equals V diag(sqrt(lambda)) V^H for such a matrix.
M3 m3_inv_sqrt(M3 h) {
  M3 v{};
  v[0] = v[4] = v[8] = 1.0;
  for (int sweep = 0; sweep < 30; ++sweep) {
    double off = std::norm(h[3]) + std::norm(h[6]) + std::norm(h[7]);
    double diag = std::norm(h[0]) + std::norm(h[4]) + std::norm(h[8]);
    if (off <= 1e-32 * diag) break;
    for (int p = 0; p < 2; ++p)
      for (int q = p + 1; q < 3; ++q) {
        cd const apq = h[p + 3 * q];
        double const r = std::abs(apq);
        if (r == 0) continue;
        cd const e = apq / r;  // phase of the element
        double const app = h[p + 3 * p].real(), aqq = h[q + 3 * q].real();
        double const th = (aqq - app) / (2 * r);
        double const t = (th >= 0 ? 1.0 : -1.0) / (std::abs(th) + std::sqrt(th * th + 1));
        double const c = 1 / std::sqrt(t * t + 1), sn = t * c;
        M3 g{};
        g[0] = g[4] = g[8] = 1.0;
        g[p + 3 * p] = c;
        g[p + 3 * q] = sn;
        g[q + 3 * p] = -sn * std::conj(e);
        g[q + 3 * q] = c * std::conj(e);
        h = m3_mul(m3_adj(g), m3_mul(h, g));
        h[p + 3 * q] = h[q + 3 * p] = 0.0;  // annihilated by the rotation
        v = m3_mul(v, g);
      }
  }
  M3 d{};
  for (int i = 0; i < 3; ++i) d[i + 3 * i] = 1 / std::sqrt(h[i + 3 * i].real());
  return m3_mul(v, m3_mul(d, m3_adj(v)));
}
// proj_to_su3_imp (src/GaugeField.cpp:203-210): M (M^H M)^(-1/2), divided by
// the principal cube root of its determinant.
M3 proj_su3(M3 const &m) {
  M3 out = m3_mul(m, m3_inv_sqrt(m3_mul(m3_adj(m), m)));
  cd const f = 1. / std::pow(m3_det(out), 1. / 3.);
  for (auto &x : out) x *= f;
  return out;
}

// GaugeField::smearing_hyp (src/GaugeField.cpp:322-427) on one timeslice:
// U [site][dir][9], in place.
void smear_hyp(cd *U, long V3, double alpha1, double alpha2, int iter,
               std::vector<int> const &iup, std::vector<int> const &idown) {
  auto link = [&](long s, int d) {
    M3 m;
    std::copy(U + (3 * s + d) * 9, U + (3 * s + d) * 9 + 9, m.begin());
    return m;
  };
  static int const perp[3][2] = {{1, 2}, {0, 2}, {0, 1}};
  auto decor = [](int dir, int plane) {
    if (dir == 0) return plane == 1 ? 0 : 3;
    if (dir == 1) return plane == 0 ? 1 : 4;
    return plane == 0 ? 2 : 5;
  };
  std::vector<M3> dec(static_cast<size_t>(V3) * 6), fresh(static_cast<size_t>(V3) * 3);
  for (int run = 0; run < iter; ++run) {
    for (long v = 0; v < V3; ++v)
      for (int dir = 0; dir < 3; ++dir)
        for (int n = 0; n < 2; ++n) {
          int const pd = perp[dir][n];
          long mu = iup[3 * v + pd];
          long const eta = iup[3 * v + dir];
          M3 inner = m3_mul(link(v, pd), m3_mul(link(mu, dir), m3_adj(link(eta, pd))));
          mu = idown[3 * v + pd];
          long const nu = iup[3 * mu + dir];
          M3 const down = m3_mul(m3_adj(link(mu, pd)), m3_mul(link(mu, dir), link(nu, pd)));
          for (int i = 0; i < 9; ++i) inner[i] += down[i];
          dec[6 * v + dir + 3 * n] = proj_su3(m3_axpy(link(v, dir), 1 - alpha2, inner, alpha2 / 2.));
        }
    for (long i = 0; i < V3; ++i)
      for (int dir = 0; dir < 3; ++dir) {
        M3 outer{};
        for (int nd = 0; nd < 3; ++nd) {
          if (nd == dir) continue;
          int const plane = ((dir + 1) ^ (nd + 1)) - 1;
          long mu = iup[3 * i + nd];
          long nu = iup[3 * mu + dir];
          long const eta = idown[3 * nu + nd];
          int const a = decor(nd, plane), b = decor(dir, plane);
          M3 const up = m3_mul(dec[6 * i + a], m3_mul(dec[6 * mu + b], m3_adj(dec[6 * eta + a])));
          mu = idown[3 * i + nd];
          nu = iup[3 * mu + dir];
          M3 const dn = m3_mul(m3_adj(dec[6 * mu + a]), m3_mul(dec[6 * mu + b], dec[6 * nu + a]));
          for (int k = 0; k < 9; ++k) outer[k] += up[k] + dn[k];
        }
        fresh[3 * i + dir] = m3_axpy(link(i, dir), 1 - alpha1, outer, alpha1 / 4.);
      }
    for (long i = 0; i < V3; ++i)
      for (int d = 0; d < 3; ++d) {
        M3 const p = proj_su3(fresh[3 * i + d]);
        std::copy(p.begin(), p.end(), U + (3 * i + d) * 9);
      }
  }
}

int vdaggerv_impl(const slaph_dims *dims, const slaph_vdv_op *ops, int n_ops,
                  int index_of_unity, const double *const *V, const double *const *U,
                  const int *ts, int n_ts, double *out) {
  return guarded([&] {
    check_dims(dims);
    int const nev = dims->nev;
    long const vol = static_cast<long>(dims->Lx) * dims->Ly * dims->Lz;
    long const dim_row = 3 * vol;
    bool displaced = false;
    for (int i = 0; i < n_ops; ++i) {
      if (ops[i].id != i) throw std::runtime_error("VdaggerV ids must be 0..n_ops-1");
      if (ops[i].n_disp != 0 && ops[i].id != index_of_unity) displaced = true;
    }
    if (displaced && !U) throw std::runtime_error("displaced operators need a gauge field");
    std::vector<int> iup, idown;
    if (displaced) gauge_neighbours(dims->Lx, dims->Ly, iup, idown);
    // momentum[op.id][x], src/OperatorFactory.cpp:209-215.
    std::vector<cd> momentum(static_cast<size_t>(n_ops) * vol);
    for (int i = 0; i < n_ops; ++i)
      create_momentum(dims->Lx, dims->Ly, dims->Lz, ops[i].momentum, &momentum[i * vol]);
    std::vector<int> tlist;
    if (ts)
      tlist.assign(ts, ts + n_ts);
    else
      for (int t = 0; t < dims->Lt; ++t) tlist.push_back(t);
    size_t const blk = static_cast<size_t>(nev) * nev;
    // The reference distributes timeslices over its threads
    // (src/OperatorFactory.cpp:263-272); the (timeslice, operator) pairs are
    // distributed here, which gives the same blocks and also keeps every
    // thread busy when only a few timeslices are asked for.
    size_t const n_items = tlist.size() * static_cast<size_t>(n_ops);
#pragma omp parallel num_threads(oracle_threads())
    {
      std::vector<cd> W(static_cast<size_t>(dim_row) * nev);
#pragma omp for schedule(dynamic)
      for (size_t it = 0; it < n_items; ++it) {
        int const t = tlist[it / n_ops];
        int const o = static_cast<int>(it % n_ops);
        cd const *Vt = reinterpret_cast<cd const *>(V[t]);
        {
          cd *dst = reinterpret_cast<cd *>(out) + (static_cast<size_t>(o) * dims->Lt + t) * blk;
          if (ops[o].id == index_of_unity) {
            for (size_t i = 0; i < blk; ++i) dst[i] = 0;  // identity, :317
            for (int i = 0; i < nev; ++i) dst[i + static_cast<size_t>(nev) * i] = 1.0;
          } else if (ops[o].n_disp != 0) {
            // W = D(V) (:289-290); the momentum is not applied to displaced operators
            Mat res(static_cast<int>(dim_row), nev);
            std::copy(Vt, Vt + dim_row * nev, res.d.begin());
            displace(res, reinterpret_cast<cd const *>(U[t]), ops[o], iup, idown);
            gemm_ah_b(Vt, res.d.data(), dim_row, nev, dst);  // :300
          } else {
            // W = diag(mom) V with mom(x) = momentum[x / 3] (:292-297)
            cd const *mom = &momentum[ops[o].id * vol];
            for (int j = 0; j < nev; ++j)
              for (long x = 0; x < dim_row; ++x)
                W[x + dim_row * j] = mul(mom[x / 3], Vt[x + dim_row * j]);
            gemm_ah_b(Vt, W.data(), dim_row, nev, dst);  // :300
          }
        }
      }
    }
  });
}

}  // namespace

extern "C" {

const char *oracle_last_error(void) { return g_err.c_str(); }

int oracle_threads(void) { return g_threads > 0 ? g_threads : omp_get_max_threads(); }
void oracle_set_threads(int n) { g_threads = n; }

void oracle_create_momentum(int Lx, int Ly, int Lz, const int p[3], double *out) {
  create_momentum(Lx, Ly, Lz, p, reinterpret_cast<cd *>(out));
}

void oracle_gamma_table(int32_t *row, double *value) {
  auto const &g = gamma_table();
  for (int m = 0; m < 16; ++m)
    for (int c = 0; c < 4; ++c) {
      row[4 * m + c] = g[m].row[c];
      value[2 * (4 * m + c)] = g[m].value[c].real();
      value[2 * (4 * m + c) + 1] = g[m].value[c].imag();
    }
}

int oracle_vdaggerv(const slaph_dims *dims, const slaph_vdv_op *ops, int n_ops,
                    int index_of_unity, const double *const *V, const int *ts, int n_ts,
                    double *out) {
  return vdaggerv_impl(dims, ops, n_ops, index_of_unity, V, nullptr, ts, n_ts, out);
}

int oracle_smear_hyp(const slaph_dims *dims, double *const *U, double alpha1, double alpha2,
                     int iterations) {
  return guarded([&] {
    check_dims(dims);
    long const V3 = static_cast<long>(dims->Lx) * dims->Ly * dims->Lz;
    std::vector<int> iup, idown;
    gauge_neighbours(dims->Lx, dims->Ly, iup, idown);
#pragma omp parallel for num_threads(oracle_threads())
    for (int t = 0; t < dims->Lt; ++t)
      smear_hyp(reinterpret_cast<cd *>(U[t]), V3, alpha1, alpha2, iterations, iup, idown);
  });
}

namespace {
// Columns of V^H W in double-double arithmetic, W = diag(mom) V (mom given)
// or W given (Wd, exact double entries).
int vdaggerv_columns_dd(const slaph_dims *dims, const int *p, const double *Vt, const double *Wd,
                        const int *cols, int n_cols, double *out) {
  return guarded([&] {
    check_dims(dims);
    int const nev = dims->nev;
    long const vol = static_cast<long>(dims->Lx) * dims->Ly * dims->Lz;
    long const dim_row = 3 * vol;
    std::vector<cd> mom(vol, cd(1.0, 0.0));
    if (p) create_momentum(dims->Lx, dims->Ly, dims->Lz, p, mom.data());
    cd const *V = reinterpret_cast<cd const *>(Vt);
    cd const *Wg = reinterpret_cast<cd const *>(Wd);
    // Error-free transformations: a b = p + e exactly (fma), a + b = s + e
    // exactly (Knuth); a double-double value is hi + lo with |lo| <= ulp(hi)/2.
    auto two_prod = [](double a, double b, double &e) {
      double const q = a * b;
      e = std::fma(a, b, -q);
      return q;
    };
    auto two_sum = [](double a, double b, double &e) {
      double const s = a + b, bb = s - a;
      e = (a - (s - bb)) + (b - bb);
      return s;
    };
    struct DD {
      double hi = 0, lo = 0;
    };
    auto dd_add = [&](DD x, double h, double l) {  // x + (h + l)
      double e;
      double const s = two_sum(x.hi, h, e);
      e += x.lo + l;
      DD r;
      r.hi = s + e;
      r.lo = e - (r.hi - s);
      return r;
    };
    for (int c = 0; c < n_cols; ++c) {
      int const j = cols[c];
      if (j < 0 || j >= nev) throw std::runtime_error("column out of range");
      // w = diag(mom) V_j in double-double: w_x = (wr + wrl) + i (wi + wil)
      std::vector<double> wr(dim_row), wrl(dim_row), wi(dim_row), wil(dim_row);
      for (long x = 0; x < dim_row; ++x) {
        cd const m = Wg ? cd(1.0, 0.0) : mom[x / 3];
        cd const v = Wg ? Wg[x + dim_row * j] : V[x + dim_row * j];
        double e1, e2, e3, e4;
        double const a = two_prod(m.real(), v.real(), e1), b = two_prod(m.imag(), v.imag(), e2);
        double const c1 = two_prod(m.real(), v.imag(), e3), d = two_prod(m.imag(), v.real(), e4);
        DD r = dd_add(DD{a, e1}, -b, -e2), i = dd_add(DD{c1, e3}, d, e4);
        wr[x] = r.hi;
        wrl[x] = r.lo;
        wi[x] = i.hi;
        wil[x] = i.lo;
      }
#pragma omp parallel for schedule(dynamic) num_threads(oracle_threads())
      for (int i = 0; i < nev; ++i) {
        DD re, im;  // sum_x conj(V(x, i)) w_x
        for (long x = 0; x < dim_row; ++x) {
          cd const v = V[x + dim_row * i];
          double e;
          double h = two_prod(v.real(), wr[x], e);
          re = dd_add(re, h, e + v.real() * wrl[x]);
          h = two_prod(v.imag(), wi[x], e);
          re = dd_add(re, h, e + v.imag() * wil[x]);
          h = two_prod(v.real(), wi[x], e);
          im = dd_add(im, h, e + v.real() * wil[x]);
          h = two_prod(v.imag(), wr[x], e);
          im = dd_add(im, -h, -e - v.imag() * wrl[x]);
        }
        out[2 * (static_cast<long>(c) * nev + i)] = re.hi + re.lo;
        out[2 * (static_cast<long>(c) * nev + i) + 1] = im.hi + im.lo;
      }
    }
  });
}
}  // namespace

int oracle_vdaggerv_columns_dd(const slaph_dims *dims, const int p[3], const double *Vt,
                               const int *cols, int n_cols, double *out) {
  return vdaggerv_columns_dd(dims, p, Vt, nullptr, cols, n_cols, out);
}

int oracle_vdaggerv_columns_dd_w(const slaph_dims *dims, const double *Vt, const double *Wt,
                                 const int *cols, int n_cols, double *out) {
  return vdaggerv_columns_dd(dims, nullptr, Vt, Wt, cols, n_cols, out);
}

int oracle_displace_eigenvectors(const slaph_dims *dims, const slaph_vdv_op *op,
                                 const double *Vt, const double *Ut, double *out) {
  return guarded([&] {
    check_dims(dims);
    if (dims->Lx != dims->Ly || dims->Lx != dims->Lz)
      throw std::runtime_error("displaced operators need a cubic lattice");
    long const dim_row = 3L * dims->Lx * dims->Ly * dims->Lz;
    std::vector<int> iup, idown;
    gauge_neighbours(dims->Lx, dims->Ly, iup, idown);
    Mat res(static_cast<int>(dim_row), dims->nev);
    cd const *V = reinterpret_cast<cd const *>(Vt);
    std::copy(V, V + dim_row * dims->nev, res.d.begin());
    displace(res, reinterpret_cast<cd const *>(Ut), *op, iup, idown);
    std::copy(res.d.begin(), res.d.end(), reinterpret_cast<cd *>(out));
  });
}

int oracle_vdaggerv_gauge(const slaph_dims *dims, const slaph_vdv_op *ops, int n_ops,
                          int index_of_unity, const double *const *V, const double *const *U,
                          const int *ts, int n_ts, double *out) {
  return vdaggerv_impl(dims, ops, n_ops, index_of_unity, V, U, ts, n_ts, out);
}

int oracle_contract(const slaph_dims *dims, const slaph_plan *plan, const double *vdv,
                    const double *const *peram, const double *noise, int accumulator,
                    int single_block_pair, double *out) {
  return guarded([&] {
    check_dims(dims);
    Inputs in{*dims, plan, vdv, peram, noise, plan->n_vdv_ops, accumulator == SLAPH_ACC_KAHAN};
    DilScheme const ds(dims->Lt, dims->dilT, DilType::block);
    int const n_bp = ds.size();
    int const Lt = dims->Lt;

    // Per block pair, the values of every (diagram, slice pair, request) in the
    // order a single-threaded run of src/Correlators.cpp:86-116 produces them.
    std::vector<std::vector<cd>> vals(n_bp);
    std::vector<std::vector<std::pair<int, int>>> slices(n_bp);
    for (int b = 0; b < n_bp; ++b) slices[b] = ds.slices(b);
    std::string err;
    bool failed = false;
#pragma omp parallel num_threads(oracle_threads())
    {
      Parts q(in, ds);
#pragma omp for schedule(dynamic)
      for (int b = 0; b < n_bp; ++b) {
        if (single_block_pair >= 0 && single_block_pair != b) continue;
        bool stop;
#pragma omp atomic read
        stop = failed;
        if (stop) continue;
        try {
          for (int d = 0; d < plan->n_diagrams; ++d) {
            auto const &dg = plan->diagrams[d];
            for (auto const &sp : slices[b])
              for (int i = 0; i < dg.n_requests; ++i)
                vals[b].push_back(resolve(dg.requests[i], sp.first, sp.second, q, in.kahan));
          }
        } catch (std::exception const &e) {
#pragma omp critical(oracle_err)
          {
            failed = true;
            err = e.what();
          }
        }
        q.clear();
      }
    }
    if (failed) throw std::runtime_error(err);

    // Diagram::assemble / write (src/Diagram.cpp:96-147): per-request values
    // summed per time difference, then divided by Lt.
    long total = 0;
    std::vector<long> offset(plan->n_diagrams);
    for (int d = 0; d < plan->n_diagrams; ++d) {
      offset[d] = total;
      total += plan->diagrams[d].n_requests;
    }
    std::vector<cd> corr(static_cast<size_t>(total) * Lt, cd(0, 0));
    for (int b = 0; b < n_bp; ++b) {
      if (single_block_pair >= 0 && single_block_pair != b) continue;
      size_t k = 0;
      for (int d = 0; d < plan->n_diagrams; ++d) {
        int const nr = plan->diagrams[d].n_requests;
        for (auto const &sp : slices[b]) {
          // get_time_delta, src/Correlators.cpp:21-23 (C++ % truncates).
          int const dt = std::abs((sp.second - sp.first - Lt) % Lt);
          for (int i = 0; i < nr; ++i) corr[(offset[d] + i) * Lt + dt] += vals[b][k++];
        }
      }
    }
    for (size_t i = 0; i < corr.size(); ++i) {
      cd const v = corr[i] / static_cast<double>(Lt);
      out[2 * i] = v.real();
      out[2 * i + 1] = v.imag();
    }
  });
}

int oracle_contract_sample(const slaph_dims *dims, const slaph_plan *plan, const double *vdv,
                           const double *const *peram, const double *noise,
                           const int *block_pairs, int n, double *cold_s, double *steady_s) {
  return guarded([&] {
    check_dims(dims);
    Inputs in{*dims, plan, vdv, peram, noise, plan->n_vdv_ops, false};
    DilScheme const ds(dims->Lt, dims->dilT, DilType::block);
    for (int i = 0; i < n; ++i)
      if (block_pairs[i] < 0 || block_pairs[i] >= ds.size())
        throw std::runtime_error("block pair out of range");
    std::string err;
    bool failed = false;
    // One block pair per thread, as the block-pair loop of
    // src/Correlators.cpp:86-116 distributes them.
#pragma omp parallel for schedule(dynamic, 1) num_threads(oracle_threads())
    for (int i = 0; i < n; ++i) {
      try {
        std::pair<int, int> sp{-1, -1};
        for (auto const &s : ds.slices(block_pairs[i]))
          if (s.first != s.second) {
            sp = s;
            break;
          }
        if (sp.first < 0) throw std::runtime_error("block pair has no off-diagonal slice pair");
        Parts q(in, ds);
        auto resolve_all = [&] {
          for (int d = 0; d < plan->n_diagrams; ++d) {
            auto const &dg = plan->diagrams[d];
            for (int r = 0; r < dg.n_requests; ++r)
              (void)resolve(dg.requests[r], sp.first, sp.second, q, false);
          }
        };
        double t0 = omp_get_wtime();
        resolve_all();
        cold_s[i] = omp_get_wtime() - t0;
        // Drop the traces that depend on both times; keep the factors and the
        // single-time traces, which later slice pairs of the block reuse.
        for (int k = 0; k < SLAPH_TR_KINDS; ++k)
          for (auto it = q.tr[k].begin(); it != q.tr[k].end();) {
            auto const &key = it->first;
            bool const pair_dep =
                std::any_of(key.begin(), key.end(), [&](int t) { return t != key[0]; });
            it = pair_dep ? q.tr[k].erase(it) : std::next(it);
          }
        t0 = omp_get_wtime();
        resolve_all();
        steady_s[i] = omp_get_wtime() - t0;
      } catch (std::exception const &e) {
#pragma omp critical(oracle_sample_err)
        {
          failed = true;
          err = e.what();
        }
      }
    }
    if (failed) throw std::runtime_error(err);
  });
}

int oracle_read_eigenvectors(const char *path, long dim_row, int nev, double *out) {
  return guarded([&] {
    FILE *fp = std::fopen(path, "rb");
    if (!fp) throw std::runtime_error("Eigenvector file does not exist!");
    for (int c = 0; c < nev; ++c) {
      size_t const n = std::fread(out + 2 * dim_row * c, sizeof(double), 2 * dim_row, fp);
      if (n != static_cast<size_t>(2 * dim_row)) {
        std::fclose(fp);
        throw std::runtime_error("Problem while reading Eigenvectors!");
      }
    }
    std::fclose(fp);
  });
}

int oracle_read_perambulator(const char *path, int Lt, int nev, int dilT, int dilE, int dilD,
                             double *out) {
  return guarded([&] {
    long const rows = 4L * nev * Lt;
    long const cols = static_cast<long>(Lt / dilT) * dilE * dilD;
    std::vector<cd> buf(static_cast<size_t>(rows) * cols);
    FILE *fp = std::fopen(path, "rb");
    if (!fp) throw std::runtime_error(std::string("failed to open file to read perambulator: ") + path);
    size_t const n = std::fread(buf.data(), sizeof(cd), buf.size(), fp);
    std::fclose(fp);
    if (n != buf.size()) throw std::runtime_error("Failed to read perambulator.");
    // Re-sort, src/Perambulator.cpp:53-64.
    long const nb_inv = static_cast<long>(Lt) * dilE * dilD / dilT;
    cd *P = reinterpret_cast<cd *>(out);
    for (long i = 0; i < rows * cols; ++i) P[i] = 0;
    for (long t1 = 0; t1 < Lt; ++t1)
      for (long ev1 = 0; ev1 < nev; ++ev1)
        for (long d1 = 0; d1 < 4; ++d1)
          for (long t2 = 0; t2 < Lt / dilT; ++t2)
            for (long ev2 = 0; ev2 < dilE; ++ev2)
              for (long d2 = 0; d2 < dilD; ++d2) {
                long const row_i = 4 * nev * t1 + 4 * ev1 + d1;
                long const col_i = dilD * dilE * t2 + dilD * ev2 + d2;
                long const r = 4 * nev * t1 + nev * d1 + ev1;
                long const c = dilE * dilD * t2 + dilE * d2 + ev2;
                P[r + rows * c] = buf[row_i * nb_inv + col_i];
              }
  });
}

int oracle_read_random_vector(const char *path, long length, double *out) {
  return guarded([&] {
    FILE *fp = std::fopen(path, "rb");
    if (!fp) throw std::runtime_error(std::string("failed to open file to read random vector: ") + path);
    size_t const n = std::fread(out, sizeof(cd), length, fp);
    std::fclose(fp);
    if (n != static_cast<size_t>(length))
      throw std::runtime_error("It seems that not all data are read from random vector file");
  });
}

long oracle_dilution_text(int num_slice, int num_block, int type, char *buf, long len) {
  std::string s;
  char line[256];
  DilType const ty = type == 0 ? DilType::block : DilType::interlace;
  char const *name = type == 0 ? "B" : "I";
  int const block_size = num_slice / num_block;
  std::snprintf(line, sizeof line, "T = %d, T%s%d (Morningstar), T%s%d (Other):\n\n", num_slice,
                name, num_block, name, block_size);
  s += line;
  DilScheme ds(num_slice, block_size, ty);
  for (int b = 0; b < ds.size(); ++b) {
    auto bl = ds.blocks(b);
    std::snprintf(line, sizeof line, "%2d => %2d\n", bl.first, bl.second);
    s += line;
    for (auto const &sp : ds.slices(b)) {
      std::snprintf(line, sizeof line, "  %2d -> %2d\n", sp.first, sp.second);
      s += line;
    }
  }
  s += "\n\n";
  if (buf && len > 0) {
    std::strncpy(buf, s.c_str(), len - 1);
    buf[len - 1] = 0;
  }
  return static_cast<long>(s.size()) + 1;
}

int oracle_block_pair_slices(int Lt, int dilT, int i, int *out, int cap) {
  if (Lt <= 0 || dilT <= 0 || Lt % dilT != 0) return -1;
  DilScheme const ds(Lt, dilT, DilType::block);
  if (i < 0 || i >= ds.size()) return -1;
  auto const sl = ds.slices(i);
  for (size_t k = 0; k < sl.size() && static_cast<int>(k) < cap; ++k) {
    out[2 * k] = sl[k].first;
    out[2 * k + 1] = sl[k].second;
  }
  return static_cast<int>(sl.size());
}

double oracle_kahan_sum(const double *xs, long n) {
  double sum = 0, c = 0;
  for (long i = 0; i < n; ++i) {
    double const t = sum + xs[i];
    if (std::abs(sum) >= std::abs(xs[i]))
      c += (sum - t) + xs[i];
    else
      c += (xs[i] - t) + sum;
    sum = t;
  }
  return sum + c;
}

}  // extern "C"
