// Symbolic schedule of contract(): which diluted factors, factor products,
// diluted traces and correlator terms one gauge configuration needs, as flat
// work lists for the device kernels.
//
// The schedule replays the reference control flow without data:
//   contract            src/Correlators.cpp:40-127 (block pairs, slice pairs)
//   Diagram::assemble   src/Diagram.cpp:96-130, resolve_request{1,2,3} :9-94
//   DilutedTrace*Factory::build   src/DilutedTraceFactory.cpp:13-245
//   DilutedFactorFactory<Q>::build src/DilutedFactorFactory.cpp:34-253
//   operator* / multiply<1,1>     src/DilutedFactor.cpp:6-51,
//                                 include/DilutedFactor.hpp:164-187
//   factor_to_trace               src/DilutedTrace.cpp:84-165
//   inner_product                 src/DilutedTrace.cpp:5-82
// Random-vector pairs and used-index masks decide which products and traces
// exist; they depend only on the lookup tables, so the schedule is built once
// per plan on the host and reused for every gauge configuration.
//
// Work is split into waves, one per block pair, like the reference's
// per-block-pair cache clearing (src/Correlators.cpp:116): diluted factors are
// global (built once), products, traces and terms are wave-local.
#pragma once

#include <array>
#include <cstdint>
#include <string>
#include <vector>

#include "../../../include/slaph_gb300.h"

namespace slaph {

// Intermediate products shared by many factors (they do not depend on the
// gamma structure, src/DilutedFactorFactory.cpp:66-78,134-144,203-218):
//  Q0M[t, vdv, r2]     = VdV(t) * R2        (nev x 4dilE)
//  Q1R[t, vdv, r1]     = R1^H * VdV(t)      (4dilE x nev)
//  Q2M[t, b1, r1, vdv] = P_r1(t,.,b1)^H VdV (4dilE x 4nev, before gamma_5 signs)
// "vdv" is a VdaggerV id combined with its dagger flag: 2*id + dagger.
struct Q0MInst {
  int32_t t, vdv, r2;
};
struct Q1RInst {
  int32_t t, vdv, r1;
};
struct Q2MInst {
  int32_t t, b1, r1, vdv;
};

// One diluted factor matrix (4dilE x 4dilE, column-major) at matrix slot.
struct Q0Inst {
  int32_t t, m, r1, gamma, slot;  // m: Q0M index
};
struct Q1Inst {
  int32_t t, b, r, r2, gamma, slot;  // r: Q1R index
};
struct Q2Inst {
  int32_t t, b2, m, r2, gamma, slot;  // m: Q2M index
};
// c = a * b on matrix slots.
struct ProdInst {
  int32_t a, b, c;
};

// Entries of a trace list as index pairs into its operand lists: the value of
// entry e is tr(L[i[e]] * R[j[e]]), or tr(L[i[e]]) when j[e] < 0.  Shapes
// depend only on (trace kind, trace id).
struct TraceShape {
  std::vector<int32_t> i, j;
  std::vector<uint16_t> mask;  // used random-vector indices of each entry
};

// One diluted-trace list: operand lists start at matrix slots a_base / b_base
// (b_base < 0 for single-matrix traces); the value of entry e is element
// val_off + e * stride of the wave's trace-value array.
struct TraceList {
  int32_t shape;
  int32_t a_base, b_base;
  int32_t stride;
  int64_t val_off;
};

// Two-matrix trace lists of one shape whose operand groups form a complete
// bipartite set: every A group (a_base) with every B group (b_base).  For each
// entry (i, j) of the shape, the values of all n_a x n_b lists are one complex
// matrix product sum_k A[a + i]_k B[b + j]^T_k, a GEMM of n_a x n_b dot
// products.  The value of list (ia, ib), entry e, is at
// val_base + e * n_a * n_b + ib * n_a + ia.
struct TraceGroup {
  int32_t shape, n_a, n_b, pad;
  int64_t a_off, b_off;  // A bases at group_bases[a_off...], B at [b_off...]
  int64_t val_base;
};

// resolve_request for one (request, slice pair): a combination of n trace
// lists, added to output[out][dt].
struct Term {
  int32_t n;
  int32_t list[3];  // wave-local trace list ids
  int32_t out;      // global request index
  int32_t dt;       // get_time_delta, src/Correlators.cpp:21-23
};

struct Wave {
  int32_t block_pair;
  std::vector<ProdInst> prods;        // ordered by dependency level
  std::vector<int64_t> prod_level_off;  // prods of level k: [off[k], off[k+1])
  std::vector<TraceList> lists;
  int64_t n_values = 0;
  // Lists that repeat the operands of an earlier list share its values.  Of
  // the distinct lists, those in groups are dense GEMMs; the rest, residual,
  // are computed entry by entry.  Group values come first: [0, n_group_values).
  std::vector<TraceGroup> groups;
  std::vector<int32_t> group_bases;
  int64_t n_group_values = 0, n_group_entries = 0;
  std::vector<int32_t> unique_lists;    // one list per distinct operand set
  std::vector<int32_t> residual_lists;  // distinct lists outside groups
  std::vector<Term> terms;            // reference order within the block pair
  int64_t n_prod_slots = 0;           // product slots used (after factor slots)
  // Work of this wave (flops, 8 per complex multiply-add).
  double flops_products = 0, flops_traces = 0;
  int64_t n_trace_entries = 0;
};

struct Schedule {
  slaph_dims dims{};
  int32_t eds = 0;  // 4 * dilE, side of every factor matrix
  int32_t n_vdv = 0;

  std::vector<Q0MInst> q0m;
  std::vector<Q1RInst> q1r;
  std::vector<Q2MInst> q2m;
  std::vector<Q0Inst> q0;
  std::vector<Q1Inst> q1;
  std::vector<Q2Inst> q2;
  int64_t n_factor_slots = 0;

  std::vector<TraceShape> shapes;
  std::vector<Wave> waves;
  int64_t n_outputs = 0;  // total requests
  int64_t max_prod_slots = 0, max_values = 0, max_terms = 0, max_lists = 0;

  double flops_factors = 0, flops_products = 0, flops_traces = 0;
  int64_t n_terms = 0, n_trace_entries = 0, n_prods = 0;
  // Trace entries computed after merging repeated lists, and those in groups.
  int64_t n_unique_entries = 0, n_group_entries = 0;
};

// Smallest operand-group counts for a dense trace group (GEMM tiles hold 64 A
// and 80 B groups); smaller bipartite sets stay residual.
constexpr int32_t kMinGroupA = 16, kMinGroupB = 16;

// Tensor-core plan of the products of one dependency level (operator*,
// src/DilutedFactor.cpp:6-51).  Left matrices are taken in order of first
// appearance; a group starts with the next unused one and adds, up to
// 64 / eds, the unused left matrix that shares the most right matrices with
// the group so far.  Column block u of group g is right matrix
// r_slots[u_list[g.u_off + u]]; out_tab[4 (g.u_off + u) + l] is the slot of
// product (left matrix l of g) x (that right matrix), or -1 when the level
// does not ask for it.  n_tiles counts the GEMM tiles of 80 columns.
struct ProductGroup {
  int32_t l[4];  // left-matrix slots, n_l of them
  int32_t n_l, n_u, u_off;
};
struct ProductPlan {
  std::vector<ProductGroup> groups;
  std::vector<int32_t> r_slots, u_list, out_tab;
  int64_t n_tiles = 0;
};
ProductPlan plan_products(ProdInst const *prods, int64_t n, int32_t eds);

// Builds the schedule; throws EmptyError with the reference's messages when a
// random-vector combination is empty.  single_block_pair >= 0 restricts the
// work to that block pair.
Schedule build_schedule(slaph_dims const &dims, slaph_plan const &plan, int single_block_pair);

}  // namespace slaph
