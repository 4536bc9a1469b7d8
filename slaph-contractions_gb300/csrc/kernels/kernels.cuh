// Launch wrappers of the engine's CUDA kernels (sm_103a).  All pointers are
// device pointers; complex numbers are double2 (re, im); matrices are
// column-major like Eigen::MatrixXcd.  Every wrapper enqueues on `stream` and
// returns the cudaError_t of the launch.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace slaph {
namespace dev {

struct Q0MInst {
  int32_t t, vdv, r2;
};
struct Q1RInst {
  int32_t t, vdv, r1;
};
struct Q2MInst {
  int32_t t, b1, r1, vdv;
};
struct Q0Inst {
  int32_t t, m, r1, gamma, slot;
};
struct Q1Inst {
  int32_t t, b, r, r2, gamma, slot;
};
struct Q2Inst {
  int32_t t, b2, m, r2, gamma, slot;
};
struct ProdInst {
  int32_t a, b, c;
};
struct TraceList {
  int32_t shape;
  int32_t a_base, b_base;
  int32_t stride;
  int64_t val_off;
};
struct Term {
  int32_t n;
  int32_t list[3];
  int32_t out;
  int32_t dt;
};

// Sizes every kernel needs.
struct Geometry {
  int32_t Lt, Lx, Ly, Lz, nev, dilE, n_rnd;
  int32_t nb;       // number of time-dilution blocks (Lt / dilT)
  int64_t dim_row;  // 3 * L^3
};

// Gamma table (src/Gamma.cpp:18-246) into constant memory.
// Gamma_m column c: row of its nonzero, and its value as a phase code
// (0: +1, 1: +i, 2: -1, 3: -i), for host-side planning.
int32_t gamma_row_host(int32_t m, int32_t c);
int32_t gamma_phase_host(int32_t m, int32_t c);
cudaError_t upload_gamma(cudaStream_t stream);

// One displacement step of W (a copy of V_t) in place on a cubic lattice, in
// the reference's sweep order (displace_eigenvectors,
// src/OperatorFactory.cpp:33-55); U: the timeslice's links [site][dir][a + 3 b].
// One HYP smearing iteration (GaugeField::smearing_hyp, src/GaugeField.cpp:
// 322-427) of n_t consecutive timeslices of links U ([t][site][dir][9]) of a
// cubic L^3 lattice, in place; dec: scratch of n_t
// hyp_scratch_doubles_per_timeslice(L) doubles (the decorated links).
int64_t hyp_scratch_doubles_per_timeslice(int32_t L);
cudaError_t hyp_smear(double2 *U, double2 *dec, int32_t L, int32_t n_t, double alpha1,
                      double alpha2, cudaStream_t stream);
cudaError_t displace(double2 *W, double2 const *U, int32_t dir, int32_t forward, Geometry g,
                     cudaStream_t stream);
// VdaggerV[2 op][t] = V_t^H W in FP64 (*op: device pointer to the operator id).
cudaError_t vdaggerv_fp64_w(double2 *vdv, double2 const *V, double2 const *W,
                            int32_t const *op, int32_t t, Geometry g, cudaStream_t stream,
                            int32_t v_t0 = 0);
// exp(-i p.x) for every op: phase[op][x] (create_momenta,
// src/OperatorFactory.cpp:64-95).  mom: [n_ops][3].
cudaError_t momenta(double2 *phase, int32_t const *mom, int32_t n_ops, Geometry g,
                    cudaStream_t stream);

// VdaggerV[vdv code 2*op][t] = V_t^H diag(phase[op] per site) V_t for every op
// in ops[0..n) (src/OperatorFactory.cpp:292-300), FP64.  V: consecutive
// timeslices [t][nev][dim_row] (each column-major), V[0] holding timeslice
// v_t0 (0: all Lt resident; a ring slot otherwise).  vdv: [2*n_ops][Lt][nev][nev].
cudaError_t vdaggerv_fp64(double2 *vdv, double2 const *V, double2 const *phase,
                          int32_t const *ops, int32_t n, int32_t t0, int32_t nt, Geometry g,
                          cudaStream_t stream, int32_t v_t0 = 0);
// Split-BF16 tensor-core VdaggerV (vdv_tc.cu): same result as vdaggerv_fp64
// to ~1e-13 relative.  scratch: device buffer of at least
// vdaggerv_tc_scratch_bytes(g, n, batch) bytes, where batch timeslices are
// processed per launch (vdaggerv_tc_batch picks it from the SM count, the
// timeslice count and a memory cap); err: device int, set non-zero when a bounded wait gave up.
size_t vdaggerv_tc_scratch_bytes(Geometry g, int32_t n_ops, int32_t batch);
// phase_fx[k] = round(phase[k] 2^62) per component, the fixed-point phases the
// split-precision VdaggerV multiplies with integer arithmetic.
cudaError_t phase_fixed(longlong2 *phase_fx, double2 const *phase, int64_t n,
                        cudaStream_t stream);
// Timeslices per GEMM launch for n_t timeslices: at most what max_bytes of
// scratch holds, chosen for the fewest rounds of one tile per SM over all
// launches (the last round of each launch is the partly idle one).
int32_t vdaggerv_tc_batch(Geometry g, int32_t n_ops, int32_t sm_count, size_t max_bytes,
                          int32_t n_t);
// Displaced operators of the split-precision VdaggerV: ops[n_comp + d] is
// V_t^H D_d(V_t), D_d the displacement steps of operator d applied in place to
// a copy W of V_t (displace above), momentum not applied.
constexpr int kMaxDispSteps = 8;
struct VdvDisplaced {
  int32_t n;                     // number of displaced operators
  int32_t const *n_steps;        // host: steps per operator
  int32_t const *steps;          // host: [n][kMaxDispSteps][2] (dir 0..2, forward 0/1)
  double2 const *U;              // device: links [Lt][site][dir][9]
  double2 *W;                    // device: nev x dim_row scratch
  longlong2 const *unit_phase;   // device: phase 1 in fixed point (2^62, 0) per site
  int32_t const *unit_op;        // device: {0}, the operator index into unit_phase
};
// ops: device list of n_comp momentum operators followed by disp->n displaced
// ones; scratch sized by vdaggerv_tc_scratch_bytes for all of them.
cudaError_t vdaggerv_tc(double2 *vdv, double2 const *V, longlong2 const *phase_fx,
                        int32_t const *ops, int32_t n_comp, int32_t t0, int32_t nt, Geometry g,
                        void *scratch, size_t scratch_bytes, int *err, cudaStream_t stream,
                        cudaEvent_t const *t_ready = nullptr,
                        VdvDisplaced const *disp = nullptr,
                        cudaEvent_t const *gemm_ev = nullptr, int32_t n_gemm_ev = 0,
                        int32_t v_t0 = 0, bool clear_scratch = true);
// (V: consecutive timeslices, V[0] holding timeslice v_t0.  clear_scratch:
// zero the scratch slots first (their padding rows must be zero); a later
// call on the same scratch in the same build may skip it.  t_ready[t], when
// given and non-null: event after which timeslice t of V is valid; the
// slicing of t waits for it on `stream`.  gemm_ev: when given, the
// events 2k and 2k+1 are recorded on `stream` just before and after the k-th
// GEMM launch, for k < n_gemm_ev / 2; vdaggerv_tc_gemm_launches gives k's range.)
int32_t vdaggerv_tc_gemm_launches(int32_t nt, int32_t batch);
// One bounded mbarrier wait that nothing completes (selftest.cu): *err = 1
// once it gives up after `cycles` clock cycles.
cudaError_t bounded_wait_selftest(int *err, long long cycles, cudaStream_t stream);
// Identity blocks for code 2*op (and 2*op+1).
cudaError_t vdaggerv_identity(double2 *vdv, int32_t op, Geometry g, cudaStream_t stream);
// vdv[2*op+1][t] = vdv[2*op][t]^H for all ops, t.
cudaError_t vdaggerv_daggers(double2 *vdv, int32_t n_ops, Geometry g, cudaStream_t stream);

// Factor intermediates and factors (src/DilutedFactorFactory.cpp:34-253).
cudaError_t q0m(double2 *out, Q0MInst const *inst, int64_t n, double2 const *vdv,
                double2 const *noise, Geometry g, cudaStream_t stream);
cudaError_t q1r(double2 *out, Q1RInst const *inst, int64_t n, double2 const *vdv,
                double2 const *noise, Geometry g, cudaStream_t stream);
cudaError_t q2m(double2 *out, Q2MInst const *inst, int64_t n, double2 const *vdv,
                double2 const *peram, Geometry g, cudaStream_t stream);
cudaError_t q0(double2 *slots, Q0Inst const *inst, int64_t n, double2 const *q0m,
               double2 const *noise, Geometry g, cudaStream_t stream);
cudaError_t q1(double2 *slots, Q1Inst const *inst, int64_t n, double2 const *q1r,
               double2 const *peram, Geometry g, cudaStream_t stream);
cudaError_t q2(double2 *slots, Q2Inst const *inst, int64_t n, double2 const *q2m,
               double2 const *peram, Geometry g, cudaStream_t stream);

// slots[c] = slots[a] * slots[b] (operator*, src/DilutedFactor.cpp:6-51).
cudaError_t products(double2 *slots, ProdInst const *p, int64_t n, int32_t eds,
                     cudaStream_t stream);

// Trace values of every entry of the lists lists[which[0..n_which)]
// (factor_to_trace, src/DilutedTrace.cpp:84-165), entry e of list L at
// values[L.val_off + e * L.stride].  shape_i/shape_j: entry operand indices,
// shape_off: [n_shapes+1] offsets into them.
cudaError_t traces(double2 *values, TraceList const *lists, int32_t const *which,
                   int64_t n_which, int32_t const *shape_i, int32_t const *shape_j,
                   int64_t const *shape_off, double2 const *slots, int32_t eds,
                   cudaStream_t stream);

// Mixed path: matrices in double-float form (float4 = re hi, re lo, im hi,
// im lo per complex), written as stored (dst_n) and transposed (dst_t); traces
// as compensated FP32 dot products over unit-stride operands.
cudaError_t split_df(float4 *dst_n, float4 *dst_t, double2 const *src, int64_t n, int32_t eds,
                     cudaStream_t stream);
// Mixed path: FP64 -> double-float (float4) copy.
cudaError_t to_df(float4 *dst, double2 const *src, int64_t n, cudaStream_t stream);
// Mixed path: all factor intermediates and factors in double-float; factors
// written into the slot buffers in both layouts (sn stored, st transposed).
cudaError_t factors_df(float4 *sn, float4 *st, float4 *q0m_buf, float4 *q1r_buf,
                       float4 *q2m_buf, Q0MInst const *q0m_i, int64_t n_q0m,
                       Q1RInst const *q1r_i, int64_t n_q1r, Q2MInst const *q2m_i, int64_t n_q2m,
                       Q0Inst const *q0_i, int64_t n_q0, Q1Inst const *q1_i, int64_t n_q1,
                       Q2Inst const *q2_i, int64_t n_q2, float4 const *vdv,
                       float4 const *noise, float4 const *peram, Geometry g,
                       cudaStream_t stream);
// slots[c] = slots[a] * slots[b] in double-float, both layouts written.
cudaError_t products_df(float4 *slots_n, float4 *slots_t, ProdInst const *p, int64_t n,
                        int32_t eds, cudaStream_t stream);
// The same products on the tensor cores (product_tc.cu), for eds = 16, 32 or
// 64.  The products of one dependency level come in groups of up to 64 / eds
// left matrices (slots l[0..n_l)) with the union of their right matrices:
// column block u of group g is right matrix u_list[g.u_off + u] (an index into
// the level's r_slots) and out_tab[4 (g.u_off + u) + l] is the slot of product
// l x u, or -1 when the level does not ask for it.  Tiles: (group, n tile of
// 80 columns).  Scratch: the groups' A regions (prod_tc_a_bytes each) from 0,
// the right-matrix streams (prod_tc_r_bytes each) from r_off; exponents: 64
// per group from 0, eds per right matrix from r_expo.  slot_bits (as
// slot_maxbits; zero for the level's product slots before the call) receives
// the largest |re|, |im| of every product written.
struct ProdGroup {
  int32_t l[4];   // left-matrix slots
  int32_t n_l;    // left matrices in the group (1 .. 64 / eds)
  int32_t n_u;    // right matrices in the union
  int32_t u_off;  // first column block in u_list / out_tab
  int32_t ea;     // exponent index of the group's row 0 (64 g)
};
struct ProdTile {
  int32_t group, nt;
};
__host__ __device__ inline int64_t prod_tc_r_bytes(int32_t eds) {
  return 24LL * eds * eds;  // (eds / 16) k-tiles x 6 slices x eds columns x 32 bytes
}
bool prod_tc_supported(int32_t eds);
int64_t prod_tc_a_bytes(int32_t eds);
cudaError_t products_tc(float4 *slots_n, float4 *slots_t, uint8_t *scratch, int64_t r_off,
                        int32_t *expo, int64_t r_expo, ProdGroup const *groups, int64_t n_groups,
                        int32_t const *r_slots, int64_t n_r, int32_t const *u_list,
                        int32_t const *out_tab, ProdTile const *tiles, int64_t n_tiles,
                        int32_t eds, unsigned int *slot_bits, int *err, cudaStream_t stream);
// Trace values as double-float pairs (re_hi, re_lo, im_hi, im_lo) into
// values_df, laid out as for traces().
cudaError_t traces_df(float4 *values_df, TraceList const *lists, int32_t const *which,
                      int64_t n_which, int32_t const *shape_i, int32_t const *shape_j,
                      int64_t const *shape_off, float4 const *slots_n, float4 const *slots_t,
                      int32_t eds, cudaStream_t stream);
// Dense trace groups on the tensor cores (trace_tc.cu).  One matrix slot
// sliced into the operand stream of a GEMM region:
struct TrSlice {
  int64_t dst;   // byte offset of the region in the scratch buffer
  int32_t slot;  // matrix slot
  int32_t row;   // complex row (A region) or column (B region) of the matrix
  int32_t expo;  // index of the matrix's exponent in the exponent array
  int32_t pad;
};
// Matrices of one 8-row core-matrix group of a region, sliced together so that
// every store covers whole core matrices: kTrSliceRowsA consecutive complex
// rows of an A region (eight rows of A', two per matrix) or kTrSliceRowsB
// consecutive columns of a B region, from a row that is a multiple of that
// count; exponent indices expo0, expo0 + 1, ...
constexpr int32_t kTrSliceRowsA = 4, kTrSliceRowsB = 8;
struct TrSliceGroup {
  int64_t dst;    // byte offset of the region in the scratch buffer
  int32_t row0;   // first row (A) or column (B) of the group
  int32_t n;      // matrices in the group (1 .. 4 for A, 1 .. 8 for B)
  int32_t expo0;  // exponent index of the first matrix
  int32_t slot[8];
  int32_t pad;
};
// One output tile of 64 A groups x 80 B groups of one (group, entry) GEMM.
struct TrTile {
  int64_t a_src, b_src;  // byte offsets of the tile's A and B operand streams
  int64_t out;           // value index of tile row 0, column 0
  int32_t ea, eb;        // exponent indices of tile row 0 and column 0
  int32_t rows, cols;    // valid rows (<= 64) and columns (<= 80)
  int32_t ld;            // value index distance between columns
  int32_t pad;
};
constexpr int32_t kTrTileRows = 64, kTrTileCols = 80;
int64_t trace_tc_k_tiles(int32_t eds);
size_t trace_tc_a_bytes(int32_t rows, int32_t eds);  // A region of `rows` matrices
size_t trace_tc_b_bytes(int32_t cols, int32_t eds);  // B region of `cols` matrices
// Largest |re|, |im| of each matrix slot first..first+n (double-float,
// natural layout, high words) as float bits: the slicing of the trace
// operands takes each matrix's exponent from it instead of scanning the
// matrix again for each group region it appears in.
cudaError_t slot_maxbits(unsigned int *bits, float4 const *slots, int64_t first, int64_t n,
                         int32_t eds, cudaStream_t stream);
// Slices the A matrices (natural layout, conjugated) and B matrices
// (transposed layout) of a batch into their regions of `scratch`, one row
// group per CTA, with the largest entries of their slots (slot_maxbits).
cudaError_t trace_tc_slice(uint8_t *scratch, int32_t *expo, TrSliceGroup const *a_groups,
                           int64_t n_a, TrSliceGroup const *b_groups, int64_t n_b,
                           float4 const *slots_n, float4 const *slots_t,
                           unsigned int const *slot_bits, int32_t eds, cudaStream_t stream);
// The GEMM tiles of a batch; FP64 trace values into `values`.
cudaError_t trace_tc_gemm(double2 *values, uint8_t const *scratch, int32_t const *expo,
                          TrTile const *tiles, int64_t n_tiles, int32_t eds, int *err,
                          cudaStream_t stream);

// Generic form of the same GEMM (factor_tc.cu): k_tiles k-tiles of 16
// complex entries; region sizes for `rows` A rows / `cols` B columns.
size_t tc_a_bytes(int32_t rows, int32_t k_tiles);
size_t tc_b_bytes(int32_t cols, int32_t k_tiles);
int32_t gemm_k_tiles(int64_t K);
cudaError_t tc_gemm(double2 *out, uint8_t const *scratch, int32_t const *expo,
                    TrTile const *tiles, int64_t n_tiles, int32_t k_tiles, int *err,
                    cudaStream_t stream);

// One GEMM operand row (A) or column (B) gathered from up to four strided
// segments of a source array, each with an exact factor (0: +1, 1: +i, 2: -1,
// 3: -i).  K = n_seg * seg_len, zero-padded to the region's k-tiles.
struct GSeg {
  int64_t src;
  int32_t factor;
  int32_t pad;
};
constexpr int kGMaxSeg = 4;
struct GVec {
  int64_t dst;     // byte offset of the region in the scratch buffer
  int64_t stride;  // element stride along K inside a segment
  int32_t row;     // row (A) or column (B) within the region
  int32_t expo;    // index of its exponent
  int32_t n_seg, seg_len;
  GSeg seg[kGMaxSeg];
};
// Slices operand vectors (A rows with put conj(v) when conj, or B columns)
// from an FP64 or a double-float source.
cudaError_t gvec_slice_f64(uint8_t *scratch, int32_t *expo, GVec const *items, int64_t n,
                           bool is_a, bool conj, double2 const *src, int32_t k_tiles,
                           cudaStream_t stream);
cudaError_t gvec_slice_df(uint8_t *scratch, int32_t *expo, GVec const *items, int64_t n,
                          bool is_a, bool conj, float4 const *src, int32_t k_tiles,
                          cudaStream_t stream);
// Q1 factor slots from the dense product X1 (factor_tc.cu); Q2 slots from the
// dense Q2 GEMM output.
struct Q1Gather {
  int64_t x_off;  // element offset of X1 of the factor's timeslice
  int32_t ld, row0, col0, gamma, slot, pad;
};
struct Q2Gather {
  int64_t off;  // element offset of the factor's (0, 0) entry
  int32_t ld, slot;
};
cudaError_t upload_gamma_tc(cudaStream_t stream);
cudaError_t q1_gather(float4 *sn, float4 *st, Q1Gather const *g, int64_t n, double2 const *x,
                      int32_t dilE, cudaStream_t stream);
cudaError_t q2_gather(float4 *sn, float4 *st, Q2Gather const *g, int64_t n, double2 const *y,
                      int32_t eds, cudaStream_t stream);

// values[i] = hi + lo of values_df[i] for i < n_values, the FP64 trace values
// the terms read.
cudaError_t df_values_to_fp64(double2 *values, float4 const *values_df, int64_t n_values,
                              cudaStream_t stream);

// Term values (resolve_request / inner_product, src/Diagram.cpp:9-94,
// src/DilutedTrace.cpp:5-82) with the native (0) or Kahan (1) accumulator.
cudaError_t terms(double2 *term_val, Term const *t, int64_t n, TraceList const *lists,
                  double2 const *values, uint16_t const *shape_mask,
                  int64_t const *shape_off, int32_t kahan, cudaStream_t stream);

// running[o] += term_val[idx[k]] for k in [seg[o], seg[o+1]) in order
// (Diagram::assemble, src/Diagram.cpp:96-114).
cudaError_t accumulate(double2 *running, int32_t const *seg_out, int64_t const *seg_off,
                       int64_t n_seg, int32_t const *idx, double2 const *term_val,
                       cudaStream_t stream);

}  // namespace dev
}  // namespace slaph
