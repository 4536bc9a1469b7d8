/*
 * oracle.h — FP64 CPU oracle for the sLapH contraction hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a restatement, in plain C++ with OpenMP,
 * of the reference algorithm (pittlerf/sLapH-contractions) for VdaggerV, the
 * diluted factors Q0/Q1/Q2, factor products, diluted traces and correlator
 * assembly.  It is used by the tests (as the checker), by the smoke check and
 * by the CPU-baseline leg of bench.py.  The engine never links or calls it.
 *
 * Parity of this oracle is pinned against the reference's own goldens:
 * the 18 HDF5 files of tests/integration-L4/correlators-reference (checked with
 * h5diff -d 1e-12 by tests/integration-L4/compare:16), the gamma table test
 * tests/gtest/gamma.cpp, the Kahan tests tests/gtest/KahanAccumulatorTest.cpp,
 * the momentum test tests/gtest/create_momenta.cpp and the dilution-iterator
 * control text tests/dilution-iterator/control.txt.
 *
 * The lookup tables are taken as input in the flat slaph_plan form of
 * include/slaph_gb300.h, exactly as contract() takes them as arguments
 * (include/Correlators.hpp:41-54).
 */
#ifndef SLAPH_ORACLE_H
#define SLAPH_ORACLE_H

#include "../include/slaph_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Message of the last failed oracle call on this thread. */
const char *oracle_last_error(void);

/* Number of OpenMP threads the oracle will use (after oracle_set_threads). */
int oracle_threads(void);
void oracle_set_threads(int n);

/* create_momenta (src/OperatorFactory.cpp:64-95) for one momentum:
 * out[2*L^3] = exp(-i 2pi (px x/Lx + py y/Ly + pz z/Lz)), x slowest. */
void oracle_create_momentum(int Lx, int Ly, int Lz, const int p[3], double *out);

/* Gamma table (src/Gamma.cpp:18-246), derived here from the dense tmLQCD
 * gamma_0..gamma_3 and their products: row[16][4], value[16][4][2]. */
void oracle_gamma_table(int32_t *row, double *value);

/* OperatorFactory::build_vdaggerv (src/OperatorFactory.cpp:220-326).
 * V[t] points to 2*3L^3*nev doubles (column-major).  out receives
 * [n_ops][Lt][nev][nev] complex column-major, identity for index_of_unity.
 * ts: which timeslices to compute (NULL = all); n_ts their count. */
int oracle_vdaggerv(const slaph_dims *dims, const slaph_vdv_op *ops, int n_ops,
                    int index_of_unity, const double *const *V, const int *ts, int n_ts,
                    double *out);

/* The same with displaced operators (src/OperatorFactory.cpp:33-55,289-290):
 * U[t] points to the timeslice's gauge links, [site][dir x,y,z][3x3 column-
 * major] complex (the GaugeField::tslices layout, src/GaugeField.cpp:108-149),
 * neighbours as GaugeField::init builds them (src/GaugeField.cpp:39-98). */
int oracle_vdaggerv_gauge(const slaph_dims *dims, const slaph_vdv_op *ops, int n_ops,
                          int index_of_unity, const double *const *V, const double *const *U,
                          const int *ts, int n_ts, double *out);

/* Columns cols[0..n_cols) of V_t^H diag(exp(-ipx)) V_t (the VdaggerV product
 * of src/OperatorFactory.cpp:292-300) in double-double arithmetic (error-free
 * products by fma, two-sum accumulation), a reference far more accurate than
 * FP64 for checking large-K VdaggerV blocks.  Vt: 2*3L^3*nev doubles
 * (column-major); out: [n_cols][nev][2]. */
int oracle_vdaggerv_columns_dd(const slaph_dims *dims, const int p[3], const double *Vt,
                               const int *cols, int n_cols, double *out);

/* The same for V_t^H W with W given (e.g. displaced eigenvectors from
 * oracle_displace_eigenvectors), W: 2*3L^3*nev doubles column-major. */
int oracle_vdaggerv_columns_dd_w(const slaph_dims *dims, const double *Vt, const double *Wt,
                                 const int *cols, int n_cols, double *out);

/* D(V_t) of one displaced operator (displace_eigenvectors,
 * src/OperatorFactory.cpp:33-55, in the reference's in-place sweep order) on
 * the timeslice's links Ut ([site][dir x,y,z][3x3 column-major]).
 * out: 2*3L^3*nev doubles column-major. */
int oracle_displace_eigenvectors(const slaph_dims *dims, const slaph_vdv_op *op,
                                 const double *Vt, const double *Ut, double *out);

/* GaugeField::smearing_hyp (src/GaugeField.cpp:322-427) of every timeslice,
 * in place on U[t] (layout as above), with proj_to_su3_imp (:203-210) taking
 * (M^H M)^(-1/2) from a Jacobi eigen-decomposition. */
int oracle_smear_hyp(const slaph_dims *dims, double *const *U, double alpha1, double alpha2,
                     int iterations);

/* contract() (src/Correlators.cpp:40-127) with the given VdaggerV array
 * ([n_ops][Lt][nev][nev]), perambulators peram[r] ((4 nev Lt) x
 * (Lt/dilT * dilE * 4) column-major) and noise ([n_rnd][Lt*4*nev]).
 * out: [total_requests][Lt][2] as slaph_contract writes it. */
int oracle_contract(const slaph_dims *dims, const slaph_plan *plan, const double *vdv,
                    const double *const *peram, const double *noise, int accumulator,
                    int single_block_pair, double *out);

/* Bounded timing sample of contract() for the CPU baseline.  For each listed
 * block pair (one per OpenMP thread) the first slice pair with distinct source
 * and sink times is resolved for every diagram and request from empty caches
 * (cold_s[i], seconds), then again after dropping only the traces that depend
 * on both times (steady_s[i]): the cost of a further slice pair of the same
 * block pair once its factors and single-time traces are cached. */
int oracle_contract_sample(const slaph_dims *dims, const slaph_plan *plan, const double *vdv,
                           const double *const *peram, const double *noise,
                           const int *block_pairs, int n, double *cold_s, double *steady_s);

/* Slice pairs (source, sink) of block pair i of the block dilution scheme, in
 * iteration order.  Returns the count; writes at most cap pairs to out. */
int oracle_block_pair_slices(int Lt, int dilT, int i, int *out, int cap);

/* The reference binary readers, restated (src/EigenVector.cpp:35-76,
 * src/Perambulator.cpp:12-71, src/RandomVector.cpp:87-113). */
int oracle_read_eigenvectors(const char *path, long dim_row, int nev, double *out);
int oracle_read_perambulator(const char *path, int Lt, int nev, int dilT, int dilE,
                             int dilD, double *out);
int oracle_read_random_vector(const char *path, long length, double *out);

/* Dilution scheme enumeration (include/dilution-iterator.hpp:21-356) in the
 * text format of main/test-iterator.cpp / src/dilution-iterator.cpp:19-35.
 * type: 0 block, 1 interlace.  Returns the bytes needed (incl. NUL). */
long oracle_dilution_text(int num_slice, int num_block, int type, char *buf, long len);

/* Neumaier sum of xs as KahanAccumulator<double> does it
 * (include/KahanAccumulator.hpp:14-48). */
double oracle_kahan_sum(const double *xs, long n);

#ifdef __cplusplus
}
#endif

#endif
