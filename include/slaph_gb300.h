/*
 * slaph_gb300.h — C ABI of the GB300 engine for the sLapH contraction hot path.
 *
 * The reference (pittlerf/sLapH-contractions) has no plugin or FFI layer: its
 * hot path sits behind ordinary C++ classes that main/contract.cpp calls.  Each
 * entry point below replaces one of those seams; the reference file:line it
 * stands in for is given beside it.  Everything is plain C: opaque handles,
 * plain pointers and sizes, int status codes (0 = ok), no exceptions across
 * the boundary.  Complex numbers are interleaved (re, im) doubles, exactly the
 * std::complex<double> byte layout the reference stores.
 *
 * Ownership: the caller owns every buffer it passes; the engine copies what it
 * needs to device memory before a call returns.  The engine owns all device
 * memory (eigenvectors, perambulators, noise, VdaggerV, factor caches).
 *
 * Threading: one host thread drives one engine.  Distinct engines are
 * independent.
 */
#ifndef SLAPH_GB300_H
#define SLAPH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define SLAPH_OK 0
#define SLAPH_ERR_ARG 1         /* invalid argument or size mismatch            */
#define SLAPH_ERR_CUDA 2        /* CUDA runtime error                           */
#define SLAPH_ERR_STATE 3       /* call out of order (e.g. contract before VdV) */
#define SLAPH_ERR_IO 4          /* file could not be opened / read / written    */
#define SLAPH_ERR_EMPTY 5       /* empty random-vector combination; the
                                   reference throws std::runtime_error here
                                   (src/DilutedFactor.cpp:44-48,
                                    src/DilutedTrace.cpp:37-41,131-135)          */
#define SLAPH_ERR_UNSUPPORTED 6 /* feature not provided by this engine          */
#define SLAPH_ERR_NOMEM 7       /* device or host allocation failed             */
#define SLAPH_ERR_PARSE 8       /* infile could not be parsed                   */
#define SLAPH_ERR_TIMEOUT 9     /* a bounded device wait gave up                */

/* ---- enums ------------------------------------------------------------- */
enum slaph_precision {
  SLAPH_FP64 = 0,  /* every product in FP64                                   */
  SLAPH_MIXED = 1  /* VdaggerV and the traces of dense trace groups as
                      split-BF16 tensor-core products with exact FP32 partial
                      sums; diluted factors, factor products and the other
                      traces in compensated double-float (2 x FP32)
                      arithmetic; terms and correlator sums in FP64.
                      Correlators agree with SLAPH_FP64 to about 1e-12
                      relative (tested at 1e-10)                                */
};

/* How long the diluted factors of a contraction live (slaph_engine_set_factor_lifetime). */
enum slaph_factor_lifetime {
  SLAPH_FACTORS_CONFIGURATION = 0, /* built once per configuration and kept for
                                      every block pair (the default)           */
  SLAPH_FACTORS_BLOCK_PAIR = 1     /* built per block pair and dropped after it,
                                      as the reference clears its factor caches
                                      per block pair (src/Correlators.cpp:116)  */
};

enum slaph_accumulator {
  SLAPH_ACC_NATIVE = 0, /* NativeAccumulator (include/KahanAccumulator.hpp:50-72) */
  SLAPH_ACC_KAHAN = 1   /* KahanAccumulator  (include/KahanAccumulator.hpp:14-48) */
};

/* Trace kinds, one per DilutedTrace*Factory of include/Diagram.hpp:44-89. */
enum slaph_trace_kind {
  SLAPH_TR_Q1 = 0,          /* "trQ1"            arity 1 */
  SLAPH_TR_Q1Q1 = 1,        /* "trQ1Q1"          arity 2 */
  SLAPH_TR_Q0Q2 = 2,        /* "trQ0Q2"          arity 2 */
  SLAPH_TR_Q1Q1Q1 = 3,      /* "trQ1Q1Q1"        arity 3 */
  SLAPH_TR_Q1Q0Q2 = 4,      /* "trQ1Q0Q2"        arity 3 */
  SLAPH_TR_Q1Q1Q1Q1 = 5,    /* "trQ1Q1Q1Q1"      arity 4 */
  SLAPH_TR_Q2Q0Q2Q0 = 6,    /* "trQ2Q0Q2Q0"      arity 4 */
  SLAPH_TR_Q2Q0Q2Q0Q2Q0 = 7,/* "trQ2Q0Q2Q0Q2Q0"  arity 6 */
  SLAPH_TR_KINDS = 8
};

#define SLAPH_MAX_DISP 8

/* ---- plain-data mirrors of the reference lookup tables ----------------- */

/* Lattice and dilution sizes shared by every call.  dilT is the number of
 * time slices per dilution block, as contract() uses it
 * (src/Correlators.cpp:65; DilutionScheme(Lt, dilT) in
 *  include/dilution-iterator.hpp:312-313).  n_rnd is the total number of
 * random vectors over all quark flavours (src/global_data.cpp:271-273). */
typedef struct {
  int32_t Lt, Lx, Ly, Lz;
  int32_t nev;
  int32_t dilT, dilE;
  int32_t n_rnd;
} slaph_dims;

/* VdaggerVQuantumNumbers (include/typedefs.hpp:44-55).  disp holds n_disp
 * (direction, axis) character pairs such as ('>', 'x'). */
typedef struct {
  int32_t id;
  int32_t momentum[3];
  int32_t n_disp;
  char disp[2 * SLAPH_MAX_DISP];
} slaph_vdv_op;

/* DilutedFactorIndex (include/typedefs.hpp:105-121).  Only gamma[0] is used
 * by the factor builders (src/DilutedFactorFactory.cpp:44,132,228). */
typedef struct {
  int32_t id_vdaggerv;
  int32_t need_vdaggerv_daggering;
  int32_t gamma;
  int32_t n_rnd_pairs;
  const int32_t *rnd_pairs; /* [n_rnd_pairs][2]: (first, second) */
} slaph_factor_index;

/* TraceRequest (include/global_data.hpp:72-81).  loc[i] is 0 for
 * Location::source and 1 for Location::sink. */
typedef struct {
  int32_t kind; /* enum slaph_trace_kind */
  int32_t tr_id;
  int32_t n_loc;
  int32_t loc[6];
} slaph_trace_request;

/* CorrelatorRequest (include/global_data.hpp:83-90). */
typedef struct {
  int32_t n_traces; /* 1, 2 or 3 */
  slaph_trace_request traces[3];
  const char *dataset_name;
} slaph_correlator_request;

/* One entry of CorrelatorRequestsMap (include/global_data.hpp:92). */
typedef struct {
  const char *name; /* "C2c", "C4cD", ... */
  int32_t n_requests;
  const slaph_correlator_request *requests;
} slaph_diagram;

/* All lookup tables that contract() receives (include/Correlators.hpp:41-54):
 * OperatorLookup, DilutedFactorIndicesCollection ("Q0","Q1","Q2"),
 * TraceIndicesCollection and CorrelatorRequestsMap, flattened.
 * trace_ql_ids[k] is [n_trace_ids[k]][arity(k)] row-major.  Diagrams appear in
 * the std::map order of the reference (sorted by name). */
typedef struct {
  int32_t n_vdv_ops;
  const slaph_vdv_op *vdv_ops;
  int32_t index_of_unity; /* -1 if absent */
  int32_t need_gaugefield;
  int32_t n_factors[3];
  const slaph_factor_index *factors[3];
  int32_t n_trace_ids[SLAPH_TR_KINDS];
  const int32_t *trace_ql_ids[SLAPH_TR_KINDS];
  int32_t n_diagrams;
  const slaph_diagram *diagrams;
} slaph_plan;

/* Arity (number of quark lines) of a trace kind. */
int slaph_trace_kind_arity(int kind);
/* Name ("trQ0Q2", ...) of a trace kind, or NULL. */
const char *slaph_trace_kind_name(int kind);

/* ---- error reporting --------------------------------------------------- */
/* Message of the last failed call made on this thread (never NULL). */
const char *slaph_last_error(void);

/* ---- front end: infile -> lookup tables -------------------------------- */
/* Replaces read_parameters() (src/global_data.cpp:61-390) together with
 * input_handling() (src/global_data_input_handling.cpp:249-275) and
 * init_lookup_tables() (src/init_lookup_tables.cpp:470-556).
 * argv (may be NULL) holds command-line overrides in the reference's
 * "--key value" form, e.g. {"--start_config", "1000"}. */
typedef struct slaph_frontend slaph_frontend;

int slaph_frontend_create(const char *infile_path, int argc, const char *const *argv,
                          slaph_frontend **out);
int slaph_frontend_destroy(slaph_frontend *fe);
/* Lattice and dilution sizes (dilT, dilE of quark 0, as main/contract.cpp:147,
 * 180-181 passes them). */
int slaph_frontend_dims(const slaph_frontend *fe, slaph_dims *out);
/* Flattened lookup tables; the pointer stays valid until destroy. */
int slaph_frontend_plan(const slaph_frontend *fe, const slaph_plan **out);
/* Integer settings: "start_config", "end_config", "delta_config",
 * "single_time_slice_combination", "n_quarks", "nb_eigen_threads",
 * "iterations" (HYP smearing steps). */
int slaph_frontend_get_int(const slaph_frontend *fe, const char *key, int64_t *out);
/* Floating-point settings: "alpha1", "alpha2" (HYP smearing strengths,
 * src/global_data.cpp:127-135). */
int slaph_frontend_get_double(const slaph_frontend *fe, const char *key, double *out);
/* String settings: "output_path", "path_eigenvectors", "name_eigenvectors",
 * "handling_vdaggerv", "path_vdaggerv", "path_config". */
int slaph_frontend_get_str(const slaph_frontend *fe, const char *key, char *buf, size_t len);
/* File names for one gauge configuration (build_IO_names,
 * src/global_data_build_IO_names.cpp:76-85).  which: 0 = eigenvector prefix
 * (append "%03d" t), 1 = perambulator of random vector index, 2 = random
 * vector of index, 3 = correlator file suffix ("_cnfg%04d.h5"), 4 = gauge
 * configuration ("<path_config>/conf.%04d", src/GaugeField.cpp:765-766). */
int slaph_frontend_io_name(const slaph_frontend *fe, int config, int which, int index,
                           char *buf, size_t len);

/* ---- input staging: the reference binary formats ------------------------ */
/* EigenVector::read_eigen_vector (src/EigenVector.cpp:35-76): one timeslice,
 * nev columns of 3*L^3 complex, column-major.  out: 2*3*L^3*nev doubles. */
int slaph_read_eigenvectors(const char *path, int64_t dim_row, int32_t nev, double *out);
/* Perambulator::read_perambulator (src/Perambulator.cpp:12-71) including the
 * re-sort into (4*nev*Lt) x (Lt/dilT*dilE*dilD) column-major. */
int slaph_read_perambulator(const char *path, int32_t Lt, int32_t nev, int32_t dilT,
                            int32_t dilE, int32_t dilD, double *out);
/* RandomVector::read_random_vector (src/RandomVector.cpp:87-113): Lt*4*nev
 * complex entries, index dirac + 4*(ev + nev*t). */
int slaph_read_random_vector(const char *path, int64_t length, double *out);
/* GaugeField::read_gauge_field with map_timeslice_to_eigen
 * (src/GaugeField.cpp:108-149,762-928): the double-precision ILDG field of a
 * LIME file, written per timeslice as [site][dir][3x3 column-major] complex
 * with site x*Ly*Lz + y*Lz + z and the spatial directions x, y, z (the layout
 * slaph_engine_set_gauge takes); n_dir = 4 adds the temporal link as a fourth
 * direction.  out: Lt*Lx*Ly*Lz*n_dir*18 doubles.  Single-precision files are
 * refused with SLAPH_ERR_UNSUPPORTED, as the reference refuses them. */
int slaph_read_gauge_lime(const char *path, int32_t Lt, int32_t Lx, int32_t Ly, int32_t Lz,
                          int32_t n_dir, double *out);

/* ---- output: the reference HDF5 layout --------------------------------- */
/* WriteHDF5Correlator (include/h5-wrapper.hpp:106-200,
 * src/h5-wrapper.cpp:18-26): one file per diagram; one 1-D dataset of Lt
 * compound {re f64, im f64} per correlator request.  data is
 * [n_datasets][Lt][2].  Existing files are replaced. */
int slaph_write_correlators_h5(const char *file_path, int32_t n_datasets,
                               const char *const *dataset_names, int32_t Lt,
                               const double *data);

/* ---- engine ------------------------------------------------------------ */
typedef struct slaph_engine slaph_engine;

/* Creates an engine on the current CUDA device.  Allocates the device arrays
 * for perambulators and noise; the eigenvectors of all timeslices are
 * allocated by the first slaph_engine_set_eigenvectors (or a ring of a few
 * timeslices by slaph_engine_set_eigenvector_slots). */
int slaph_engine_create(const slaph_dims *dims, slaph_engine **out);
int slaph_engine_destroy(slaph_engine *eng);

/* OperatorFactory ctor (src/OperatorFactory.cpp:184-218): the VdaggerV lookup
 * table and the identity index.  Momentum phases are built on the device
 * (create_momenta, src/OperatorFactory.cpp:64-95). */
int slaph_engine_set_operators(slaph_engine *eng, const slaph_vdv_op *ops, int32_t n_ops,
                               int32_t index_of_unity);
/* Host -> device copies of the inputs (layouts as the readers above).  The
 * plain forms return when the copy is done.  The _async forms only enqueue it
 * on the engine's upload stream and return at once: slaph_vdaggerv_build then
 * waits for each eigenvector timeslice just before it needs it (overlapping
 * the remaining copies with VdaggerV work) and slaph_contract for the
 * perambulators and noise.  The host buffer of an _async call must stay valid
 * and unchanged until the build (eigenvectors) or contract (perambulators,
 * noise) that consumes it returns; page-locked buffers (slaph_host_alloc) make
 * the copy asynchronous, pageable ones are copied before the call returns.
 * The reference reads each eigenvector timeslice inside the VdaggerV loop
 * (src/OperatorFactory.cpp:274-278); these calls are the device-side
 * counterpart of that overlap.  slaph_contract uses the VdaggerV of the last
 * slaph_vdaggerv_build, so the next configuration's eigenvectors may be
 * uploaded between a build and the contraction that follows it. */
int slaph_engine_set_eigenvectors(slaph_engine *eng, int32_t t, const double *V);
/* Eigenvectors streamed per timeslice, as the reference reads them inside its
 * VdaggerV loop (src/OperatorFactory.cpp:263-300), for lattices whose
 * eigenvectors do not fit on the device next to everything else (48^3 x 96,
 * Nev 220: 112 GB).  n_slots >= 2: the engine keeps a ring of n_slots
 * timeslices instead of all Lt; both eigenvector setters then only record the
 * host buffer of timeslice t, and slaph_vdaggerv_build copies the timeslices
 * n_slots / 2 at a time into one half of the ring while it computes the other,
 * so every host buffer must stay valid and unchanged until the build returns
 * (page-locked buffers from slaph_host_alloc copy at the full link rate).
 * n_slots = 0 returns to all timeslices resident (the default).  Earlier
 * eigenvector uploads and VdaggerV are discarded by a change. */
int slaph_engine_set_eigenvector_slots(slaph_engine *eng, int32_t n_slots);

/* Factor lifetime of the following contractions (enum slaph_factor_lifetime).
 * With SLAPH_FACTORS_CONFIGURATION every diluted factor of the configuration
 * is built once and kept, which is fastest but needs device memory for all of
 * them (two double-float layouts of (4 dilE)^2 entries each: about 60 GB at
 * 32^3 x 64 pipi I=1, 207 GB at 48^3 x 96 with pipi I=1 + KK).  With
 * SLAPH_FACTORS_BLOCK_PAIR the contraction runs block pair by block pair, each
 * with the factors it uses, built for it and dropped after it, as the
 * reference's DiagramParts caches are (src/Correlators.cpp:69-116): factors
 * used by several block pairs are built several times, device memory holds
 * one block pair's.  Correlators are summed in the same order either way. */
int slaph_engine_set_factor_lifetime(slaph_engine *eng, int mode);
int slaph_engine_set_perambulator(slaph_engine *eng, int32_t rnd_id, const double *peram);
int slaph_engine_set_random_vector(slaph_engine *eng, int32_t rnd_id, const double *noise);
int slaph_engine_set_eigenvectors_async(slaph_engine *eng, int32_t t, const double *V);
int slaph_engine_set_perambulator_async(slaph_engine *eng, int32_t rnd_id, const double *peram);
int slaph_engine_set_random_vector_async(slaph_engine *eng, int32_t rnd_id, const double *noise);

/* Gauge links of timeslice t for displaced operators: V3 x 3 x 9 complex
 * doubles, link (site s, direction d = x, y, z) as a column-major 3x3 matrix at
 * (3 s + d) 9 — the GaugeField::tslices layout (src/GaugeField.cpp:108-149)
 * without its unused fourth direction, unsmeared (slaph_engine_smear_gauge_hyp
 * smears the stored links afterwards).  Sites and neighbours
 * are those of GaugeField::init (src/GaugeField.cpp:39-98); displaced
 * operators need a cubic spatial lattice.  A displaced VdaggerV is
 * V_t^H D(V_t) with the displacement steps applied in the reference's in-place
 * sweep order (displace_eigenvectors, src/OperatorFactory.cpp:33-55); the
 * momentum of a displaced operator is not applied, as in the reference
 * (:289-298).  Needed for every timeslice before slaph_vdaggerv_build when the
 * operator table holds displaced operators. */
int slaph_engine_set_gauge(slaph_engine *eng, int32_t t, const double *U);

/* The time dilution (slices per block) for the contractions that follow.  In
 * the reference it is an argument of contract() (include/Correlators.hpp:41-54,
 * DilutionScheme at src/Correlators.cpp:65), given after OperatorFactory has
 * built VdaggerV without it (src/OperatorFactory.cpp:184-218): a caller that
 * creates the engine before it knows dilT sets it here.  dilT must divide Lt.
 * VdaggerV, eigenvectors and noise stay; a change re-makes the perambulator
 * buffer, whose columns depend on the number of time blocks, so the
 * perambulators are uploaded after this call. */
int slaph_engine_set_time_dilution(slaph_engine *eng, int32_t dilT);

/* Replaces the smearing step of OperatorFactory::create_operators
 * (src/OperatorFactory.cpp:253-260): GaugeField::smearing_hyp
 * (src/GaugeField.cpp:322-427) with (alpha1, alpha2, iterations) applied on
 * the device to the stored links of every timeslice, in place, in FP64.  The
 * SU(3) back-projection proj_to_su3_imp (:203-210) takes (M^H M)^(-1/2) from a
 * Jacobi eigen-decomposition, equal to the reference's Eigen matrix square
 * root to rounding.  Needs slaph_engine_set_gauge for every timeslice first;
 * iterations = 0 leaves the links unchanged (the reference's default). */
int slaph_engine_smear_gauge_hyp(slaph_engine *eng, double alpha1, double alpha2,
                                 int32_t iterations);
/* Copy the stored (possibly smeared) links of timeslice t back to the host, in
 * the slaph_engine_set_gauge layout. */
int slaph_engine_gauge_fetch(slaph_engine *eng, int32_t t, double *out);

/* Self-test of the bounded device waits that every tensor-core pipeline stage
 * uses: one kernel waits on an mbarrier that nothing completes, gives up after
 * `cycles` clock cycles and reports it (*device_code = 1); the context stays
 * usable.  Returns SLAPH_OK when the wait gave up as designed.  No
 * counterpart in the reference (it has no device code). */
int slaph_selftest_bounded_wait(int64_t cycles, int32_t *device_code);

/* Page-locked host memory for the inputs, so that the set_* copies above run
 * at the full host-device link rate.  slaph_host_alloc returns driver-pinned
 * memory (cudaHostAlloc) that keeps that rate for its whole lifetime; free it
 * with slaph_host_free.  slaph_host_register / _unregister instead register a
 * caller-owned buffer; on systems whose GPU reads host page tables (Grace),
 * pages the kernel later moves (e.g. huge-page collapse of large anonymous
 * mappings) fall back to a slow staged copy, so long-lived input buffers are
 * better taken from slaph_host_alloc.  No counterpart in the reference (its
 * inputs never leave host memory). */
int slaph_host_alloc(size_t bytes, void **out);
int slaph_host_free(void *ptr);
int slaph_host_register(void *ptr, size_t bytes);
int slaph_host_unregister(void *ptr);

/* OperatorFactory::build_vdaggerv (src/OperatorFactory.cpp:220-326):
 * VdaggerV[op][t] = V_t^dagger diag(exp(-ipx)) V_t for every op of the lookup,
 * identity for index_of_unity.  precision: enum slaph_precision. */
int slaph_vdaggerv_build(slaph_engine *eng, int precision);
/* OperatorFactory::return_vdaggerv (include/OperatorsForMesons.hpp:66-69):
 * nev x nev column-major complex into out (2*nev*nev doubles). */
int slaph_vdaggerv_fetch(slaph_engine *eng, int32_t op_id, int32_t t, double *out);

/* VdaggerV files: the handling_vdaggerv modes of
 * OperatorFactory::create_operators (src/OperatorFactory.cpp:507-520).
 * "write" (:225-237, 302-312, write_vdaggerv :144-168): after a build, every
 * operator but the unity is written per timeslice to
 * "/<path>/cnfg%04d/operators.%04d.p_<p>.d_<d>.t_%03d" as nev x nev
 * column-major complex doubles (the directory is created).  "read"
 * (read_vdaggerv, :328-393): the blocks are read from
 * "/<path>/cnfg%04d/operators.%04d.p_<p>_.t_%03d" (no displacement; not the
 * name "write" produces).  "liuming" (read_vdaggerv_liuming, :395-490): one
 * file "/<path>/VdaggerV.p<x>p<y>p<z>.conf%04d" holds all timeslices as
 * row-major blocks; the file of -p is read and adjointed, else the file of +p
 * is read as is.  <p> is the concatenation of std::to_string of the momentum
 * components, <d> the displacement pairs ("000" for none).  After a read the
 * unity operator and the dagger copies are set as after a build, and
 * slaph_contract may follow.  Missing or short files give SLAPH_ERR_IO (the
 * reference constructs the same message without throwing it). */
#define SLAPH_VDV_FILE_WRITE 0
#define SLAPH_VDV_FILE_READ 1
#define SLAPH_VDV_FILE_LIUMING_MINUS 2
#define SLAPH_VDV_FILE_LIUMING_PLUS 3
int slaph_vdaggerv_write(slaph_engine *eng, const char *path_vdaggerv, int32_t config);
/* liuming: 0 for the "read" mode, 1 for the "liuming" mode. */
int slaph_vdaggerv_read(slaph_engine *eng, const char *path_vdaggerv, int32_t config,
                        int32_t liuming);
/* The file name of one operator (and timeslice, for kinds WRITE and READ). */
int slaph_vdaggerv_file_name(const char *path_vdaggerv, int32_t config, const slaph_vdv_op *op,
                             int32_t t, int32_t kind, char *buf, size_t len);

/* contract() (src/Correlators.cpp:40-127, include/Correlators.hpp:41-54).
 * corr_out receives, for every diagram of plan (plan order) and every request
 * (request order), Lt complex values C[t] = sum / Lt exactly as Diagram::write
 * stores them (src/Diagram.cpp:132-147): [total_requests][Lt][2] doubles.
 * single_block_pair >= 0 restricts the work to that block pair, as the
 * reference's --single_time_slice_combination (src/Correlators.cpp:88-90). */
int slaph_contract(slaph_engine *eng, const slaph_plan *plan, int precision, int accumulator,
                   int single_block_pair, double *corr_out);
/* Number of doubles slaph_contract writes for this plan. */
int64_t slaph_plan_output_doubles(const slaph_plan *plan, int32_t Lt);

/* Host-only view of the schedule slaph_contract builds for a plan (no GPU
 * needed): out[0] waves (block pairs), [1] trace lists, [2] lists with
 * distinct operands, [3] of those outside dense groups, [4] dense groups,
 * [5] trace entries, [6] entries after merging equal lists, [7] entries in
 * dense groups, [8] correlator terms, [9] factor products, [10..12] Q0, Q1, Q2
 * factors, [13] correlator requests, [14] (check_layout != 0) 1 if every
 * trace-value index is written exactly once and every list reads the values
 * of a list with its operands, else 0, [15] tiles of the tensor-core product
 * plan, [16] (check_layout != 0) 1 if that plan computes every product of
 * every dependency level exactly once, into its slot, from its left and right
 * matrices, else 0.  Writes min(n, 17) values. */
int slaph_plan_schedule_stats(const slaph_dims *dims, const slaph_plan *plan,
                              int32_t single_block_pair, int32_t check_layout, double *out,
                              int32_t n);

/* Per-stage device times of the last build / contract, in milliseconds,
 * measured with CUDA events on the engine stream.  out[0] VdaggerV,
 * out[1] factors Q0/Q1/Q2, out[2] products + traces, out[3] assembly,
 * out[4] host planning (wall clock), out[5] kernel launches issued,
 * out[6] the per-entry trace kernel alone (summed over its launches), out[7]
 * its launch count, out[8] the tensor-core trace GEMM (mixed precision),
 * out[9] its launch count, out[10] the slicing of its operands, out[11] the
 * split-precision VdaggerV GEMM alone (summed over its launches; set by the
 * build), out[12] its launch count, out[13] the last HYP smearing
 * (slaph_engine_smear_gauge_hyp), out[14] the factor products (summed over
 * their dependency levels), out[15] the number of those levels.  Returns the
 * number of values written (<= n, at most 16). */
int slaph_engine_timings(const slaph_engine *eng, double *out, int n);

/* VdaggerV of one operator on one timeslice for callers that cannot let a
 * library allocate device memory: hosts whose own allocator has reserved the
 * device up front, and latency-critical loops that cannot afford the device
 * synchronisation cudaMalloc/cudaFree may imply.  No counterpart in the
 * reference (it has no GPU code); the result equals slaph_vdaggerv_fetch of
 * slaph_vdaggerv_build(SLAPH_FP64).
 *   V_t:  DEVICE pointer, 3*L^3 x nev complex, column-major (one timeslice)
 *   out:  DEVICE pointer, nev x nev complex, column-major
 *   momentum: host array of 3 ints, read during the call and handed to the
 *             device as kernel arguments (the GPU reads no host memory);
 *   stream:   a cudaStream_t (NULL = legacy)
 * Allocates nothing: the phase table lives in a static device array of
 * 4 MiB + 256 B, which every GPU that loads the library holds until the
 * process exits, so L^3 may not exceed 262144 (64^3); larger lattices (and
 * any single extent above that) are rejected with SLAPH_ERR_ARG.  The first call on a device looks up that
 * array's device address (once per device); make that first call before any
 * stream capture.  The work is enqueued on `stream` and not waited for.
 * Every call shares the one array: calls whose work overlaps on the GPU (other
 * streams, or other host threads) race on it and must be serialised by the
 * caller. */
int slaph_vdaggerv_noalloc(const slaph_dims *dims, const double *V_t, const int32_t *momentum,
                           double *out, void *stream);

/* Device-resident statistics of the last contract: out[0] factors built,
 * out[1] products, out[2] traces, out[3] correlator terms, out[4] flops of
 * the factor stage, out[5] flops of products+traces, out[6] trace entries
 * computed after merging lists with equal operands, out[7] of those, the
 * entries in dense groups (tensor-core GEMMs in mixed precision). */
int slaph_engine_stats(const slaph_engine *eng, double *out, int n);

#ifdef __cplusplus
}
#endif

#endif /* SLAPH_GB300_H */
