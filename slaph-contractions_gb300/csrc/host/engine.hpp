// Engine: device state for one lattice geometry and the per-configuration
// calls of the hot path (VdaggerV build, contraction).
#pragma once

#include <cuda_runtime.h>

#include <chrono>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../../include/slaph_gb300.h"
#include "../kernels/kernels.cuh"
#include "capi_util.hpp"
#include "schedule.hpp"

namespace slaph {

void cuda_check(cudaError_t e, char const *what);
#define SLAPH_CK(call) ::slaph::cuda_check((call), #call)

// Owning device allocation.
class DevBuf {
 public:
  DevBuf() = default;
  ~DevBuf() { release(); }
  DevBuf(DevBuf const &) = delete;
  DevBuf &operator=(DevBuf const &) = delete;
  void reserve(size_t bytes);  // grows, never shrinks; contents undefined
  void release();
  template <typename T>
  T *as() const {
    return static_cast<T *>(p_);
  }
  size_t size() const { return n_; }

 private:
  void *p_ = nullptr;
  size_t n_ = 0;
};

// Page-locked host memory for the engine's read-backs (error flags,
// correlators): a device-to-host copy into it goes straight to the
// device-to-host copy engine, instead of waiting behind the host-to-device
// uploads that pageable copies share their staging with.
class HostBuf {
 public:
  HostBuf() = default;
  ~HostBuf() { release(); }
  HostBuf(HostBuf const &) = delete;
  HostBuf &operator=(HostBuf const &) = delete;
  void reserve(size_t bytes);  // grows, never shrinks; contents undefined
  void release();
  template <typename T>
  T *as() const {
    return static_cast<T *>(p_);
  }

 private:
  void *p_ = nullptr;
  size_t n_ = 0;
};

// A schedule plus its work lists resident on the device.
struct DeviceSchedule {
  Schedule s;
  DevBuf q0m, q1r, q2m, q0, q1, q2;
  DevBuf shape_i, shape_j, shape_mask, shape_off;
  // Dense trace groups of a wave cut into batches that fit the tensor-core
  // scratch buffer: slicing row groups (a_off, n_a / b_off, n_b index tc_a /
  // tc_b) and GEMM tiles per batch.
  struct TcBatch {
    int64_t a_off, n_a, b_off, n_b, tile_off, n_tiles;
  };
  // Products of one dependency level on the tensor cores: offsets into the
  // wave's product-GEMM lists.
  struct PLevel {
    int64_t g_off, n_g, r_off, n_r, t_off, n_t;
  };
  struct WaveBufs {
    DevBuf prods, lists, terms, seg_out, seg_off, idx, unique, residual;
    int64_t n_seg = 0;
    DevBuf tc_a, tc_b, tc_tiles;
    std::vector<TcBatch> tc_batches;
    DevBuf p_groups, p_rslots, p_ulist, p_out, p_tiles;
    std::vector<PLevel> p_levels;
  };
  std::vector<std::unique_ptr<WaveBufs>> waves;
  double plan_seconds = 0;
  // Q1/Q2 factors on the tensor cores (mixed precision), in batches of
  // timeslices.  Phase 1: X1 = Q1R x perambulator blocks and the Q2M
  // intermediates (K = nev); phase 2: Q2 (K = 4 nev); then gathers into slots.
  struct FBatch {
    int64_t a_x1[2], a_q2m[2], b_x1[2], b_q2m[2], a_q2[2], b_q2[2];  // (offset, count) in fvec
    int64_t t1[2], t2[2];  // in ftiles
    int64_t g1[2], g2[2];  // in fg1 / fg2
  };
  bool f_ready = false;
  std::vector<FBatch> f_batches;
  DevBuf fvec, ftiles, fg1, fg2;
  size_t f_scratch = 0;
  int64_t f_out = 0, f_expo = 0;  // doubles2 of dense outputs, exponents per batch
  bool tc_ready = false;
  // Products on the tensor cores: scratch bytes and exponents of the largest level.
  bool p_ready = false;
  size_t p_scratch = 0;
  int64_t p_expo = 0;
  size_t tc_scratch = 0;   // bytes of scratch the batches need
  int64_t tc_expo = 0;     // exponents per batch (maximum)
};

class Engine {
 public:
  explicit Engine(slaph_dims const &dims);
  ~Engine();

  void set_operators(slaph_vdv_op const *ops, int32_t n, int32_t index_of_unity);
  // Host -> device copies on the upload stream; the blocking forms wait for
  // their copy, the asynchronous ones return at once (the host buffer must stay
  // valid until the next vdaggerv_build / contract that consumes it returns).
  void set_eigenvectors(int32_t t, double const *V, bool async = false);
  void set_perambulator(int32_t r, double const *peram, bool async = false);
  void set_random_vector(int32_t r, double const *noise, bool async = false);
  // Gauge links of timeslice t, [site][dir x,y,z][3x3 column-major] complex,
  // for displaced operators.
  void set_gauge(int32_t t, double const *U);
  void set_time_dilution(int32_t dilT);
  // 0: every eigenvector timeslice resident on the device (the default);
  // n >= 2: a ring of n timeslice slots, filled from the host buffers given to
  // set_eigenvectors during vdaggerv_build, n / 2 timeslices at a time.
  void set_eigenvector_slots(int32_t n);
  // SLAPH_FACTORS_CONFIGURATION or SLAPH_FACTORS_BLOCK_PAIR.
  void set_factor_lifetime(int mode);
  // HYP smearing of the stored links of every timeslice, in place.
  void smear_gauge_hyp(double alpha1, double alpha2, int32_t iterations);
  void gauge_fetch(int32_t t, double *out);
  void vdaggerv_build(int precision);
  void vdaggerv_fetch(int32_t op, int32_t t, double *out);
  // VdaggerV files of the reference's handling_vdaggerv modes.
  void vdaggerv_write(char const *path, int32_t config);
  void vdaggerv_read(char const *path, int32_t config, int32_t liuming);
  void contract(slaph_plan const *plan, int precision, int accumulator, int single_block_pair,
                double *corr_out);

  double timings[16] = {};
  double stats[8] = {};

 private:
  slaph_dims dims_;
  dev::Geometry geo_{};
  int device_ = 0;
  cudaStream_t stream_ = nullptr;
  cudaEvent_t ev_[8] = {};
  // Input uploads: their own stream, one completion event per timeslice /
  // random vector, and the compute stream's last use of each input buffer.
  cudaStream_t up_stream_ = nullptr;
  std::vector<cudaEvent_t> ev_v_, ev_p_, ev_n_;
  std::vector<char> pend_v_, pend_p_, pend_n_;
  cudaEvent_t ev_v_used_ = nullptr, ev_pn_used_ = nullptr;
  std::vector<cudaEvent_t> tc_ev_;  // three per tensor-core trace batch
  std::vector<cudaEvent_t> vdv_ev_;  // two per split-precision VdaggerV GEMM launch

  DevBuf V_, peram_, noise_, phase_, phase_fx_, vdv_, ops_dev_, mom_dev_, tc_scratch_, err_;
  HostBuf host_rb_;  // read-back staging
  DevBuf slot_bits_;  // largest |re|, |im| of every double-float matrix slot (mixed path)
  int read_err_flag();  // the device error flag, through host_rb_ on the engine stream
  std::vector<slaph_vdv_op> ops_;
  DevBuf U_, W_, disp_ops_;  // gauge links, displaced eigenvector scratch, displaced op ids
  DevBuf hyp_dec_;           // decorated links of a chunk of timeslices (HYP smearing)
  DevBuf phase_unit_, unit_op_;  // phase 1 per site and its operator index (displaced, mixed)
  std::vector<char> gauge_set_;
  // Eigenvector ring (set_eigenvector_slots): host buffer per timeslice and
  // the compute stream's last use of each half of the ring.
  int32_t ring_slots_ = 0;
  std::vector<double const *> host_v_;
  cudaEvent_t ev_half_[2] = {};
  int32_t index_of_unity_ = -1;
  bool ops_set_ = false, vdv_built_ = false;
  int64_t launches_ = 0;

  // Working buffers of the contraction.
  DevBuf slots_, df_slots_, df_slots_t_, values_, values_df_, term_val_, running_, tr_expo_,
      f_out_;

  std::unique_ptr<DeviceSchedule> sched_;
  slaph_plan const *sched_plan_ = nullptr;
  int sched_bp_ = -2;
  // Factors per block pair: one schedule per block pair of bp_plan_.
  int factor_lifetime_ = SLAPH_FACTORS_CONFIGURATION;
  std::map<int, std::unique_ptr<DeviceSchedule>> bp_scheds_;
  slaph_plan const *bp_plan_ = nullptr;

  int64_t peram_elems() const;
  void prepare_schedule(slaph_plan const *plan, int single_block_pair);
  std::unique_ptr<DeviceSchedule> make_schedule(slaph_plan const *plan, int single_block_pair);
  void prepare_trace_tc(DeviceSchedule &ds);
  void prepare_factor_tc(DeviceSchedule &ds);
  void prepare_product_tc(DeviceSchedule &ds);
  void launch(cudaError_t e, char const *what) {
    cuda_check(e, what);
    ++launches_;
  }
};

}  // namespace slaph
