// Engine host logic: device memory, schedule upload, kernel sequencing.
#include "engine.hpp"

#include <algorithm>
#include <climits>
#include <array>
#include <map>
#include <cstdio>
#include <cstring>
#include <numeric>

namespace slaph {

static_assert(sizeof(Q0MInst) == sizeof(dev::Q0MInst), "layout");
static_assert(sizeof(Q1RInst) == sizeof(dev::Q1RInst), "layout");
static_assert(sizeof(Q2MInst) == sizeof(dev::Q2MInst), "layout");
static_assert(sizeof(Q0Inst) == sizeof(dev::Q0Inst), "layout");
static_assert(sizeof(Q1Inst) == sizeof(dev::Q1Inst), "layout");
static_assert(sizeof(Q2Inst) == sizeof(dev::Q2Inst), "layout");
static_assert(sizeof(ProdInst) == sizeof(dev::ProdInst), "layout");
static_assert(sizeof(TraceList) == sizeof(dev::TraceList), "layout");
static_assert(sizeof(Term) == sizeof(dev::Term), "layout");

void cuda_check(cudaError_t e, char const *what) {
  if (e == cudaSuccess) return;
  std::string const msg = std::string(what) + ": " + cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation) throw NoMemError(msg);
  throw CudaError(msg);
}

void DevBuf::reserve(size_t bytes) {
  if (bytes <= n_) return;
  release();
  if (bytes == 0) return;
  cudaError_t const e = cudaMalloc(&p_, bytes);
  if (e != cudaSuccess) {
    p_ = nullptr;
    (void)cudaGetLastError();
    throw NoMemError("device allocation of " + std::to_string(bytes) + " bytes failed: " +
                     cudaGetErrorString(e));
  }
  n_ = bytes;
}

void DevBuf::release() {
  if (p_) cudaFree(p_);
  p_ = nullptr;
  n_ = 0;
}

void HostBuf::reserve(size_t bytes) {
  if (bytes <= n_) return;
  release();
  SLAPH_CK(cudaHostAlloc(&p_, bytes, cudaHostAllocPortable));
  n_ = bytes;
}

void HostBuf::release() {
  if (p_) cudaFreeHost(p_);
  p_ = nullptr;
  n_ = 0;
}

int Engine::read_err_flag() {
  host_rb_.reserve(sizeof(int));
  SLAPH_CK(cudaMemcpyAsync(host_rb_.as<int>(), err_.as<void>(), sizeof(int),
                           cudaMemcpyDeviceToHost, stream_));
  SLAPH_CK(cudaStreamSynchronize(stream_));
  return *host_rb_.as<int>();
}

namespace {

// Bounds of the split-precision VdaggerV scratch (timeslice batches): at
// least kTcScratchCap, up to a third of the free device memory and at most
// kTcScratchMax (larger batches leave less of the last round of tiles idle).
constexpr size_t kTcScratchCap = 24ULL << 30;
constexpr size_t kTcScratchMax = 64ULL << 30;
// Smallest batch capacity of the tensor-core traces (the VdaggerV scratch is
// reused when it is larger).
constexpr size_t kTraceScratchMin = 1ULL << 30;

template <typename T>
void upload(DevBuf &b, std::vector<T> const &v, cudaStream_t s) {
  b.reserve(std::max<size_t>(1, v.size()) * sizeof(T));
  if (!v.empty())
    SLAPH_CK(cudaMemcpyAsync(b.as<void>(), v.data(), v.size() * sizeof(T),
                             cudaMemcpyHostToDevice, s));
}

double elapsed_ms(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0;
  SLAPH_CK(cudaEventElapsedTime(&ms, a, b));
  return ms;
}


// Row groups of the slicing items [b, e) of one batch: consecutive items of
// one region with consecutive rows and exponent indices, cut at multiples of
// `rows` (one 8-row core-matrix group of the operand stream).
void slice_groups(std::vector<dev::TrSlice> const &it, size_t b, size_t e, int32_t rows,
                  std::vector<dev::TrSliceGroup> &out) {
  for (size_t k = b; k < e;) {
    dev::TrSliceGroup g{};
    g.dst = it[k].dst;
    g.row0 = it[k].row;
    g.expo0 = it[k].expo;
    do {
      g.slot[g.n++] = it[k].slot;
      ++k;
    } while (k < e && g.n < rows && it[k].dst == g.dst && it[k].row == g.row0 + g.n &&
             it[k].expo == g.expo0 + g.n && it[k].row % rows != 0);
    out.push_back(g);
  }
}
}  // namespace

Engine::Engine(slaph_dims const &d) : dims_(d) {
  if (d.Lt < 1 || d.Lx < 1 || d.Ly < 1 || d.Lz < 1 || d.nev < 1 || d.dilT < 1 || d.dilE < 1 ||
      d.n_rnd < 1)
    throw ArgError("invalid slaph_dims: every size must be positive");
  if (d.Lt % d.dilT != 0) throw ArgError("Lt must be a multiple of dilT");
  if (d.n_rnd > 16) throw UnsupportedError("at most 16 random vectors (16-bit used masks)");
  if (4 * d.dilE > 64) throw UnsupportedError("4*dilE above 64 is not supported");
  geo_.Lt = d.Lt;
  geo_.Lx = d.Lx;
  geo_.Ly = d.Ly;
  geo_.Lz = d.Lz;
  geo_.nev = d.nev;
  geo_.dilE = d.dilE;
  geo_.n_rnd = d.n_rnd;
  geo_.nb = d.Lt / d.dilT;
  geo_.dim_row = 3LL * d.Lx * d.Ly * d.Lz;
  SLAPH_CK(cudaGetDevice(&device_));
  SLAPH_CK(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
  SLAPH_CK(cudaStreamCreateWithFlags(&up_stream_, cudaStreamNonBlocking));
  for (auto &e : ev_) SLAPH_CK(cudaEventCreate(&e));
  auto make_events = [](std::vector<cudaEvent_t> &v, int n) {
    v.assign(n, nullptr);
    for (auto &e : v) SLAPH_CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  };
  make_events(ev_v_, d.Lt);
  make_events(ev_p_, d.n_rnd);
  make_events(ev_n_, d.n_rnd);
  pend_v_.assign(d.Lt, 0);
  pend_p_.assign(d.n_rnd, 0);
  pend_n_.assign(d.n_rnd, 0);
  SLAPH_CK(cudaEventCreateWithFlags(&ev_v_used_, cudaEventDisableTiming));
  SLAPH_CK(cudaEventCreateWithFlags(&ev_pn_used_, cudaEventDisableTiming));
  SLAPH_CK(cudaEventRecord(ev_v_used_, stream_));
  SLAPH_CK(cudaEventRecord(ev_pn_used_, stream_));
  for (auto &e : ev_half_) SLAPH_CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  // The eigenvectors are allocated by the first set_eigenvectors (all
  // timeslices) or by set_eigenvector_slots (a ring).
  peram_.reserve(sizeof(double2) * peram_elems() * d.n_rnd);
  noise_.reserve(sizeof(double2) * 4LL * d.nev * d.Lt * d.n_rnd);
  SLAPH_CK(cudaMemsetAsync(noise_.as<void>(), 0, noise_.size(), stream_));
  SLAPH_CK(cudaMemsetAsync(peram_.as<void>(), 0, peram_.size(), stream_));
  SLAPH_CK(dev::upload_gamma(stream_));
  SLAPH_CK(dev::upload_gamma_tc(stream_));
  SLAPH_CK(cudaStreamSynchronize(stream_));
}

Engine::~Engine() {
  if (up_stream_) cudaStreamSynchronize(up_stream_);
  if (stream_) cudaStreamSynchronize(stream_);
  for (auto &e : ev_)
    if (e) cudaEventDestroy(e);
  for (auto *v : {&ev_v_, &ev_p_, &ev_n_})
    for (auto &e : *v)
      if (e) cudaEventDestroy(e);
  if (ev_v_used_) cudaEventDestroy(ev_v_used_);
  for (auto &e : ev_half_)
    if (e) cudaEventDestroy(e);
  if (ev_pn_used_) cudaEventDestroy(ev_pn_used_);
  if (up_stream_) cudaStreamDestroy(up_stream_);
  for (auto *v : {&tc_ev_, &vdv_ev_})
    for (auto &e : *v)
      if (e) cudaEventDestroy(e);
  if (stream_) cudaStreamDestroy(stream_);
}

int64_t Engine::peram_elems() const {
  return 4LL * dims_.nev * dims_.Lt * (dims_.Lt / dims_.dilT) * dims_.dilE * 4;
}

void Engine::set_operators(slaph_vdv_op const *ops, int32_t n, int32_t index_of_unity) {
  if (n < 0 || (n > 0 && !ops)) throw ArgError("invalid operator list");
  for (int32_t i = 0; i < n; ++i) {
    if (ops[i].id != i) throw ArgError("VdaggerV ids must be 0..n_ops-1 in order");
    if (ops[i].n_disp < 0 || ops[i].n_disp > SLAPH_MAX_DISP)
      throw ArgError("invalid displacement length");
    for (int32_t k = 0; k < ops[i].n_disp; ++k) {
      char const fb = ops[i].disp[2 * k], ax = ops[i].disp[2 * k + 1];
      if ((fb != '<' && fb != '>') || (ax != 'x' && ax != 'y' && ax != 'z'))
        throw ArgError("displacement steps are ('<' | '>', 'x' | 'y' | 'z') pairs");
    }
    if (ops[i].n_disp > 0 && (dims_.Lx != dims_.Ly || dims_.Lx != dims_.Lz))
      throw UnsupportedError("displaced operators need a cubic spatial lattice");
  }
  if (index_of_unity >= n) throw ArgError("index_of_unity out of range");
  ops_.assign(ops, ops + n);
  index_of_unity_ = index_of_unity;
  std::vector<int32_t> mom(3 * std::max(n, 1), 0);
  for (int32_t i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c) mom[3 * i + c] = ops[i].momentum[c];
  upload(mom_dev_, mom, stream_);
  int64_t const vol = geo_.dim_row / 3;
  phase_.reserve(sizeof(double2) * vol * std::max(n, 1));
  launch(dev::momenta(phase_.as<double2>(), mom_dev_.as<int32_t>(), n, geo_, stream_),
         "momenta");
  phase_fx_.reserve(sizeof(longlong2) * vol * std::max(n, 1));
  launch(dev::phase_fixed(phase_fx_.as<longlong2>(), phase_.as<double2>(), vol * n, stream_),
         "phase_fixed");
  vdv_.reserve(sizeof(double2) * 2LL * std::max(n, 1) * dims_.Lt * dims_.nev * dims_.nev);
  SLAPH_CK(cudaStreamSynchronize(stream_));
  ops_set_ = true;
  vdv_built_ = false;
}

void Engine::set_eigenvector_slots(int32_t n) {
  if (n < 0 || n == 1) throw ArgError("eigenvector slots: 0 (all resident) or at least 2");
  SLAPH_CK(cudaStreamSynchronize(up_stream_));
  SLAPH_CK(cudaStreamSynchronize(stream_));
  ring_slots_ = n;
  V_.release();
  std::fill(pend_v_.begin(), pend_v_.end(), 0);
  host_v_.assign(dims_.Lt, nullptr);
  if (n > 0) V_.reserve(sizeof(double2) * geo_.dim_row * dims_.nev * n);
  vdv_built_ = false;
}

void Engine::set_eigenvectors(int32_t t, double const *V, bool async) {
  if (t < 0 || t >= dims_.Lt || !V) throw ArgError("invalid timeslice or null pointer");
  size_t const n = static_cast<size_t>(geo_.dim_row) * dims_.nev;
  if (ring_slots_ > 0) {
    // Streamed: the build copies timeslice t from this buffer when it needs it.
    host_v_[t] = V;
    return;
  }
  if (V_.size() < sizeof(double2) * n * dims_.Lt) {
    SLAPH_CK(cudaStreamSynchronize(stream_));
    V_.reserve(sizeof(double2) * n * dims_.Lt);
  }
  // The previous VdaggerV build must be done with V before it is overwritten.
  SLAPH_CK(cudaStreamWaitEvent(up_stream_, ev_v_used_, 0));
  SLAPH_CK(cudaMemcpyAsync(V_.as<double2>() + n * t, V, n * sizeof(double2),
                           cudaMemcpyHostToDevice, up_stream_));
  SLAPH_CK(cudaEventRecord(ev_v_[t], up_stream_));
  pend_v_[t] = 1;
  if (!async) SLAPH_CK(cudaEventSynchronize(ev_v_[t]));
  // The VdaggerV of the last build stays valid for contract(): it lives in its
  // own buffer, so the next configuration's eigenvectors may be uploaded while
  // this one contracts.
}

void Engine::set_perambulator(int32_t r, double const *P, bool async) {
  if (r < 0 || r >= dims_.n_rnd || !P) throw ArgError("invalid random vector index");
  size_t const n = static_cast<size_t>(peram_elems());
  SLAPH_CK(cudaStreamWaitEvent(up_stream_, ev_pn_used_, 0));
  SLAPH_CK(cudaMemcpyAsync(peram_.as<double2>() + n * r, P, n * sizeof(double2),
                           cudaMemcpyHostToDevice, up_stream_));
  SLAPH_CK(cudaEventRecord(ev_p_[r], up_stream_));
  pend_p_[r] = 1;
  if (!async) SLAPH_CK(cudaEventSynchronize(ev_p_[r]));
}

void Engine::set_random_vector(int32_t r, double const *noise, bool async) {
  if (r < 0 || r >= dims_.n_rnd || !noise) throw ArgError("invalid random vector index");
  size_t const n = 4ULL * dims_.nev * dims_.Lt;
  SLAPH_CK(cudaStreamWaitEvent(up_stream_, ev_pn_used_, 0));
  SLAPH_CK(cudaMemcpyAsync(noise_.as<double2>() + n * r, noise, n * sizeof(double2),
                           cudaMemcpyHostToDevice, up_stream_));
  SLAPH_CK(cudaEventRecord(ev_n_[r], up_stream_));
  pend_n_[r] = 1;
  if (!async) SLAPH_CK(cudaEventSynchronize(ev_n_[r]));
}

void Engine::set_time_dilution(int32_t dilT) {
  if (dilT < 1 || dims_.Lt % dilT != 0)
    throw ArgError("Lt must be a positive multiple of dilT");
  if (dilT == dims_.dilT) return;
  // The perambulators' column count depends on the number of time blocks:
  // their buffer is re-made (to be uploaded again); VdaggerV and the
  // eigenvectors do not depend on it and stay.
  SLAPH_CK(cudaStreamSynchronize(up_stream_));
  SLAPH_CK(cudaStreamSynchronize(stream_));
  dims_.dilT = dilT;
  geo_.nb = dims_.Lt / dilT;
  peram_.release();
  peram_.reserve(sizeof(double2) * peram_elems() * dims_.n_rnd);
  SLAPH_CK(cudaMemsetAsync(peram_.as<void>(), 0, peram_.size(), stream_));
  SLAPH_CK(cudaStreamSynchronize(stream_));
  std::fill(pend_p_.begin(), pend_p_.end(), 0);
  sched_.reset();
  sched_plan_ = nullptr;
  bp_scheds_.clear();
  bp_plan_ = nullptr;
}

void Engine::set_gauge(int32_t t, double const *U) {
  if (t < 0 || t >= dims_.Lt || !U) throw ArgError("invalid timeslice or null pointer");
  if (dims_.Lx != dims_.Ly || dims_.Lx != dims_.Lz)
    throw UnsupportedError("displaced operators need a cubic spatial lattice");
  size_t const per = static_cast<size_t>(geo_.dim_row / 3) * 27;  // links of one timeslice
  if (U_.size() == 0) {
    U_.reserve(sizeof(double2) * per * dims_.Lt);
    gauge_set_.assign(dims_.Lt, 0);
  }
  SLAPH_CK(cudaStreamWaitEvent(up_stream_, ev_v_used_, 0));
  SLAPH_CK(cudaMemcpyAsync(U_.as<double2>() + per * t, U, per * sizeof(double2),
                           cudaMemcpyHostToDevice, up_stream_));
  SLAPH_CK(cudaStreamSynchronize(up_stream_));
  gauge_set_[t] = 1;
}

void Engine::smear_gauge_hyp(double alpha1, double alpha2, int32_t iterations) {
  if (iterations < 0) throw ArgError("negative number of smearing iterations");
  if (U_.size() == 0 || std::find(gauge_set_.begin(), gauge_set_.end(), 0) != gauge_set_.end())
    throw StateError("slaph_engine_set_gauge must be called for every timeslice before smearing");
  if (iterations == 0) return;
  // Scratch for the decorated links of up to 256 MiB worth of timeslices.
  size_t const per_dec = sizeof(double) * dev::hyp_scratch_doubles_per_timeslice(dims_.Lx);
  int32_t const chunk = static_cast<int32_t>(
      std::max<size_t>(1, std::min<size_t>(dims_.Lt, (size_t{256} << 20) / per_dec)));
  hyp_dec_.reserve(per_dec * chunk);
  size_t const per = static_cast<size_t>(geo_.dim_row / 3) * 27;
  SLAPH_CK(cudaStreamWaitEvent(stream_, ev_v_used_, 0));
  SLAPH_CK(cudaEventRecord(ev_[6], stream_));
  for (int32_t it = 0; it < iterations; ++it)
    for (int32_t t0 = 0; t0 < dims_.Lt; t0 += chunk)
      SLAPH_CK(dev::hyp_smear(U_.as<double2>() + per * t0, hyp_dec_.as<double2>(), dims_.Lx,
                              std::min(chunk, dims_.Lt - t0), alpha1, alpha2, stream_));
  SLAPH_CK(cudaEventRecord(ev_[7], stream_));
  SLAPH_CK(cudaStreamSynchronize(stream_));
  timings[13] = elapsed_ms(ev_[6], ev_[7]);
}

void Engine::gauge_fetch(int32_t t, double *out) {
  if (t < 0 || t >= dims_.Lt || !out) throw ArgError("invalid timeslice or null pointer");
  if (U_.size() == 0 || !gauge_set_[t]) throw StateError("no gauge links for this timeslice");
  size_t const per = static_cast<size_t>(geo_.dim_row / 3) * 27;
  SLAPH_CK(cudaMemcpyAsync(out, U_.as<double2>() + per * t, per * sizeof(double2),
                           cudaMemcpyDeviceToHost, stream_));
  SLAPH_CK(cudaStreamSynchronize(stream_));
}

void Engine::vdaggerv_build(int precision) {
  if (!ops_set_) throw StateError("slaph_engine_set_operators must be called first");
  if (precision != SLAPH_FP64 && precision != SLAPH_MIXED)
    throw ArgError("unknown precision mode");
  launches_ = 0;
  // Momentum operators (the GEMM paths below) and displaced operators (V^H D(V)).
  std::vector<int32_t> computed, displaced;
  for (auto const &o : ops_) {
    if (o.id == index_of_unity_) continue;
    (o.n_disp > 0 ? displaced : computed).push_back(o.id);
  }
  if (!displaced.empty()) {
    bool all = gauge_set_.size() == static_cast<size_t>(dims_.Lt);
    for (char c : gauge_set_) all = all && c;
    if (!all)
      throw StateError("displaced operators need slaph_engine_set_gauge for every timeslice");
  }
  DevBuf list;
  int32_t const n_comp = static_cast<int32_t>(computed.size());
  // The split-precision build takes the displaced operators too (after the
  // momentum ones); the FP64 build handles them separately below.
  bool const tc_disp = precision == SLAPH_MIXED && !displaced.empty();
  std::vector<int32_t> all = computed;
  if (tc_disp) all.insert(all.end(), displaced.begin(), displaced.end());
  upload(list, all, stream_);
  int32_t const n_all = static_cast<int32_t>(all.size());
  dev::VdvDisplaced dd{};
  std::vector<int32_t> d_steps, d_n;
  if (tc_disp) {
    size_t const sites = static_cast<size_t>(geo_.dim_row / 3);
    if (phase_unit_.size() < sites * sizeof(longlong2)) {
      std::vector<longlong2> one(sites, make_longlong2(1LL << 62, 0));
      upload(phase_unit_, one, stream_);
      upload(unit_op_, std::vector<int32_t>{0}, stream_);
    }
    W_.reserve(sizeof(double2) * static_cast<size_t>(geo_.dim_row) * dims_.nev);
    d_steps.assign(2 * dev::kMaxDispSteps * displaced.size(), 0);
    for (size_t k = 0; k < displaced.size(); ++k) {
      slaph_vdv_op const &op = ops_[displaced[k]];
      if (op.n_disp > dev::kMaxDispSteps) throw UnsupportedError("too many displacement steps");
      d_n.push_back(op.n_disp);
      for (int32_t s = 0; s < op.n_disp; ++s) {
        char const ax = op.disp[2 * s + 1];
        d_steps[2 * (k * dev::kMaxDispSteps + s)] = ax == 'x' ? 0 : ax == 'y' ? 1 : 2;
        d_steps[2 * (k * dev::kMaxDispSteps + s) + 1] = op.disp[2 * s] == '>' ? 1 : 0;
      }
    }
    dd = dev::VdvDisplaced{static_cast<int32_t>(displaced.size()), d_n.data(), d_steps.data(),
                           U_.as<double2>(), W_.as<double2>(), phase_unit_.as<longlong2>(),
                           unit_op_.as<int32_t>()};
  }
  int32_t n_gemm = 0;     // GEMM launches of the whole build
  int64_t batch_fit = 1;  // timeslices per GEMM launch that the scratch holds
  if (precision == SLAPH_MIXED) {
    int sms = 0;
    SLAPH_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_));
    size_t free_b = 0, total_b = 0;
    SLAPH_CK(cudaMemGetInfo(&free_b, &total_b));
    size_t const cap = std::max(kTcScratchCap, std::min(kTcScratchMax, free_b / 3));
    int32_t const n_t = ring_slots_ > 0 ? std::max(1, ring_slots_ / 2) : dims_.Lt;
    int32_t const batch = dev::vdaggerv_tc_batch(geo_, std::max(n_all, 1), sms, cap, n_t);
    tc_scratch_.reserve(dev::vdaggerv_tc_scratch_bytes(geo_, std::max(n_all, 1), batch));
    // The scratch may be larger than this batch needs (kept from an earlier
    // call): the launch count follows from what it holds.
    batch_fit = std::max<int64_t>(
        1, static_cast<int64_t>(tc_scratch_.size() /
                                dev::vdaggerv_tc_scratch_bytes(geo_, std::max(n_all, 1), 1)));
    err_.reserve(sizeof(int));
    SLAPH_CK(cudaMemsetAsync(err_.as<void>(), 0, sizeof(int), stream_));
  }
  // Timeslice ranges: all of them at once with resident eigenvectors, chunks
  // of half the ring when they are streamed (one half is copied while the
  // other is computed).
  int32_t const chunk = ring_slots_ > 0 ? ring_slots_ / 2 : dims_.Lt;
  std::vector<std::pair<int32_t, int32_t>> ranges;
  for (int32_t t0 = 0; t0 < dims_.Lt; t0 += chunk)
    ranges.emplace_back(t0, std::min(chunk, dims_.Lt - t0));
  if (precision == SLAPH_MIXED && n_all > 0)
    for (auto const &r : ranges)
      n_gemm += dev::vdaggerv_tc_gemm_launches(r.second, static_cast<int32_t>(batch_fit));
  while (vdv_ev_.size() < 2 * static_cast<size_t>(n_gemm)) {
    cudaEvent_t e = nullptr;
    SLAPH_CK(cudaEventCreate(&e));
    vdv_ev_.push_back(e);
  }
  bool const needs_v = n_all > 0 || !displaced.empty();
  if (ring_slots_ > 0 && needs_v)
    for (int32_t t = 0; t < dims_.Lt; ++t)
      if (!host_v_[t])
        throw StateError("streamed eigenvectors: slaph_engine_set_eigenvectors is needed for "
                         "every timeslice before the build");
  if (ring_slots_ == 0 && needs_v && V_.size() == 0)
    throw StateError("slaph_engine_set_eigenvectors must be called before the build");
  SLAPH_CK(cudaEventRecord(ev_[0], stream_));
  // Eigenvectors uploaded asynchronously: the split-precision build waits for
  // each timeslice just before slicing it (overlapping the remaining copies),
  // the FP64 build for the timeslices of its range.
  std::vector<cudaEvent_t> ready(dims_.Lt, nullptr);
  if (ring_slots_ == 0)
    for (int32_t t = 0; t < dims_.Lt; ++t)
      if (pend_v_[t]) ready[t] = ev_v_[t];
  size_t const n_v = static_cast<size_t>(geo_.dim_row) * dims_.nev;  // per timeslice
  size_t const links = static_cast<size_t>(geo_.dim_row / 3) * 27;
  bool const fp64_disp = !displaced.empty() && !tc_disp;
  if (fp64_disp) {
    W_.reserve(sizeof(double2) * n_v);
    upload(disp_ops_, displaced, stream_);
  }
  int64_t disp_launches = 0;  // per timeslice, split-precision displaced operators
  for (int32_t n : d_n) disp_launches += n + 2;
  int32_t gemm_done = 0;
  for (size_t c = 0; c < ranges.size(); ++c) {
    int32_t const t0 = ranges[c].first, nt = ranges[c].second;
    double2 *Vb = V_.as<double2>();  // consecutive timeslices from v_t0 on
    int32_t v_t0 = 0;
    if (ring_slots_ > 0) {
      int const h = static_cast<int>(c % 2);
      Vb = V_.as<double2>() + n_v * static_cast<size_t>(chunk) * h;
      v_t0 = t0;
      if (needs_v) {
        // This half was last read by the range two before this one.
        if (c >= 2) SLAPH_CK(cudaStreamWaitEvent(up_stream_, ev_half_[h], 0));
        for (int32_t t = t0; t < t0 + nt; ++t) {
          SLAPH_CK(cudaMemcpyAsync(Vb + n_v * (t - t0), host_v_[t], n_v * sizeof(double2),
                                   cudaMemcpyHostToDevice, up_stream_));
          SLAPH_CK(cudaEventRecord(ev_v_[t], up_stream_));
          ready[t] = ev_v_[t];
        }
      }
    }
    if (precision == SLAPH_MIXED) {
      int32_t const k =
          n_all > 0 ? dev::vdaggerv_tc_gemm_launches(nt, static_cast<int32_t>(batch_fit)) : 0;
      launch(dev::vdaggerv_tc(vdv_.as<double2>(), Vb, phase_fx_.as<longlong2>(),
                              list.as<int32_t>(), n_comp, t0, nt, geo_, tc_scratch_.as<void>(),
                              tc_scratch_.size(), err_.as<int>(), stream_, ready.data(),
                              tc_disp ? &dd : nullptr, vdv_ev_.data() + 2 * gemm_done, 2 * k,
                              v_t0, c == 0),
             "vdaggerv_tc");
      gemm_done += k;
      // per timeslice the exponents, A slices and (with momentum operators)
      // B slices, per displaced operator its steps, exponents and slices; one
      // GEMM per batch of timeslices
      if (n_all > 0)
        launches_ += (2LL + (n_comp > 0 ? 1 : 0) + disp_launches) * nt + k - 1;
    } else {
      for (int32_t t = t0; t < t0 + nt; ++t)
        if (ready[t]) SLAPH_CK(cudaStreamWaitEvent(stream_, ready[t], 0));
      launch(dev::vdaggerv_fp64(vdv_.as<double2>(), Vb, phase_.as<double2>(), list.as<int32_t>(),
                                n_comp, t0, nt, geo_, stream_, v_t0),
             "vdaggerv_fp64");
    }
    // Displaced operators of the FP64 build: W = D(V_t) step by step, then
    // V_t^H W in FP64 (src/OperatorFactory.cpp:289-290, 300); the momentum is
    // not applied.
    if (fp64_disp) {
      for (int32_t t = t0; t < t0 + nt; ++t)
        for (size_t k = 0; k < displaced.size(); ++k) {
          slaph_vdv_op const &op = ops_[displaced[k]];
          SLAPH_CK(cudaMemcpyAsync(W_.as<double2>(), Vb + n_v * (t - v_t0),
                                   n_v * sizeof(double2), cudaMemcpyDeviceToDevice, stream_));
          for (int32_t st = 0; st < op.n_disp; ++st) {
            char const ax = op.disp[2 * st + 1];
            launch(dev::displace(W_.as<double2>(), U_.as<double2>() + links * t,
                                 ax == 'x' ? 0 : ax == 'y' ? 1 : 2,
                                 op.disp[2 * st] == '>' ? 1 : 0, geo_, stream_),
                   "displace");
          }
          launch(dev::vdaggerv_fp64_w(vdv_.as<double2>(), Vb, W_.as<double2>(),
                                      disp_ops_.as<int32_t>() + k, t, geo_, stream_, v_t0),
                 "vdaggerv_fp64_w");
        }
    }
    if (ring_slots_ > 0) SLAPH_CK(cudaEventRecord(ev_half_[c % 2], stream_));
  }
  // V is not read after this point: later uploads may overwrite it.
  SLAPH_CK(cudaEventRecord(ev_v_used_, stream_));
  std::fill(pend_v_.begin(), pend_v_.end(), 0);
  if (index_of_unity_ >= 0)
    launch(dev::vdaggerv_identity(vdv_.as<double2>(), index_of_unity_, geo_, stream_),
           "vdaggerv_identity");
  launch(dev::vdaggerv_daggers(vdv_.as<double2>(), static_cast<int32_t>(ops_.size()), geo_,
                               stream_),
         "vdaggerv_daggers");
  SLAPH_CK(cudaEventRecord(ev_[1], stream_));
  SLAPH_CK(cudaEventSynchronize(ev_[1]));
  timings[0] = elapsed_ms(ev_[0], ev_[1]);
  timings[5] = static_cast<double>(launches_);
  double t_gemm = 0;
  for (int32_t k = 0; k < n_gemm; ++k) t_gemm += elapsed_ms(vdv_ev_[2 * k], vdv_ev_[2 * k + 1]);
  timings[11] = t_gemm;
  timings[12] = static_cast<double>(n_gemm);
  if (precision == SLAPH_MIXED) {
    int const code = read_err_flag();
    if (code != 0)
      throw TimeoutError("split-precision VdaggerV: a bounded device wait gave up (stage " +
                         std::to_string(code) + ")");
  }
  vdv_built_ = true;
}

void Engine::vdaggerv_write(char const *path, int32_t config) {
  if (!vdv_built_) throw StateError("VdaggerV has not been built");
  if (!path) throw ArgError("null path");
  size_t const blk = static_cast<size_t>(dims_.nev) * dims_.nev;
  std::vector<double2> host(blk * dims_.Lt);
  for (auto const &op : ops_) {
    if (op.id == index_of_unity_) continue;  // not written (src/OperatorFactory.cpp:315-318)
    SLAPH_CK(cudaMemcpyAsync(host.data(), vdv_.as<double2>() + 2ULL * op.id * dims_.Lt * blk,
                             host.size() * sizeof(double2), cudaMemcpyDeviceToHost, stream_));
    SLAPH_CK(cudaStreamSynchronize(stream_));
    for (int32_t t = 0; t < dims_.Lt; ++t)
      write_vdaggerv_file(vdaggerv_file_name(path, config, op, t, SLAPH_VDV_FILE_WRITE),
                          reinterpret_cast<double const *>(host.data() + blk * t), dims_.nev);
  }
}

void Engine::vdaggerv_read(char const *path, int32_t config, int32_t liuming) {
  if (!ops_set_) throw StateError("slaph_engine_set_operators must be called first");
  if (!path) throw ArgError("null path");
  size_t const blk = static_cast<size_t>(dims_.nev) * dims_.nev;
  int32_t const nev = dims_.nev;
  std::vector<double2> host(blk * dims_.Lt), file(blk * dims_.Lt);
  // The previous contraction may still read the VdaggerV buffer.
  SLAPH_CK(cudaStreamSynchronize(stream_));
  for (auto const &op : ops_) {
    if (op.id == index_of_unity_) continue;  // identity below
    if (!liuming) {
      // read_vdaggerv (src/OperatorFactory.cpp:328-393): one column-major block
      // per timeslice.  The reference constructs but does not throw its
      // exception for a missing file (leaving zeros); the engine raises it.
      for (int32_t t = 0; t < dims_.Lt; ++t)
        read_vdaggerv_file(vdaggerv_file_name(path, config, op, t, SLAPH_VDV_FILE_READ),
                           reinterpret_cast<double *>(host.data() + blk * t),
                           static_cast<int64_t>(2 * blk));
    } else {
      // read_vdaggerv_liuming (:395-490): all timeslices in one file of -p
      // (row-major blocks, adjoint taken) or else of +p (row-major blocks).
      std::string const minus =
          vdaggerv_file_name(path, config, op, 0, SLAPH_VDV_FILE_LIUMING_MINUS);
      std::string const plus =
          vdaggerv_file_name(path, config, op, 0, SLAPH_VDV_FILE_LIUMING_PLUS);
      bool adjoint = true;
      std::FILE *probe = std::fopen(minus.c_str(), "rb");
      if (!probe) {
        adjoint = false;
        probe = std::fopen(plus.c_str(), "rb");
        if (!probe) throw IoError("can't open " + minus + " NOR " + plus);
      }
      std::fclose(probe);
      read_vdaggerv_file(adjoint ? minus : plus, reinterpret_cast<double *>(file.data()),
                         static_cast<int64_t>(2 * file.size()));
      for (int32_t t = 0; t < dims_.Lt; ++t)
        for (int32_t i = 0; i < nev; ++i)
          for (int32_t j = 0; j < nev; ++j) {
            // file: M(r, c) at r nev + c; stored: X(i, j) at i + nev j
            size_t const o = blk * t;
            double2 const v = adjoint ? file[o + static_cast<size_t>(j) * nev + i]
                                      : file[o + static_cast<size_t>(i) * nev + j];
            host[o + i + static_cast<size_t>(nev) * j] =
                adjoint ? make_double2(v.x, -v.y) : v;
          }
    }
    SLAPH_CK(cudaMemcpyAsync(vdv_.as<double2>() + 2ULL * op.id * dims_.Lt * blk, host.data(),
                             host.size() * sizeof(double2), cudaMemcpyHostToDevice, stream_));
    SLAPH_CK(cudaStreamSynchronize(stream_));
  }
  if (index_of_unity_ >= 0)
    launch(dev::vdaggerv_identity(vdv_.as<double2>(), index_of_unity_, geo_, stream_),
           "vdaggerv_identity");
  launch(dev::vdaggerv_daggers(vdv_.as<double2>(), static_cast<int32_t>(ops_.size()), geo_,
                               stream_),
         "vdaggerv_daggers");
  SLAPH_CK(cudaStreamSynchronize(stream_));
  vdv_built_ = true;
}

void Engine::vdaggerv_fetch(int32_t op, int32_t t, double *out) {
  if (!vdv_built_) throw StateError("VdaggerV has not been built");
  if (op < 0 || op >= static_cast<int32_t>(ops_.size()) || t < 0 || t >= dims_.Lt || !out)
    throw ArgError("invalid operator id or timeslice");
  size_t const blk = static_cast<size_t>(dims_.nev) * dims_.nev;
  SLAPH_CK(cudaMemcpyAsync(out, vdv_.as<double2>() + (2ULL * op * dims_.Lt + t) * blk,
                           blk * sizeof(double2), cudaMemcpyDeviceToHost, stream_));
  SLAPH_CK(cudaStreamSynchronize(stream_));
}

void Engine::prepare_schedule(slaph_plan const *plan, int bp) {
  if (sched_ && sched_plan_ == plan && sched_bp_ == bp) return;
  sched_.reset();
  sched_ = make_schedule(plan, bp);
  sched_plan_ = plan;
  sched_bp_ = bp;
}

void Engine::set_factor_lifetime(int mode) {
  if (mode != SLAPH_FACTORS_CONFIGURATION && mode != SLAPH_FACTORS_BLOCK_PAIR)
    throw ArgError("unknown factor lifetime");
  factor_lifetime_ = mode;
}

std::unique_ptr<DeviceSchedule> Engine::make_schedule(slaph_plan const *plan, int bp) {
  auto const t0 = std::chrono::steady_clock::now();
  auto ds = std::make_unique<DeviceSchedule>();
  ds->s = build_schedule(dims_, *plan, bp);
  Schedule const &s = ds->s;
  upload(ds->q0m, s.q0m, stream_);
  upload(ds->q1r, s.q1r, stream_);
  upload(ds->q2m, s.q2m, stream_);
  upload(ds->q0, s.q0, stream_);
  upload(ds->q1, s.q1, stream_);
  upload(ds->q2, s.q2, stream_);
  std::vector<int64_t> off{0};
  std::vector<int32_t> si, sj;
  std::vector<uint16_t> sm;
  for (auto const &sh : s.shapes) {
    si.insert(si.end(), sh.i.begin(), sh.i.end());
    sj.insert(sj.end(), sh.j.begin(), sh.j.end());
    sm.insert(sm.end(), sh.mask.begin(), sh.mask.end());
    off.push_back(static_cast<int64_t>(si.size()));
  }
  upload(ds->shape_i, si, stream_);
  upload(ds->shape_j, sj, stream_);
  upload(ds->shape_mask, sm, stream_);
  upload(ds->shape_off, off, stream_);
  int64_t const Lt = dims_.Lt;
  for (auto const &w : s.waves) {
    auto wb = std::make_unique<DeviceSchedule::WaveBufs>();
    upload(wb->prods, w.prods, stream_);
    upload(wb->lists, w.lists, stream_);
    upload(wb->terms, w.terms, stream_);
    upload(wb->unique, w.unique_lists, stream_);
    upload(wb->residual, w.residual_lists, stream_);
    // Stable counting sort of the terms by output (request, dt) gives the
    // per-output summation order of Diagram::assemble.
    int64_t const n_out = s.n_outputs * Lt;
    std::vector<int64_t> count(n_out + 1, 0);
    for (auto const &t : w.terms) ++count[t.out * Lt + t.dt + 1];
    std::vector<int32_t> seg_out;
    std::vector<int64_t> seg_off{0};
    std::vector<int64_t> start(n_out, 0);
    int64_t acc = 0;
    for (int64_t o = 0; o < n_out; ++o) {
      start[o] = acc;
      if (count[o + 1]) {
        seg_out.push_back(static_cast<int32_t>(o));
        acc += count[o + 1];
        seg_off.push_back(acc);
      }
    }
    std::vector<int32_t> idx(w.terms.size());
    for (size_t k = 0; k < w.terms.size(); ++k) {
      auto const &t = w.terms[k];
      idx[start[t.out * Lt + t.dt]++] = static_cast<int32_t>(k);
    }
    wb->n_seg = static_cast<int64_t>(seg_out.size());
    upload(wb->seg_out, seg_out, stream_);
    upload(wb->seg_off, seg_off, stream_);
    upload(wb->idx, idx, stream_);
    SLAPH_CK(cudaStreamSynchronize(stream_));
    ds->waves.push_back(std::move(wb));
  }
  SLAPH_CK(cudaStreamSynchronize(stream_));
  ds->plan_seconds =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return ds;
}

// Tensor-core plan of the dense trace groups: per group, one A region per
// distinct entry row i (the matrices a + i of all A groups) and one B region
// per distinct entry column j; one GEMM per entry (i, j) over its regions, cut
// into 64 x 80 tiles.  Groups are packed into batches of at most the scratch
// capacity (a group larger than that raises it).
void Engine::prepare_trace_tc(DeviceSchedule &ds) {
  if (ds.tc_ready) return;
  Schedule const &s = ds.s;
  int32_t const eds = s.eds;
  // Bytes of one 64-row A tile stream and one 80-column B tile stream.
  int64_t const a_tile = static_cast<int64_t>(dev::trace_tc_a_bytes(1, eds));
  int64_t const b_tile = static_cast<int64_t>(dev::trace_tc_b_bytes(1, eds));
  size_t cap = std::max(tc_scratch_.size(), kTraceScratchMin);
  for (auto const &w : s.waves)
    for (auto const &g : w.groups) {
      auto const &sh = s.shapes[g.shape];
      std::vector<int32_t> is(sh.i.begin(), sh.i.end()), js(sh.j.begin(), sh.j.end());
      std::sort(is.begin(), is.end());
      std::sort(js.begin(), js.end());
      size_t const ni = std::unique(is.begin(), is.end()) - is.begin();
      size_t const nj = std::unique(js.begin(), js.end()) - js.begin();
      cap = std::max(cap, ni * dev::trace_tc_a_bytes(g.n_a, eds) +
                              nj * dev::trace_tc_b_bytes(g.n_b, eds));
    }
  size_t need = 0;
  int64_t max_expo = 0;
  for (size_t wi = 0; wi < s.waves.size(); ++wi) {
    Wave const &w = s.waves[wi];
    auto &wb = *ds.waves[wi];
    std::vector<dev::TrSlice> av, bv;
    std::vector<dev::TrSliceGroup> ag, bg;
    std::vector<dev::TrTile> tiles;
    wb.tc_batches.clear();
    DeviceSchedule::TcBatch cur{0, 0, 0, 0, 0, 0};
    size_t used = 0;
    int64_t expo = 0;
    auto close = [&] {
      // the batch's slicing items as row groups: offsets into ag / bg
      int64_t const ga = static_cast<int64_t>(ag.size()), gb = static_cast<int64_t>(bg.size());
      slice_groups(av, static_cast<size_t>(cur.a_off), av.size(), dev::kTrSliceRowsA, ag);
      slice_groups(bv, static_cast<size_t>(cur.b_off), bv.size(), dev::kTrSliceRowsB, bg);
      cur.n_tiles = static_cast<int64_t>(tiles.size()) - cur.tile_off;
      if (cur.n_tiles > 0)
        wb.tc_batches.push_back({ga, static_cast<int64_t>(ag.size()) - ga, gb,
                                 static_cast<int64_t>(bg.size()) - gb, cur.tile_off,
                                 cur.n_tiles});
      need = std::max(need, used);
      max_expo = std::max(max_expo, expo);
      cur = {static_cast<int64_t>(av.size()), 0, static_cast<int64_t>(bv.size()), 0,
             static_cast<int64_t>(tiles.size()), 0};
      used = 0;
      expo = 0;
    };
    for (auto const &g : w.groups) {
      auto const &sh = s.shapes[g.shape];
      std::vector<int32_t> is(sh.i.begin(), sh.i.end()), js(sh.j.begin(), sh.j.end());
      std::sort(is.begin(), is.end());
      is.erase(std::unique(is.begin(), is.end()), is.end());
      std::sort(js.begin(), js.end());
      js.erase(std::unique(js.begin(), js.end()), js.end());
      size_t const ab = dev::trace_tc_a_bytes(g.n_a, eds), bb = dev::trace_tc_b_bytes(g.n_b, eds);
      size_t const gb = is.size() * ab + js.size() * bb;
      if (used > 0 && used + gb > cap) close();
      // Regions and exponents of this group, by operand index.
      size_t const ni = static_cast<size_t>(is.back()) + 1, nj = static_cast<size_t>(js.back()) + 1;
      std::vector<int64_t> a_reg(ni, -1), b_reg(nj, -1), a_exp(ni, -1), b_exp(nj, -1);
      for (int32_t i : is) {
        a_reg[i] = static_cast<int64_t>(used);
        a_exp[i] = expo;
        for (int32_t ia = 0; ia < g.n_a; ++ia)
          av.push_back({static_cast<int64_t>(used), w.group_bases[g.a_off + ia] + i, ia,
                        static_cast<int32_t>(expo + ia), 0});
        used += ab;
        expo += g.n_a;
      }
      for (int32_t j : js) {
        b_reg[j] = static_cast<int64_t>(used);
        b_exp[j] = expo;
        for (int32_t ib = 0; ib < g.n_b; ++ib)
          bv.push_back({static_cast<int64_t>(used), w.group_bases[g.b_off + ib] + j, ib,
                        static_cast<int32_t>(expo + ib), 0});
        used += bb;
        expo += g.n_b;
      }
      // GEMM tiles, entries in order of their A region (consecutive tiles share
      // operand streams in L2).
      int64_t const n_e = static_cast<int64_t>(sh.i.size());
      std::vector<int64_t> eo(n_e);
      std::iota(eo.begin(), eo.end(), 0);
      std::stable_sort(eo.begin(), eo.end(),
                       [&](int64_t x, int64_t y) { return sh.i[x] < sh.i[y]; });
      int32_t const mts = (g.n_a + dev::kTrTileRows - 1) / dev::kTrTileRows;
      int32_t const nts = (g.n_b + dev::kTrTileCols - 1) / dev::kTrTileCols;
      int64_t const plane = static_cast<int64_t>(g.n_a) * g.n_b;
      for (int64_t e : eo) {
        int32_t const i = sh.i[e], j = sh.j[e];
        for (int32_t mt = 0; mt < mts; ++mt)
          for (int32_t nt = 0; nt < nts; ++nt) {
            dev::TrTile t{};
            t.a_src = a_reg[i] + static_cast<int64_t>(mt) * a_tile;
            t.b_src = b_reg[j] + static_cast<int64_t>(nt) * b_tile;
            t.out = g.val_base + e * plane + static_cast<int64_t>(nt) * dev::kTrTileCols * g.n_a +
                    static_cast<int64_t>(mt) * dev::kTrTileRows;
            t.ea = static_cast<int32_t>(a_exp[i] + mt * dev::kTrTileRows);
            t.eb = static_cast<int32_t>(b_exp[j] + nt * dev::kTrTileCols);
            t.rows = std::min(dev::kTrTileRows, g.n_a - mt * dev::kTrTileRows);
            t.cols = std::min(dev::kTrTileCols, g.n_b - nt * dev::kTrTileCols);
            t.ld = g.n_a;
            tiles.push_back(t);
          }
      }
    }
    close();
    upload(wb.tc_a, ag, stream_);
    upload(wb.tc_b, bg, stream_);
    upload(wb.tc_tiles, tiles, stream_);
    SLAPH_CK(cudaStreamSynchronize(stream_));
  }
  ds.tc_scratch = need;
  ds.tc_expo = max_expo;
  ds.tc_ready = true;
}

// Tensor-core plan of the factor products (product_tc.cu), per wave and
// dependency level: the groups of plan_products, their tiles of 80 columns
// and the scratch they need.
void Engine::prepare_product_tc(DeviceSchedule &ds) {
  if (ds.p_ready) return;
  Schedule const &s = ds.s;
  int32_t const eds = s.eds;
  int64_t const a_bytes = dev::prod_tc_a_bytes(eds), r_bytes = dev::prod_tc_r_bytes(eds);
  size_t need = 0;
  int64_t max_expo = 0;
  for (size_t wi = 0; wi < s.waves.size(); ++wi) {
    Wave const &w = s.waves[wi];
    auto &wb = *ds.waves[wi];
    std::vector<dev::ProdGroup> groups;
    std::vector<int32_t> r_slots, u_list, out_tab;
    std::vector<dev::ProdTile> tiles;
    wb.p_levels.clear();
    for (size_t lv = 0; lv + 1 < w.prod_level_off.size(); ++lv) {
      int64_t const b = w.prod_level_off[lv], e = w.prod_level_off[lv + 1];
      DeviceSchedule::PLevel pl{static_cast<int64_t>(groups.size()), 0,
                                static_cast<int64_t>(r_slots.size()), 0,
                                static_cast<int64_t>(tiles.size()), 0};
      ProductPlan const pp = plan_products(w.prods.data() + b, e - b, eds);
      int32_t const n_r = static_cast<int32_t>(pp.r_slots.size());
      r_slots.insert(r_slots.end(), pp.r_slots.begin(), pp.r_slots.end());
      int32_t const u_base = static_cast<int32_t>(u_list.size());
      u_list.insert(u_list.end(), pp.u_list.begin(), pp.u_list.end());
      out_tab.insert(out_tab.end(), pp.out_tab.begin(), pp.out_tab.end());
      for (auto const &pg : pp.groups) {
        dev::ProdGroup g{};
        for (int x = 0; x < 4; ++x) g.l[x] = pg.l[x];
        g.n_l = pg.n_l;
        g.n_u = pg.n_u;
        g.u_off = u_base + pg.u_off;
        int32_t const gi = static_cast<int32_t>(groups.size() - pl.g_off);
        g.ea = 64 * gi;
        int32_t const n_t = (eds * g.n_u + dev::kTrTileCols - 1) / dev::kTrTileCols;
        for (int32_t nt = 0; nt < n_t; ++nt) tiles.push_back({gi, nt});
        groups.push_back(g);
      }
      pl.n_g = static_cast<int64_t>(groups.size()) - pl.g_off;
      pl.n_r = n_r;
      pl.n_t = static_cast<int64_t>(tiles.size()) - pl.t_off;
      wb.p_levels.push_back(pl);
      size_t const r_off = static_cast<size_t>((pl.n_g * a_bytes + 1023) / 1024 * 1024);
      need = std::max(need, r_off + static_cast<size_t>(n_r) * r_bytes);
      max_expo = std::max(max_expo, 64 * pl.n_g + static_cast<int64_t>(n_r) * eds);
    }
    if (u_list.size() > 0x7fffffffULL) throw UnsupportedError("product GEMM lists above 2^31");
    upload(wb.p_groups, groups, stream_);
    upload(wb.p_rslots, r_slots, stream_);
    upload(wb.p_ulist, u_list, stream_);
    upload(wb.p_out, out_tab, stream_);
    upload(wb.p_tiles, tiles, stream_);
    SLAPH_CK(cudaStreamSynchronize(stream_));
  }
  ds.p_scratch = need;
  ds.p_expo = max_expo;
  ds.p_ready = true;
}

// Tensor-core plan of the Q1/Q2 factors (factor_tc.cu).  Per timeslice t:
//   X1[t]  rows (Q1R r at t, a), columns (r2, b, d, c), K = v:
//          A = conj(Q1R_r(a, v)), B = P_r2((4t+d) nev + v, b eds + c)
//   Q2M[t] rows (pair (b1, r1), a, bd), columns (VdaggerV code, v), K = w:
//          A = P_r1((4t+bd) nev + w, b1 eds + a) (conjugated by the GEMM form),
//          B = VdV_code(t)(w, v)
//   Q2     per complete bipartite set of (Q2M instance m) x (gamma, r2, b2):
//          rows (m, a), columns (gamma, r2, b2, c), K = (bd, v):
//          A = conj(s(bd, a) Q2M_m(a, bd nev + v)),
//          B = Gval[gamma][bd] P_r2((4t+Grow[gamma][bd]) nev + v, b2 eds + c)
// Dense FP64 outputs go to f_out_; gathers write the factor slots.
void Engine::prepare_factor_tc(DeviceSchedule &ds) {
  if (ds.f_ready) return;
  Schedule const &s = ds.s;
  int32_t const eds = s.eds, nev = dims_.nev, dilE = dims_.dilE, nb = geo_.nb;
  int32_t const n_rnd = dims_.n_rnd, Lt = dims_.Lt;
  int64_t const prow = 4LL * nev * Lt;            // perambulator rows
  int64_t const prs = prow * nb * eds;            // perambulator elements per random vector
  int64_t const blk = static_cast<int64_t>(nev) * nev;
  int32_t const kt1 = dev::gemm_k_tiles(nev), kt2 = dev::gemm_k_tiles(4LL * nev);
  size_t const a_tile1 = dev::tc_a_bytes(1, kt1), b_tile1 = dev::tc_b_bytes(1, kt1);
  size_t const a_tile2 = dev::tc_a_bytes(1, kt2), b_tile2 = dev::tc_b_bytes(1, kt2);
  size_t const cap = std::max(tc_scratch_.size(), kTraceScratchMin);
  int64_t const out_cap = int64_t{1} << 29;  // double2 per batch (8 GiB)

  // Instances per timeslice.
  std::vector<std::vector<int32_t>> q1r_t(Lt), q2m_t(Lt), q1_t(Lt), q2_t(Lt);
  for (size_t i = 0; i < s.q1r.size(); ++i) q1r_t[s.q1r[i].t].push_back(static_cast<int32_t>(i));
  for (size_t i = 0; i < s.q2m.size(); ++i) q2m_t[s.q2m[i].t].push_back(static_cast<int32_t>(i));
  for (size_t i = 0; i < s.q1.size(); ++i) q1_t[s.q1[i].t].push_back(static_cast<int32_t>(i));
  for (size_t i = 0; i < s.q2.size(); ++i) q2_t[s.q2[i].t].push_back(static_cast<int32_t>(i));

  std::vector<dev::GVec> vec;
  std::vector<dev::TrTile> tiles;
  std::vector<dev::Q1Gather> g1;
  std::vector<dev::Q2Gather> g2;
  ds.f_batches.clear();
  size_t need = 0;
  int64_t need_out = 0, need_expo = 0;

  auto add_vec = [&](int64_t dst, int32_t row, int32_t expo, int64_t stride, int32_t seg_len,
                     std::initializer_list<dev::GSeg> segs) {
    dev::GVec v{};
    v.dst = dst;
    v.stride = stride;
    v.row = row;
    v.expo = expo;
    v.n_seg = static_cast<int32_t>(segs.size());
    v.seg_len = seg_len;
    int k = 0;
    for (auto const &g : segs) v.seg[k++] = g;
    vec.push_back(v);
  };
  auto add_tiles = [&](int64_t a_reg, int64_t b_reg, size_t a_tile, size_t b_tile, int32_t rows,
                       int32_t cols, int64_t out, int32_t ea, int32_t eb) {
    int32_t const mts = (rows + dev::kTrTileRows - 1) / dev::kTrTileRows;
    int32_t const nts = (cols + dev::kTrTileCols - 1) / dev::kTrTileCols;
    for (int32_t mt = 0; mt < mts; ++mt)
      for (int32_t nt = 0; nt < nts; ++nt) {
        dev::TrTile t{};
        t.a_src = a_reg + static_cast<int64_t>(mt) * static_cast<int64_t>(a_tile);
        t.b_src = b_reg + static_cast<int64_t>(nt) * static_cast<int64_t>(b_tile);
        t.out = out + static_cast<int64_t>(nt) * dev::kTrTileCols * rows +
                static_cast<int64_t>(mt) * dev::kTrTileRows;
        t.ea = ea + mt * dev::kTrTileRows;
        t.eb = eb + nt * dev::kTrTileCols;
        t.rows = std::min(dev::kTrTileRows, rows - mt * dev::kTrTileRows);
        t.cols = std::min(dev::kTrTileCols, cols - nt * dev::kTrTileCols);
        t.ld = rows;
        tiles.push_back(t);
      }
  };

  // Per-timeslice pieces, appended to the current batch until a cap is hit.
  struct TPlan {
    size_t s1 = 0, s2 = 0;  // scratch bytes of phase 1 / 2
    int64_t out = 0;        // dense output doubles2
  };
  auto t_sizes = [&](int t, std::vector<std::vector<int32_t>> &bic_rows,
                     std::vector<std::vector<std::array<int32_t, 3>>> &bic_cols) {
    TPlan p;
    int32_t const nr = static_cast<int32_t>(q1r_t[t].size());
    int32_t const x1_rows = nr * eds, x1_cols = n_rnd * nb * 4 * eds;
    std::map<std::pair<int32_t, int32_t>, int32_t> pairs;
    std::map<int32_t, int32_t> codes;
    for (int32_t m : q2m_t[t]) {
      pairs.emplace(std::make_pair(s.q2m[m].b1, s.q2m[m].r1), 0);
      codes.emplace(s.q2m[m].vdv, 0);
    }
    int32_t const q2m_rows = static_cast<int32_t>(pairs.size()) * eds * 4;
    int32_t const q2m_cols = static_cast<int32_t>(codes.size()) * nev;
    if (nr > 0)
      p.s1 += dev::tc_a_bytes(x1_rows, kt1) + dev::tc_b_bytes(x1_cols, kt1);
    if (!q2m_t[t].empty())
      p.s1 += dev::tc_a_bytes(q2m_rows, kt1) + dev::tc_b_bytes(q2m_cols, kt1);
    p.out += static_cast<int64_t>(x1_rows) * x1_cols + static_cast<int64_t>(q2m_rows) * q2m_cols;
    // Q2 bicliques: Q2M instances with equal sets of (gamma, r2, b2).
    std::map<int32_t, std::vector<std::array<int32_t, 3>>> cols_of;
    for (int32_t q : q2_t[t]) cols_of[s.q2[q].m].push_back({s.q2[q].gamma, s.q2[q].r2, s.q2[q].b2});
    std::map<std::vector<std::array<int32_t, 3>>, std::vector<int32_t>> groups;
    for (auto &kv : cols_of) {
      auto v = kv.second;
      std::sort(v.begin(), v.end());
      v.erase(std::unique(v.begin(), v.end()), v.end());
      groups[v].push_back(kv.first);
    }
    bic_rows.clear();
    bic_cols.clear();
    for (auto &kv : groups) {
      bic_rows.push_back(kv.second);
      bic_cols.push_back(kv.first);
      int32_t const rows = static_cast<int32_t>(kv.second.size()) * eds;
      int32_t const cols = static_cast<int32_t>(kv.first.size()) * eds;
      p.s2 += dev::tc_a_bytes(rows, kt2) + dev::tc_b_bytes(cols, kt2);
      p.out += static_cast<int64_t>(rows) * cols;
    }
    return p;
  };

  size_t used1 = 0, used2 = 0;
  int64_t used_out = 0;
  int32_t expo = 0;
  std::vector<int> batch_ts;
  auto flush = [&](void) {
    if (batch_ts.empty()) return;
    // Phase 1 then phase 2 items of every timeslice of the batch.
    DeviceSchedule::FBatch b{};
    int64_t out = 0;
    size_t off1 = 0, off2 = 0;
    expo = 0;
    struct TOut {
      int64_t x1, q2m;
      int32_t x1_rows, q2m_rows;
      std::map<std::pair<int32_t, int32_t>, int32_t> pairs;
      std::map<int32_t, int32_t> codes;
      std::vector<std::vector<int32_t>> bic_rows;
      std::vector<std::vector<std::array<int32_t, 3>>> bic_cols;
      std::map<int32_t, int32_t> rloc;
    };
    std::vector<TOut> tos(batch_ts.size());
    // -- phase 1 vectors: X1 A (df source), Q2M A (f64), X1 B (f64), Q2M B (f64)
    auto begin = [&](int64_t (&r)[2]) { r[0] = static_cast<int64_t>(vec.size()); };
    auto end = [&](int64_t (&r)[2]) { r[1] = static_cast<int64_t>(vec.size()) - r[0]; };
    std::vector<int64_t> regA_x1(batch_ts.size()), regB_x1(batch_ts.size()),
        regA_q2m(batch_ts.size()), regB_q2m(batch_ts.size());
    std::vector<int32_t> eA_x1(batch_ts.size()), eB_x1(batch_ts.size()),
        eA_q2m(batch_ts.size()), eB_q2m(batch_ts.size());
    for (size_t k = 0; k < batch_ts.size(); ++k) {
      int const t = batch_ts[k];
      TOut &o = tos[k];
      for (int32_t r : q1r_t[t]) o.rloc.emplace(r, static_cast<int32_t>(o.rloc.size()));
      for (int32_t m : q2m_t[t]) {
        o.pairs.emplace(std::make_pair(s.q2m[m].b1, s.q2m[m].r1), 0);
        o.codes.emplace(s.q2m[m].vdv, 0);
      }
      int32_t i = 0;
      for (auto &kv : o.pairs) kv.second = i++;
      i = 0;
      for (auto &kv : o.codes) kv.second = i++;
      o.x1_rows = static_cast<int32_t>(o.rloc.size()) * eds;
      o.q2m_rows = static_cast<int32_t>(o.pairs.size()) * eds * 4;
      o.x1 = out;
      out += static_cast<int64_t>(o.x1_rows) * n_rnd * nb * 4 * eds;
      o.q2m = out;
      out += static_cast<int64_t>(o.q2m_rows) * static_cast<int64_t>(o.codes.size()) * nev;
    }
    begin(b.a_x1);
    for (size_t k = 0; k < batch_ts.size(); ++k) {
      TOut &o = tos[k];
      regA_x1[k] = static_cast<int64_t>(off1);
      eA_x1[k] = expo;
      for (auto const &kv : o.rloc)
        for (int32_t a = 0; a < eds; ++a)
          add_vec(regA_x1[k], kv.second * eds + a, expo++, eds, nev,
                  {{static_cast<int64_t>(kv.first) * nev * eds + a, 0, 0}});
      off1 += dev::tc_a_bytes(std::max(o.x1_rows, 1), kt1);
    }
    end(b.a_x1);
    begin(b.a_q2m);
    for (size_t k = 0; k < batch_ts.size(); ++k) {
      int const t = batch_ts[k];
      TOut &o = tos[k];
      regA_q2m[k] = static_cast<int64_t>(off1);
      eA_q2m[k] = expo;
      for (auto const &kv : o.pairs) {
        int32_t const b1 = kv.first.first, r1 = kv.first.second, p = kv.second;
        for (int32_t a = 0; a < eds; ++a)
          for (int32_t bd = 0; bd < 4; ++bd)
            add_vec(regA_q2m[k], (p * eds + a) * 4 + bd, eA_q2m[k] + (p * eds + a) * 4 + bd, 1,
                    nev,
                    {{r1 * prs + (4LL * t + bd) * nev + prow * (static_cast<int64_t>(b1) * eds + a),
                      0, 0}});
      }
      expo += o.q2m_rows;
      off1 += dev::tc_a_bytes(std::max(o.q2m_rows, 1), kt1);
    }
    end(b.a_q2m);
    begin(b.b_x1);
    for (size_t k = 0; k < batch_ts.size(); ++k) {
      int const t = batch_ts[k];
      regB_x1[k] = static_cast<int64_t>(off1);
      eB_x1[k] = expo;
      int32_t const cols = n_rnd * nb * 4 * eds;
      if (tos[k].x1_rows > 0) {
        for (int32_t r2 = 0; r2 < n_rnd; ++r2)
          for (int32_t b2 = 0; b2 < nb; ++b2)
            for (int32_t d = 0; d < 4; ++d)
              for (int32_t c = 0; c < eds; ++c)
                add_vec(regB_x1[k], ((r2 * nb + b2) * 4 + d) * eds + c, expo++, 1, nev,
                        {{r2 * prs + (4LL * t + d) * nev + prow * (static_cast<int64_t>(b2) * eds + c),
                          0, 0}});
        off1 += dev::tc_b_bytes(cols, kt1);
      }
    }
    end(b.b_x1);
    begin(b.b_q2m);
    for (size_t k = 0; k < batch_ts.size(); ++k) {
      int const t = batch_ts[k];
      TOut &o = tos[k];
      regB_q2m[k] = static_cast<int64_t>(off1);
      eB_q2m[k] = expo;
      for (auto const &kv : o.codes)
        for (int32_t v = 0; v < nev; ++v)
          add_vec(regB_q2m[k], kv.second * nev + v, expo++, 1, nev,
                  {{(static_cast<int64_t>(kv.first) * Lt + t) * blk + static_cast<int64_t>(nev) * v,
                    0, 0}});
      if (!o.codes.empty())
        off1 += dev::tc_b_bytes(static_cast<int32_t>(o.codes.size()) * nev, kt1);
    }
    end(b.b_q2m);
    b.t1[0] = static_cast<int64_t>(tiles.size());
    for (size_t k = 0; k < batch_ts.size(); ++k) {
      TOut &o = tos[k];
      if (o.x1_rows > 0)
        add_tiles(regA_x1[k], regB_x1[k], a_tile1, b_tile1, o.x1_rows, n_rnd * nb * 4 * eds, o.x1,
                  eA_x1[k], eB_x1[k]);
      if (o.q2m_rows > 0)
        add_tiles(regA_q2m[k], regB_q2m[k], a_tile1, b_tile1, o.q2m_rows,
                  static_cast<int32_t>(o.codes.size()) * nev, o.q2m, eA_q2m[k], eB_q2m[k]);
    }
    b.t1[1] = static_cast<int64_t>(tiles.size()) - b.t1[0];
    need = std::max(need, off1);
    // -- phase 2: Q2 bicliques (A from the Q2M outputs, B from the perambulators)
    std::vector<std::vector<int64_t>> regA2(batch_ts.size()), regB2(batch_ts.size()),
        out2(batch_ts.size());
    std::vector<std::vector<int32_t>> eA2(batch_ts.size()), eB2(batch_ts.size());
    for (size_t k = 0; k < batch_ts.size(); ++k) t_sizes(batch_ts[k], tos[k].bic_rows, tos[k].bic_cols);
    begin(b.a_q2);
    for (size_t k = 0; k < batch_ts.size(); ++k) {
      TOut &o = tos[k];
      int64_t const ld = o.q2m_rows;
      for (size_t g = 0; g < o.bic_rows.size(); ++g) {
        regA2[k].push_back(static_cast<int64_t>(off2));
        eA2[k].push_back(expo);
        int32_t const rows = static_cast<int32_t>(o.bic_rows[g].size()) * eds;
        for (size_t mi = 0; mi < o.bic_rows[g].size(); ++mi) {
          auto const &q = s.q2m[o.bic_rows[g][mi]];
          int32_t const p = o.pairs.at({q.b1, q.r1}), ci = o.codes.at(q.vdv);
          for (int32_t a = 0; a < eds; ++a) {
            int32_t const r = a / dilE;
            dev::GVec v{};
            v.dst = static_cast<int64_t>(off2);
            v.stride = ld;
            v.row = static_cast<int32_t>(mi) * eds + a;
            v.expo = expo++;
            v.n_seg = 4;
            v.seg_len = nev;
            for (int32_t bd = 0; bd < 4; ++bd) {
              bool const flip = (bd + r == 3) || (bd - r > 1) || (r - bd > 1);
              v.seg[bd].src = o.q2m + ((p * eds + a) * 4 + bd) + ld * (static_cast<int64_t>(ci) * nev);
              v.seg[bd].factor = flip ? 2 : 0;
            }
            vec.push_back(v);
          }
        }
        off2 += dev::tc_a_bytes(rows, kt2);
      }
    }
    end(b.a_q2);
    begin(b.b_q2);
    for (size_t k = 0; k < batch_ts.size(); ++k) {
      int const t = batch_ts[k];
      TOut &o = tos[k];
      for (size_t g = 0; g < o.bic_cols.size(); ++g) {
        regB2[k].push_back(static_cast<int64_t>(off2));
        eB2[k].push_back(expo);
        int32_t const cols = static_cast<int32_t>(o.bic_cols[g].size()) * eds;
        for (size_t ci = 0; ci < o.bic_cols[g].size(); ++ci) {
          auto const &cg = o.bic_cols[g][ci];  // (gamma, r2, b2)
          for (int32_t c = 0; c < eds; ++c) {
            dev::GVec v{};
            v.dst = static_cast<int64_t>(off2);
            v.stride = 1;
            v.row = static_cast<int32_t>(ci) * eds + c;
            v.expo = expo++;
            v.n_seg = 4;
            v.seg_len = nev;
            for (int32_t bd = 0; bd < 4; ++bd) {
              v.seg[bd].src = cg[1] * prs + (4LL * t + dev::gamma_row_host(cg[0], bd)) * nev +
                              prow * (static_cast<int64_t>(cg[2]) * eds + c);
              v.seg[bd].factor = dev::gamma_phase_host(cg[0], bd);
            }
            vec.push_back(v);
          }
        }
        off2 += dev::tc_b_bytes(cols, kt2);
      }
    }
    end(b.b_q2);
    b.t2[0] = static_cast<int64_t>(tiles.size());
    for (size_t k = 0; k < batch_ts.size(); ++k) {
      TOut &o = tos[k];
      for (size_t g = 0; g < o.bic_rows.size(); ++g) {
        int32_t const rows = static_cast<int32_t>(o.bic_rows[g].size()) * eds;
        int32_t const cols = static_cast<int32_t>(o.bic_cols[g].size()) * eds;
        out2[k].push_back(out);
        add_tiles(regA2[k][g], regB2[k][g], a_tile2, b_tile2, rows, cols, out, eA2[k][g],
                  eB2[k][g]);
        out += static_cast<int64_t>(rows) * cols;
      }
    }
    b.t2[1] = static_cast<int64_t>(tiles.size()) - b.t2[0];
    need = std::max(need, off2);
    // -- gathers
    b.g1[0] = static_cast<int64_t>(g1.size());
    for (size_t k = 0; k < batch_ts.size(); ++k) {
      TOut &o = tos[k];
      for (int32_t qi : q1_t[batch_ts[k]]) {
        auto const &q = s.q1[qi];
        dev::Q1Gather g{};
        g.x_off = o.x1;
        g.ld = o.x1_rows;
        g.row0 = o.rloc.at(q.r) * eds;
        g.col0 = (q.r2 * nb + q.b) * 4 * eds;
        g.gamma = q.gamma;
        g.slot = q.slot;
        g1.push_back(g);
      }
    }
    b.g1[1] = static_cast<int64_t>(g1.size()) - b.g1[0];
    b.g2[0] = static_cast<int64_t>(g2.size());
    for (size_t k = 0; k < batch_ts.size(); ++k) {
      TOut &o = tos[k];
      std::map<int32_t, std::pair<size_t, size_t>> where;  // Q2M m -> (biclique, row)
      for (size_t g = 0; g < o.bic_rows.size(); ++g)
        for (size_t mi = 0; mi < o.bic_rows[g].size(); ++mi) where[o.bic_rows[g][mi]] = {g, mi};
      for (int32_t qi : q2_t[batch_ts[k]]) {
        auto const &q = s.q2[qi];
        auto const w = where.at(q.m);
        auto const &cols = o.bic_cols[w.first];
        std::array<int32_t, 3> const key{q.gamma, q.r2, q.b2};
        size_t const ci = std::lower_bound(cols.begin(), cols.end(), key) - cols.begin();
        int32_t const rows = static_cast<int32_t>(o.bic_rows[w.first].size()) * eds;
        dev::Q2Gather g{};
        g.off = out2[k][w.first] + static_cast<int64_t>(w.second) * eds +
                static_cast<int64_t>(rows) * (static_cast<int64_t>(ci) * eds);
        g.ld = rows;
        g.slot = q.slot;
        g2.push_back(g);
      }
    }
    b.g2[1] = static_cast<int64_t>(g2.size()) - b.g2[0];
    need_out = std::max(need_out, out);
    need_expo = std::max<int64_t>(need_expo, expo);
    ds.f_batches.push_back(b);
    batch_ts.clear();
    used1 = used2 = 0;
    used_out = 0;
  };
  std::vector<std::vector<int32_t>> br;
  std::vector<std::vector<std::array<int32_t, 3>>> bc;
  for (int t = 0; t < Lt; ++t) {
    if (q1r_t[t].empty() && q2m_t[t].empty() && q2_t[t].empty()) continue;
    TPlan const p = t_sizes(t, br, bc);
    if (!batch_ts.empty() &&
        (used1 + p.s1 > cap || used2 + p.s2 > cap || used_out + p.out > out_cap))
      flush();
    batch_ts.push_back(t);
    used1 += p.s1;
    used2 += p.s2;
    used_out += p.out;
  }
  flush();
  upload(ds.fvec, vec, stream_);
  upload(ds.ftiles, tiles, stream_);
  upload(ds.fg1, g1, stream_);
  upload(ds.fg2, g2, stream_);
  SLAPH_CK(cudaStreamSynchronize(stream_));
  ds.f_scratch = need;
  ds.f_out = need_out;
  ds.f_expo = need_expo;
  ds.f_ready = true;
}

void Engine::contract(slaph_plan const *plan, int precision, int accumulator,
                      int single_block_pair, double *corr_out) {
  if (!plan || !corr_out) throw ArgError("null plan or output");
  if (!vdv_built_) throw StateError("slaph_vdaggerv_build must be called before contract");
  if (precision != SLAPH_FP64 && precision != SLAPH_MIXED)
    throw ArgError("unknown precision mode");
  if (accumulator != SLAPH_ACC_NATIVE && accumulator != SLAPH_ACC_KAHAN)
    throw ArgError("unknown accumulator");
  if (plan->n_vdv_ops != static_cast<int32_t>(ops_.size()))
    throw ArgError("plan VdaggerV table does not match slaph_engine_set_operators");
  for (int32_t d = 0; d < plan->n_diagrams; ++d)
    if (plan->diagrams[d].n_requests > 0 && !plan->diagrams[d].requests)
      throw ArgError("diagram without request array");
  // launches_ continues the count of the preceding VdaggerV build: one gauge
  // configuration = build + contract.
  auto const tp = std::chrono::steady_clock::now();
  // The schedules to run: one for the whole configuration (factors built once
  // and kept for every block pair), or one per block pair (factors built for
  // that block pair and dropped after it, as the reference clears its factor
  // caches per block pair, src/Correlators.cpp:116); the correlator sums run
  // over the block pairs in the same order either way.
  std::vector<DeviceSchedule *> scheds;
  if (factor_lifetime_ == SLAPH_FACTORS_BLOCK_PAIR) {
    if (bp_plan_ != plan) {
      bp_scheds_.clear();
      bp_plan_ = plan;
    }
    int const nb = dims_.Lt / dims_.dilT;
    for (int b = 0; b < nb * (nb + 1) / 2; ++b) {
      if (single_block_pair >= 0 && b != single_block_pair) continue;
      auto &sp = bp_scheds_[b];
      if (!sp) sp = make_schedule(plan, b);
      scheds.push_back(sp.get());
    }
    if (scheds.empty()) throw ArgError("block pair out of range");
  } else {
    prepare_schedule(plan, single_block_pair);
    scheds.push_back(sched_.get());
  }
  double const plan_wall =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - tp).count();
  bool const mixed = precision == SLAPH_MIXED;
  // Perambulators and noise uploaded asynchronously are waited for here.
  for (int32_t r = 0; r < dims_.n_rnd; ++r) {
    if (pend_p_[r]) SLAPH_CK(cudaStreamWaitEvent(stream_, ev_p_[r], 0));
    if (pend_n_[r]) SLAPH_CK(cudaStreamWaitEvent(stream_, ev_n_[r], 0));
  }
  std::fill(pend_p_.begin(), pend_p_.end(), 0);
  std::fill(pend_n_.begin(), pend_n_.end(), 0);
  int64_t const n_outputs = scheds.front()->s.n_outputs;
  int64_t const n_run = std::max<int64_t>(1, n_outputs * dims_.Lt);
  running_.reserve(sizeof(double2) * n_run);
  SLAPH_CK(cudaMemsetAsync(running_.as<void>(), 0, sizeof(double2) * n_run, stream_));
  double t_f = 0, t_pt = 0, t_as = 0, t_tr = 0, t_sl = 0, t_gm = 0, t_pr = 0;
  int64_t n_pr = 0;
  int64_t n_tr = 0, n_gm = 0;
  double st[8] = {};
  for (DeviceSchedule *dsp : scheds) {
    DeviceSchedule &ds = *dsp;
    Schedule const &s = ds.s;
    int32_t const eds = s.eds;
    int64_t const ms = static_cast<int64_t>(eds) * eds;
    int64_t const nev = dims_.nev;

    // ---- factors
    SLAPH_CK(cudaEventRecord(ev_[0], stream_));
    if (!mixed) {
      slots_.reserve(sizeof(double2) * ms *
                     std::max<int64_t>(1, s.n_factor_slots + s.max_prod_slots));
      DevBuf q0m, q1r, q2m;
      q0m.reserve(sizeof(double2) * std::max<int64_t>(1, s.q0m.size()) * nev * eds);
      q1r.reserve(sizeof(double2) * std::max<int64_t>(1, s.q1r.size()) * nev * eds);
      q2m.reserve(sizeof(double2) * std::max<int64_t>(1, s.q2m.size()) * eds * 4 * nev);
      double2 const *vdv = vdv_.as<double2>();
      launch(dev::q0m(q0m.as<double2>(), ds.q0m.as<dev::Q0MInst>(), s.q0m.size(), vdv,
                      noise_.as<double2>(), geo_, stream_),
             "q0m");
      launch(dev::q1r(q1r.as<double2>(), ds.q1r.as<dev::Q1RInst>(), s.q1r.size(), vdv,
                      noise_.as<double2>(), geo_, stream_),
             "q1r");
      launch(dev::q2m(q2m.as<double2>(), ds.q2m.as<dev::Q2MInst>(), s.q2m.size(), vdv,
                      peram_.as<double2>(), geo_, stream_),
             "q2m");
      launch(dev::q0(slots_.as<double2>(), ds.q0.as<dev::Q0Inst>(), s.q0.size(),
                     q0m.as<double2>(), noise_.as<double2>(), geo_, stream_),
             "q0");
      launch(dev::q1(slots_.as<double2>(), ds.q1.as<dev::Q1Inst>(), s.q1.size(),
                     q1r.as<double2>(), peram_.as<double2>(), geo_, stream_),
             "q1");
      launch(dev::q2(slots_.as<double2>(), ds.q2.as<dev::Q2Inst>(), s.q2.size(),
                     q2m.as<double2>(), peram_.as<double2>(), geo_, stream_),
             "q2");
      SLAPH_CK(cudaEventRecord(ev_[1], stream_));
      SLAPH_CK(cudaEventSynchronize(ev_[1]));  // intermediates are freed here
    } else {
      // Double-float matrices in both layouts: factors now, products per wave.
      size_t const df_bytes =
          sizeof(float4) * ms * std::max<int64_t>(1, s.n_factor_slots + s.max_prod_slots);
      df_slots_.reserve(df_bytes);
      df_slots_t_.reserve(df_bytes);
      slot_bits_.reserve(sizeof(unsigned int) *
                         std::max<int64_t>(1, s.n_factor_slots + s.max_prod_slots));
      int64_t const n_vdv = 2LL * static_cast<int64_t>(ops_.size()) * dims_.Lt * nev * nev;
      int64_t const n_noise = 4LL * nev * dims_.Lt * dims_.n_rnd;
      DevBuf vdv_df, noise_df, q0m, q1r;
      vdv_df.reserve(sizeof(float4) * std::max<int64_t>(1, n_vdv));
      noise_df.reserve(sizeof(float4) * n_noise);
      launch(dev::to_df(vdv_df.as<float4>(), vdv_.as<double2>(), n_vdv, stream_), "to_df");
      launch(dev::to_df(noise_df.as<float4>(), noise_.as<double2>(), n_noise, stream_), "to_df");
      q0m.reserve(sizeof(float4) * std::max<int64_t>(1, s.q0m.size()) * nev * eds);
      q1r.reserve(sizeof(float4) * std::max<int64_t>(1, s.q1r.size()) * nev * eds);
      // Q0 and the Q1R intermediates in double-float; Q2M, Q1 and Q2 on the
      // tensor cores below.
      launch(dev::factors_df(df_slots_.as<float4>(), df_slots_t_.as<float4>(), q0m.as<float4>(),
                             q1r.as<float4>(), nullptr, ds.q0m.as<dev::Q0MInst>(),
                             s.q0m.size(), ds.q1r.as<dev::Q1RInst>(), s.q1r.size(), nullptr, 0,
                             ds.q0.as<dev::Q0Inst>(), s.q0.size(), nullptr, 0, nullptr, 0,
                             vdv_df.as<float4>(), noise_df.as<float4>(), nullptr, geo_, stream_),
             "factors_df");
      launches_ += 2;
      prepare_factor_tc(ds);
      tc_scratch_.reserve(std::max<size_t>(1, ds.f_scratch));
      f_out_.reserve(sizeof(double2) * std::max<int64_t>(1, ds.f_out));
      tr_expo_.reserve(sizeof(int32_t) * std::max<int64_t>(1, ds.f_expo));
      err_.reserve(sizeof(int));
      SLAPH_CK(cudaMemsetAsync(err_.as<void>(), 0, sizeof(int), stream_));
      int32_t const kt1 = dev::gemm_k_tiles(nev), kt2 = dev::gemm_k_tiles(4 * nev);
      uint8_t *scr = tc_scratch_.as<uint8_t>();
      int32_t *ex = tr_expo_.as<int32_t>();
      double2 *fo = f_out_.as<double2>();
      auto const *fv = ds.fvec.as<dev::GVec>();
      auto const *ft = ds.ftiles.as<dev::TrTile>();
      auto count = [&](int64_t n) { launches_ += n > 0 ? 1 : 0; };
      for (auto const &b : ds.f_batches) {
        cuda_check(dev::gvec_slice_df(scr, ex, fv + b.a_x1[0], b.a_x1[1], true, true,
                                      q1r.as<float4>(), kt1, stream_),
                   "slice X1 A");
        cuda_check(dev::gvec_slice_f64(scr, ex, fv + b.a_q2m[0], b.a_q2m[1], true, false,
                                       peram_.as<double2>(), kt1, stream_),
                   "slice Q2M A");
        cuda_check(dev::gvec_slice_f64(scr, ex, fv + b.b_x1[0], b.b_x1[1], false, false,
                                       peram_.as<double2>(), kt1, stream_),
                   "slice X1 B");
        cuda_check(dev::gvec_slice_f64(scr, ex, fv + b.b_q2m[0], b.b_q2m[1], false, false,
                                       vdv_.as<double2>(), kt1, stream_),
                   "slice Q2M B");
        count(b.a_x1[1]); count(b.a_q2m[1]); count(b.b_x1[1]); count(b.b_q2m[1]);
        cuda_check(dev::tc_gemm(fo, scr, ex, ft + b.t1[0], b.t1[1], kt1, err_.as<int>(), stream_),
                   "factor GEMM (X1, Q2M)");
        count(b.t1[1]);
        cuda_check(dev::gvec_slice_f64(scr, ex, fv + b.a_q2[0], b.a_q2[1], true, true, fo, kt2,
                                       stream_),
                   "slice Q2 A");
        cuda_check(dev::gvec_slice_f64(scr, ex, fv + b.b_q2[0], b.b_q2[1], false, false,
                                       peram_.as<double2>(), kt2, stream_),
                   "slice Q2 B");
        count(b.a_q2[1]); count(b.b_q2[1]);
        cuda_check(dev::tc_gemm(fo, scr, ex, ft + b.t2[0], b.t2[1], kt2, err_.as<int>(), stream_),
                   "factor GEMM (Q2)");
        count(b.t2[1]);
        cuda_check(dev::q1_gather(df_slots_.as<float4>(), df_slots_t_.as<float4>(),
                                  ds.fg1.as<dev::Q1Gather>() + b.g1[0], b.g1[1], fo, dims_.dilE,
                                  stream_),
                   "q1_gather");
        cuda_check(dev::q2_gather(df_slots_.as<float4>(), df_slots_t_.as<float4>(),
                                  ds.fg2.as<dev::Q2Gather>() + b.g2[0], b.g2[1], fo, eds, stream_),
                   "q2_gather");
        count(b.g1[1]); count(b.g2[1]);
      }
      // largest entries of the factor slots for the trace-operand slicing
      launch(dev::slot_maxbits(slot_bits_.as<unsigned int>(), df_slots_.as<float4>(), 0,
                               s.n_factor_slots, eds, stream_),
             "slot_maxbits");
      SLAPH_CK(cudaEventRecord(ev_[1], stream_));
      SLAPH_CK(cudaEventSynchronize(ev_[1]));  // intermediates are freed here
    }
    t_f += elapsed_ms(ev_[0], ev_[1]);

    // ---- waves: products, traces, terms, accumulation
    values_.reserve(sizeof(double2) * std::max<int64_t>(1, s.max_values));
    term_val_.reserve(sizeof(double2) * std::max<int64_t>(1, s.max_terms));
    bool const p_tc = mixed && dev::prod_tc_supported(eds);
    if (mixed) {
      prepare_trace_tc(ds);
      if (p_tc) prepare_product_tc(ds);
      tc_scratch_.reserve(std::max<size_t>(1, std::max(ds.tc_scratch, ds.p_scratch)));
      tr_expo_.reserve(sizeof(int32_t) * std::max<int64_t>(1, std::max(ds.tc_expo, ds.p_expo)));
      err_.reserve(sizeof(int));
      SLAPH_CK(cudaMemsetAsync(err_.as<void>(), 0, sizeof(int), stream_));
    }
    for (size_t wi = 0; wi < s.waves.size(); ++wi) {
      Wave const &w = s.waves[wi];
      auto &wb = *ds.waves[wi];
      SLAPH_CK(cudaEventRecord(ev_[2], stream_));
      auto const *prods = wb.prods.as<dev::ProdInst>();
      // the tensor-core products take the largest entries of their slots by
      // atomicMax from zero
      if (p_tc && w.n_prod_slots > 0)
        SLAPH_CK(cudaMemsetAsync(slot_bits_.as<unsigned int>() + s.n_factor_slots, 0,
                                 sizeof(unsigned int) * w.n_prod_slots, stream_));
      for (size_t lv = 0; lv + 1 < w.prod_level_off.size(); ++lv) {
        int64_t const b = w.prod_level_off[lv], e = w.prod_level_off[lv + 1];
        if (e <= b) continue;
        if (mixed && p_tc) {
          auto const &pl = wb.p_levels[lv];
          int64_t const r_off =
              (pl.n_g * dev::prod_tc_a_bytes(eds) + 1023) / 1024 * 1024;
          launch(dev::products_tc(df_slots_.as<float4>(), df_slots_t_.as<float4>(),
                                  tc_scratch_.as<uint8_t>(), r_off, tr_expo_.as<int32_t>(),
                                  64 * pl.n_g, wb.p_groups.as<dev::ProdGroup>() + pl.g_off,
                                  pl.n_g, wb.p_rslots.as<int32_t>() + pl.r_off, pl.n_r,
                                  wb.p_ulist.as<int32_t>(), wb.p_out.as<int32_t>(),
                                  wb.p_tiles.as<dev::ProdTile>() + pl.t_off, pl.n_t, eds,
                                  slot_bits_.as<unsigned int>(), err_.as<int>(), stream_),
                 "products_tc");
          launches_ += 2;
        } else if (mixed) {
          launch(dev::products_df(df_slots_.as<float4>(), df_slots_t_.as<float4>(), prods + b,
                                  e - b, eds, stream_),
                 "products_df");
        } else
          launch(dev::products(slots_.as<double2>(), prods + b, e - b, eds, stream_), "products");
      }
      if (mixed && !p_tc && w.n_prod_slots > 0)  // largest entries of the product slots
        launch(dev::slot_maxbits(slot_bits_.as<unsigned int>(), df_slots_.as<float4>(),
                                 s.n_factor_slots, w.n_prod_slots, eds, stream_),
               "slot_maxbits");
      int64_t const n_res = static_cast<int64_t>(w.residual_lists.size());
      int64_t const n_uni = static_cast<int64_t>(w.unique_lists.size());
      SLAPH_CK(cudaEventRecord(ev_[5], stream_));
      if (mixed) {
        values_df_.reserve(sizeof(float4) * std::max<int64_t>(1, s.max_values));
        if (n_res > 0)
          launch(dev::traces_df(values_df_.as<float4>(), wb.lists.as<dev::TraceList>(),
                                wb.residual.as<int32_t>(), n_res, ds.shape_i.as<int32_t>(),
                                ds.shape_j.as<int32_t>(), ds.shape_off.as<int64_t>(),
                                df_slots_.as<float4>(), df_slots_t_.as<float4>(), eds, stream_),
                 "traces_df");
        SLAPH_CK(cudaEventRecord(ev_[6], stream_));
        int64_t const gv = w.n_group_values;
        if (w.n_values > gv)
          launch(dev::df_values_to_fp64(values_.as<double2>() + gv, values_df_.as<float4>() + gv,
                                        w.n_values - gv, stream_),
                 "df_values_to_fp64");
        // Dense groups on the tensor cores: slice, then GEMM, per batch.
        while (tc_ev_.size() < 3 * wb.tc_batches.size()) {
          cudaEvent_t e = nullptr;
          SLAPH_CK(cudaEventCreate(&e));
          tc_ev_.push_back(e);
        }
        for (size_t bi = 0; bi < wb.tc_batches.size(); ++bi) {
          auto const &b = wb.tc_batches[bi];
          SLAPH_CK(cudaEventRecord(tc_ev_[3 * bi], stream_));
          cuda_check(dev::trace_tc_slice(tc_scratch_.as<uint8_t>(), tr_expo_.as<int32_t>(),
                                         wb.tc_a.as<dev::TrSliceGroup>() + b.a_off, b.n_a,
                                         wb.tc_b.as<dev::TrSliceGroup>() + b.b_off, b.n_b,
                                         df_slots_.as<float4>(), df_slots_t_.as<float4>(),
                                         slot_bits_.as<unsigned int>(), eds, stream_),
                     "trace_tc_slice");
          launches_ += (b.n_a > 0 ? 1 : 0) + (b.n_b > 0 ? 1 : 0);
          SLAPH_CK(cudaEventRecord(tc_ev_[3 * bi + 1], stream_));
          launch(dev::trace_tc_gemm(values_.as<double2>(), tc_scratch_.as<uint8_t>(),
                                    tr_expo_.as<int32_t>(), wb.tc_tiles.as<dev::TrTile>() + b.tile_off,
                                    b.n_tiles, eds, err_.as<int>(), stream_),
                 "trace_tc_gemm");
          SLAPH_CK(cudaEventRecord(tc_ev_[3 * bi + 2], stream_));
        }
      } else {
        if (n_uni > 0)
          launch(dev::traces(values_.as<double2>(), wb.lists.as<dev::TraceList>(),
                             wb.unique.as<int32_t>(), n_uni, ds.shape_i.as<int32_t>(),
                             ds.shape_j.as<int32_t>(), ds.shape_off.as<int64_t>(),
                             slots_.as<double2>(), eds, stream_),
                 "traces");
        SLAPH_CK(cudaEventRecord(ev_[6], stream_));
      }
      bool const traced = mixed ? n_res > 0 : n_uni > 0;
      SLAPH_CK(cudaEventRecord(ev_[3], stream_));
      launch(dev::terms(term_val_.as<double2>(), wb.terms.as<dev::Term>(),
                        static_cast<int64_t>(w.terms.size()), wb.lists.as<dev::TraceList>(),
                        values_.as<double2>(), ds.shape_mask.as<uint16_t>(),
                        ds.shape_off.as<int64_t>(), accumulator == SLAPH_ACC_KAHAN ? 1 : 0,
                        stream_),
             "terms");
      launch(dev::accumulate(running_.as<double2>(), wb.seg_out.as<int32_t>(),
                             wb.seg_off.as<int64_t>(), wb.n_seg, wb.idx.as<int32_t>(),
                             term_val_.as<double2>(), stream_),
             "accumulate");
      SLAPH_CK(cudaEventRecord(ev_[4], stream_));
      SLAPH_CK(cudaEventSynchronize(ev_[4]));
      t_pt += elapsed_ms(ev_[2], ev_[3]);
      t_as += elapsed_ms(ev_[3], ev_[4]);
      t_pr += elapsed_ms(ev_[2], ev_[5]);
      n_pr += static_cast<int64_t>(w.prod_level_off.size() > 0 ? w.prod_level_off.size() - 1 : 0);
      if (traced) {
        t_tr += elapsed_ms(ev_[5], ev_[6]);
        ++n_tr;
      }
      if (mixed)
        for (size_t bi = 0; bi < wb.tc_batches.size(); ++bi) {
          t_sl += elapsed_ms(tc_ev_[3 * bi], tc_ev_[3 * bi + 1]);
          t_gm += elapsed_ms(tc_ev_[3 * bi + 1], tc_ev_[3 * bi + 2]);
          ++n_gm;
        }
    }
    if (mixed) {
      int const code = read_err_flag();
      if (code != 0)
        throw TimeoutError("tensor-core factors or traces: a bounded device wait gave up "
                           "(stage " + std::to_string(code) + ")");
    }
    st[6] += static_cast<double>(s.n_unique_entries);
    st[7] += static_cast<double>(s.n_group_entries);
    st[0] += static_cast<double>(s.q0.size() + s.q1.size() + s.q2.size());
    st[1] += static_cast<double>(s.n_prods);
    st[2] += static_cast<double>(s.n_trace_entries);
    st[3] += static_cast<double>(s.n_terms);
    st[4] += s.flops_factors;
    st[5] += s.flops_products + s.flops_traces;
  }
  // Perambulators and noise are not read after the factor stages.
  SLAPH_CK(cudaEventRecord(ev_pn_used_, stream_));
  timings[1] = t_f;
  timings[2] = t_pt;
  timings[3] = t_as;
  timings[4] = plan_wall * 1e3;
  timings[5] = static_cast<double>(launches_);
  timings[6] = t_tr;
  timings[7] = static_cast<double>(n_tr);
  timings[8] = t_gm;
  timings[9] = static_cast<double>(n_gm);
  timings[10] = t_sl;
  timings[14] = t_pr;
  timings[15] = static_cast<double>(n_pr);

  // ---- output: C[t] = correlator[t][i] / Lt (src/Diagram.cpp:141-143)
  size_t const n_host = static_cast<size_t>(n_outputs * dims_.Lt);
  host_rb_.reserve(std::max<size_t>(1, n_host) * sizeof(double2));
  double2 const *host = host_rb_.as<double2>();
  if (n_host > 0)
    SLAPH_CK(cudaMemcpyAsync(host_rb_.as<double2>(), running_.as<double2>(),
                             n_host * sizeof(double2), cudaMemcpyDeviceToHost, stream_));
  SLAPH_CK(cudaStreamSynchronize(stream_));
  double const inv = static_cast<double>(dims_.Lt);
  for (size_t i = 0; i < n_host; ++i) {
    corr_out[2 * i] = host[i].x / inv;
    corr_out[2 * i + 1] = host[i].y / inv;
  }
  for (int k = 0; k < 8; ++k) stats[k] = st[k];
}

}  // namespace slaph
