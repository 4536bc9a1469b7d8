// C ABI of the engine (include/slaph_gb300.h).
#include <memory>
#include <string>

#include "capi_util.hpp"
#include "engine.hpp"

struct slaph_engine {
  std::unique_ptr<slaph::Engine> e;
};

namespace {
slaph::Engine &get(slaph_engine *eng) {
  if (!eng || !eng->e) throw slaph::ArgError("null engine");
  return *eng->e;
}
}  // namespace

extern "C" {

int slaph_engine_create(const slaph_dims *dims, slaph_engine **out) {
  return slaph::guarded([&] {
    if (!dims || !out) throw slaph::ArgError("null argument");
    *out = nullptr;
    auto eng = std::make_unique<slaph_engine>();
    eng->e = std::make_unique<slaph::Engine>(*dims);
    *out = eng.release();
  });
}

int slaph_engine_destroy(slaph_engine *eng) {
  delete eng;
  return SLAPH_OK;
}

int slaph_engine_set_operators(slaph_engine *eng, const slaph_vdv_op *ops, int32_t n_ops,
                               int32_t index_of_unity) {
  return slaph::guarded([&] { get(eng).set_operators(ops, n_ops, index_of_unity); });
}

int slaph_engine_set_eigenvectors(slaph_engine *eng, int32_t t, const double *V) {
  return slaph::guarded([&] { get(eng).set_eigenvectors(t, V); });
}

int slaph_engine_set_perambulator(slaph_engine *eng, int32_t rnd_id, const double *peram) {
  return slaph::guarded([&] { get(eng).set_perambulator(rnd_id, peram); });
}

int slaph_engine_set_random_vector(slaph_engine *eng, int32_t rnd_id, const double *noise) {
  return slaph::guarded([&] { get(eng).set_random_vector(rnd_id, noise); });
}

int slaph_engine_set_eigenvectors_async(slaph_engine *eng, int32_t t, const double *V) {
  return slaph::guarded([&] { get(eng).set_eigenvectors(t, V, true); });
}

int slaph_engine_set_perambulator_async(slaph_engine *eng, int32_t rnd_id, const double *peram) {
  return slaph::guarded([&] { get(eng).set_perambulator(rnd_id, peram, true); });
}

int slaph_engine_set_random_vector_async(slaph_engine *eng, int32_t rnd_id,
                                         const double *noise) {
  return slaph::guarded([&] { get(eng).set_random_vector(rnd_id, noise, true); });
}

int slaph_engine_set_eigenvector_slots(slaph_engine *eng, int32_t n_slots) {
  return slaph::guarded([&] { get(eng).set_eigenvector_slots(n_slots); });
}

int slaph_engine_set_factor_lifetime(slaph_engine *eng, int mode) {
  return slaph::guarded([&] { get(eng).set_factor_lifetime(mode); });
}

int slaph_engine_set_time_dilution(slaph_engine *eng, int32_t dilT) {
  return slaph::guarded([&] { get(eng).set_time_dilution(dilT); });
}

int slaph_engine_set_gauge(slaph_engine *eng, int32_t t, const double *U) {
  return slaph::guarded([&] { get(eng).set_gauge(t, U); });
}

int slaph_engine_smear_gauge_hyp(slaph_engine *eng, double alpha1, double alpha2,
                                 int32_t iterations) {
  return slaph::guarded([&] { get(eng).smear_gauge_hyp(alpha1, alpha2, iterations); });
}

int slaph_engine_gauge_fetch(slaph_engine *eng, int32_t t, double *out) {
  return slaph::guarded([&] { get(eng).gauge_fetch(t, out); });
}

int slaph_selftest_bounded_wait(int64_t cycles, int32_t *device_code) {
  return slaph::guarded([&] {
    if (!device_code || cycles < 0) throw slaph::ArgError("invalid argument");
    int *err = nullptr;
    slaph::cuda_check(cudaMalloc(&err, sizeof(int)), "cudaMalloc");
    int code = 0;
    cudaError_t e = cudaMemset(err, 0, sizeof(int));
    if (e == cudaSuccess) e = slaph::dev::bounded_wait_selftest(err, cycles, nullptr);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(&code, err, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(err);
    slaph::cuda_check(e, "bounded wait self-test");
    *device_code = code;
    if (code != 1)
      throw slaph::CudaError("bounded wait self-test: the device wait did not give up as designed");
  });
}

int slaph_host_alloc(size_t bytes, void **out) {
  return slaph::guarded([&] {
    if (!out || bytes == 0) throw slaph::ArgError("null output or empty size");
    *out = nullptr;
    cudaError_t const e = cudaHostAlloc(out, bytes, cudaHostAllocPortable);
    if (e != cudaSuccess) {
      *out = nullptr;
      (void)cudaGetLastError();
      throw slaph::NoMemError(std::string("cudaHostAlloc of ") + std::to_string(bytes) +
                              " bytes failed: " + cudaGetErrorString(e));
    }
  });
}

int slaph_host_free(void *ptr) {
  return slaph::guarded([&] {
    if (!ptr) throw slaph::ArgError("null host buffer");
    slaph::cuda_check(cudaFreeHost(ptr), "cudaFreeHost");
  });
}

int slaph_host_register(void *ptr, size_t bytes) {
  return slaph::guarded([&] {
    if (!ptr || bytes == 0) throw slaph::ArgError("null or empty host buffer");
    slaph::cuda_check(cudaHostRegister(ptr, bytes, cudaHostRegisterDefault), "cudaHostRegister");
  });
}

int slaph_host_unregister(void *ptr) {
  return slaph::guarded([&] {
    if (!ptr) throw slaph::ArgError("null host buffer");
    slaph::cuda_check(cudaHostUnregister(ptr), "cudaHostUnregister");
  });
}

int slaph_vdaggerv_build(slaph_engine *eng, int precision) {
  return slaph::guarded([&] { get(eng).vdaggerv_build(precision); });
}

int slaph_vdaggerv_fetch(slaph_engine *eng, int32_t op_id, int32_t t, double *out) {
  return slaph::guarded([&] { get(eng).vdaggerv_fetch(op_id, t, out); });
}

int slaph_vdaggerv_write(slaph_engine *eng, const char *path_vdaggerv, int32_t config) {
  return slaph::guarded([&] { get(eng).vdaggerv_write(path_vdaggerv, config); });
}

int slaph_vdaggerv_read(slaph_engine *eng, const char *path_vdaggerv, int32_t config,
                        int32_t liuming) {
  return slaph::guarded([&] { get(eng).vdaggerv_read(path_vdaggerv, config, liuming); });
}

int slaph_contract(slaph_engine *eng, const slaph_plan *plan, int precision, int accumulator,
                   int single_block_pair, double *corr_out) {
  return slaph::guarded(
      [&] { get(eng).contract(plan, precision, accumulator, single_block_pair, corr_out); });
}

int slaph_engine_timings(const slaph_engine *eng, double *out, int n) {
  if (!eng || !eng->e || !out || n < 0) {
    slaph::set_last_error("invalid argument");
    return -1;
  }
  int const m = n < 16 ? n : 16;
  for (int i = 0; i < m; ++i) out[i] = eng->e->timings[i];
  return m;
}

int slaph_engine_stats(const slaph_engine *eng, double *out, int n) {
  if (!eng || !eng->e || !out || n < 0) {
    slaph::set_last_error("invalid argument");
    return -1;
  }
  int const m = n < 8 ? n : 8;
  for (int i = 0; i < m; ++i) out[i] = eng->e->stats[i];
  return m;
}

}  // extern "C"
