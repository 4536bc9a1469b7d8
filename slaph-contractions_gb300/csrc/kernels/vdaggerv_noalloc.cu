// slaph_vdaggerv_noalloc: VdaggerV of one operator on one timeslice without
// any device allocation.
//
// The engine's VdaggerV path keeps its momentum-phase table in engine-owned
// device memory.  Some callers cannot let a library allocate: hosts whose own
// allocator has reserved the device memory up front (a cudaMalloc here would
// fail or fight their pool), and latency-critical loops that cannot afford
// the device synchronisation cudaMalloc/cudaFree may imply.  This variant runs
// the same two kernels (phases, then V^H diag(phase) V) with all scratch in
// the file-scope array below, which every GPU that loads the library holds
// until the process exits.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <mutex>

#include "../host/capi_util.hpp"
#include "kernels.cuh"

namespace {

void check(cudaError_t e, char const *what) {
  if (e != cudaSuccess) throw slaph::CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}

// Scratch layout: [0, 256) launch metadata (operator list, momentum),
// [256, 256 + 16 * L^3) the phase table of one momentum.
constexpr size_t kMetaBytes = 256;
constexpr size_t kMaxVolume = 262144;  // L^3 up to 64^3
constexpr size_t kScratchBytes = kMetaBytes + kMaxVolume * sizeof(double2);

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
void *g_scratch_ptr[kMaxDevices] = {};

// Device address of g_scratch on the current device, looked up once per
// device (host code cannot use the symbol itself as a device address).
void *scratch_for_current_device() {
  int dev = -1;
  check(cudaGetDevice(&dev), "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) throw slaph::UnsupportedError("device index above 63");
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    check(cudaGetSymbolAddress(&p, g_scratch), "cudaGetSymbolAddress");
    if (!p) throw slaph::CudaError("cudaGetSymbolAddress returned a null address");
    g_scratch_ptr[dev] = p;
  }
  return g_scratch_ptr[dev];
}

// Writes the launch metadata into the scratch from kernel arguments, so that
// no host memory is read by the GPU: meta[0] = operator index 0 (the output
// block), meta[1..3] = momentum.
__global__ void noalloc_meta_kernel(int32_t *meta, int32_t px, int32_t py, int32_t pz) {
  if (threadIdx.x == 0) {
    meta[0] = 0;
    meta[1] = px;
    meta[2] = py;
    meta[3] = pz;
  }
}

}  // namespace

extern "C" int slaph_vdaggerv_noalloc(const slaph_dims *dims, const double *V_t,
                                      const int32_t *momentum, double *out, void *stream) {
  return slaph::guarded([&] {
    if (!dims || !V_t || !momentum || !out) throw slaph::ArgError("null argument");
    if (dims->Lx < 1 || dims->Ly < 1 || dims->Lz < 1 || dims->nev < 1)
      throw slaph::ArgError("invalid lattice or eigenvector count");
    // Each extent is bounded before the product is formed, so the product
    // (at most 2^54) cannot wrap.
    if (static_cast<size_t>(dims->Lx) > kMaxVolume || static_cast<size_t>(dims->Ly) > kMaxVolume ||
        static_cast<size_t>(dims->Lz) > kMaxVolume)
      throw slaph::ArgError("slaph_vdaggerv_noalloc: a lattice extent exceeds the static "
                            "scratch limit of " + std::to_string(kMaxVolume) + " sites (64^3)");
    size_t const vol = static_cast<size_t>(dims->Lx) * dims->Ly * dims->Lz;
    if (vol > kMaxVolume)
      throw slaph::ArgError("slaph_vdaggerv_noalloc: L^3 = " + std::to_string(vol) +
                            " exceeds the static scratch limit of " +
                            std::to_string(kMaxVolume) + " sites (64^3)");
    auto *base = static_cast<unsigned char *>(scratch_for_current_device());
    auto *meta = reinterpret_cast<int32_t *>(base);
    auto *phase = reinterpret_cast<double2 *>(base + kMetaBytes);
    cudaStream_t const s = static_cast<cudaStream_t>(stream);

    noalloc_meta_kernel<<<1, 32, 0, s>>>(meta, momentum[0], momentum[1], momentum[2]);
    check(cudaGetLastError(), "metadata kernel");
    slaph::dev::Geometry g{};
    g.Lt = 1;
    g.Lx = dims->Lx;
    g.Ly = dims->Ly;
    g.Lz = dims->Lz;
    g.nev = dims->nev;
    g.dilE = dims->dilE > 0 ? dims->dilE : 1;
    g.n_rnd = 1;
    g.nb = 1;
    g.dim_row = 3LL * static_cast<int64_t>(vol);
    check(slaph::dev::momenta(phase, meta + 1, 1, g, s), "momenta kernel");
    check(
        slaph::dev::vdaggerv_fp64(reinterpret_cast<double2 *>(out),
                                  reinterpret_cast<double2 const *>(V_t), phase, meta, 1, 0, 1,
                                  g, s),
        "vdaggerv kernel");
  });
}
