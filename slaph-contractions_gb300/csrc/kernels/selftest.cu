// Self-test of the bounded waits of the tensor-core pipelines: one thread
// waits on a shared-memory mbarrier that nothing completes, with a limit of
// `cycles` clock cycles; the wait gives up, records code 1 in *err and the
// kernel exits, as the GEMM pipelines do when a copy or an MMA never lands.
#include <cuda_runtime.h>

#include <cstdint>

#include "kernels.cuh"
#include "tc_common.cuh"

namespace slaph {
namespace dev {
namespace {

__global__ void bounded_wait_kernel(int *err, long long cycles) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar, 1);  // one arrival expected, none comes
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    if (tc::mbar_wait_for(&bar, 0, err, 1, cycles)) atomicExch(err, -1);  // completed: wrong
  }
}

}  // namespace

cudaError_t bounded_wait_selftest(int *err, long long cycles, cudaStream_t stream) {
  if (cycles < 0) return cudaErrorInvalidValue;
  bounded_wait_kernel<<<1, 32, 0, stream>>>(err, cycles);
  return cudaGetLastError();
}

}  // namespace dev
}  // namespace slaph
