// Self-check of the bounded device waits.
//
// Every wait of the persistent solvers (the team barrier GroupTeam::sync and
// the reductions built on it) gives up after kBarrierSpinLimit polls, sets the
// team's error flag and makes the solve return VFVM_ERR_TIMEOUT, the code the
// host maps to the reference's exception path (src/vfvm_logging_exceptions.jl:6-29).
// This entry point runs that same barrier in a team told to expect one CTA
// more than the launch has, so the barrier's generation word is never
// advanced and every CTA's wait must run out: the host gets VFVM_ERR_TIMEOUT
// back and the CUDA context stays usable.  Nothing traps or faults.
#include "vfvm_team.cuh"

namespace vfvm {

__global__ void waitcheck_kernel(GridSync gs, int nblk_claimed, int* status) {
  GroupTeam team{gs, nblk_claimed, (int)blockIdx.x, 0u};
  const bool ok = team.sync();
  if (threadIdx.x == 0 && !ok) atomicExch(status, VFVM_ERR_TIMEOUT);
}

}  // namespace vfvm

using namespace vfvm;

extern "C" int vfvm_check_bounded_wait(int32_t ctas, int32_t* wait_status, float* ms) {
  if (ctas < 1 || ctas > 1024 || !wait_status) return VFVM_ERR_INPUT;
  unsigned* bar = nullptr;
  int* st = nullptr;
  VFVM_CUDA(cudaMalloc(&bar, 4 * sizeof(unsigned) + sizeof(int)));
  st = reinterpret_cast<int*>(bar + 4);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = VFVM_OK;
  do {
    if (cudaMemset(bar, 0, 4 * sizeof(unsigned) + sizeof(int)) != cudaSuccess) { rc = VFVM_ERR_CUDA; break; }
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) { rc = VFVM_ERR_CUDA; break; }
    // the barrier needs no partials; the team claims one CTA more than launched
    GridSync gs{bar, nullptr};
    cudaEventRecord(e0, 0);
    waitcheck_kernel<<<ctas, 64>>>(gs, ctas + 1, st);
    cudaEventRecord(e1, 0);
    if (cudaGetLastError() != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) { rc = VFVM_ERR_CUDA; break; }
    int h = 0;
    if (cudaMemcpy(&h, st, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) { rc = VFVM_ERR_CUDA; break; }
    *wait_status = h;
    if (ms) cudaEventElapsedTime(ms, e0, e1);
  } while (0);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(bar);
  return rc;
}
