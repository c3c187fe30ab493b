// Allocation-free variant of vfvm_linsolve_csr.
//
// Some callers cannot call cudaMalloc at the point where they need a linear
// solve: code running under a framework that owns all device memory through its
// own pool (and forbids or cannot see outside allocations), callers inside a
// region where allocation would synchronise the device or break a running
// schedule, and embedded hosts that hand out only fixed, pre-reserved buffers.
// They pass their matrix, right hand side and solution buffers; the solver's
// work vectors come from the fixed array below instead of cudaMalloc.
//
// The work array is a file-scope __device__ array of a fixed size, so every GPU
// that loads this library holds it (about 7.7 MB) until the process exits, and
// it limits the system size to VFVM_NOALLOC_MAX_ROWS rows.  All calls share it:
// calls whose work overlaps on the GPU (other host threads, other streams)
// race on it and must be serialised by the caller.
#include <cstdio>
#include "vfvm_linsolve.cuh"

namespace vfvm {

constexpr int kNoallocMaxRows = VFVM_NOALLOC_MAX_ROWS;
constexpr int kNoallocMaxGrid = 1024;  // largest cooperative grid the scratch layout reserves room for

constexpr size_t a256(size_t b) { return (b + 255) & ~(size_t)255; }
constexpr size_t kNoallocBytes = a256(7 * (size_t)kNoallocMaxRows * sizeof(double)) +
                                 a256((size_t)kNoallocMaxRows * sizeof(int)) +
                                 a256((size_t)2 * kNoallocMaxGrid * 8 * sizeof(double)) + a256(8 * sizeof(unsigned)) +
                                 a256(sizeof(int)) + a256(64);

// The work memory.  In host code `g_noalloc_scratch` names a host-side shadow,
// not a device address; its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) char g_noalloc_scratch[kNoallocBytes];

namespace {
// Device address of the work array in the CUDA context current on this thread.
// It is looked up on every call rather than cached: a __device__ symbol's
// address belongs to the context that loaded the module, and the context of a
// device ordinal can change (cudaDeviceReset, a driver-API caller making its
// own context current).  The lookup allocates nothing; the first one in a
// context loads the module, which is why the first call should come before any
// stream capture.
int scratch_address(char** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) {
    fprintf(stderr, "vfvm_linsolve_csr_noalloc: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
    return VFVM_ERR_CUDA;
  }
  *out = static_cast<char*>(p);
  return VFVM_OK;
}
}  // namespace

}  // namespace vfvm

using namespace vfvm;

extern "C" int vfvm_linsolve_csr_noalloc(int32_t n, int64_t nnz, const int32_t* rowptr, const int32_t* colind,
                                         const double* vals, const double* b, double* x, double reltol, double abstol,
                                         int32_t maxiters, int32_t* iters, double* resnorm) {
  if (n > kNoallocMaxRows) {
    fprintf(stderr, "vfvm_linsolve_csr_noalloc: %d rows exceed the fixed work memory (at most %d rows)\n", (int)n,
            kNoallocMaxRows);
    return VFVM_ERR_NOALLOC_LIMIT;
  }
  if (n < 1 || nnz < n || !rowptr || !colind || !vals || !b || !x || maxiters < 0 || !(reltol >= 0) || !(abstol >= 0))
    return VFVM_ERR_INPUT;
  const int grid = linsolve_grid(n);
  if (grid < 1) return VFVM_ERR_CUDA;
  if (grid > kNoallocMaxGrid || linsolve_scratch_bytes(n, grid) > kNoallocBytes) return VFVM_ERR_NOALLOC_LIMIT;
  char* scratch = nullptr;
  const int rc = scratch_address(&scratch);
  if (rc != VFVM_OK) return rc;
  return linsolve_run(n, nnz, rowptr, colind, vals, b, x, reltol, abstol, maxiters, iters, resnorm, scratch, grid, 0);
}
