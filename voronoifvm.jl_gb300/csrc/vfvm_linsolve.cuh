// Shared pieces of the CSR linear-solve entry points.
#pragma once
#include "vfvm_common.cuh"

namespace vfvm {

constexpr int kLinThreads = 512;

inline size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// bytes of device scratch one solve of n rows needs with `grid` blocks
size_t linsolve_scratch_bytes(int64_t n, int grid);
// cooperative grid size for n rows on the current device (0 on error)
int linsolve_grid(int n);
// runs the solve with the given scratch (no allocation)
int linsolve_run(int32_t n, int64_t nnz, const int32_t* rowptr, const int32_t* colind, const double* vals,
                 const double* b, double* x, double reltol, double abstol, int32_t maxiters, int32_t* iters,
                 double* resnorm, char* scratch, int grid, cudaStream_t stream);

}  // namespace vfvm
