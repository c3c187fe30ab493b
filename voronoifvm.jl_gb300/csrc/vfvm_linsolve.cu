// Standalone device linear solve for a caller-assembled CSR matrix.
//
// This is the linear-solver plug point of the reference: _solve_linear!
// (src/vfvm_linsolve.jl:6-61) hands state.matrix and the residual to a
// LinearSolve algorithm chosen by control.method_linear
// (src/vfvm_solvercontrol.jl:106).  vfvm_linsolve_csr is such an algorithm on the
// device: left-Jacobi-preconditioned BiCGStab in one persistent cooperative launch.
#include <mutex>

#include "vfvm_krylov.cuh"
#include "vfvm_linsolve.cuh"

namespace vfvm {

constexpr int kMaxGridDevices = 64;

// Validates the CSR structure (row pointers inside [0, nnz], monotone, columns
// inside [0, n)) and records the diagonal slot of every row.  err bit 1: bad
// structure, bit 2: missing diagonal.
__global__ void csr_check_kernel(int n, int64_t nnz, const int32_t* __restrict__ rowptr,
                                 const int32_t* __restrict__ col, int* __restrict__ diag, int* __restrict__ err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t b = rowptr[i], e = rowptr[i + 1];
  if ((i == 0 && b != 0) || (i == n - 1 && e != nnz) || b < 0 || e < b || e > nnz) {
    atomicOr(err, 1);
    diag[i] = 0;
    return;
  }
  int dg = -1;
  for (int64_t s = b; s < e; ++s) {
    const int c = col[s];
    if (c < 0 || c >= n) atomicOr(err, 1);
    if (c == i) dg = (int)s;
  }
  if (dg < 0) { atomicOr(err, 2); dg = 0; }
  diag[i] = dg;
}

template <int LPR>
__global__ void __launch_bounds__(kLinThreads) linsolve_kernel(KrylovData<1, double> d, KrylovCtl c, GridSync gs,
                                                               KrylovOut* out, const int* err) {
  if (*err) return;  // invalid input: every block leaves before the first barrier
  GridTeam team = grid_team(gs);
  const bool ok = team_bicgstab_jacobi<GridTeam, 1, LPR, double>(team, d, c, out);
  if (!ok && blockIdx.x == 0 && threadIdx.x == 0) out->status = VFVM_ERR_TIMEOUT;
}

size_t linsolve_scratch_bytes(int64_t n, int grid) {
  // 7 vectors of doubles (r, r0, p, v, s, t, dinv), diag (int), partials, barrier words, output record
  return align256(7 * n * sizeof(double)) + align256(n * sizeof(int)) + align256((size_t)2 * grid * 8 * sizeof(double)) +
         align256(8 * sizeof(unsigned)) + align256(sizeof(int)) + align256(sizeof(KrylovOut));
}

int linsolve_grid(int n) {
  // grid size per device ordinal, computed once; guarded because both CSR entry
  // points are context-free and may be called from several host threads
  static std::mutex mu;
  static int cached[kMaxGridDevices] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return 0;
  int full = 0;
  {
    std::lock_guard<std::mutex> lock(mu);
    if (dev < kMaxGridDevices) full = cached[dev];
  }
  if (full == 0) {
    int sms = 0, per_sm = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, linsolve_kernel<8>, kLinThreads, 0) != cudaSuccess) return 0;
    full = sms * (per_sm < 2 ? per_sm : 2);
    if (full < 1) return 0;
    std::lock_guard<std::mutex> lock(mu);
    if (dev < kMaxGridDevices) cached[dev] = full;
  }
  const int need = (int)((n + kLinThreads - 1) / kLinThreads);
  return need < full ? (need > 0 ? need : 1) : full;
}

int linsolve_run(int32_t n, int64_t nnz, const int32_t* rowptr, const int32_t* colind, const double* vals,
                 const double* b, double* x, double reltol, double abstol, int32_t maxiters, int32_t* iters,
                 double* resnorm, char* scratch, int grid, cudaStream_t stream) {
  char* q = scratch;
  double* vec = reinterpret_cast<double*>(q);
  q += align256(7 * (size_t)n * sizeof(double));
  int* diag = reinterpret_cast<int*>(q);
  q += align256((size_t)n * sizeof(int));
  double* partials = reinterpret_cast<double*>(q);
  q += align256((size_t)2 * grid * 8 * sizeof(double));
  unsigned* bar = reinterpret_cast<unsigned*>(q);
  q += align256(8 * sizeof(unsigned));
  int* err = reinterpret_cast<int*>(q);
  q += align256(sizeof(int));
  KrylovOut* out = reinterpret_cast<KrylovOut*>(q);

  // state that must start at zero on every call
  VFVM_CUDA(cudaMemsetAsync(bar, 0, 8 * sizeof(unsigned), stream));
  VFVM_CUDA(cudaMemsetAsync(err, 0, sizeof(int), stream));
  VFVM_CUDA(cudaMemsetAsync(out, 0, sizeof(KrylovOut), stream));
  csr_check_kernel<<<(n + 255) / 256, 256, 0, stream>>>(n, nnz, rowptr, colind, diag, err);
  VFVM_CUDA(cudaGetLastError());

  KrylovData<1, double> d;
  d.N = n; d.rowptr = rowptr; d.col = colind; d.A = vals; d.diag = diag;
  d.dinv = vec + 6 * (size_t)n; d.b = b; d.x = x;
  d.r = vec; d.r0 = vec + n; d.p = vec + 2 * (size_t)n; d.v = vec + 3 * (size_t)n; d.s = vec + 4 * (size_t)n;
  d.t = vec + 5 * (size_t)n;
  KrylovCtl c{reltol, abstol, maxiters};
  GridSync gs{bar, partials};
  void* args[] = {&d, &c, &gs, &out, &err};
  VFVM_CUDA(cudaLaunchCooperativeKernel((void*)linsolve_kernel<8>, dim3(grid), dim3(kLinThreads), args, 0, stream));
  KrylovOut h;
  int herr = 0;
  VFVM_CUDA(cudaMemcpyAsync(&h, out, sizeof(KrylovOut), cudaMemcpyDeviceToHost, stream));
  VFVM_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, stream));
  VFVM_CUDA(cudaStreamSynchronize(stream));
  if (herr) return VFVM_ERR_INPUT;
  if (iters) *iters = h.iters;
  if (resnorm) *resnorm = h.res;
  if (h.status) return h.status;
  if (h.breakdown && !(h.res <= fmax(abstol, reltol * h.res0))) return VFVM_ERR_LINEAR;
  return VFVM_OK;
}

}  // namespace vfvm

using namespace vfvm;

extern "C" int vfvm_linsolve_csr(int32_t n, int64_t nnz, const int32_t* rowptr, const int32_t* colind,
                                 const double* vals, const double* b, double* x, double reltol, double abstol,
                                 int32_t maxiters, int32_t* iters, double* resnorm) {
  if (n < 1 || nnz < n || !rowptr || !colind || !vals || !b || !x || maxiters < 0 || !(reltol >= 0) || !(abstol >= 0))
    return VFVM_ERR_INPUT;
  const int grid = linsolve_grid(n);
  if (grid < 1) return VFVM_ERR_CUDA;
  char* scratch = nullptr;
  VFVM_CUDA(cudaMalloc(&scratch, linsolve_scratch_bytes(n, grid)));
  const int rc = linsolve_run(n, nnz, rowptr, colind, vals, b, x, reltol, abstol, maxiters, iters, resnorm, scratch,
                              grid, 0);
  cudaFree(scratch);
  return rc;
}
