// Residual + Jacobian assembly kernels (the reference's eval_and_assemble,
// src/vfvm_assembly.jl:520-643, with assemble_nodes :38-126, assemble_edges
// :128-200 and assemble_bnodes :318-407).
//
// Layout: node-centric gather.  One thread owns one node K: it evaluates the
// node physics, then every edge incident to K (walking K's block row of the
// Jacobian, whose columns are sorted by node index -- which is also the edge
// numbering order, so F[K] is summed in the reference's order), then K's
// boundary-face items.  It writes F[K], its off-diagonal Jacobian blocks (each
// contributed by exactly one edge) and its diagonal block.  No atomics, no
// colouring, one writer per output element, deterministic.
#include "vfvm_assembly.cuh"

namespace vfvm {

template <class Ph, typename P, bool MR>
__global__ void __launch_bounds__(128) assemble_kernel(const AsmTables t, const double* __restrict__ U,
                                                       const double* __restrict__ Uold, const double* __restrict__ tv,
                                                       double* __restrict__ F, P* __restrict__ J,
                                                       int* __restrict__ err) {
  const int K = blockIdx.x * blockDim.x + threadIdx.x;
  if (K >= t.N) return;
  Ph ph;
  ph.load(t.params);
  if (assemble_node<Ph, P, MR>(t, ph, K, U, Uold, tv[0], tv[1], tv[2], F, J)) atomicOr(err, 1);
}

// _initialize_dirichlet! (src/vfvm_system.jl:947-1003): per node, its boundary
// items in bface order; the last Dirichlet value set wins, as in the reference.
template <class Ph>
__global__ void init_dirichlet_kernel(const AsmTables t, double* __restrict__ U, const double* __restrict__ tv) {
  const int K = blockIdx.x * blockDim.x + threadIdx.x;
  if (K >= t.N) return;
  Ph ph;
  ph.load(t.params);
  init_dirichlet_node<Ph>(t, ph, K, U, tv[0], tv[2]);
}

__global__ void gather_kernel(const double* __restrict__ J, const int64_t* __restrict__ pmap, double* __restrict__ out, int64_t n) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k < n) out[k] = J[pmap[k]];
}

int launch_assemble(vfvm_ctx* c, const double* U, const double* Uold, const double* tv, double* F, double* J,
                    float* Jf, cudaStream_t s) {
  const AsmTables t = c->tables();
  const int threads = 128;
  const int blocks = (c->N + threads - 1) / threads;
  return dispatch_physics(c->phys, [&](auto ph) {
    using Ph = decltype(ph);
    if (Jf) {
      if (c->multireg)
        assemble_kernel<Ph, float, true><<<blocks, threads, 0, s>>>(t, U, Uold, tv, F, Jf, c->errflag.p);
      else
        assemble_kernel<Ph, float, false><<<blocks, threads, 0, s>>>(t, U, Uold, tv, F, Jf, c->errflag.p);
    } else {
      if (c->multireg)
        assemble_kernel<Ph, double, true><<<blocks, threads, 0, s>>>(t, U, Uold, tv, F, J, c->errflag.p);
      else
        assemble_kernel<Ph, double, false><<<blocks, threads, 0, s>>>(t, U, Uold, tv, F, J, c->errflag.p);
    }
    return cudaGetLastError() == cudaSuccess ? VFVM_OK : VFVM_ERR_CUDA;
  });
}

int launch_init_dirichlet(vfvm_ctx* c, double* U, const double* tv, cudaStream_t s) {
  const AsmTables t = c->tables();
  const int threads = 128;
  const int blocks = (c->N + threads - 1) / threads;
  return dispatch_physics(c->phys, [&](auto ph) {
    init_dirichlet_kernel<decltype(ph)><<<blocks, threads, 0, s>>>(t, U, tv);
    return cudaGetLastError() == cudaSuccess ? VFVM_OK : VFVM_ERR_CUDA;
  });
}

int launch_pattern_gather(vfvm_ctx* c, const double* J, double* out, cudaStream_t s) {
  if (c->nnz == 0) return VFVM_OK;
  const int threads = 256;
  const int64_t blocks = (c->nnz + threads - 1) / threads;
  gather_kernel<<<(unsigned)blocks, threads, 0, s>>>(J, c->pmap.p, out, c->nnz);
  return cudaGetLastError() == cudaSuccess ? VFVM_OK : VFVM_ERR_CUDA;
}

}  // namespace vfvm
