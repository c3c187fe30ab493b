// The mass matrix of the ODE/DAE form of a system (the reference's
// mass_matrix, src/vfvm_diffeq_interface.jl:60-112): the Jacobian of the
// storage terms at U = 0, node items with their factors (storage) and boundary
// items with theirs (bstorage), in the rows and columns of the species of the
// item's region or node.  Together with the residual at tstep = Inf
// (vfvm_assemble) it gives the ODE right hand side -F and its Jacobian -J.
#include "vfvm_assembly.cuh"

namespace vfvm {

template <class Ph, bool MR>
__global__ void __launch_bounds__(128) mass_kernel(const AsmTables t, double* __restrict__ J) {
  constexpr int NS = Ph::NS;
  const int K = blockIdx.x * blockDim.x + threadIdx.x;
  if (K >= t.N) return;
  Ph ph;
  ph.load(t.params);
  double jd[NS * NS];
#pragma unroll
  for (int k = 0; k < NS * NS; ++k) jd[k] = 0.0;
  const double* xK = t.coord + (size_t)K * t.dim;
  const double* dK = t.nodedata ? t.nodedata + (size_t)K * t.nnd : nullptr;
  Dual<NS, double> u[NS], s[NS];
#pragma unroll
  for (int i = 0; i < NS; ++i) u[i] = dseed<NS, double>(0.0, i);
  if (Ph::has_storage) {
    const int nbeg = MR ? t.nitem_ptr[K] : 0, nend = MR ? t.nitem_ptr[K + 1] : 1;
    for (int it = nbeg; it < nend; ++it) {
      const int reg = MR ? t.nitem_reg[it] : t.region;
      const double fac = MR ? t.nitem_fac[it] : t.node_fac[K];
      const unsigned m = (MR && t.reg_spec) ? t.reg_spec[reg - 1] : ~0u;
      NodeItem ni{K, reg, xK, 0.0, 0.0, dK};
#pragma unroll
      for (int i = 0; i < NS; ++i) s[i] = dconst<NS, double>(0.0);
      ph.storage(s, u, ni);
#pragma unroll
      for (int i = 0; i < NS; ++i)
#pragma unroll
        for (int j = 0; j < NS; ++j)
          if (((m >> i) & 1u) && ((m >> j) & 1u)) jd[i * NS + j] += s[i].d[j] * fac;
    }
  }
  if (Ph::has_bstorage) {
    const unsigned m = t.node_spec ? t.node_spec[K] : ~0u;
    for (int it = t.bn_ptr[K]; it < t.bn_ptr[K + 1]; ++it) {
      const double fac = t.bn_fac[it];
      BNodeItem bi{K, t.bn_reg[it], xK, 0.0, 0.0, fac, kDirichlet, nullptr};
#pragma unroll
      for (int i = 0; i < NS; ++i) s[i] = dconst<NS, double>(0.0);
      ph.bstorage(s, u, bi);
#pragma unroll
      for (int i = 0; i < NS; ++i)
#pragma unroll
        for (int j = 0; j < NS; ++j)
          if (((m >> i) & 1u) && ((m >> j) & 1u)) jd[i * NS + j] += s[i].d[j] * fac;
    }
  }
  double* Jd = J + (size_t)t.diag[K] * NS * NS;
#pragma unroll
  for (int k = 0; k < NS * NS; ++k) Jd[k] = jd[k];
}

}  // namespace vfvm

using namespace vfvm;

extern "C" int vfvm_mass_matrix(vfvm_ctx* c, double* vals) {
  if (!c || !vals) return VFVM_ERR_INPUT;
  const size_t nb = (size_t)c->nnzb * c->ns * c->ns;
  DBuf<double> J, out;
  VFVM_CUDA(J.alloc(nb));
  VFVM_CUDA(cudaMemsetAsync(J.p, 0, nb * sizeof(double), c->stream));
  const AsmTables t = c->tables();
  const int threads = 128, blocks = (c->N + threads - 1) / threads;
  int rc = dispatch_physics(c->phys, [&](auto ph) {
    using Ph = decltype(ph);
    if (c->multireg) mass_kernel<Ph, true><<<blocks, threads, 0, c->stream>>>(t, J.p);
    else mass_kernel<Ph, false><<<blocks, threads, 0, c->stream>>>(t, J.p);
    return cudaGetLastError() == cudaSuccess ? VFVM_OK : VFVM_ERR_CUDA;
  });
  if (rc) return rc;
  if (c->nnz > 0) {
    VFVM_CUDA(out.alloc((size_t)c->nnz));
    if ((rc = launch_pattern_gather(c, J.p, out.p, c->stream))) return rc;
    VFVM_CUDA(cudaMemcpyAsync(vals, out.p, (size_t)c->nnz * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  }
  VFVM_CUDA(cudaStreamSynchronize(c->stream));
  return VFVM_OK;
}
