// Parameter derivatives of the residual: the reference's dudp, accumulated by
// the asm_param closures of the assembly loops (src/vfvm_assembly.jl:116-120
// node terms, :194-198 edges, :232-236 edge reactions, :296-304 outflow, :403-405 breaction,
// :434-436 bstorage, assemble_bedges :497-501), for physics whose first NPD
// parameters carry derivatives (the reference's nparams, parameters(u)).
//
// dudp[k][K] = sum over node items fac * d(reaction + storage * tstepinv)/dp_k
//            + sum over edges +- fac * d flux / dp_k (first node +, second -)
//            + sum over edges fac * d edgereaction / dp_k (both nodes)
//            + sum over boundary items fac * d(breaction + bstorage * tstepinv)/dp_k
//            + sum over boundary edges +- fac * d bflux / dp_k
// (source and bsource carry no parameter derivative there, nor the old
// storage).  The physics is rebound to dual-number parameters of width one,
// parameter k seeded; the unknowns enter as constants.  One thread per node,
// the node-centric gather of the assembly, species masks as there.
#include "vfvm_assembly.cuh"

namespace vfvm {

template <class PhD, bool MR>
__global__ void __launch_bounds__(128) dparams_kernel(const AsmTables t, const double* __restrict__ U,
                                                      const double* __restrict__ tv, int k, double* __restrict__ out) {
  constexpr int NS = PhD::NS;
  using D = Dual<1, double>;
  const int K = blockIdx.x * blockDim.x + threadIdx.x;
  if (K >= t.N) return;
  PhD ph;
  ph.load(t.params);
  ph.seed(k);
  const double time = tv[0], tstepinv = tv[1], lambda = tv[2];
  const double* xK = t.coord + (size_t)K * t.dim;
  const double* dK = t.nodedata ? t.nodedata + (size_t)K * t.nnd : nullptr;
  D uK[NS], y[NS], s[NS];
#pragma unroll
  for (int i = 0; i < NS; ++i) uK[i] = dconst<1, double>(U[(size_t)K * NS + i]);
  double acc[NS];
#pragma unroll
  for (int i = 0; i < NS; ++i) acc[i] = 0.0;
  // node items
  const int nbeg = MR ? t.nitem_ptr[K] : 0, nend = MR ? t.nitem_ptr[K + 1] : 1;
  for (int it = nbeg; it < nend; ++it) {
    const int reg = MR ? t.nitem_reg[it] : t.region;
    const double fac = MR ? t.nitem_fac[it] : t.node_fac[K];
    const unsigned m = (MR && t.reg_spec) ? t.reg_spec[reg - 1] : ~0u;
    NodeItem ni{K, reg, xK, time, lambda, dK};
#pragma unroll
    for (int i = 0; i < NS; ++i) { y[i] = dconst<1, double>(0.0); s[i] = dconst<1, double>(0.0); }
    if (PhD::has_reaction) ph.reaction(y, uK, ni);
    if (PhD::has_storage) ph.storage(s, uK, ni);
#pragma unroll
    for (int i = 0; i < NS; ++i)
      if ((m >> i) & 1u) acc[i] += (y[i].d[0] + s[i].d[0] * tstepinv) * fac;
  }
  // edges incident to K, in column order
  for (int sl = t.browptr[K]; sl < t.browptr[K + 1]; ++sl) {
    const int M = t.bcol[sl];
    if (M == K) continue;
    const bool kfirst = K < M;
    const int A = kfirst ? K : M, B = kfirst ? M : K;
    D uA[NS], uB[NS];
#pragma unroll
    for (int i = 0; i < NS; ++i) {
      uA[i] = dconst<1, double>(U[(size_t)A * NS + i]);
      uB[i] = dconst<1, double>(U[(size_t)B * NS + i]);
    }
    const int ebeg = MR ? t.sitem_ptr[sl] : 0, eend = MR ? t.sitem_ptr[sl + 1] : 1;
    for (int it = ebeg; it < eend; ++it) {
      const int reg = MR ? t.sitem_reg[it] : t.region;
      const double fac = MR ? t.sitem_fac[it] : t.slot_fac[sl];
      const unsigned m = (MR && t.reg_spec) ? t.reg_spec[reg - 1] : ~0u;
      EdgeItem ei{A, B, reg, t.coord + (size_t)A * t.dim, t.coord + (size_t)B * t.dim, time, lambda,
                  t.nodedata ? t.nodedata + (size_t)A * t.nnd : nullptr,
                  t.nodedata ? t.nodedata + (size_t)B * t.nnd : nullptr};
#pragma unroll
      for (int i = 0; i < NS; ++i) y[i] = dconst<1, double>(0.0);
      ph.flux(y, uA, uB, ei);
#pragma unroll
      for (int i = 0; i < NS; ++i)
        if ((m >> i) & 1u) acc[i] += kfirst ? fac * y[i].d[0] : -(fac * y[i].d[0]);
      if constexpr (PhD::has_boutflow) {  // outflowasm_param, src/vfvm_assembly.jl:296-304 (+ for both nodes)
        const bool oA = t.outflow_node && t.outflow_node[A], oB = t.outflow_node && t.outflow_node[B];
        if (kfirst ? oA : oB) {
          ei.outflownode = oB ? 2 : 1;
#pragma unroll
          for (int i = 0; i < NS; ++i) y[i] = dconst<1, double>(0.0);
          ph.boutflow(y, uA, uB, ei);
          ei.outflownode = 0;
#pragma unroll
          for (int i = 0; i < NS; ++i)
            if ((m >> i) & 1u) acc[i] += fac * y[i].d[0];
        }
      }
      if constexpr (PhD::has_edgereaction) {
#pragma unroll
        for (int i = 0; i < NS; ++i) y[i] = dconst<1, double>(0.0);
        ph.edgereaction(y, uA, uB, ei);
#pragma unroll
        for (int i = 0; i < NS; ++i)
          if ((m >> i) & 1u) acc[i] += fac * y[i].d[0];
      }
    }
    if constexpr (PhD::has_bflux) {
      if (t.sbe_ptr) {
        const unsigned m = t.node_spec ? t.node_spec[A] : ~0u;
        for (int it = t.sbe_ptr[sl]; it < t.sbe_ptr[sl + 1]; ++it) {
          const double fac = t.sbe_fac[it];
          BEdgeItem be{A, B, t.sbe_reg[it], t.coord + (size_t)A * t.dim, t.coord + (size_t)B * t.dim, time, lambda};
#pragma unroll
          for (int i = 0; i < NS; ++i) y[i] = dconst<1, double>(0.0);
          ph.bflux(y, uA, uB, be);
#pragma unroll
          for (int i = 0; i < NS; ++i)
            if ((m >> i) & 1u) acc[i] += kfirst ? fac * y[i].d[0] : -(fac * y[i].d[0]);
        }
      }
    }
  }
  // boundary items
  const unsigned nm = t.node_spec ? t.node_spec[K] : ~0u;
  for (int it = t.bn_ptr[K]; it < t.bn_ptr[K + 1]; ++it) {
    const int reg = t.bn_reg[it];
    const double fac = t.bn_fac[it];
    const double Dir = (t.has_legacy && reg - 1 < t.nbregions) ? kDirichlet / fac : kDirichlet;
    BNodeItem bi{K, reg, xK, time, lambda, fac, Dir, nullptr};
#pragma unroll
    for (int i = 0; i < NS; ++i) { y[i] = dconst<1, double>(0.0); s[i] = dconst<1, double>(0.0); }
    if (PhD::has_breaction) ph.breaction(y, uK, bi);
    if (PhD::has_bstorage) ph.bstorage(s, uK, bi);
#pragma unroll
    for (int i = 0; i < NS; ++i)
      if ((nm >> i) & 1u) acc[i] += y[i].d[0] * fac + s[i].d[0] * fac * tstepinv;
  }
#pragma unroll
  for (int i = 0; i < NS; ++i) out[(size_t)K * NS + i] = acc[i];
}

}  // namespace vfvm

using namespace vfvm;

extern "C" int vfvm_parameter_derivatives(vfvm_ctx* c, const double* U, double time, double tstep, double lambda,
                                          double* dudp, int32_t* npd) {
  if (!c || !U || !npd) return VFVM_ERR_INPUT;
  const size_t n = (size_t)c->N * c->ns;
  int np = dispatch_physics(c->phys, [](auto ph) { return decltype(ph)::NPD; });
  if (np < 0) return VFVM_ERR_INPUT;
  *npd = np;
  if (np == 0 || !dudp) return VFVM_OK;
  DBuf<double> dU, dT, dO;
  VFVM_CUDA(dU.alloc(n));
  VFVM_CUDA(dT.alloc(3));
  VFVM_CUDA(dO.alloc((size_t)np * n));
  const double tv[3] = {time, 1.0 / tstep, lambda};
  VFVM_CUDA(cudaMemcpyAsync(dU.p, U, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  VFVM_CUDA(cudaMemcpyAsync(dT.p, tv, sizeof(tv), cudaMemcpyHostToDevice, c->stream));
  const AsmTables t = c->tables();
  const int threads = 128, blocks = (c->N + threads - 1) / threads;
  int rc = dispatch_physics(c->phys, [&](auto ph) {
    using Ph = decltype(ph);
    if constexpr (Ph::NPD > 0) {
      using PhD = typename Ph::template rebind<Dual<1, double>>;
      for (int k = 0; k < Ph::NPD; ++k) {
        if (c->multireg)
          dparams_kernel<PhD, true><<<blocks, threads, 0, c->stream>>>(t, dU.p, dT.p, k, dO.p + (size_t)k * n);
        else
          dparams_kernel<PhD, false><<<blocks, threads, 0, c->stream>>>(t, dU.p, dT.p, k, dO.p + (size_t)k * n);
      }
      return cudaGetLastError() == cudaSuccess ? VFVM_OK : VFVM_ERR_CUDA;
    }
    return VFVM_OK;
  });
  if (rc) return rc;
  VFVM_CUDA(cudaMemcpyAsync(dudp, dO.p, (size_t)np * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  VFVM_CUDA(cudaStreamSynchronize(c->stream));
  return VFVM_OK;
}
