// Test-function integrals: the reference's integrate(system, T, U) and
// integrate(system, T, U, Uold, tstep) (src/vfvm_testfunctions.jl:125-380),
// the post-processing that turns solutions into boundary currents.
//
// Per species, over the node items (node, region, factor):
//   react  = sum fac * reaction(U_K) * T_K        (integrate_TxFunc)
//   src    = sum fac * source * T_K               (integrate_TxSrc)
//   stor   = sum fac * storage(U_K) * T_K, oldstor with Uold
// and over the edge items (edge, region, factor), first node K < second L:
//   flux   = sum fac * flux(U_K, U_L) * (T_K - T_L)        (integrate_∇TxFlux)
//   erea   = sum fac * edgereaction(U_K, U_L) * (T_K + T_L) (integrate_TxEdgefunc)
// One thread per node K: its node items and the edges to its higher-numbered
// neighbours, so every edge once.  The physics runs on dual numbers of width
// one (their values are the plain-double evaluation).  Each block writes its
// sums (a fixed-order tree in shared memory); the host adds the blocks in
// order, so the result is deterministic.
#include <vector>

#include "vfvm_assembly.cuh"

namespace vfvm {

constexpr int kTfThreads = 128;

template <class Ph, bool MR>
__global__ void __launch_bounds__(kTfThreads) tf_integrals_kernel(const AsmTables t, const double* __restrict__ T,
                                                                  const double* __restrict__ U,
                                                                  const double* __restrict__ Uold, double time,
                                                                  double lambda, double* __restrict__ partials) {
  constexpr int NS = Ph::NS, NV = 6 * NS;
  using D = Dual<1, double>;
  __shared__ double sh[NV][kTfThreads];
  Ph ph;
  ph.load(t.params);
  double acc[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) acc[k] = 0.0;
  const int K = blockIdx.x * blockDim.x + threadIdx.x;
  if (K < t.N) {
    const double* xK = t.coord + (size_t)K * t.dim;
    const double* dK = t.nodedata ? t.nodedata + (size_t)K * t.nnd : nullptr;
    D uK[NS], uoK[NS], y[NS];
#pragma unroll
    for (int i = 0; i < NS; ++i) {
      uK[i] = dconst<1, double>(U[(size_t)K * NS + i]);
      uoK[i] = dconst<1, double>(Uold[(size_t)K * NS + i]);
    }
    const double TK = T[K];
    const int nbeg = MR ? t.nitem_ptr[K] : 0, nend = MR ? t.nitem_ptr[K + 1] : 1;
    for (int it = nbeg; it < nend; ++it) {
      const int reg = MR ? t.nitem_reg[it] : t.region;
      const double fac = MR ? t.nitem_fac[it] : t.node_fac[K];
      NodeItem ni{K, reg, xK, time, lambda, dK};
      if (Ph::has_reaction) {
#pragma unroll
        for (int i = 0; i < NS; ++i) y[i] = dconst<1, double>(0.0);
        ph.reaction(y, uK, ni);
#pragma unroll
        for (int i = 0; i < NS; ++i) acc[1 * NS + i] += fac * y[i].v * TK;
      }
      if (Ph::has_source) {
        double src[NS];
#pragma unroll
        for (int i = 0; i < NS; ++i) src[i] = 0.0;
        ph.source(src, ni);
#pragma unroll
        for (int i = 0; i < NS; ++i) acc[2 * NS + i] += fac * src[i] * TK;
      }
      if (Ph::has_storage) {
#pragma unroll
        for (int i = 0; i < NS; ++i) y[i] = dconst<1, double>(0.0);
        ph.storage(y, uK, ni);
#pragma unroll
        for (int i = 0; i < NS; ++i) acc[3 * NS + i] += fac * y[i].v * TK;
#pragma unroll
        for (int i = 0; i < NS; ++i) y[i] = dconst<1, double>(0.0);
        ph.storage(y, uoK, ni);
#pragma unroll
        for (int i = 0; i < NS; ++i) acc[4 * NS + i] += fac * y[i].v * TK;
      }
    }
    for (int s = t.browptr[K]; s < t.browptr[K + 1]; ++s) {
      const int M = t.bcol[s];
      if (M <= K) continue;  // every edge once, from its first (lower) node
      D uM[NS];
#pragma unroll
      for (int i = 0; i < NS; ++i) uM[i] = dconst<1, double>(U[(size_t)M * NS + i]);
      const double TM = T[M];
      const double* xM = t.coord + (size_t)M * t.dim;
      const double* dM = t.nodedata ? t.nodedata + (size_t)M * t.nnd : nullptr;
      const int ebeg = MR ? t.sitem_ptr[s] : 0, eend = MR ? t.sitem_ptr[s + 1] : 1;
      for (int it = ebeg; it < eend; ++it) {
        const int reg = MR ? t.sitem_reg[it] : t.region;
        const double fac = MR ? t.sitem_fac[it] : t.slot_fac[s];
        EdgeItem ei{K, M, reg, xK, xM, time, lambda, dK, dM};
#pragma unroll
        for (int i = 0; i < NS; ++i) y[i] = dconst<1, double>(0.0);
        ph.flux(y, uK, uM, ei);
#pragma unroll
        for (int i = 0; i < NS; ++i) acc[0 * NS + i] += fac * y[i].v * (TK - TM);
        if constexpr (Ph::has_edgereaction) {
#pragma unroll
          for (int i = 0; i < NS; ++i) y[i] = dconst<1, double>(0.0);
          ph.edgereaction(y, uK, uM, ei);
#pragma unroll
          for (int i = 0; i < NS; ++i) acc[5 * NS + i] += fac * y[i].v * (TK + TM);
        }
      }
    }
  }
#pragma unroll
  for (int k = 0; k < NV; ++k) sh[k][threadIdx.x] = acc[k];
  __syncthreads();
  for (int h = kTfThreads / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h)
#pragma unroll
      for (int k = 0; k < NV; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) partials[(size_t)blockIdx.x * NV + k] = sh[k][0];
}

}  // namespace vfvm

using namespace vfvm;

extern "C" int vfvm_integrate(vfvm_ctx* c, const double* T, const double* U, const double* Uold, double time,
                              double lambda, double* out) {
  if (!c || !T || !U || !out) return VFVM_ERR_INPUT;
  const size_t n = (size_t)c->N * c->ns;
  const int blocks = (c->N + kTfThreads - 1) / kTfThreads;
  const int nv = 6 * c->ns;
  DBuf<double> dT, dU, dUo, dP;
  VFVM_CUDA(dT.alloc(c->N));
  VFVM_CUDA(dU.alloc(n));
  VFVM_CUDA(dUo.alloc(n));
  VFVM_CUDA(dP.alloc((size_t)blocks * nv));
  VFVM_CUDA(cudaMemcpyAsync(dT.p, T, c->N * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  VFVM_CUDA(cudaMemcpyAsync(dU.p, U, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  VFVM_CUDA(cudaMemcpyAsync(dUo.p, Uold ? Uold : U, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  const AsmTables t = c->tables();
  int rc = dispatch_physics(c->phys, [&](auto ph) {
    using Ph = decltype(ph);
    if (c->multireg)
      tf_integrals_kernel<Ph, true><<<blocks, kTfThreads, 0, c->stream>>>(t, dT.p, dU.p, dUo.p, time, lambda, dP.p);
    else
      tf_integrals_kernel<Ph, false><<<blocks, kTfThreads, 0, c->stream>>>(t, dT.p, dU.p, dUo.p, time, lambda, dP.p);
    return cudaGetLastError() == cudaSuccess ? VFVM_OK : VFVM_ERR_CUDA;
  });
  if (rc) return rc;
  std::vector<double> h((size_t)blocks * nv);
  VFVM_CUDA(cudaMemcpyAsync(h.data(), dP.p, h.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  VFVM_CUDA(cudaStreamSynchronize(c->stream));
  for (int k = 0; k < nv; ++k) out[k] = 0.0;
  for (int b = 0; b < blocks; ++b)
    for (int k = 0; k < nv; ++k) out[k] += h[(size_t)b * nv + k];
  return VFVM_OK;
}
