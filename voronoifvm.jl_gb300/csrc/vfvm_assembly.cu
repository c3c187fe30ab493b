// Residual + Jacobian assembly kernels (the reference's eval_and_assemble,
// src/vfvm_assembly.jl:520-643, with assemble_nodes :38-126, assemble_edges
// :128-200 and assemble_bnodes :318-407).
//
// Two kernels, both deterministic, atomic-free, one writer per output element,
// F[K] summed in the reference's edge order (a block row's columns are sorted
// by node index, which is also the edge numbering order):
//
// * assemble_tile_kernel (single-region grids, the default): edge-once
//   evaluation over node tiles staged in shared memory (below);
// * assemble_kernel (multi-region grids): node-centric gather.  One thread
//   owns one node K: it evaluates the node physics, then every edge incident to
//   K (so each edge flux is evaluated from both ends), then K's boundary-face
//   items.
#include <cstdlib>
#include <cstring>

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

// Edge-once assembly over node tiles (single-region grids).  One CTA per tile:
//   stage    the unknowns of the tile's owned and halo nodes into shared memory
//            (FP64 values and, in the mixed form, their FP32 shadows, each
//            converted once);
//   items    every edge of the tile once: flux(u_first, u_second) on duals,
//            storing fac * f (FP64) and the two partial blocks d/du_first,
//            d/du_second (times fac) in shared memory; and, as further work
//            items of the same loop, every owned node's node terms (reaction,
//            source, storage), stored alongside;
//   nodes    every owned node starts from its node terms and gathers its
//            edges' results in the reference's edge order (its block row's
//            columns are sorted by node index): F[K] += +-fac f, the diagonal
//            block accumulates d/du_K, and each off-diagonal block is written
//            once; then its boundary terms.
// Signs and factor placement follow assemble_edges (src/vfvm_assembly.jl:169-192):
// the first node gets +f, the second -f.  No atomics; one writer per output.
template <class Ph, typename P>
__global__ void __launch_bounds__(256) assemble_tile_kernel(const AsmTables t, const TileTables tt,
                                                            const double* __restrict__ U,
                                                            const double* __restrict__ Uold,
                                                            const double* __restrict__ tv, double* __restrict__ F,
                                                            P* __restrict__ J, int* __restrict__ err) {
  constexpr int NS = Ph::NS;
  constexpr bool kSh = kShadow<P>;
  extern __shared__ __align__(16) unsigned char smem[];
  const TileSmem L = tile_smem_layout<NS, P>(tt.maxloc, tt.maxedges);
  int* sl = reinterpret_cast<int*>(smem + L.lnodes);
  double* uv = reinterpret_cast<double*>(smem + L.uv);
  P* us = reinterpret_cast<P*>(smem + L.us);
  double* ef = reinterpret_cast<double*>(smem + L.ef);
  P* ja = reinterpret_cast<P*>(smem + L.ja);
  P* jb = reinterpret_cast<P*>(smem + L.jb);
  double* nf = reinterpret_cast<double*>(smem + L.nf);
  P* nj = reinterpret_cast<P*>(smem + L.nj);

  const int tile = blockIdx.x;
  const int lbeg = tt.tile_ptr[tile], nloc = tt.tile_ptr[tile + 1] - lbeg, nown = tt.tile_nown[tile];
  const int ebeg = tt.tile_eptr[tile], ne = tt.tile_eptr[tile + 1] - ebeg;
  const double time = tv[0], tstepinv = tv[1], lambda = tv[2];
  Ph ph;
  ph.load(t.params);

  // ---- stage the tile's unknowns
  for (int l = threadIdx.x; l < nloc; l += blockDim.x) {
    const int K = tt.lnodes[lbeg + l];
    sl[l] = K;
#pragma unroll
    for (int i = 0; i < NS; ++i) {
      const double v = U[(size_t)K * NS + i];
      uv[l * NS + i] = v;
      if constexpr (kSh) us[l * NS + i] = P(v);
    }
  }
  __syncthreads();

  // ---- work items: every edge of the tile once, then the owned nodes' node terms
  for (int item = threadIdx.x; item < ne + nown; item += blockDim.x) {
    if (item >= ne) {
      const int l = item - ne;
      const int K = sl[l];
      double uK[NS], fK[NS];
      P uKs[NS], jd[NS * NS];
#pragma unroll
      for (int i = 0; i < NS; ++i) {
        uK[i] = uv[l * NS + i];
        if constexpr (kSh) uKs[i] = us[l * NS + i];
        else uKs[i] = uK[i];
        fK[i] = 0.0;
      }
#pragma unroll
      for (int i = 0; i < NS * NS; ++i) jd[i] = P(0);
      node_terms<Ph, P, false>(t, ph, K, uK, uKs, Uold, time, tstepinv, lambda, fK, jd);
#pragma unroll
      for (int i = 0; i < NS; ++i) nf[l * NS + i] = fK[i];
#pragma unroll
      for (int i = 0; i < NS * NS; ++i) nj[l * NS * NS + i] = jd[i];
      continue;
    }
    const int e = item;
    const unsigned ab = tt.edge_ab[ebeg + e];
    const int la = (int)(ab & 0xffffu), lb = (int)(ab >> 16);
    const int A = sl[la], B = sl[lb];
    const double fac = tt.edge_fac[ebeg + e];
    P facp;
    if constexpr (kSh) facp = tt.edge_facf[ebeg + e];
    else facp = fac;
    EdgeItem ei{A, B, t.region, t.coord + (size_t)A * t.dim, t.coord + (size_t)B * t.dim, time, lambda,
                t.nodedata ? t.nodedata + (size_t)A * t.nnd : nullptr,
                t.nodedata ? t.nodedata + (size_t)B * t.nnd : nullptr};
    Dual<2 * NS, P> ua[NS], ub[NS], f[NS];
#pragma unroll
    for (int i = 0; i < NS; ++i) {
      if constexpr (kSh) {
        ua[i] = dseed<2 * NS, P>(uv[la * NS + i], us[la * NS + i], i);
        ub[i] = dseed<2 * NS, P>(uv[lb * NS + i], us[lb * NS + i], NS + i);
      } else {
        ua[i] = dseed<2 * NS, P>(uv[la * NS + i], P(uv[la * NS + i]), i);
        ub[i] = dseed<2 * NS, P>(uv[lb * NS + i], P(uv[lb * NS + i]), NS + i);
      }
      f[i] = dconst<2 * NS, P>(0.0);
    }
    ph.flux(f, ua, ub, ei);
#pragma unroll
    for (int i = 0; i < NS; ++i) {
      ef[e * NS + i] = fac * f[i].v;
#pragma unroll
      for (int j = 0; j < NS; ++j) {
        ja[(e * NS + i) * NS + j] = f[i].d[j] * facp;
        jb[(e * NS + i) * NS + j] = f[i].d[NS + j] * facp;
      }
    }
  }
  __syncthreads();

  // ---- owned nodes: node terms, edges in row order, boundary terms
  bool bad = false;
  for (int l = threadIdx.x; l < nown; l += blockDim.x) {
    const int K = sl[l];
    double uK[NS], fK[NS];
    P uKs[NS], jd[NS * NS];
#pragma unroll
    for (int i = 0; i < NS; ++i) {
      uK[i] = uv[l * NS + i];
      if constexpr (kSh) uKs[i] = us[l * NS + i];
      else uKs[i] = uK[i];
      fK[i] = nf[l * NS + i];
    }
#pragma unroll
    for (int i = 0; i < NS * NS; ++i) jd[i] = nj[l * NS * NS + i];
    const int sbeg = t.browptr[K], send = t.browptr[K + 1], dg = t.diag[K];
    for (int s = sbeg; s < send; ++s) {
      if (s == dg) continue;
      const int le = tt.slot_le[s];
      P* Js = J ? J + (size_t)s * NS * NS : nullptr;
      if (s > dg) {  // K is the edge's first node
#pragma unroll
        for (int i = 0; i < NS; ++i) {
          fK[i] += ef[le * NS + i];
#pragma unroll
          for (int j = 0; j < NS; ++j) {
            jd[i * NS + j] += ja[(le * NS + i) * NS + j];
            if (Js) Js[i * NS + j] = jb[(le * NS + i) * NS + j];
          }
        }
      } else {       // K is the edge's second node
#pragma unroll
        for (int i = 0; i < NS; ++i) {
          fK[i] += -ef[le * NS + i];
#pragma unroll
          for (int j = 0; j < NS; ++j) {
            jd[i * NS + j] += -jb[(le * NS + i) * NS + j];
            if (Js) Js[i * NS + j] = -ja[(le * NS + i) * NS + j];
          }
        }
      }
    }
    bnode_terms<Ph, P>(t, ph, K, uK, uKs, Uold, time, tstepinv, lambda, fK, jd);
#pragma unroll
    for (int i = 0; i < NS; ++i) {
      F[(size_t)K * NS + i] = fK[i];
      bad |= nan_bits(fK[i]);
    }
    if (J) {
      P* Jd = J + (size_t)dg * NS * NS;
#pragma unroll
      for (int i = 0; i < NS * NS; ++i) {
        Jd[i] = jd[i];
        bad |= nan_bits(jd[i]);
      }
    }
  }
  if (bad) atomicOr(err, 1);
}

// Largest dynamic shared memory a CTA may use on the current device.
static int max_dynamic_smem() {
  int dev = 0, v = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
  return v;
}

// Shared memory of the tiled kernel for this context and precision, 0 if it
// does not fit (the node-centric kernel is used then).
template <class Ph, typename P>
static size_t tile_smem_bytes(const vfvm_ctx* c) {
  if (c->ntiles == 0) return 0;
  const size_t b = tile_smem_layout<Ph::NS, P>(c->tile_maxloc, c->tile_maxedges).total;
  return b <= (size_t)max_dynamic_smem() ? b : 0;
}

// VFVM_ASSEMBLY_KERNEL=node selects the node-centric kernel on every grid (a
// comparison of the two kernels; both do the whole assembly).  Read at each
// launch, so a process can time both.
static bool use_node_kernel() {
  const char* e = std::getenv("VFVM_ASSEMBLY_KERNEL");
  return e && std::strcmp(e, "node") == 0;
}

int prepare_tiled_assembly(vfvm_ctx* c) {
  if (c->ntiles == 0) return VFVM_OK;
  return dispatch_physics(c->phys, [&](auto ph) {
    using Ph = decltype(ph);
    const size_t b64 = tile_smem_bytes<Ph, double>(c), b32 = tile_smem_bytes<Ph, float>(c);
    if (b64) VFVM_CUDA(cudaFuncSetAttribute((const void*)assemble_tile_kernel<Ph, double>,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b64));
    if (b32) VFVM_CUDA(cudaFuncSetAttribute((const void*)assemble_tile_kernel<Ph, float>,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b32));
    return VFVM_OK;
  });
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
    // the tiled kernel has no boundary-edge terms: physics with bflux use the node kernel
    if (!Ph::has_bflux && !Ph::has_edgereaction && !Ph::has_boutflow && !c->multireg && c->ntiles > 0 &&
        !use_node_kernel()) {
      const TileTables tt = c->tile_tables();
      const size_t b = Jf ? tile_smem_bytes<Ph, float>(c) : tile_smem_bytes<Ph, double>(c);
      if (b) {
        if (Jf)
          assemble_tile_kernel<Ph, float><<<c->ntiles, c->tile_threads, b, s>>>(t, tt, U, Uold, tv, F, Jf,
                                                                                c->errflag.p);
        else
          assemble_tile_kernel<Ph, double><<<c->ntiles, c->tile_threads, b, s>>>(t, tt, U, Uold, tv, F, J,
                                                                                 c->errflag.p);
        return cudaGetLastError() == cudaSuccess ? VFVM_OK : VFVM_ERR_CUDA;
      }
    }
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
