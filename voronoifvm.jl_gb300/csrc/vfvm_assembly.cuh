// Per-node assembly and Dirichlet initialisation, shared by the standalone
// kernels (vfvm_assembly.cu) and the persistent solvers.
//
// One call owns node K: node terms (reaction - source + storage/tstep), every
// edge incident to K in edge order (the block row's columns are sorted by node
// index), then K's boundary-face items; it writes F[K], K's off-diagonal
// Jacobian blocks and its diagonal block.  Returns true if a NaN was produced
// (AssemblyError in the reference, src/vfvm_assembly.jl:10-12).
#pragma once
#include "vfvm_context.cuh"
#include "vfvm_physics.cuh"

namespace vfvm {

// NaN test on the bit pattern (integer instructions; keeps the check off the
// FP64 pipe, which GB300 runs at a small fraction of the FP32 rate)
__device__ __forceinline__ bool nan_bits(double x) {
  return (__double_as_longlong(x) & 0x7fffffffffffffffll) > 0x7ff0000000000000ll;
}
__device__ __forceinline__ bool nan_bits(float x) { return (__float_as_uint(x) & 0x7fffffffu) > 0x7f800000u; }

// Node terms of K: reaction - source + (storage - oldstorage)/tstep
// (src/vfvm_assembly.jl:38-126), added to fK and the diagonal block jd.  With
// species restricted to regions (MR and t.reg_spec) only the rows and columns
// of the species of the item's region (src/vfvm_assemblydata.jl:245-269).
template <class Ph, typename P, bool MR>
__device__ __forceinline__ void node_terms(const AsmTables& t, const Ph& ph, int K, const double* uK, const P* uKs,
                                           const double* __restrict__ Uold, double time, double tstepinv,
                                           double lambda, double* fK, P* jd) {
  constexpr int NS = Ph::NS;
  const double* xK = t.coord + (size_t)K * t.dim;
  const double* dK = t.nodedata ? t.nodedata + (size_t)K * t.nnd : nullptr;
  const int nbeg = MR ? t.nitem_ptr[K] : 0, nend = MR ? t.nitem_ptr[K + 1] : 1;
  for (int it = nbeg; it < nend; ++it) {
    const int reg = MR ? t.nitem_reg[it] : t.region;
    const double fac = MR ? t.nitem_fac[it] : t.node_fac[K];
    const unsigned rm = (MR && t.reg_spec) ? t.reg_spec[reg - 1] : ~0u;
    NodeItem ni{K, reg, xK, time, lambda, dK};
    Dual<NS, P> u[NS], r[NS], s[NS];
#pragma unroll
    for (int i = 0; i < NS; ++i) { u[i] = dseed<NS, P>(uK[i], uKs[i], i); r[i] = dconst<NS, P>(0.0); s[i] = dconst<NS, P>(0.0); }
    double src[NS], ostor[NS];
#pragma unroll
    for (int i = 0; i < NS; ++i) { src[i] = 0.0; ostor[i] = 0.0; }
    if (Ph::has_source) ph.source(src, ni);
    if (Ph::has_reaction) ph.reaction(r, u, ni);
    if (Ph::has_storage) {
      ph.storage(s, u, ni);
      double uo[NS];
#pragma unroll
      for (int i = 0; i < NS; ++i) uo[i] = Uold[(size_t)K * NS + i];
      ph.storage(ostor, uo, ni);
    }
    const P facp = P(fac), tip = P(tstepinv);
#pragma unroll
    for (int i = 0; i < NS; ++i) {
      if (!((rm >> i) & 1u)) continue;
      fK[i] += fac * (r[i].v - src[i] + (s[i].v - ostor[i]) * tstepinv);
#pragma unroll
      for (int j = 0; j < NS; ++j)
        if ((rm >> j) & 1u) jd[i * NS + j] += (r[i].d[j] + s[i].d[j] * tip) * facp;
    }
  }
}

// Boundary-face items of K in bface order: legacy Dirichlet/Robin data
// (src/vfvm_assembly.jl:355-387, every species of the dense layout),
// breaction - bsource (:388-407) and (bstorage - old bstorage) / tstep
// (:409-440) in the rows and columns of the node's species nm
// (src/vfvm_assemblydata.jl:278-301).
template <class Ph, typename P>
__device__ __forceinline__ void bnode_terms(const AsmTables& t, const Ph& ph, int K, const double* uK, const P* uKs,
                                            const double* __restrict__ Uold, double time, double tstepinv,
                                            double lambda, double* fK, P* jd, unsigned nm = ~0u) {
  constexpr int NS = Ph::NS;
  const double* xK = t.coord + (size_t)K * t.dim;
  const int bbeg = t.bn_ptr[K], bend = t.bn_ptr[K + 1];
  for (int it = bbeg; it < bend; ++it) {
    const int reg = t.bn_reg[it];
    const double fac = t.bn_fac[it];
    double Dir = kDirichlet;
    if (t.has_legacy && reg - 1 < t.nbregions) {
      Dir = kDirichlet / fac;
#pragma unroll
      for (int i = 0; i < NS; ++i) {
        const double bf = t.bfactors[i + NS * (reg - 1)], bv = t.bvalues[i + NS * (reg - 1)];
        if (bf == kDirichlet) {
          fK[i] += bf * (uK[i] - bv);
          jd[i * NS + i] += P(bf);
        } else {
          fK[i] += fac * (bf * uK[i] - bv);
          if (bf != 0.0) jd[i * NS + i] += P(bf) * P(fac);
        }
      }
    }
    BNodeItem bi{K, reg, xK, time, lambda, fac, Dir, nullptr};
    if (Ph::has_breaction || Ph::has_bsource) {
      Dual<NS, P> u[NS], y[NS];
      double bsrc[NS];
#pragma unroll
      for (int i = 0; i < NS; ++i) { u[i] = dseed<NS, P>(uK[i], uKs[i], i); y[i] = dconst<NS, P>(0.0); bsrc[i] = 0.0; }
      if (Ph::has_breaction) ph.breaction(y, u, bi);
      if (Ph::has_bsource) ph.bsource(bsrc, bi);
      const P facp = P(fac);
#pragma unroll
      for (int i = 0; i < NS; ++i) {
        if (!((nm >> i) & 1u)) continue;
        fK[i] += fac * (y[i].v - bsrc[i]);
#pragma unroll
        for (int j = 0; j < NS; ++j)
          if ((nm >> j) & 1u) jd[i * NS + j] += y[i].d[j] * facp;
      }
    }
    if (Ph::has_bstorage) {
      Dual<NS, P> u[NS], s[NS];
      double uo[NS], so[NS];
#pragma unroll
      for (int i = 0; i < NS; ++i) {
        u[i] = dseed<NS, P>(uK[i], uKs[i], i);
        s[i] = dconst<NS, P>(0.0);
        uo[i] = Uold[(size_t)K * NS + i];
        so[i] = 0.0;
      }
      ph.bstorage(s, u, bi);
      ph.bstorage(so, uo, bi);
      const P ft = P(fac * tstepinv);
#pragma unroll
      for (int i = 0; i < NS; ++i) {
        if (!((nm >> i) & 1u)) continue;
        fK[i] += fac * (s[i].v - so[i]) * tstepinv;
#pragma unroll
        for (int j = 0; j < NS; ++j)
          if ((nm >> j) & 1u) jd[i * NS + j] += s[i].d[j] * ft;
      }
    }
  }
}

// Boundary-edge items of Jacobian slot s (edge A-B, A < B), evaluated from
// node K's end: assemble_bedges (src/vfvm_assembly.jl:444-510), the same sign
// and factor placement as a bulk edge (first node +f, second -f); with species
// restricted to regions, the rows and columns of the first node's species
// (src/vfvm_assemblydata.jl:391-420).
template <class Ph, typename P>
__device__ __forceinline__ void bedge_terms(const AsmTables& t, const Ph& ph, int s, int A, int B, bool kfirst,
                                            const double* uA, const P* uAs, const double* uB, const P* uBs,
                                            double time, double lambda, double* fK, P* jd, P* jo) {
  constexpr int NS = Ph::NS;
  const unsigned m = t.node_spec ? t.node_spec[A] : ~0u;
  for (int it = t.sbe_ptr[s]; it < t.sbe_ptr[s + 1]; ++it) {
    const double fac = t.sbe_fac[it];
    BEdgeItem be{A, B, t.sbe_reg[it], t.coord + (size_t)A * t.dim, t.coord + (size_t)B * t.dim, time, lambda};
    Dual<2 * NS, P> ua[NS], ub[NS], f[NS];
#pragma unroll
    for (int i = 0; i < NS; ++i) {
      ua[i] = dseed<2 * NS, P>(uA[i], uAs[i], i);
      ub[i] = dseed<2 * NS, P>(uB[i], uBs[i], NS + i);
      f[i] = dconst<2 * NS, P>(0.0);
    }
    ph.bflux(f, ua, ub, be);
    const P facp = P(fac);
#pragma unroll
    for (int i = 0; i < NS; ++i) {
      if (!((m >> i) & 1u)) continue;
      if (kfirst) {
        fK[i] += fac * f[i].v;
#pragma unroll
        for (int j = 0; j < NS; ++j)
          if ((m >> j) & 1u) { jd[i * NS + j] += f[i].d[j] * facp; jo[i * NS + j] += f[i].d[NS + j] * facp; }
      } else {
        fK[i] += -(fac * f[i].v);
#pragma unroll
        for (int j = 0; j < NS; ++j)
          if ((m >> j) & 1u) { jd[i * NS + j] += (-f[i].d[NS + j]) * facp; jo[i * NS + j] += (-f[i].d[j]) * facp; }
      }
    }
  }
}

template <class Ph, typename P, bool MR>
__device__ __forceinline__ bool assemble_node(const AsmTables& t, const Ph& ph, int K, const double* __restrict__ U,
                                              const double* __restrict__ Uold, double time, double tstepinv,
                                              double lambda, double* __restrict__ F, P* __restrict__ J) {
  constexpr int NS = Ph::NS;
  double uK[NS];
  P uKs[NS];  // the values in the partials' precision, converted once per node
#pragma unroll
  for (int i = 0; i < NS; ++i) { uK[i] = U[(size_t)K * NS + i]; uKs[i] = P(uK[i]); }
  double fK[NS];
  P jd[NS * NS];
#pragma unroll
  for (int i = 0; i < NS; ++i) fK[i] = 0.0;
#pragma unroll
  for (int i = 0; i < NS * NS; ++i) jd[i] = P(0);

  node_terms<Ph, P, MR>(t, ph, K, uK, uKs, Uold, time, tstepinv, lambda, fK, jd);

  // ---- edges incident to K, in edge order (columns sorted by node index)
  const int sbeg = t.browptr[K], send = t.browptr[K + 1];
  for (int s = sbeg; s < send; ++s) {
    const int M = t.bcol[s];
    if (M == K) continue;
    double uM[NS];
    P uMs[NS];
#pragma unroll
    for (int i = 0; i < NS; ++i) { uM[i] = U[(size_t)M * NS + i]; uMs[i] = P(uM[i]); }
    const bool kfirst = K < M;
    const int A = kfirst ? K : M, B = kfirst ? M : K;
    P jo[NS * NS];
#pragma unroll
    for (int i = 0; i < NS * NS; ++i) jo[i] = P(0);
    const int ebeg = MR ? t.sitem_ptr[s] : 0, eend = MR ? t.sitem_ptr[s + 1] : 1;
    for (int it = ebeg; it < eend; ++it) {
      const int reg = MR ? t.sitem_reg[it] : t.region;
      const double fac = MR ? t.sitem_fac[it] : t.slot_fac[s];
      const unsigned rm = (MR && t.reg_spec) ? t.reg_spec[reg - 1] : ~0u;  // src/vfvm_assemblydata.jl:346-381
      EdgeItem ei{A, B, reg, t.coord + (size_t)A * t.dim, t.coord + (size_t)B * t.dim, time, lambda,
                  t.nodedata ? t.nodedata + (size_t)A * t.nnd : nullptr,
                  t.nodedata ? t.nodedata + (size_t)B * t.nnd : nullptr};
      Dual<2 * NS, P> ua[NS], ub[NS], f[NS];
#pragma unroll
      for (int i = 0; i < NS; ++i) {
        ua[i] = dseed<2 * NS, P>(kfirst ? uK[i] : uM[i], kfirst ? uKs[i] : uMs[i], i);
        ub[i] = dseed<2 * NS, P>(kfirst ? uM[i] : uK[i], kfirst ? uMs[i] : uKs[i], NS + i);
        f[i] = dconst<2 * NS, P>(0.0);
      }
      ph.flux(f, ua, ub, ei);
      P facp;
      if constexpr (kShadow<P>) facp = MR ? P(fac) : t.slot_facf[s];  // no conversion on the edge path
      else facp = fac;
      if (kfirst) {
#pragma unroll
        for (int i = 0; i < NS; ++i) {
          if (!((rm >> i) & 1u)) continue;
          fK[i] += fac * f[i].v;
#pragma unroll
          for (int j = 0; j < NS; ++j) {
            if (!((rm >> j) & 1u)) continue;
            jd[i * NS + j] += f[i].d[j] * facp;
            jo[i * NS + j] += f[i].d[NS + j] * facp;
          }
        }
      } else {
#pragma unroll
        for (int i = 0; i < NS; ++i) {
          if (!((rm >> i) & 1u)) continue;
          fK[i] += -(fac * f[i].v);
#pragma unroll
          for (int j = 0; j < NS; ++j) {
            if (!((rm >> j) & 1u)) continue;
            jd[i * NS + j] += (-f[i].d[NS + j]) * facp;
            jo[i * NS + j] += (-f[i].d[j]) * facp;
          }
        }
      }
      if constexpr (Ph::has_boutflow) {
        // boutflow (src/vfvm_assembly.jl:239-313): on an edge with a node on an
        // outflow boundary region, fac * r to the first node's residual (+) when
        // it is an outflow node and to the second's (-) when that one is; the
        // edge's outflow node is the second if both are
        const bool oA = t.outflow_node && t.outflow_node[A], oB = t.outflow_node && t.outflow_node[B];
        if (oA || oB) {
          ei.outflownode = oB ? 2 : 1;
          Dual<2 * NS, P> r[NS];
#pragma unroll
          for (int i = 0; i < NS; ++i) r[i] = dconst<2 * NS, P>(0.0);
          ph.boutflow(r, ua, ub, ei);
          if (kfirst ? oA : oB) {
#pragma unroll
            for (int i = 0; i < NS; ++i) {
              if (!((rm >> i) & 1u)) continue;
              fK[i] += kfirst ? fac * r[i].v : -(fac * r[i].v);
#pragma unroll
              for (int j = 0; j < NS; ++j) {
                if (!((rm >> j) & 1u)) continue;
                if (kfirst) {
                  jd[i * NS + j] += r[i].d[j] * facp;
                  jo[i * NS + j] += r[i].d[NS + j] * facp;
                } else {
                  jd[i * NS + j] += (-r[i].d[NS + j]) * facp;
                  jo[i * NS + j] += (-r[i].d[j]) * facp;
                }
              }
            }
          }
          ei.outflownode = 0;
        }
      }
      if constexpr (Ph::has_edgereaction) {
        // edgereaction (src/vfvm_assembly.jl:202-238): fac * r added to both end
        // nodes, the Jacobian entries placed as the reference places them (first
        // node's row: +dr/du_first, -dr/du_second; second node's row:
        // -dr/du_first, +dr/du_second)
        Dual<2 * NS, P> r[NS];
#pragma unroll
        for (int i = 0; i < NS; ++i) r[i] = dconst<2 * NS, P>(0.0);
        ph.edgereaction(r, ua, ub, ei);
#pragma unroll
        for (int i = 0; i < NS; ++i) {
          if (!((rm >> i) & 1u)) continue;
          fK[i] += fac * r[i].v;
#pragma unroll
          for (int j = 0; j < NS; ++j) {
            if (!((rm >> j) & 1u)) continue;
            if (kfirst) {
              jd[i * NS + j] += r[i].d[j] * facp;
              jo[i * NS + j] += (-r[i].d[NS + j]) * facp;
            } else {
              jd[i * NS + j] += r[i].d[NS + j] * facp;
              jo[i * NS + j] += (-r[i].d[j]) * facp;
            }
          }
        }
      }
    }
    if constexpr (Ph::has_bflux) {
      if (t.sbe_ptr) {
        if (kfirst) bedge_terms<Ph, P>(t, ph, s, K, M, true, uK, uKs, uM, uMs, time, lambda, fK, jd, jo);
        else bedge_terms<Ph, P>(t, ph, s, M, K, false, uM, uMs, uK, uKs, time, lambda, fK, jd, jo);
      }
    }
    if (J) {
      P* Js = J + (size_t)s * NS * NS;
#pragma unroll
      for (int i = 0; i < NS * NS; ++i) Js[i] = jo[i];
    }
  }

  const unsigned nm = (MR && t.node_spec) ? t.node_spec[K] : ~0u;
  bnode_terms<Ph, P>(t, ph, K, uK, uKs, Uold, time, tstepinv, lambda, fK, jd, nm);
  if (MR && t.node_spec) {
    // the species K does not carry: F += U - Uold, unit diagonal
    // (_eval_and_assemble_inactive_species, src/vfvm_system.jl:1012-1026)
#pragma unroll
    for (int i = 0; i < NS; ++i)
      if (!((nm >> i) & 1u)) {
        fK[i] += uK[i] - Uold[(size_t)K * NS + i];
        jd[i * NS + i] += P(1);
      }
  }

  bool bad = false;
#pragma unroll
  for (int i = 0; i < NS; ++i) {
    F[(size_t)K * NS + i] = fK[i];
    bad |= nan_bits(fK[i]);
  }
  if (J) {
    P* Jd = J + (size_t)t.diag[K] * NS * NS;
#pragma unroll
    for (int i = 0; i < NS * NS; ++i) {
      Jd[i] = jd[i];
      bad |= nan_bits(jd[i]);
    }
  }
  return bad;
}


template <class Ph>
__device__ __forceinline__ void init_dirichlet_node(const AsmTables& t, const Ph& ph, int K, double* __restrict__ U,
                                                    double time, double lambda) {
  constexpr int NS = Ph::NS;
  const int bbeg = t.bn_ptr[K], bend = t.bn_ptr[K + 1];
  const unsigned nm = t.node_spec ? t.node_spec[K] : ~0u;
  if (bbeg == bend && !t.node_spec) return;
  const double* xK = t.coord + (size_t)K * t.dim;
  double u[NS];
#pragma unroll
  for (int i = 0; i < NS; ++i) u[i] = U[(size_t)K * NS + i];
  for (int it = bbeg; it < bend; ++it) {
    const int reg = t.bn_reg[it];
    double dv[NS], y[NS];
#pragma unroll
    for (int i = 0; i < NS; ++i) { dv[i] = INFINITY; y[i] = 0.0; }
    BNodeItem bi{K, reg, xK, time, lambda, t.bn_fac[it], kDirichlet, dv};
    if (Ph::has_breaction) ph.breaction(y, u, bi);
#pragma unroll
    for (int i = 0; i < NS; ++i) {
      if (!isinf(dv[i])) u[i] = dv[i];
      if (t.has_legacy && reg - 1 < t.nbregions) {
        const double bf = t.bfactors[i + NS * (reg - 1)];
        if (fabs(bf - kDirichlet) <= 1.4901161193847656e-8 * kDirichlet) u[i] = t.bvalues[i + NS * (reg - 1)];
      }
    }
  }
  // species K does not carry start at 0 (_initialize_inactive_dof!, src/vfvm_system.jl:1030-1042)
#pragma unroll
  for (int i = 0; i < NS; ++i)
    if (!((nm >> i) & 1u)) u[i] = 0.0;
#pragma unroll
  for (int i = 0; i < NS; ++i) U[(size_t)K * NS + i] = u[i];
}

}  // namespace vfvm
