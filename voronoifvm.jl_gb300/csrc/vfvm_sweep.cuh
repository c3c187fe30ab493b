// Sweep engine: many systems on one grid (parameter sweeps, training data, the
// learned-start evaluation) solved together by whole-GPU kernels.
//
// Every kernel runs over all systems at once (grid: blocks per system x
// systems, blockIdx.y = system), so each phase of Newton and BiCGStab is one
// wide, bandwidth-bound launch instead of a barrier-separated phase of a small
// CTA team.  Per-system control flow (Newton and Krylov convergence, damping,
// the guarded start) lives in a state record per system; the kernels skip
// systems that are done, and CUDA-graph conditional WHILE nodes loop while any
// system is still iterating.  Per-system reductions are deterministic: block
// partials in a fixed slot, summed in block order by the system's last block.
//
// Newton logic: solve_step!, src/vfvm_solver.jl:13-222 (as team_newton);
// linear solve: left-preconditioned BiCGStab, multicolour ILU0 in ELL layout,
// optional Galerkin coarse stage.
#pragma once
#include "vfvm_newton_team.cuh"

namespace vfvm {

constexpr int kSweepThreads = 256;
constexpr int kSweepMaxBpi = 1024;  // blocks per system at most (reduction slots per system)

struct SweepState {
  double damp, oldnorm, tolx, rnorm, norm, resnorm, updnorm, prev_resnorm;
  double rho, alpha, omega, beta, tol2, rr;
  int niter, nround, status, nnewton, nlin, nactive, kactive, early;
  int guard, from_guess, restart, kit, kbreak, pad0, pad1, pad2;
};

// per-call values (device memory, written before each graph launch)
struct SweepCall {
  DevControl ctl;
  double time, tstepinv, lambda;
  const double* start;     // S * n initial values (the guess when guarded)
  const double* fallback;  // S * n user's inival for the guard (nullptr: no guard)
  int guard, pad[3];
};

template <class Ph, typename KT>
struct SweepArgs {
  static constexpr int NS = Ph::NS;
  AsmTables t;                 // shared grid tables (params/nodedata: instance 0, replaced per system)
  int S, N, nb, bpi;           // systems, nodes, block slots, blocks per system
  int64_t n;                   // unknowns per system
  double *U, *Uold, *F;        // S * n
  const double* params; int np;     // S * np
  const double* nodedata;           // S * N * nnd
  const uint8_t* dirdof;
  KT *J, *ilu, *dinv, *ell_val, *lo_val, *up_val;  // per system: nb*B, nb*B, N*B, ew*N*B, lw*N*B, uw*N*B
  KT *b, *x, *r, *r0, *p, *v, *s, *t2, *y;          // per system: n
  KrylovData<NS, KT> kd0;      // shared index tables (value pointers set per system)
  IluData<KT> il0;
  CoarseData cd0;              // shared aggregation tables; A/rc/zc per system (stride nc*nc / nc)
  SweepState* st;
  double* partials;            // S * bpi * 8
  unsigned* tickets;           // S
  const SweepCall* call;
  int ncolors;
  int* klist;                  // systems still in BiCGStab (built before each iteration)
  int* kcount;
  unsigned* runs;              // loop-condition evaluations [BiCGStab, Newton] (launch accounting),
                               // systems that entered the current BiCGStab loop
};

// The work unit of a block: system i, block lb of the nb blocks serving it.
struct SwUnit {
  int i, lb, nb;
  __device__ __forceinline__ int tid() const { return lb * blockDim.x + threadIdx.x; }
  __device__ __forceinline__ int nt() const { return nb * blockDim.x; }
};
// 2D grid (blocks per system x systems): one unit per block
__device__ __forceinline__ SwUnit sw_unit2d() { return SwUnit{(int)blockIdx.y, (int)blockIdx.x, (int)gridDim.x}; }

// Runs body(unit) for the work units this block serves.  use_list = 0: the 2D
// grid (bpi x S) covers every system, blocks of finished systems return at
// once.  use_list = 1 (BiCGStab iterations): a 1D grid strides over the units
// (bpi per system) of the compact list of systems still iterating, so late
// iterations, when few systems are left, launch few busy blocks.  (Spreading
// the last systems over more blocks per system was measured slower.)
template <class Ph, typename KT, class Body>
__device__ __forceinline__ void sw_for_active(const SweepArgs<Ph, KT>& a, int use_list, Body&& body) {
  if (!use_list) {
    const SwUnit u = sw_unit2d();
    if (a.st[u.i].kactive) body(u);
    return;
  }
  const int cnt = *a.kcount;
  if (cnt <= 0) return;
  const int nb = a.bpi;
  for (int64_t w = blockIdx.x; w < (int64_t)cnt * nb; w += gridDim.x) {
    body(SwUnit{a.klist[w / nb], (int)(w % nb), nb});
    __syncthreads();
  }
}

template <class Ph, typename KT>
__device__ __forceinline__ KrylovData<Ph::NS, KT> sw_kd(const SweepArgs<Ph, KT>& a, int i) {
  constexpr int B = Ph::NS * Ph::NS;
  KrylovData<Ph::NS, KT> d = a.kd0;
  const int64_t n = a.n;
  d.A = a.J + (int64_t)i * a.nb * B;
  d.dinv = a.dinv + (int64_t)i * a.N * B;
  d.b = a.b + i * n; d.x = a.x + i * n; d.r = a.r + i * n; d.r0 = a.r0 + i * n;
  d.p = a.p + i * n; d.v = a.v + i * n; d.s = a.s + i * n; d.t = a.t2 + i * n;
  d.ell_val = a.ell_val + (int64_t)i * a.kd0.ew * a.N * B;
  d.cd = a.cd0;
  if (d.cd.nc) {
    d.cd.A = a.cd0.A + (int64_t)i * d.cd.nc * d.cd.nc;
    d.cd.rc = a.cd0.rc + (int64_t)i * d.cd.nc;
    d.cd.zc = a.cd0.zc + (int64_t)i * d.cd.nc;
  }
  return d;
}

template <class Ph, typename KT>
__device__ __forceinline__ IluData<KT> sw_il(const SweepArgs<Ph, KT>& a, int i) {
  constexpr int B = Ph::NS * Ph::NS;
  IluData<KT> il = a.il0;
  il.ilu = a.ilu + (int64_t)i * a.nb * B;
  il.lo_val = a.lo_val + (int64_t)i * a.il0.lw * a.N * B;
  il.up_val = a.up_val + (int64_t)i * a.il0.uw * a.N * B;
  il.y = a.y + i * a.n;
  return il;
}

template <class Ph, typename KT>
__device__ __forceinline__ AsmTables sw_tables(const SweepArgs<Ph, KT>& a, int i) {
  AsmTables t = a.t;
  t.params = a.params + (int64_t)i * a.np;
  t.nodedata = a.t.nnd ? a.nodedata + (int64_t)i * a.N * a.t.nnd : nullptr;
  return t;
}



// Block reduction of NV values into the system's partial slot; returns true in
// thread 0 of the system's last block, with out[] = the totals in block order.
template <int NV>
__device__ __forceinline__ bool sw_reduce(double (&v)[NV], unsigned maxmask, double* partials, unsigned* tickets,
                                          int i, int lb, int bpi, double (&out)[NV]) {
  __shared__ double sh[NV][kTeamMaxWarps];
  __shared__ int last;
  block_allreduce<NV>(v, maxmask, sh);
  if (threadIdx.x == 0) {
    double* slot = partials + ((int64_t)i * kSweepMaxBpi + lb) * 8;
#pragma unroll
    for (int k = 0; k < NV; ++k) slot[k] = v[k];
    __threadfence();
    last = atomicAdd(&tickets[i], 1u) == (unsigned)bpi - 1u;
  }
  __syncthreads();
  if (!last || threadIdx.x >= 32) return false;
  // the system's last block: warp 0 combines the partials (lane j takes blocks
  // j, j+32, ...; then a fixed shuffle tree), so the order is fixed
  __threadfence();
  const int lane = threadIdx.x;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    const bool mx = (maxmask >> k) & 1;
    double acc = 0.0;
    for (int bx = lane; bx < bpi; bx += 32) {
      const double pv = __ldcg(&partials[((int64_t)i * kSweepMaxBpi + bx) * 8 + k]);
      acc = mx ? fmax(acc, pv) : acc + pv;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double ov = __shfl_xor_sync(0xffffffffu, acc, o);
      acc = mx ? fmax(acc, ov) : acc + ov;
    }
    out[k] = acc;
  }
  if (lane != 0) return false;
  tickets[i] = 0u;
  return true;
}

// ---- Newton-level kernels ----

// U = start (Dirichlet values set), Uold = fallback or start; state reset
template <class Ph, typename KT>
__global__ void __launch_bounds__(kSweepThreads) sw_init_kernel(SweepArgs<Ph, KT> a) {
  constexpr int NS = Ph::NS;
  const SwUnit u = sw_unit2d();
  const int i = u.i;
  const SweepCall& c = *a.call;
  const AsmTables t = sw_tables(a, i);
  Ph ph;
  ph.load(t.params);
  double* U = a.U + i * a.n;
  double* Uold = a.Uold + i * a.n;
  const double* src = c.start + i * a.n;
  const double* old = (c.fallback ? c.fallback : c.start) + i * a.n;
  double acc[1] = {0.0}, out[1];
  for (int K = u.tid(); K < a.N; K += u.nt()) {
#pragma unroll
    for (int k = 0; k < NS; ++k) { U[(int64_t)K * NS + k] = src[(int64_t)K * NS + k]; Uold[(int64_t)K * NS + k] = old[(int64_t)K * NS + k]; }
    init_dirichlet_node<Ph>(t, ph, K, U, c.time, c.lambda);
#pragma unroll
    for (int k = 0; k < NS; ++k) acc[0] += fabs(U[(int64_t)K * NS + k]);
  }
  if (sw_reduce<1>(acc, 0u, a.partials, a.tickets, i, u.lb, u.nb, out)) {
    SweepState& s = a.st[i];
    s.rnorm = out[0];
    s.damp = c.ctl.is_linear ? 1.0 : c.ctl.damp_initial;
    s.oldnorm = 1.0; s.tolx = 0.0; s.norm = 0.0; s.resnorm = 0.0; s.updnorm = 0.0;
    s.prev_resnorm = INFINITY;
    s.niter = 1; s.nround = 0; s.status = VFVM_OK; s.nnewton = 0; s.nlin = 0; s.early = 0;
    s.guard = c.guard; s.from_guess = c.guard; s.restart = 0; s.kactive = 0;
    s.nactive = c.ctl.maxiters >= 1 ? 1 : 0;
    if (!s.nactive) s.status = VFVM_ERR_CONVERGENCE;
  }
}

// guarded start abandoned: U = fallback (Dirichlet values set), state reset
template <class Ph, typename KT>
__global__ void __launch_bounds__(kSweepThreads) sw_restart_kernel(SweepArgs<Ph, KT> a) {
  constexpr int NS = Ph::NS;
  const SwUnit u = sw_unit2d();
  const int i = u.i;
  if (!a.st[i].restart) return;
  const SweepCall& c = *a.call;
  const AsmTables t = sw_tables(a, i);
  Ph ph;
  ph.load(t.params);
  double* U = a.U + i * a.n;
  const double* fb = c.fallback + i * a.n;
  double acc[1] = {0.0}, out[1];
  for (int K = u.tid(); K < a.N; K += u.nt()) {
#pragma unroll
    for (int k = 0; k < NS; ++k) U[(int64_t)K * NS + k] = fb[(int64_t)K * NS + k];
    init_dirichlet_node<Ph>(t, ph, K, U, c.time, c.lambda);
#pragma unroll
    for (int k = 0; k < NS; ++k) acc[0] += fabs(U[(int64_t)K * NS + k]);
  }
  if (sw_reduce<1>(acc, 0u, a.partials, a.tickets, i, u.lb, u.nb, out)) {
    SweepState& s = a.st[i];
    s.rnorm = out[0];
    s.damp = c.ctl.is_linear ? 1.0 : c.ctl.damp_initial;
    s.oldnorm = 1.0; s.tolx = 0.0; s.norm = 0.0; s.prev_resnorm = INFINITY;
    s.niter = 1; s.nround = 0; s.status = VFVM_OK; s.early = 0;
    s.guard = 0; s.from_guess = 0; s.restart = 0; s.nactive = 1;
  }
}

// assembly of every active system; then b = F, x = 0, residual norm, NaN check,
// residual-control exit and the guard test (in the system's last block)
template <class Ph, typename KT>
__global__ void __launch_bounds__(kSweepThreads) sw_assemble_kernel(SweepArgs<Ph, KT> a) {
  const SwUnit u = sw_unit2d();
  const int i = u.i;
  if (!a.st[i].nactive) return;
  constexpr int NS = Ph::NS;
  const SweepCall& c = *a.call;
  const AsmTables t = sw_tables(a, i);
  Ph ph;
  ph.load(t.params);
  int bad = 0;
  for (int K = u.tid(); K < a.N; K += u.nt())
    if (assemble_node<Ph, KT, false>(t, ph, K, a.U + i * a.n, a.Uold + i * a.n, c.time, c.tstepinv, c.lambda,
                                     a.F + i * a.n, a.J + (int64_t)i * a.nb * NS * NS))
      bad = 1;
  double acc[1] = {double(bad)}, out[1];
  if (sw_reduce<1>(acc, 1u, a.partials, a.tickets, i, u.lb, u.nb, out) && out[0] != 0.0) {
    a.st[i].status = VFVM_ERR_ASSEMBLY;
  }
}

template <class Ph, typename KT>
__global__ void __launch_bounds__(kSweepThreads) sw_prep_kernel(SweepArgs<Ph, KT> a) {
  const SwUnit u = sw_unit2d();
  const int i = u.i;
  SweepState& s = a.st[i];
  if (!s.nactive) return;
  const SweepCall& c = *a.call;
  const double* F = a.F + i * a.n;
  KT* b = a.b + i * a.n;
  KT* x = a.x + i * a.n;
  const uint8_t* dd = a.dirdof;
  double acc[2] = {0.0, 0.0}, out[2];
  for (int64_t q = u.tid(); q < a.n; q += u.nt()) {
    const double f = F[q];
    b[q] = KT(f);
    x[q] = KT(0);
    acc[0] += f * f;
    if (!dd[q]) acc[1] = fmax(acc[1], fabs(f));
  }
  if (sw_reduce<2>(acc, 2u, a.partials, a.tickets, i, u.lb, u.nb, out)) {
    s.resnorm = out[1];
    s.kactive = 0;
    if (s.status != VFVM_OK || isnan(out[0])) {
      s.status = VFVM_ERR_ASSEMBLY;
      if (s.guard) { s.restart = 1; s.status = VFVM_OK; }
      return;
    }
    if (!c.ctl.updatecontrol) s.norm = out[1];
    if (!c.ctl.updatecontrol && !c.ctl.is_linear && (out[1] < c.ctl.abstol || out[1] < s.tolx)) {
      s.early = 1;  // converged: no linear solve
      return;
    }
    if (s.guard && s.nnewton > 0 && !(out[1] < s.prev_resnorm)) {
      s.restart = 1;  // the guess does not reduce the residual: plain Newton from the fallback
      return;
    }
    s.prev_resnorm = out[1];
    s.kactive = 1;
  }
}

// ---- preconditioner setup ----

template <class Ph, typename KT>
__global__ void __launch_bounds__(kSweepThreads) sw_ilu_copy_kernel(SweepArgs<Ph, KT> a) {
  const SwUnit u = sw_unit2d();
  const int i = u.i;
  if (!a.st[i].kactive) return;
  constexpr int B = Ph::NS * Ph::NS;
  const int64_t m = (int64_t)a.nb * B;
  const KT* J = a.J + i * m;
  KT* L = a.ilu + i * m;
  for (int64_t q = u.tid(); q < m; q += u.nt()) L[q] = J[q];
}

template <class Ph, typename KT>
__global__ void __launch_bounds__(kSweepThreads) sw_ilu_factor_kernel(SweepArgs<Ph, KT> a, int c) {
  const SwUnit u = sw_unit2d();
  const int i = u.i;
  if (!a.st[i].kactive) return;
  const KrylovData<Ph::NS, KT> d = sw_kd(a, i);
  const IluData<KT> il = sw_il(a, i);
  for (int p = il.color_ptr[c] + u.tid(); p < il.color_ptr[c + 1]; p += u.nt())
    ilu_factor_row<Ph::NS, KT>(il.color_nodes[p], d, il);
}

template <class Ph, typename KT>
__global__ void __launch_bounds__(kSweepThreads) sw_pack_kernel(SweepArgs<Ph, KT> a) {
  const SwUnit u = sw_unit2d();
  const int i = u.i;
  if (!a.st[i].kactive) return;
  const KrylovData<Ph::NS, KT> d = sw_kd(a, i);
  const IluData<KT> il = sw_il(a, i);
  pack_ell_rows<Ph::NS, KT>(d, 0, a.N, u.tid(), u.nt());
  pack_ilu_positions<Ph::NS, KT>(il, a.N, 0, a.N, u.tid(), u.nt(), 0, a.N);
}

template <class Ph, typename KT>
__global__ void __launch_bounds__(kSweepThreads) sw_galerkin_kernel(SweepArgs<Ph, KT> a) {
  const SwUnit u = sw_unit2d();
  const int i = u.i;
  if (!a.st[i].kactive) return;
  const KrylovData<Ph::NS, KT> d = sw_kd(a, i);
  for (int64_t e = u.tid(); e < (int64_t)d.cd.nc * d.cd.nc; e += u.nt()) d.cd.A[e] = 0.f;
}

template <class Ph, typename KT>
__global__ void __launch_bounds__(kSweepThreads) sw_galerkin2_kernel(SweepArgs<Ph, KT> a) {
  const SwUnit u = sw_unit2d();
  const int i = u.i;
  if (!a.st[i].kactive) return;
  const KrylovData<Ph::NS, KT> d = sw_kd(a, i);
  coarse_galerkin_warps<Ph::NS, KT>(d.cd, d.col, d.A, u.tid() >> 5, u.nt() >> 5);
}

// one CTA per system: the dense inverse of its coarse matrix in shared memory
template <class Ph, typename KT>
__global__ void __launch_bounds__(1024) sw_coarse_invert_kernel(SweepArgs<Ph, KT> a) {
  const int i = blockIdx.x;
  if (!a.st[i].kactive) return;
  extern __shared__ float sw_csm[];
  const int nc = a.cd0.nc;
  float* A = a.cd0.A + (int64_t)i * nc * nc;
  for (int e = threadIdx.x; e < nc * nc; e += blockDim.x) sw_csm[e] = A[e];
  __syncthreads();
  coarse_invert_smem(sw_csm, nc, sw_csm + (size_t)nc * nc);
  for (int e = threadIdx.x; e < nc * nc; e += blockDim.x) A[e] = sw_csm[e];
}

// ---- BiCGStab kernels ----

// z = ILU0 forward sweep of colour c (fwd) or backward sweep (bwd); which = 0: b -> r,
// 1: y -> v, 2: y -> t
template <class Ph, typename KT>
__device__ __forceinline__ void sw_vectors(const SweepArgs<Ph, KT>& a, int i, int which, const KT*& in, KT*& out) {
  const int64_t o = i * a.n;
  if (which == 0) { in = a.b + o; out = a.r + o; }
  else if (which == 1) { in = a.y + o; out = a.v + o; }
  else { in = a.y + o; out = a.t2 + o; }
}

template <class Ph, typename KT>
__global__ void __launch_bounds__(kSweepThreads) sw_ilu_fwd_kernel(SweepArgs<Ph, KT> a, int c, int which,
                                                                   int use_list) {
  sw_for_active(a, use_list, [&](const SwUnit& u) {
    const int i = u.i;
    const IluData<KT> il = sw_il(a, i);
    const KT* in; KT* out;
    sw_vectors(a, i, which, in, out);
    ilu_fwd_positions<Ph::NS, KT>(il, a.N, in, out, il.color_ptr[c], il.color_ptr[c + 1], u.tid(), u.nt());
  });
}

template <class Ph, typename KT>
__global__ void __launch_bounds__(kSweepThreads) sw_ilu_bwd_kernel(SweepArgs<Ph, KT> a, int c, int which,
                                                                   int use_list) {
  sw_for_active(a, use_list, [&](const SwUnit& u) {
    const int i = u.i;
    const IluData<KT> il = sw_il(a, i);
    const KT* in; KT* out;
    sw_vectors(a, i, which, in, out);
    ilu_bwd_positions<Ph::NS, KT>(il, a.dinv + (int64_t)i * a.N * Ph::NS * Ph::NS, a.N, out, il.color_ptr[c],
                                  il.color_ptr[c + 1], u.tid(), u.nt());
  });
}

template <class Ph, typename KT>
__global__ void __launch_bounds__(kSweepThreads) sw_coarse_restrict_kernel(SweepArgs<Ph, KT> a, int which,
                                                                           int use_list) {
  sw_for_active(a, use_list, [&](const SwUnit& u) {
    const int i = u.i;
    const KrylovData<Ph::NS, KT> d = sw_kd(a, i);
    const KT* in; KT* out;
    sw_vectors(a, i, which, in, out);
    coarse_restrict_warps<Ph::NS, KT>(d.cd, in, u.tid() >> 5, u.nt() >> 5);
  });
}

template <class Ph, typename KT>
__global__ void __launch_bounds__(kSweepThreads) sw_coarse_matvec_kernel(SweepArgs<Ph, KT> a, int use_list) {
  sw_for_active(a, use_list, [&](const SwUnit& u) {
    const int i = u.i;
    const KrylovData<Ph::NS, KT> d = sw_kd(a, i);
    coarse_matvec_warps(d.cd, u.tid() >> 5, u.nt() >> 5);
  });
}

// r0 = r, rho = r.r: start of BiCGStab on the preconditioned right hand side
template <class Ph, typename KT>
__global__ void __launch_bounds__(kSweepThreads) sw_kstart_kernel(SweepArgs<Ph, KT> a) {
  const SwUnit u = sw_unit2d();
  const int i = u.i;
  SweepState& s = a.st[i];
  if (!s.kactive) return;
  const int64_t o = i * a.n;
  KT* r = a.r + o;
  KT* r0 = a.r0 + o;
  KT* p = a.p + o;
  KT* v = a.v + o;
  double acc[1] = {0.0}, out[1];
  acc_t<KT> a0 = 0;
  const float* zc = a.cd0.nc ? a.cd0.zc + (int64_t)i * a.cd0.nc : nullptr;
  for (int64_t q = u.tid(); q < a.n; q += u.nt()) {
    KT rq = r[q];
    if (zc && !a.dirdof[q]) {  // r += P zc (coarse prolongation of M^-1 b)
      const int64_t K = q / Ph::NS;
      rq += KT(__ldcg(&zc[a.cd0.agg_of_node[K] * Ph::NS + (int)(q - K * Ph::NS)]));
      r[q] = rq;
    }
    r0[q] = rq; p[q] = KT(0); v[q] = KT(0);
    a0 += acc_t<KT>(rq) * acc_t<KT>(rq);
  }
  acc[0] = double(a0);
  if (sw_reduce<1>(acc, 0u, a.partials, a.tickets, i, u.lb, u.nb, out)) {
    const DevControl& ctl = a.call->ctl;
    s.rho = out[0]; s.rr = out[0]; s.alpha = 1.0; s.omega = 1.0; s.beta = 0.0; s.kit = 0; s.kbreak = 0;
    const double tol = fmax(ctl.abstol_linear, ctl.reltol_linear * sqrt(out[0]));
    s.tol2 = tol * tol;
    if (!(out[0] > s.tol2) || ctl.maxiters_linear <= 0 || isnan(out[0])) s.kactive = 0;
  }
}

template <class Ph, typename KT>
__global__ void __launch_bounds__(kSweepThreads) sw_p_kernel(SweepArgs<Ph, KT> a) {
  sw_for_active(a, 1, [&](const SwUnit& u) {
    const int i = u.i;
    const SweepState& s = a.st[i];
    const int64_t o = i * a.n;
    vec_p_update<KT>(a.p + o, a.r + o, a.v + o, KT(s.beta), KT(s.omega), u.tid(), a.n, u.nt());
  });
}

// y = A p (which 1) or y = A s (which 2)
template <class Ph, typename KT>
__global__ void __launch_bounds__(kSweepThreads) sw_spmv_kernel(SweepArgs<Ph, KT> a, int which) {
  sw_for_active(a, 1, [&](const SwUnit& u) {
    const int i = u.i;
    const KrylovData<Ph::NS, KT> d = sw_kd(a, i);
    const int64_t o = i * a.n;
    spmv_ell_rows<Ph::NS, KT>(d, which == 1 ? a.p + o : a.s + o, a.y + o, 0, a.N, u.tid(), u.nt());
  });
}

// z += P zc (coarse prolongation) fused with acc += (w.z, z.z); the system's
// coarse solution is staged in shared memory first (one L2 read per block
// instead of one per unknown)
template <class Ph, typename KT>
__device__ __forceinline__ void sw_prolong_dot(const SweepArgs<Ph, KT>& a, const SwUnit& u, const KT* __restrict__ w,
                                               KT* __restrict__ z, double (&acc)[2]) {
  constexpr int NS = Ph::NS;
  __shared__ float zcs[kCoarseMax];
  const int i = u.i;
  const int nc = a.cd0.nc;
  const float* zc = a.cd0.zc + (int64_t)i * nc;
  for (int k = threadIdx.x; k < nc; k += blockDim.x) zcs[k] = __ldcg(&zc[k]);
  __syncthreads();
  const int* __restrict__ agg = a.cd0.agg_of_node;
  const uint8_t* __restrict__ dd = a.dirdof;
  acc_t<KT> a0 = 0, a1 = 0;
  const int64_t st = u.nt();
  // kVecU elements per thread and pass, all loads issued before the first use
  // (the element order of each thread's sums is unchanged)
  for (int64_t q = u.tid(); q < a.n; q += kVecU * st) {
    KT zz[kVecU], ww[kVecU];
    uint8_t dq[kVecU];
    int ag[kVecU];
#pragma unroll
    for (int v = 0; v < kVecU; ++v) {
      const int64_t e = q + v * st;
      if (e < a.n) { zz[v] = z[e]; ww[v] = w[e]; dq[v] = dd[e]; ag[v] = agg[e / NS]; }
      else { zz[v] = KT(0); ww[v] = KT(0); dq[v] = 1; ag[v] = 0; }
    }
#pragma unroll
    for (int v = 0; v < kVecU; ++v) {
      const int64_t e = q + v * st;
      if (e < a.n) {
        if (!dq[v]) {
          zz[v] += KT(zcs[ag[v] * NS + (int)(e - (e / NS) * NS)]);
          z[e] = zz[v];
        }
        a0 += acc_t<KT>(ww[v]) * acc_t<KT>(zz[v]);
        a1 += acc_t<KT>(zz[v]) * acc_t<KT>(zz[v]);
      }
    }
  }
  acc[0] += double(a0);
  acc[1] += double(a1);
  __syncthreads();  // zcs is reloaded by the block's next unit
}

// alpha = rho / (r0 . v); s = r - alpha v happens in the next kernel
template <class Ph, typename KT>
__global__ void __launch_bounds__(kSweepThreads) sw_alpha_kernel(SweepArgs<Ph, KT> a) {
  sw_for_active(a, 1, [&](const SwUnit& u) {
    const int i = u.i;
    SweepState& s = a.st[i];
    const int64_t o = i * a.n;
    double acc[2] = {0.0, 0.0}, out[2];
    if (a.cd0.nc) sw_prolong_dot<Ph, KT>(a, u, a.r0 + o, a.v + o, acc);  // v += P zc, then r0.v
    else vec_dots<KT>(a.r0 + o, a.v + o, u.tid(), a.n, u.nt(), acc);
    acc[1] = 0.0;
    if (sw_reduce<2>(acc, 0u, a.partials, a.tickets, i, u.lb, u.nb, out)) {
      if (out[0] == 0.0 || isnan(out[0])) { s.kbreak = 1; s.alpha = 0.0; }
      else s.alpha = s.rho / out[0];
    }
  });
}

template <class Ph, typename KT>
__global__ void __launch_bounds__(kSweepThreads) sw_s_kernel(SweepArgs<Ph, KT> a) {
  sw_for_active(a, 1, [&](const SwUnit& u) {
    const int i = u.i;
    const SweepState& s = a.st[i];
    const int64_t o = i * a.n;
    vec_s_update<KT>(a.s + o, a.r + o, a.v + o, KT(s.alpha), u.tid(), a.n, u.nt());
  });
}

// omega = (s . t) / (t . t)
template <class Ph, typename KT>
__global__ void __launch_bounds__(kSweepThreads) sw_omega_kernel(SweepArgs<Ph, KT> a) {
  sw_for_active(a, 1, [&](const SwUnit& u) {
    const int i = u.i;
    SweepState& s = a.st[i];
    const int64_t o = i * a.n;
    double acc[2] = {0.0, 0.0}, out[2];
    if (a.cd0.nc) sw_prolong_dot<Ph, KT>(a, u, a.s + o, a.t2 + o, acc);  // t += P zc, then s.t, t.t
    else vec_dots<KT>(a.s + o, a.t2 + o, u.tid(), a.n, u.nt(), acc);
    if (sw_reduce<2>(acc, 0u, a.partials, a.tickets, i, u.lb, u.nb, out)) s.omega = out[1] > 0.0 ? out[0] / out[1] : 0.0;
  });
}

// x += alpha p + omega s, r = s - omega t, convergence and the next beta
template <class Ph, typename KT>
__global__ void __launch_bounds__(kSweepThreads) sw_xr_kernel(SweepArgs<Ph, KT> a) {
  sw_for_active(a, 1, [&](const SwUnit& u) {
    const int i = u.i;
    SweepState& s = a.st[i];
    const int64_t o = i * a.n;
    double acc[2] = {0.0, 0.0}, out[2];
    vec_xr_update<KT>(a.x + o, a.r + o, a.p + o, a.s + o, a.t2 + o, a.r0 + o, KT(s.alpha), KT(s.omega), u.tid(),
                      a.n, u.nt(), acc);
    if (sw_reduce<2>(acc, 0u, a.partials, a.tickets, i, u.lb, u.nb, out)) {
      s.kit += 1;
      s.rr = out[1];
      const int brk = s.kbreak || out[0] == 0.0 || s.omega == 0.0 || isnan(out[1]);
      if (brk || !(out[1] > s.tol2) || s.kit >= a.call->ctl.maxiters_linear) {
        s.kactive = 0;
      } else {
        s.beta = (out[0] / s.rho) * (s.alpha / s.omega);
        s.rho = out[0];
      }
    }
  });
}

// Newton update U -= damp x and the solve_step! logic per system
template <class Ph, typename KT>
__global__ void __launch_bounds__(kSweepThreads) sw_update_kernel(SweepArgs<Ph, KT> a) {
  const SwUnit u = sw_unit2d();
  const int i = u.i;
  SweepState& s = a.st[i];
  // the BiCGStab loop is over for every system (those cut short by the
  // batch-level tail rule keep their current iterate)
  if (u.lb == 0 && threadIdx.x == 0) s.kactive = 0;
  if (!s.nactive || s.restart) return;
  const int64_t o = i * a.n;
  const bool apply = s.status == VFVM_OK && !s.early;
  const double damp = s.damp;
  double* U = a.U + o;
  const KT* x = a.x + o;
  double acc[2] = {0.0, 0.0}, out[2];
  for (int64_t q = u.tid(); q < a.n; q += u.nt()) {
    double u = U[q];
    if (apply) {
      const double dx = double(x[q]);
      u -= damp * dx;
      U[q] = u;
      acc[0] = fmax(acc[0], fabs(dx));
    }
    acc[1] += fabs(u);
  }
  if (sw_reduce<2>(acc, 1u, a.partials, a.tickets, i, u.lb, u.nb, out)) {
    const DevControl& ctl = a.call->ctl;
    s.nlin += s.kit;
    s.kit = 0;
    if (!apply) { s.nactive = 0; return; }  // converged before the solve, or failed
    s.nnewton += 1;
    s.updnorm = out[0];
    if (ctl.is_linear) { s.nactive = 0; return; }
    s.damp = fmin(s.damp * ctl.damp_growth, 1.0);
    const double norm = ctl.updatecontrol ? out[0] : s.resnorm;
    s.norm = norm;
    if (s.tolx == 0.0) s.tolx = norm * ctl.reltol;
    double dnorm = 1.0;
    const double rnorm_new = out[1];
    if (s.rnorm > 1.0e-50) dnorm = fabs((s.rnorm - rnorm_new) / s.rnorm);
    s.nround = (dnorm < ctl.tol_round) ? s.nround + 1 : 0;
    if (s.niter > 1 && norm / s.oldnorm > 1.0 / ctl.tol_mono) {
      if (s.guard) s.restart = 1;
      else { s.status = VFVM_ERR_CONVERGENCE; s.nactive = 0; }
      return;
    }
    if (norm < ctl.abstol || norm < s.tolx) { s.nactive = 0; return; }
    s.oldnorm = norm;
    s.rnorm = rnorm_new;
    if (s.nround > ctl.max_round) { s.nactive = 0; return; }
    s.niter += 1;
    if (s.niter > ctl.maxiters) {
      if (s.guard) s.restart = 1;
      else { s.status = VFVM_ERR_CONVERGENCE; s.nactive = 0; }
    }
  }
}

// Loop conditions: any system with kactive (which 0) / nactive or restart
// (which 1).  For which 0 also the compact list of systems still in BiCGStab,
// in system order (one block; each thread takes a contiguous chunk).
// Loop condition of the sweep graph: which = 1, any system still in Newton;
// which = 0, any system still in BiCGStab (and the compact list of them) --
// unless at most call->ctl.batch_tail systems are and they are at most a tenth
// of the systems that entered this BiCGStab loop (the batch-level inexact
// Newton rule: the loop ends and the stragglers keep their current iterate).
// runs[0..1]: loop bodies executed; runs[2]: systems that entered the current
// BiCGStab loop (set by its first evaluation, cleared by the Newton condition).
static __global__ void __launch_bounds__(1024) sw_cond_kernel(const SweepState* st, int S, int which,
                                                             cudaGraphConditionalHandle h, int* klist, int* kcount,
                                                             unsigned* runs, const SweepCall* call) {
  if (threadIdx.x == 0) atomicAdd(&runs[which], 1u);  // loop bodies executed (launch accounting)
  __shared__ int wsum[32];
  __shared__ int total;
  const int t = threadIdx.x, nt = blockDim.x;
  const int chunk = (S + nt - 1) / nt;
  const int b = min(S, t * chunk), e = min(S, b + chunk);
  int cnt = 0;
  for (int i = b; i < e; ++i) cnt += which == 0 ? (st[i].kactive != 0) : (st[i].nactive || st[i].restart);
  // exclusive scan of the per-thread counts
  const int lane = t & 31, w = t >> 5;
  int incl = cnt;
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) wsum[w] = incl;
  __syncthreads();
  if (t == 0) {
    int acc = 0;
    for (int k = 0; k < (nt + 31) / 32; ++k) { const int v = wsum[k]; wsum[k] = acc; acc += v; }
    total = acc;
  }
  __syncthreads();
  if (which == 0) {
    int pos = wsum[w] + incl - cnt;
    for (int i = b; i < e; ++i)
      if (st[i].kactive) klist[pos++] = i;
    if (t == 0) *kcount = total;
  }
  if (t == 0) {
    bool go = total > 0;
    if (which == 1) {
      runs[2] = 0u;
    } else {
      if (runs[2] == 0u) runs[2] = (unsigned)total;
      if (total <= call->ctl.batch_tail && 10u * (unsigned)total <= runs[2]) go = false;
    }
    cudaGraphSetConditional(h, go ? 1u : 0u);
  }
}

}  // namespace vfvm
