// Restarted GMRES(m) with left preconditioning for the team engines: the
// Krylov method behind LinearSolve.jl's KrylovJL_GMRES (Krylov.jl `gmres`),
// which the reference pairs with ILU(0) preconditioners in
// examples/DevEx004_EquationBlock3D.jl:187 and examples/DevEx005_Mixture.jl:290.
//
// Each Arnoldi vector is orthogonalised by block classical Gram-Schmidt with
// one re-orthogonalisation pass (CGS2): the projections onto up to eight basis
// vectors are reduced together, so iteration j costs 2 ceil((j+1)/8) + 1 team
// reductions besides the preconditioned operator.  The Hessenberg columns are
// brought to triangular form by Givens rotations, computed redundantly by one
// thread of every CTA from the same deterministic reductions, so every CTA
// takes the same decisions.  Convergence test (shared with the BiCGStab
// solvers of this engine): ||M^-1 (b - A x)|| <= max(abstol, reltol ||M^-1 b||),
// where the left-preconditioned least-squares residual |g_{j+1}| is that norm.
#pragma once
#include "vfvm_team_ilu.cuh"

namespace vfvm {

constexpr int kGmresMaxRestart = 32;  // VFVM_GMRES_MAX_RESTART
constexpr int kGmresChunk = 8;        // projections per team reduction (8 partial slots per CTA)

struct GmresShared {
  double R[kGmresMaxRestart][kGmresMaxRestart];  // R[j][i], i <= j: column j of the triangular factor
  double h[kGmresMaxRestart + 1];                 // Hessenberg column being rotated
  double g[kGmresMaxRestart + 1];                 // rotated beta e_1
  double cs[kGmresMaxRestart], sn[kGmresMaxRestart];
  double y[kGmresMaxRestart];
};

// Solves M^-1 A x = zb (zb = M^-1 b, already formed) from x = 0 with the basis
// in V ((m + 1) vectors of n) and r as restart scratch.  op(in, out) computes
// out = M^-1 A in; it starts with a team barrier (it reads `in` across the
// team) and leaves every out[q] readable by the thread of team rank q mod size.
// `iters` (Arnoldi steps) is set on every thread.  Returns false if a team
// barrier expired.
template <class Team, typename KT, class Op>
__device__ bool team_gmres_core(Team& team, int64_t n, const KT* __restrict__ zb, KT* __restrict__ x,
                                KT* __restrict__ r, KT* __restrict__ V, int m, const KrylovCtl& c, Op&& op,
                                int& iters) {
  __shared__ GmresShared sh;
  const int64_t q0 = team.rank(), qs = team.size();
  iters = 0;
  m = m < 1 ? 1 : (m > kGmresMaxRestart ? kGmresMaxRestart : m);
  double a1[1] = {0.0}, r1[1];
  for (int64_t q = q0; q < n; q += qs) {
    const KT z = zb[q];
    x[q] = KT(0);
    r[q] = z;
    a1[0] += double(z) * double(z);
  }
  if (!team.template reduce<1>(a1, 0u, r1)) return false;
  const double tol = fmax(c.abstol, c.reltol * sqrt(r1[0]));
  double beta = sqrt(r1[0]);
  if (!(beta > tol) || c.maxiters <= 0) return true;
  for (int64_t q = q0; q < n; q += qs) V[q] = KT(double(r[q]) / beta);
  if (threadIdx.x == 0) sh.g[0] = beta;
  int it = 0, k = 0;       // Arnoldi steps in total / in this cycle
  bool restart = false;    // the next operator application forms the restart residual
  while (true) {
    // one call site of the operator: Arnoldi step (w = M^-1 A V_k) or restart (r = M^-1 A x)
    KT* __restrict__ w = restart ? r : V + (size_t)(k + 1) * n;
    if (!op(restart ? (const KT*)x : (const KT*)(V + (size_t)k * n), w)) return false;
    if (restart) {
      // true preconditioned residual r = zb - M^-1 A x, then a new cycle from V_0 = r / beta
      a1[0] = 0.0;
      for (int64_t q = q0; q < n; q += qs) {
        const KT rq = KT(double(zb[q]) - double(r[q]));
        r[q] = rq;
        a1[0] += double(rq) * double(rq);
      }
      if (!team.template reduce<1>(a1, 0u, r1)) return false;
      beta = sqrt(r1[0]);
      if (!(beta > tol)) break;
      for (int64_t q = q0; q < n; q += qs) V[q] = KT(double(r[q]) / beta);
      if (threadIdx.x == 0) sh.g[0] = beta;
      k = 0;
      restart = false;
      continue;
    }
    // w -= V_i (V_i . w), i <= k, in chunks of kGmresChunk, twice
    for (int pass = 0; pass < 2; ++pass) {
      for (int i0 = 0; i0 <= k; i0 += kGmresChunk) {
        const int nb = min(kGmresChunk, k + 1 - i0);
        const KT* __restrict__ Vc = V + (size_t)i0 * n;
        double acc[kGmresChunk], red[kGmresChunk];
#pragma unroll
        for (int j = 0; j < kGmresChunk; ++j) acc[j] = 0.0;
        for (int64_t q = q0; q < n; q += qs) {
          const double wq = double(w[q]);
#pragma unroll
          for (int j = 0; j < kGmresChunk; ++j)
            if (j < nb) acc[j] += double(Vc[(size_t)j * n + q]) * wq;
        }
        if (!team.template reduce<kGmresChunk>(acc, 0u, red)) return false;
        for (int64_t q = q0; q < n; q += qs) {
          double wq = double(w[q]);
#pragma unroll
          for (int j = 0; j < kGmresChunk; ++j)
            if (j < nb) wq -= red[j] * double(Vc[(size_t)j * n + q]);
          w[q] = KT(wq);
        }
        if (threadIdx.x == 0)
          for (int j = 0; j < nb; ++j) sh.h[i0 + j] = (pass ? sh.h[i0 + j] : 0.0) + red[j];
      }
    }
    double a[1] = {0.0}, rn[1];
    for (int64_t q = q0; q < n; q += qs) a[0] += double(w[q]) * double(w[q]);
    if (!team.template reduce<1>(a, 0u, rn)) return false;
    const double hn = sqrt(rn[0]);
    if (hn > 0.0)
      for (int64_t q = q0; q < n; q += qs) w[q] = KT(double(w[q]) / hn);
    if (threadIdx.x == 0) {
      double* h = sh.h;
      for (int i = 0; i < k; ++i) {
        const double t = sh.cs[i] * h[i] + sh.sn[i] * h[i + 1];
        h[i + 1] = -sh.sn[i] * h[i] + sh.cs[i] * h[i + 1];
        h[i] = t;
      }
      const double rr = hypot(h[k], hn);
      const double cs = rr > 0.0 ? h[k] / rr : 1.0, sn = rr > 0.0 ? hn / rr : 0.0;
      sh.cs[k] = cs;
      sh.sn[k] = sn;
      h[k] = rr;
      sh.g[k + 1] = -sn * sh.g[k];
      sh.g[k] = cs * sh.g[k];
      for (int i = 0; i <= k; ++i) sh.R[k][i] = h[i];
    }
    __syncthreads();
    const double res = fabs(sh.g[k + 1]);
    ++k;
    ++it;
    // converged, NaN, out of iterations, or an invariant subspace (hn == 0: x is exact)
    const bool stop = !(res > tol) || !(hn > 0.0) || it >= c.maxiters;
    if (!stop && k < m) continue;
    // end of a cycle: y = R^-1 g;  x += V y
    if (threadIdx.x == 0) {
      for (int i = k - 1; i >= 0; --i) {
        double s = sh.g[i];
        for (int j = i + 1; j < k; ++j) s -= sh.R[j][i] * sh.y[j];
        sh.y[i] = sh.R[i][i] != 0.0 ? s / sh.R[i][i] : 0.0;
      }
    }
    __syncthreads();
    for (int64_t q = q0; q < n; q += qs) {
      double xq = double(x[q]);
      for (int j = 0; j < k; ++j) xq += sh.y[j] * double(V[(size_t)j * n + q]);
      x[q] = KT(xq);
    }
    if (stop) break;
    restart = true;
  }
  iters = it;
  return true;
}

// GMRES(m) on the Newton matrix with the engine's preconditioners: block
// Jacobi, multicolour ILU(0) or subdomain ILU(0), each with the coarse stage
// when d.cd.nc > 0 (not with block Jacobi).  Same contract as the BiCGStab
// solvers: A, b in d, result in d.x, `iters` set on every thread.
// Not inlined: the Newton kernels that carry it keep their register budget for
// the assembly and BiCGStab paths.
template <class Team, int NS, int LPR, typename KT, int PRECON>
__device__ __noinline__ bool team_gmres(Team& team, const KrylovData<NS, KT>& d, const IluData<KT>& il, const KrylovCtl& c,
                           int64_t nvals, int m, int& iters) {
  const int64_t n = (int64_t)d.N * NS;
  iters = 0;
  if constexpr (PRECON == VFVM_PRECON_JACOBI) {
    // Dinv = inverse diagonal blocks; zb = Dinv b
    for (int K = team.rank(); K < d.N; K += team.size()) {
      double a[NS * NS], inv[NS * NS];
      const KT* Ad = d.A + (size_t)d.diag[K] * NS * NS;
#pragma unroll
      for (int i = 0; i < NS * NS; ++i) a[i] = double(Ad[i]);
      small_inverse<NS>(a, inv);
#pragma unroll
      for (int i = 0; i < NS * NS; ++i) d.dinv[(size_t)K * NS * NS + i] = KT(inv[i]);
#pragma unroll
      for (int i = 0; i < NS; ++i) {
        double z = 0.0;
#pragma unroll
        for (int j = 0; j < NS; ++j) z += inv[i * NS + j] * double(d.b[(size_t)K * NS + j]);
        d.r0[(size_t)K * NS + i] = KT(z);
      }
    }
    if (!team.sync()) return false;
    auto op = [&](const KT* in, KT* out) -> bool {
      if (!team.sync()) return false;
      double acc[2] = {0.0, 0.0};
      team_spmv_jac<Team, NS, LPR, KT>(team, d, in, out, in, acc);
      return team.sync();
    };
    return team_gmres_core(team, n, d.r0, d.x, d.r, d.gv, m, c, op, iters);
  } else if constexpr (PRECON == VFVM_PRECON_ILU0) {
    if (!team_ilu_factor<Team, NS, KT>(team, d, il, nvals)) return false;
    pack_ell_rows<NS, KT>(d, 0, d.N, team.rank(), team.size());
    pack_ilu_positions<NS, KT>(il, d.N, 0, d.N, team.rank(), team.size(), 0, d.N);
    if (d.cd.nc && !team_coarse_setup<Team, NS, KT>(team, d.cd, d.col, d.A)) return false;  // (ends with a barrier)
    if (!d.cd.nc && !team.sync()) return false;
    if (!team_ilu_apply_ell<Team, NS, KT>(team, d, il, d.b, d.r0)) return false;  // zb = M^-1 b
    if (d.cd.nc && !team_coarse_add<Team, NS, KT>(team, d.cd, d.b, d.r0, n)) return false;
    // the ILU sweeps end with a barrier; the coarse prolongation writes entry q on team rank q mod size
    auto op = [&](const KT* in, KT* out) -> bool {
      if (!team.sync()) return false;
      spmv_ell_rows<NS, KT>(d, in, il.y, 0, d.N, team.rank(), team.size());
      if (!team.sync()) return false;
      if (!team_ilu_apply_ell<Team, NS, KT>(team, d, il, il.y, out)) return false;
      return !d.cd.nc || team_coarse_add<Team, NS, KT>(team, d.cd, il.y, out, n);
    };
    return team_gmres_core(team, n, d.r0, d.x, d.r, d.gv, m, c, op, iters);
  } else {
    __shared__ Subdomain sd;
    if (threadIdx.x == 0) make_subdomain<NS, KT>(sd, d.N, team_cta(team), team_ncta(team), il);
    __syncthreads();
    const int64_t q0 = (int64_t)sd.K0 * NS, q1 = (int64_t)sd.K1 * NS;
    bilu_factor<NS, KT>(sd, d, il);
    pack_ell_rows<NS, KT>(d, sd.K0, sd.K1, threadIdx.x, blockDim.x);
    for (int cc = 0; cc < il.ncolors && cc < kMaxColors; ++cc)
      pack_ilu_positions<NS, KT>(il, d.N, sd.cb[cc], sd.ce[cc], threadIdx.x, blockDim.x, sd.K0, sd.K1);
    __syncthreads();
    if (d.cd.nc && !team_coarse_setup<Team, NS, KT>(team, d.cd, d.col, d.A)) return false;
    bilu_apply_ell<NS, KT>(sd, d, il, d.b, d.r0);  // zb = M^-1 b (subdomain-local)
    if (d.cd.nc && !team_coarse_add_range<Team, NS, KT>(team, d.cd, d.b, d.r0, q0, q1)) return false;
    if (!team.sync()) return false;  // zb is read in team-rank order below
    auto op = [&](const KT* in, KT* out) -> bool {
      if (!team.sync()) return false;
      spmv_ell_rows<NS, KT>(d, in, il.y, sd.K0, sd.K1, threadIdx.x, blockDim.x);
      __syncthreads();
      bilu_apply_ell<NS, KT>(sd, d, il, il.y, out);
      if (d.cd.nc && !team_coarse_add_range<Team, NS, KT>(team, d.cd, il.y, out, q0, q1)) return false;
      return team.sync();
    };
    return team_gmres_core(team, n, d.r0, d.x, d.r, d.gv, m, c, op, iters);
  }
}

}  // namespace vfvm
