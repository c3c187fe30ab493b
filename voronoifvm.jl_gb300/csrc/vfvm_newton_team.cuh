// Team-generic damped Newton (solve_step!, src/vfvm_solver.jl:13-222) with
// the linear solve done by team BiCGStab or, in the single-system persistent
// kernel, GMRES (block-Jacobi, multicolour or subdomain ILU0).
// Runs inside one persistent launch: the whole grid for one system, or a group
// of CTAs per system in the batched solver.  Every decision of the Newton
// logic is taken redundantly by all threads from the same (deterministic)
// reduced values, so control flow stays uniform across the team.
#pragma once
#include "vfvm_assembly.cuh"
#include "vfvm_solver.cuh"
#include "vfvm_team_gmres.cuh"

namespace vfvm {

constexpr int kPersistThreads = 512;  // one 512-thread CTA per SM at <= 128 registers
constexpr int kPersistLPR = 8;

struct NewtonOut {
  int status, nnewton, nlin, nsteps;
  double updnorm, resnorm;
  int from_guess, pad_;  // guarded batch solves: 1 if the result was reached from the guess
};

template <class Ph, typename KT>
struct NewtonData {
  AsmTables t;
  double* U;
  double* Uold;
  double* F;
  KT* J;          // block matrix values written by the assembly
  KT* bw;         // right hand side (writable alias of kd.b)
  const uint8_t* dirdof;
  KrylovData<Ph::NS, KT> kd;
  IluData<KT> il;
  int64_t nvals;  // nnzb * NS * NS
};

// One Newton solve at (time, 1/tstep, lambda) from the values in nd.U (old
// time-step values in nd.Uold).  Returns false if a team barrier expired.
// guard: give up (VFVM_ERR_CONVERGENCE) as soon as an iteration fails to reduce
// the FP64 residual max-norm below that of the iteration before.
// GM: the kernel carries GMRES (ctl.krylov selects it; nd.kd.gv holds the basis).
template <class Team, class Ph, typename KT, int PRECON, bool GM = false>
__device__ bool team_newton(Team& team, const NewtonData<Ph, KT>& nd, const DevControl& ctl, double time,
                            double tstepinv, double lambda, NewtonOut& res, bool guard = false) {
  constexpr int NS = Ph::NS;
  const int N = nd.t.N;
  const int64_t n = (int64_t)N * NS;
  Ph ph;
  ph.load(nd.t.params);
  res.status = VFVM_OK;
  res.nnewton = 0;
  res.nlin = 0;
  // _initialize_dirichlet!
  for (int K = team.rank(); K < N; K += team.size()) init_dirichlet_node<Ph>(nd.t, ph, K, nd.U, time, lambda);
  double a1[1] = {0.0}, r1[1];
  if (!team.sync()) return false;
  for (int64_t q = team.rank(); q < n; q += team.size()) a1[0] += fabs(nd.U[q]);
  if (!team.template reduce<1>(a1, 0u, r1)) return false;
  double rnorm = r1[0];
  double damp = ctl.is_linear ? 1.0 : ctl.damp_initial;
  double oldnorm = 1.0, tolx = 0.0, norm = 0.0, prev_resnorm = INFINITY;
  int nround = 0, niter = 1;
  if (ctl.maxiters < 1) { res.status = VFVM_ERR_CONVERGENCE; return true; }
  const KrylovCtl kctl{ctl.reltol_linear, ctl.abstol_linear, ctl.maxiters_linear};
  while (true) {
    // eval_and_assemble
    int bad = 0;
    for (int K = team.rank(); K < N; K += team.size())
      if (assemble_node<Ph, KT, false>(nd.t, ph, K, nd.U, nd.Uold, time, tstepinv, lambda, nd.F, nd.J)) bad = 1;
    if (!team.sync()) return false;
    double a3[3] = {0.0, 0.0, double(bad)}, r3[3];
    for (int64_t q = team.rank(); q < n; q += team.size()) {
      const double f = nd.F[q];
      nd.bw[q] = KT(f);
      a3[0] += f * f;
      if (!nd.dirdof[q]) a3[1] = fmax(a3[1], fabs(f));
    }
    if (!team.template reduce<3>(a3, 6u, r3)) return false;
    res.resnorm = r3[1];
    if (r3[2] != 0.0 || isnan(r3[0])) { res.status = VFVM_ERR_ASSEMBLY; return true; }
    const double resnorm = r3[1];
    // residual control: the iterate already meets the tolerance, no linear solve
    if (!ctl.updatecontrol && !ctl.is_linear && (resnorm < ctl.abstol || resnorm < tolx)) break;
    if (guard) {
      if (res.nnewton > 0 && !(resnorm < prev_resnorm)) { res.status = VFVM_ERR_CONVERGENCE; return true; }
      prev_resnorm = resnorm;
    }
    // linear solve J x = F
    int kit = 0;
    bool ok = true, solved = false;
    if constexpr (GM) {
      if (ctl.krylov == VFVM_KRYLOV_GMRES) {
        ok = team_gmres<Team, NS, kPersistLPR, KT, PRECON>(team, nd.kd, nd.il, kctl, nd.nvals, ctl.gmres_restart, kit);
        solved = true;
      }
    }
    if (solved) {
    } else if (PRECON == VFVM_PRECON_JACOBI) {
      ok = team_bicgstab_jacobi<Team, NS, kPersistLPR, KT>(team, nd.kd, kctl, nullptr, &kit);
    } else if (PRECON == VFVM_PRECON_ILU0) {
      ok = team_bicgstab_ilu<Team, NS, kPersistLPR, KT>(team, nd.kd, nd.il, kctl, nd.nvals, kit);
    } else {
      ok = team_bicgstab_bilu<Team, NS, kPersistLPR, KT>(team, nd.kd, nd.il, kctl, kit);
    }
    if (!ok) return false;
    res.nlin += kit;
    // u -= damp * x
    double a2[2] = {0.0, 0.0}, r2[2];
    for (int64_t q = team.rank(); q < n; q += team.size()) {
      const double dx = double(nd.kd.x[q]);
      const double u = nd.U[q] - damp * dx;
      nd.U[q] = u;
      a2[0] = fmax(a2[0], fabs(dx));
      a2[1] += fabs(u);
    }
    if (!team.template reduce<2>(a2, 1u, r2)) return false;
    res.nnewton += 1;
    res.updnorm = r2[0];
    if (ctl.is_linear) break;
    damp = fmin(damp * ctl.damp_growth, 1.0);
    norm = ctl.updatecontrol ? r2[0] : resnorm;
    if (tolx == 0.0) tolx = norm * ctl.reltol;
    double dnorm = 1.0;
    const double rnorm_new = r2[1];
    if (rnorm > 1.0e-50) dnorm = fabs((rnorm - rnorm_new) / rnorm);
    nround = (dnorm < ctl.tol_round) ? nround + 1 : 0;
    if (niter > 1 && norm / oldnorm > 1.0 / ctl.tol_mono) { res.status = VFVM_ERR_CONVERGENCE; break; }
    if (norm < ctl.abstol || norm < tolx) break;
    oldnorm = norm;
    rnorm = rnorm_new;
    if (nround > ctl.max_round) break;
    niter += 1;
    if (niter > ctl.maxiters) { res.status = VFVM_ERR_CONVERGENCE; break; }
  }
  return true;
}

template <class Team>
__device__ __forceinline__ bool team_copy(Team& team, double* dst, const double* src, int64_t n) {
  for (int64_t q = team.rank(); q < n; q += team.size()) dst[q] = src[q];
  return team.sync();
}

// Fixed run of one system: nsteps == 0 -> one solve at (time, tstepinv, lambda);
// nsteps > 0 -> nsteps implicit Euler steps of size dt from t0 (Uold = U before each).
struct PersistRun {
  int nsteps;
  double time, tstepinv, lambda, t0, dt;
};

template <class Ph, typename KT, int PRECON>
__global__ void __launch_bounds__(kPersistThreads, 1) newton_persistent_kernel(NewtonData<Ph, KT> nd, DevControl ctl,
                                                                            GridSync gs, PersistRun run,
                                                                            NewtonOut* out) {
  GroupTeam team = grid_team(gs);
  NewtonOut tot{VFVM_OK, 0, 0, 0, 0.0, 0.0};
  bool ok = true;
  if (run.nsteps == 0) {
    ok = team_newton<GroupTeam, Ph, KT, PRECON, true>(team, nd, ctl, run.time, run.tstepinv, run.lambda, tot);
  } else {
    const int64_t n = (int64_t)nd.t.N * Ph::NS;
    double time = run.t0;
    for (int step = 0; step < run.nsteps && ok; ++step) {
      for (int64_t q = team.rank(); q < n; q += team.size()) nd.Uold[q] = nd.U[q];
      if (!(ok = team.sync())) break;
      time += run.dt;
      NewtonOut one;
      ok = team_newton<GroupTeam, Ph, KT, PRECON, true>(team, nd, ctl, time, 1.0 / run.dt, 0.0, one);
      tot.nnewton += one.nnewton;
      tot.nlin += one.nlin;
      tot.updnorm = one.updnorm;
      tot.resnorm = one.resnorm;
      tot.status = one.status;
      if (!ok || one.status != VFVM_OK) break;
      tot.nsteps += 1;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (!ok) tot.status = VFVM_ERR_TIMEOUT;
    *out = tot;
  }
}

// Batched: the grid is split into groups of `gsize` CTAs; each group takes the
// next system from a queue (largest first) and solves it with team_newton.
struct BatchSync {
  GridSync gs;    // the group's barrier words and partials
  int* slot;      // the group's current queue position
};

template <class Ph, typename KT, int PRECON>
__global__ void __launch_bounds__(kPersistThreads, 1) newton_batch_kernel(const NewtonData<Ph, KT>* __restrict__ insts,
                                                                       int ninst, const int* __restrict__ order,
                                                                       DevControl ctl, const BatchSync* __restrict__ groups,
                                                                       int gsize, unsigned* queue, double time,
                                                                       double tstepinv, double lambda, NewtonOut* outs,
                                                                       int* failed, const double* guess,
                                                                       const double* fallback, const double* ubase) {
  const int group = blockIdx.x / gsize;
  const BatchSync bs = groups[group];
  GroupTeam team{bs.gs, gsize, (int)(blockIdx.x % gsize), 0u};
  __shared__ int pos_sh;
  while (true) {
    if (team.bid == 0 && threadIdx.x == 0) *((volatile int*)bs.slot) = (int)atomicAdd(queue, 1u);
    if (!team.sync()) { if (threadIdx.x == 0) atomicExch(failed, 1); return; }
    if (threadIdx.x == 0) pos_sh = *((volatile int*)bs.slot);
    __syncthreads();
    const int pos = pos_sh;
    // everyone has read the slot before the leader may overwrite it
    if (!team.sync()) { if (threadIdx.x == 0) atomicExch(failed, 1); return; }
    if (pos >= ninst) return;
    const int inst = order[pos];
    const NewtonData<Ph, KT>& nd = insts[inst];
    NewtonOut res;
    bool ok = true;
    int from_guess = 0;
    if (guess) {
      // guarded start: Newton from the guess while every iteration reduces the
      // FP64 residual; if it does not (or fails otherwise), plain Newton from
      // the fallback (the caller's inival)
      const int64_t off = nd.U - ubase, n = (int64_t)nd.t.N * Ph::NS;
      ok = team_copy(team, nd.U, guess + off, n) &&
           team_newton<GroupTeam, Ph, KT, PRECON>(team, nd, ctl, time, tstepinv, lambda, res, true);
      from_guess = 1;
      if (ok && res.status != VFVM_OK) {
        const int nn = res.nnewton, nl = res.nlin;
        from_guess = 0;
        ok = team_copy(team, nd.U, fallback + off, n) &&
             team_newton<GroupTeam, Ph, KT, PRECON>(team, nd, ctl, time, tstepinv, lambda, res);
        res.nnewton += nn;
        res.nlin += nl;
      }
    } else {
      ok = team_newton<GroupTeam, Ph, KT, PRECON>(team, nd, ctl, time, tstepinv, lambda, res);
    }
    res.from_guess = from_guess;
    if (!ok) { if (threadIdx.x == 0) atomicExch(failed, 1); return; }
    if (team.bid == 0 && threadIdx.x == 0) outs[inst] = res;
  }
}

}  // namespace vfvm
