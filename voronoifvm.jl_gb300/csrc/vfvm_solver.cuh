// Device-resident Newton + Krylov solver: state, work buffers, graph cache.
#pragma once
#include <map>
#include "vfvm_context.cuh"

namespace vfvm {

constexpr int kThreads = 256;
constexpr int kMaxRedBlocks = 608;  // 4 per SM on 152 SMs; bounds the reduction partials

// Solver control as the kernels read it (copied from vfvm_control before a launch).
struct DevControl {
  double abstol, reltol, tol_round, tol_mono, damp_initial, damp_growth;
  double reltol_linear, abstol_linear;
  int maxiters, max_round, is_linear, updatecontrol, maxiters_linear;
  int krylov, gmres_restart;  // VFVM_KRYLOV_*; GMRES basis size (persistent engine only)
  int batch_tail;              // sweep engine: end the BiCGStab loop once at most this many systems iterate
};

// Newton (solve_step!, src/vfvm_solver.jl:13-222) and BiCGStab state kept in
// device memory so the whole loop runs without the host.
struct DevState {
  // time, tstep^-1, embedding parameter (read by the assembly kernels), fixed step size
  double time, tstepinv, lambda, dt;
  // Newton
  double damp, oldnorm, tolx, rnorm, norm, resnorm, updnorm, dnorm;
  int niter, nround, finished, status, nlin, nnewton, abort, tot_newton;
  int tot_lin, nsteps, early, pad7;  // early: residual control met before the linear solve
  double maxdiff, pad5;
  // BiCGStab
  double rho, alpha, omega, beta, tol2, rr, bnorm2, pad2;
  int kit, kbreak, pad3, pad4;
  // reduction scratch: tickets
  unsigned ticket[8];
};

struct GraphKey {
  int precision, precon, kind, coarse;
  bool operator<(const GraphKey& o) const {
    if (precision != o.precision) return precision < o.precision;
    if (precon != o.precon) return precon < o.precon;
    if (kind != o.kind) return kind < o.kind;
    return coarse < o.coarse;
  }
};

template <typename KT>
struct KVecs {
  DBuf<KT> b, x, r, r0, p, ph, v, s, sh, t, dinv, ilu;
  DBuf<KT> ell_val, lo_val, up_val;  // ELL values (matrix, ILU0 L and U couplings), packed per Newton step
  DBuf<KT> gv;                       // GMRES basis, (restart + 1) x N*NS, allocated on first use
};

// Device-side step control of vfvm_evolve_device: the step loop of
// solve_transient! (src/vfvm_solver.jl:350-513) as a state record that a
// one-thread controller kernel advances after every tentative step, inside the
// step graph (graph kind 2), with no host round trip per step.
struct StepCtl {
  // settings
  double dl_min, dl_max, dl_grow, dl_dec, du_opt, du_max_factor, time0;
  const double* lambdas;  // nlam values
  double* Ustore;         // max_store solutions of n values
  double* tstore;         // max_store times / embedding values
  double* oldsol;         // the last accepted solution (start of every tentative step)
  int64_t n;
  int nlam, transient, num_final_steps, force_first_step, handle_exceptions, store_all, max_store, max_tries;
  // state
  double lam, lam0, dl, du;
  int i, istep, status, nstored, ntries, copy_old, store_slot, store_src;
};

struct Workspace {
  KVecs<double> k64;
  KVecs<float> k32;
  DBuf<double> partials;        // kMaxRedBlocks * 4
  DBuf<double> Uinit;           // initial value / old solution for the next solve
  DBuf<int> node_color;         // colour per node
  DBuf<int> color_nodes_ptr;    // unused placeholder for symmetry
  DevState* st = nullptr;       // device
  DevState* st_host = nullptr;  // pinned mirror
  DevControl* ctl = nullptr;    // device
  StepCtl* sc = nullptr;        // device step control (vfvm_evolve_device), allocated on first use
  cudaGraphConditionalHandle ncond{}, kcond{};
  std::map<GraphKey, cudaGraphExec_t> graphs;
  std::map<GraphKey, cudaGraph_t> graph_defs;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // persistent engine: barrier words, reduction partials, result record
  DBuf<unsigned> pbar;
  DBuf<double> ppartials;
  DBuf<char> pout;
};

// persistent engine (vfvm_persist.cu): one solve (nsteps == 0) or a fixed-step run
struct PersistRunHost {
  int nsteps;
  double time, tstep, lambda, t0, dt;
};
int persistent_solve(vfvm_ctx* c, const vfvm_control* ctl, const PersistRunHost& run, vfvm_history* hist, float* ms);

int ensure_workspace(vfvm_ctx* c, int precision);
// cached, instantiated Newton graph; kind 0 = solve from Uinit, kind 1 = fixed implicit Euler step,
// kind 2 = the whole step loop with device step control (ws->sc)
int get_graph(vfvm_ctx* c, int precision, int precon, int kind, cudaGraphExec_t* out);
int launch_maxdiff(vfvm_ctx* c, const double* a, const double* b);
DevControl make_devcontrol(const vfvm_control& c);

}  // namespace vfvm
