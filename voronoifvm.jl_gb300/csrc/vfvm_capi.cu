// C ABI entry points: assembly, Newton solve, time/embedding evolution.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>
#include "vfvm_solver.cuh"
#include "vfvm_physics.cuh"

using namespace vfvm;

namespace {

// Below this many unknowns a solve is launch-latency bound: the one-launch
// persistent engine wins; above it the per-phase graph kernels (full occupancy) win.
constexpr int64_t kAutoPersistentDofs = 16384;

// Write {time, 1/tstep, lambda} (and abort = 0) into the device state.
int set_time(vfvm_ctx* c, double time, double tstep, double lambda) {
  Workspace* w = c->ws;
  DevState* h = w->st_host;
  h->time = time;
  h->tstepinv = 1.0 / tstep;  // 1/Inf = 0: stationary (src/vfvm_assembly.jl:550-554)
  h->lambda = lambda;
  VFVM_CUDA(cudaMemcpyAsync(&w->st->time, &h->time, 3 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  return VFVM_OK;
}

int set_control(vfvm_ctx* c, const vfvm_control* ctl) {
  if (ctl->precon == VFVM_PRECON_BLOCK_ILU0 && c->ncolors > kMaxBlockIluColors) return VFVM_ERR_INPUT;
  // GMRES runs on the single-system persistent engine only
  if (ctl->krylov == VFVM_KRYLOV_GMRES && (c->multireg || ctl->engine == VFVM_ENGINE_GRAPH)) return VFVM_ERR_INPUT;
  if (int rc = ensure_coarse(c, ctl->coarse)) return rc;
  static thread_local DevControl staged;
  staged = make_devcontrol(*ctl);
  VFVM_CUDA(cudaMemcpyAsync(c->ws->ctl, &staged, sizeof(DevControl), cudaMemcpyHostToDevice, c->stream));
  VFVM_CUDA(cudaStreamSynchronize(c->stream));
  return VFVM_OK;
}

int check_control(const vfvm_control* ctl) {
  if (!ctl) return VFVM_ERR_INPUT;
  if (ctl->precision != VFVM_PRECISION_FP64 && ctl->precision != VFVM_PRECISION_MIXED) return VFVM_ERR_INPUT;
  if (ctl->precon != VFVM_PRECON_JACOBI && ctl->precon != VFVM_PRECON_ILU0 && ctl->precon != VFVM_PRECON_BLOCK_ILU0)
    return VFVM_ERR_INPUT;
  if (ctl->krylov != VFVM_KRYLOV_BICGSTAB && ctl->krylov != VFVM_KRYLOV_GMRES) return VFVM_ERR_INPUT;
  if (ctl->krylov == VFVM_KRYLOV_GMRES && (ctl->gmres_restart < 1 || ctl->gmres_restart > VFVM_GMRES_MAX_RESTART))
    return VFVM_ERR_INPUT;
  if (ctl->coarse < 0 || ctl->coarse > VFVM_COARSE_MAX) return VFVM_ERR_INPUT;
  return VFVM_OK;
}

// Runs the Newton graph once from ws->Uinit (already on the device) at the time
// values set in the state; leaves the result in c->U and the state in st_host.
bool use_persistent(const vfvm_ctx* c, const vfvm_control* ctl) {
  if (c->multireg) return false;
  if (ctl->krylov == VFVM_KRYLOV_GMRES) return true;
  if (ctl->engine == VFVM_ENGINE_AUTO) return (int64_t)c->N * c->ns <= kAutoPersistentDofs;
  return ctl->engine == VFVM_ENGINE_PERSISTENT;
}

int run_newton(vfvm_ctx* c, const vfvm_control* ctl, float* ms) {
  Workspace* w = c->ws;
  if (use_persistent(c, ctl)) {
    const size_t n = (size_t)c->N * c->ns;
    VFVM_CUDA(cudaMemcpyAsync(c->U.p, w->Uinit.p, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    VFVM_CUDA(cudaMemcpyAsync(c->Uold.p, w->Uinit.p, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    const DevState* h = w->st_host;
    PersistRunHost run{0, h->time, 1.0 / h->tstepinv, h->lambda, 0.0, 0.0};
    return persistent_solve(c, ctl, run, nullptr, ms);
  }
  cudaGraphExec_t exec;
  int rc = get_graph(c, ctl->precision, ctl->precon, 0, &exec);
  if (rc != VFVM_OK) return rc;
  VFVM_CUDA(cudaMemsetAsync(&w->st->abort, 0, sizeof(int), c->stream));
  VFVM_CUDA(cudaEventRecord(w->ev0, c->stream));
  VFVM_CUDA(cudaGraphLaunch(exec, c->stream));
  VFVM_CUDA(cudaEventRecord(w->ev1, c->stream));
  VFVM_CUDA(cudaMemcpyAsync(w->st_host, w->st, sizeof(DevState), cudaMemcpyDeviceToHost, c->stream));
  VFVM_CUDA(cudaStreamSynchronize(c->stream));
  if (ms) VFVM_CUDA(cudaEventElapsedTime(ms, w->ev0, w->ev1));
  return w->st_host->status;
}

void fill_history(const DevState* h, vfvm_history* hist, float ms, bool accumulate) {
  if (!hist) return;
  if (!accumulate) std::memset(hist, 0, sizeof(*hist));
  hist->nnewton += h->nnewton;
  hist->nlin += h->nlin;
  hist->status = h->status;
  hist->updatenorm = h->updnorm;
  hist->resnorm = h->resnorm;
  hist->time_ms += ms;
}

}  // namespace

extern "C" int vfvm_init_dirichlet(vfvm_ctx* c, double* U, double time, double lambda) {
  if (!c || !U) return VFVM_ERR_INPUT;
  int rc = ensure_workspace(c, VFVM_PRECISION_FP64);
  if (rc) return rc;
  const size_t n = (size_t)c->N * c->ns;
  if ((rc = set_time(c, time, INFINITY, lambda))) return rc;
  VFVM_CUDA(cudaMemcpyAsync(c->U.p, U, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  if ((rc = launch_init_dirichlet(c, c->U.p, &c->ws->st->time, c->stream))) return rc;
  VFVM_CUDA(cudaMemcpyAsync(U, c->U.p, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  VFVM_CUDA(cudaStreamSynchronize(c->stream));
  return VFVM_OK;
}

extern "C" int vfvm_assemble(vfvm_ctx* c, const double* U, const double* Uold, double time, double tstep,
                             double lambda, double* F, double* Jvals) {
  if (!c || !U) return VFVM_ERR_INPUT;
  int rc = ensure_workspace(c, VFVM_PRECISION_FP64);
  if (rc) return rc;
  const size_t n = (size_t)c->N * c->ns;
  if ((rc = set_time(c, time, tstep, lambda))) return rc;
  VFVM_CUDA(cudaMemcpyAsync(c->U.p, U, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  VFVM_CUDA(cudaMemcpyAsync(c->Uold.p, Uold ? Uold : U, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  VFVM_CUDA(cudaMemsetAsync(c->errflag.p, 0, sizeof(int), c->stream));
  if ((rc = launch_assemble(c, c->U.p, c->Uold.p, &c->ws->st->time, c->F.p, c->J.p, nullptr, c->stream))) return rc;
  if (F) VFVM_CUDA(cudaMemcpyAsync(F, c->F.p, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (Jvals && c->nnz > 0) {
    DBuf<double> out;  // scalar-pattern values, gathered from the block matrix
    VFVM_CUDA(out.alloc((size_t)c->nnz));
    if ((rc = launch_pattern_gather(c, c->J.p, out.p, c->stream))) return rc;
    VFVM_CUDA(cudaMemcpyAsync(Jvals, out.p, (size_t)c->nnz * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    VFVM_CUDA(cudaStreamSynchronize(c->stream));
  }
  int err = 0;
  VFVM_CUDA(cudaMemcpyAsync(&err, c->errflag.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  VFVM_CUDA(cudaStreamSynchronize(c->stream));
  return err ? VFVM_ERR_ASSEMBLY : VFVM_OK;
}

extern "C" int vfvm_assemble_device(vfvm_ctx* c, const double* U_dev, const double* Uold_dev, double time,
                                    double tstep, double lambda, double* F_dev, int32_t precision) {
  if (!c || !U_dev || !F_dev) return VFVM_ERR_INPUT;
  if (precision != VFVM_PRECISION_FP64 && precision != VFVM_PRECISION_MIXED) return VFVM_ERR_INPUT;
  int rc = ensure_workspace(c, precision);
  if (rc) return rc;
  if ((rc = set_time(c, time, tstep, lambda))) return rc;
  if (precision == VFVM_PRECISION_FP64)
    return launch_assemble(c, U_dev, Uold_dev ? Uold_dev : U_dev, &c->ws->st->time, F_dev, c->J.p, nullptr, c->stream);
  return launch_assemble(c, U_dev, Uold_dev ? Uold_dev : U_dev, &c->ws->st->time, F_dev, nullptr, c->Jf.p, c->stream);
}

extern "C" int vfvm_solve_device(vfvm_ctx* c, const vfvm_control* ctl, const double* inival_dev, double* U_dev,
                                 double time, double tstep, double lambda, vfvm_history* hist) {
  if (!c || !inival_dev || !U_dev) return VFVM_ERR_INPUT;
  int rc = check_control(ctl);
  if (rc) return rc;
  if ((rc = ensure_workspace(c, ctl->precision))) return rc;
  const size_t n = (size_t)c->N * c->ns;
  if ((rc = set_control(c, ctl))) return rc;
  if ((rc = set_time(c, time, tstep, lambda))) return rc;
  VFVM_CUDA(cudaMemcpyAsync(c->ws->Uinit.p, inival_dev, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  float ms = 0;
  rc = run_newton(c, ctl, &ms);
  VFVM_CUDA(cudaMemcpyAsync(U_dev, c->U.p, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  VFVM_CUDA(cudaStreamSynchronize(c->stream));
  fill_history(c->ws->st_host, hist, ms, false);
  return rc;
}

extern "C" int vfvm_solve(vfvm_ctx* c, const vfvm_control* ctl, const double* inival, double* U, double time,
                          double tstep, double lambda, vfvm_history* hist) {
  if (!c || !inival || !U) return VFVM_ERR_INPUT;
  int rc = check_control(ctl);
  if (rc) return rc;
  if ((rc = ensure_workspace(c, ctl->precision))) return rc;
  const size_t n = (size_t)c->N * c->ns;
  if ((rc = set_control(c, ctl))) return rc;
  if ((rc = set_time(c, time, tstep, lambda))) return rc;
  VFVM_CUDA(cudaMemcpyAsync(c->ws->Uinit.p, inival, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  float ms = 0;
  rc = run_newton(c, ctl, &ms);
  VFVM_CUDA(cudaMemcpyAsync(U, c->U.p, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  VFVM_CUDA(cudaStreamSynchronize(c->stream));
  fill_history(c->ws->st_host, hist, ms, false);
  return rc;
}

// Fixed-step implicit Euler on the device: nsteps launches of the step graph,
// no host synchronisation in between.  U_dev holds the initial value on entry
// and the final solution on return.
extern "C" int vfvm_evolve_fixed_device(vfvm_ctx* c, const vfvm_control* ctl, double* U_dev, double t0, double dt,
                                        int32_t nsteps, vfvm_history* hist) {
  if (!c || !U_dev || nsteps < 0 || !(dt > 0)) return VFVM_ERR_INPUT;
  int rc = check_control(ctl);
  if (rc) return rc;
  if ((rc = ensure_workspace(c, ctl->precision))) return rc;
  Workspace* w = c->ws;
  const size_t n = (size_t)c->N * c->ns;
  if ((rc = set_control(c, ctl))) return rc;
  if (use_persistent(c, ctl)) {
    VFVM_CUDA(cudaMemcpyAsync(c->U.p, U_dev, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    PersistRunHost run{nsteps, t0, dt, 0.0, t0, dt};
    float ms = 0;
    rc = persistent_solve(c, ctl, run, hist, &ms);
    VFVM_CUDA(cudaMemcpyAsync(U_dev, c->U.p, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    VFVM_CUDA(cudaStreamSynchronize(c->stream));
    return rc;
  }
  cudaGraphExec_t exec;
  if ((rc = get_graph(c, ctl->precision, ctl->precon, 1, &exec))) return rc;
  DevState* h = w->st_host;
  std::memset(h, 0, sizeof(DevState));
  h->time = t0;
  h->tstepinv = 1.0 / dt;
  h->lambda = 0.0;
  h->dt = dt;
  VFVM_CUDA(cudaMemcpyAsync(w->st, h, sizeof(DevState), cudaMemcpyHostToDevice, c->stream));
  VFVM_CUDA(cudaMemcpyAsync(c->U.p, U_dev, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  VFVM_CUDA(cudaEventRecord(w->ev0, c->stream));
  for (int k = 0; k < nsteps; ++k) VFVM_CUDA(cudaGraphLaunch(exec, c->stream));
  VFVM_CUDA(cudaEventRecord(w->ev1, c->stream));
  VFVM_CUDA(cudaMemcpyAsync(U_dev, c->U.p, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  VFVM_CUDA(cudaMemcpyAsync(h, w->st, sizeof(DevState), cudaMemcpyDeviceToHost, c->stream));
  VFVM_CUDA(cudaStreamSynchronize(c->stream));
  float ms = 0;
  VFVM_CUDA(cudaEventElapsedTime(&ms, w->ev0, w->ev1));
  if (hist) {
    std::memset(hist, 0, sizeof(*hist));
    hist->nnewton = h->tot_newton;
    hist->nlin = h->tot_lin;
    hist->nsteps = h->abort ? 0 : nsteps;
    hist->status = h->status;
    hist->updatenorm = h->updnorm;
    hist->resnorm = h->resnorm;
    hist->time_ms = ms;
  }
  return h->status;
}

// solve_transient! (src/vfvm_solver.jl:267-537): implicit Euler (transient) or
// parameter embedding with the reference's step-size control.  Each step is one
// device-resident Newton solve; the step logic itself is host code as in the
// reference.
extern "C" int vfvm_evolve(vfvm_ctx* c, const vfvm_control* ctl, const double* inival, const double* lambdas,
                           int32_t nlambdas, int32_t transient, double time, double* U_store, double* t_store,
                           int32_t max_store, int32_t* nstored, vfvm_history* hist) {
  if (!c || !inival || !lambdas || nlambdas < 1 || !nstored) return VFVM_ERR_INPUT;
  int rc = check_control(ctl);
  if (rc) return rc;
  if ((rc = ensure_workspace(c, ctl->precision))) return rc;
  if ((rc = set_control(c, ctl))) return rc;
  Workspace* w = c->ws;
  const size_t n = (size_t)c->N * c->ns;
  DBuf<double> oldsol;
  VFVM_CUDA(oldsol.alloc(n));
  if (hist) std::memset(hist, 0, sizeof(*hist));
  *nstored = 0;
  auto store = [&](double t, const double* Udev) -> int {
    if (*nstored < max_store) {
      if (U_store) VFVM_CUDA(cudaMemcpyAsync(U_store + (size_t)(*nstored) * n, Udev, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
      if (t_store) t_store[*nstored] = t;
      (*nstored)++;
    } else if (U_store && max_store > 0) {  // keep the last solution in the last slot
      VFVM_CUDA(cudaMemcpyAsync(U_store + (size_t)(max_store - 1) * n, Udev, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
      if (t_store) t_store[max_store - 1] = t;
    }
    return VFVM_OK;
  };
  auto isapprox = [](double a, double b, double rtol, double atol) {
    return a == b || (std::isfinite(a) && std::isfinite(b) && std::fabs(a - b) <= std::max(atol, rtol * std::max(std::fabs(a), std::fabs(b))));
  };
  const double sqeps = 1.4901161193847656e-8;
  double dl, dl_min, dl_max, dl_grow, dl_dec;
  if (transient) { dl = ctl->dt; dl_min = ctl->dt_min; dl_max = ctl->dt_max; dl_grow = ctl->dt_grow; dl_dec = ctl->dt_decrease; }
  else { dl = ctl->dp; dl_min = ctl->dp_min; dl_max = ctl->dp_max; dl_grow = ctl->dp_grow; dl_dec = ctl->dp_decrease; }
  const double du_opt = ctl->du_opt, du_max_factor = ctl->du_max_factor;
  float ms = 0;
  // initial value (Dirichlet-initialised) or first embedding solve
  VFVM_CUDA(cudaMemcpyAsync(oldsol.p, inival, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  if (transient) {
    VFVM_CUDA(cudaMemcpyAsync(c->U.p, oldsol.p, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    if ((rc = store(lambdas[0], c->U.p))) return rc;
  } else {
    if ((rc = set_time(c, time, INFINITY, lambdas[0]))) return rc;
    VFVM_CUDA(cudaMemcpyAsync(w->Uinit.p, oldsol.p, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    rc = run_newton(c, ctl, &ms);
    fill_history(w->st_host, hist, ms, true);
    if (rc != VFVM_OK) return rc;
    VFVM_CUDA(cudaMemcpyAsync(oldsol.p, c->U.p, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    if ((rc = store(lambdas[0], c->U.p))) return rc;
  }
  int istep = 0;
  bool solved = false;
  double lam = lambdas[0], lam0 = lam;
  int final_status = VFVM_OK;
  for (int i = 0; i + 1 < nlambdas; ++i) {
    dl = std::max(dl, dl_min);
    const double lend = lambdas[i + 1];
    lam = lambdas[i];
    while (lam < lend) {
      solved = false;
      lam0 = lam;
      double du = 0.0;
      bool giveup = false;
      while (!solved) {
        solved = true;
        bool errored = false;
        lam = lam0 + dl;
        if (transient) { if ((rc = set_time(c, lam, dl, 0.0))) return rc; }
        else { if ((rc = set_time(c, time, INFINITY, lam))) return rc; }
        VFVM_CUDA(cudaMemcpyAsync(w->Uinit.p, oldsol.p, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
        rc = run_newton(c, ctl, &ms);
        fill_history(w->st_host, hist, ms, true);
        if (rc == VFVM_ERR_CUDA || rc == VFVM_ERR_INPUT) return rc;
        if (rc != VFVM_OK) {
          if (!ctl->handle_exceptions) return rc;
          solved = false;
          errored = true;
        }
        if (solved) {
          if ((rc = launch_maxdiff(c, c->U.p, oldsol.p))) return rc;
          VFVM_CUDA(cudaMemcpyAsync(&w->st_host->maxdiff, &w->st->maxdiff, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
          VFVM_CUDA(cudaStreamSynchronize(c->stream));
          du = w->st_host->maxdiff;
          if (du > du_max_factor * du_opt) solved = false;
        }
        if (!solved) {
          if (isapprox(dl, dl_min, sqeps, 0.0)) {
            if (!(ctl->force_first_step && istep == 0)) {
              final_status = VFVM_ERR_EMBEDDING;
              if (!ctl->handle_exceptions) return final_status;
              giveup = true;
              break;
            } else if (!errored) {
              solved = true;
            } else {
              final_status = VFVM_ERR_EMBEDDING;
              if (!ctl->handle_exceptions) return final_status;
              giveup = true;
              break;
            }
          } else {
            dl = std::max(dl_min, dl * dl_dec);
          }
        }
      }
      if (giveup) { solved = false; break; }
      if (solved) {
        istep++;
        if (hist) hist->nsteps++;
        if (ctl->store_all) if ((rc = store(lam, c->U.p))) return rc;
        VFVM_CUDA(cudaMemcpyAsync(oldsol.p, c->U.p, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
        const double steps_to_go = std::ceil((lend - lam) / dl);
        double lam_predict = lend - lam;
        if (steps_to_go < ctl->num_final_steps) lam_predict = steps_to_go > 0 ? (lend - lam) / steps_to_go : NAN;
        if (isapprox(dl_max, dl_min, sqeps, 0.0)) lam_predict = dl_max;
        if (lam < lend) {
          dl = std::min({dl_max, dl * dl_grow, dl * du_opt / (du + 1.0e-14), lam_predict, lend - lam});
          if (isapprox(lam + dl, lend, 1.0e-15, 1.0e-15)) dl = lend - lam;
        }
      }
    }
    if (!ctl->store_all) if ((rc = store(lam0, oldsol.p))) return rc;
    if (!solved) break;
  }
  VFVM_CUDA(cudaStreamSynchronize(c->stream));
  if (hist) hist->status = final_status;
  return final_status;
}

// tentative steps (accepted or rejected) of one vfvm_evolve_device call at most;
// beyond them the call returns VFVM_ERR_EMBEDDING
constexpr int kMaxDeviceSteps = 1 << 18;

// solve_transient! with the step control on the device: the whole step loop is
// one launch of the step graph (graph kind 2), with no host round trip per step;
// the stored solutions stay on the device until the loop ends.  Same decisions
// as vfvm_evolve (src/vfvm_solver.jl:350-513); lambdas must increase strictly.
// host_syncs (optional) receives the number of host synchronisations of the
// call: 3 for implicit Euler (set-up, end of the loop, stored solutions), 4 for
// embedding (the first solve at lambdas[0] comes before the loop), whatever
// the number of steps.
extern "C" int vfvm_evolve_device(vfvm_ctx* c, const vfvm_control* ctl, const double* inival, const double* lambdas,
                                  int32_t nlambdas, int32_t transient, double time, double* U_store,
                                  double* t_store, int32_t max_store, int32_t* nstored, vfvm_history* hist,
                                  int32_t* host_syncs) {
  if (!c || !inival || !lambdas || nlambdas < 1 || !nstored || max_store < 1 || !U_store || !t_store)
    return VFVM_ERR_INPUT;
  for (int i = 0; i + 1 < nlambdas; ++i)
    if (!(lambdas[i] < lambdas[i + 1])) return VFVM_ERR_INPUT;
  int rc = check_control(ctl);
  if (rc) return rc;
  if (ctl->krylov == VFVM_KRYLOV_GMRES) return VFVM_ERR_INPUT;  // the step graph runs BiCGStab
  if ((rc = ensure_workspace(c, ctl->precision))) return rc;
  if ((rc = set_control(c, ctl))) return rc;  // (one synchronisation)
  int syncs = 1;
  Workspace* w = c->ws;
  const size_t n = (size_t)c->N * c->ns;
  if (!w->sc) VFVM_CUDA(cudaMalloc(&w->sc, sizeof(StepCtl)));
  DBuf<double> dlam, ustore, tstore;
  VFVM_CUDA(dlam.alloc((size_t)nlambdas));
  VFVM_CUDA(ustore.alloc((size_t)max_store * n));
  VFVM_CUDA(tstore.alloc((size_t)max_store));
  VFVM_CUDA(cudaMemcpyAsync(dlam.p, lambdas, (size_t)nlambdas * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  if (hist) std::memset(hist, 0, sizeof(*hist));

  StepCtl h;
  std::memset(&h, 0, sizeof(h));
  if (transient) {
    h.dl = ctl->dt; h.dl_min = ctl->dt_min; h.dl_max = ctl->dt_max; h.dl_grow = ctl->dt_grow; h.dl_dec = ctl->dt_decrease;
  } else {
    h.dl = ctl->dp; h.dl_min = ctl->dp_min; h.dl_max = ctl->dp_max; h.dl_grow = ctl->dp_grow; h.dl_dec = ctl->dp_decrease;
  }
  h.du_opt = ctl->du_opt; h.du_max_factor = ctl->du_max_factor; h.time0 = time;
  h.lambdas = dlam.p; h.Ustore = ustore.p; h.tstore = tstore.p; h.oldsol = w->Uinit.p; h.n = (int64_t)n;
  h.nlam = nlambdas; h.transient = transient ? 1 : 0; h.num_final_steps = ctl->num_final_steps;
  h.force_first_step = ctl->force_first_step; h.handle_exceptions = ctl->handle_exceptions;
  h.store_all = ctl->store_all; h.max_store = max_store; h.max_tries = kMaxDeviceSteps;
  h.status = VFVM_OK; h.store_slot = -1;

  // the start value: u_old of the first step (after a first solve at lambdas[0] when embedding)
  VFVM_CUDA(cudaMemcpyAsync(w->Uinit.p, inival, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  float ms = 0;
  if (!transient) {
    if ((rc = set_time(c, time, INFINITY, lambdas[0]))) return rc;
    rc = run_newton(c, ctl, &ms);  // (one synchronisation)
    ++syncs;
    fill_history(w->st_host, hist, ms, true);
    if (rc != VFVM_OK) return rc;
    VFVM_CUDA(cudaMemcpyAsync(w->Uinit.p, c->U.p, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  }
  VFVM_CUDA(cudaMemcpyAsync(ustore.p, w->Uinit.p, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  VFVM_CUDA(cudaMemcpyAsync(tstore.p, &lambdas[0], sizeof(double), cudaMemcpyHostToDevice, c->stream));
  h.nstored = 1;
  static thread_local StepCtl staged;
  staged = h;
  VFVM_CUDA(cudaMemcpyAsync(w->sc, &staged, sizeof(StepCtl), cudaMemcpyHostToDevice, c->stream));
  {  // Newton totals of the step loop start from zero
    DevState* hs = w->st_host;
    std::memset(hs, 0, sizeof(DevState));
    VFVM_CUDA(cudaMemcpyAsync(w->st, hs, sizeof(DevState), cudaMemcpyHostToDevice, c->stream));
  }
  cudaGraphExec_t exec;
  if ((rc = get_graph(c, ctl->precision, ctl->precon, 2, &exec))) return rc;
  VFVM_CUDA(cudaEventRecord(w->ev0, c->stream));
  VFVM_CUDA(cudaGraphLaunch(exec, c->stream));
  VFVM_CUDA(cudaEventRecord(w->ev1, c->stream));
  VFVM_CUDA(cudaMemcpyAsync(&staged, w->sc, sizeof(StepCtl), cudaMemcpyDeviceToHost, c->stream));
  VFVM_CUDA(cudaMemcpyAsync(w->st_host, w->st, sizeof(DevState), cudaMemcpyDeviceToHost, c->stream));
  VFVM_CUDA(cudaStreamSynchronize(c->stream));
  ++syncs;
  h = staged;
  VFVM_CUDA(cudaEventElapsedTime(&ms, w->ev0, w->ev1));
  const int nst = std::min(h.nstored, max_store);
  VFVM_CUDA(cudaMemcpyAsync(U_store, ustore.p, (size_t)nst * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  VFVM_CUDA(cudaMemcpyAsync(t_store, tstore.p, (size_t)nst * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  VFVM_CUDA(cudaStreamSynchronize(c->stream));
  ++syncs;
  *nstored = nst;
  if (hist) {
    hist->nnewton += w->st_host->tot_newton;
    hist->nlin += w->st_host->tot_lin;
    hist->nsteps = h.istep;
    hist->status = h.status;
    hist->updatenorm = w->st_host->updnorm;
    hist->resnorm = w->st_host->resnorm;
    hist->time_ms += ms;
  }
  if (host_syncs) *host_syncs = syncs;
  return h.status;
}
