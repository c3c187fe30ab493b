// Host entry points of the persistent engine and of the batched solver: one
// system per cooperative launch, or many systems of uneven size in one
// cooperative launch (a group of CTAs per system, largest systems first).
#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>
#include "vfvm_persist.cuh"
#include "vfvm_physics.cuh"
#include "vfvm_newton_team.cuh"

namespace vfvm {

int persistent_solve(vfvm_ctx* c, const vfvm_control* ctl, const PersistRunHost& run, vfvm_history* hist, float* ms) {
  if (c->multireg) return VFVM_ERR_INPUT;
  return dispatch_physics(c->phys, [&](auto ph) { return persistent_solve_t<decltype(ph)>(c, ctl, run, hist, ms); });
}

}  // namespace vfvm

// ---------------------------------------------------------------------------
// batched solver
// ---------------------------------------------------------------------------
using namespace vfvm;


extern "C" vfvm_batch* vfvm_batch_create(int32_t ninst, const vfvm_grid* grids, const vfvm_physics_desc* phys,
                                         int* status) {
  int dummy;
  if (!status) status = &dummy;
  *status = VFVM_ERR_INPUT;
  if (ninst < 1 || !grids || !phys) return nullptr;
  for (int i = 1; i < ninst; ++i)
    if (phys[i].physics_id != phys[0].physics_id) return nullptr;  // one device functor per batch
  vfvm_batch* b = new vfvm_batch;
  b->ninst = ninst;
  b->phys = phys[0].physics_id;
  b->offsets.assign(ninst + 1, 0);
  // systems that all use the same grid arrays (and coordinate system) share one set of device tables
  bool shared = true;
  for (int i = 1; i < ninst && shared; ++i)
    shared = grids[i].dim == grids[0].dim && grids[i].nnodes == grids[0].nnodes && grids[i].ncells == grids[0].ncells &&
             grids[i].nbfaces == grids[0].nbfaces && grids[i].coord == grids[0].coord &&
             grids[i].cellnodes == grids[0].cellnodes && grids[i].cellregions == grids[0].cellregions &&
             grids[i].bfacenodes == grids[0].bfacenodes && grids[i].bfaceregions == grids[0].bfaceregions &&
             grids[i].coordsystem == grids[0].coordsystem;
  for (int i = 0; i < ninst; ++i) {
    int st = 0;
    b->shared_grid = shared;
    vfvm_ctx* c = (shared && i > 0) ? clone_context(b->ctx[0], &phys[i], &st) : vfvm_create(&grids[i], &phys[i], &st);
    if (!c || c->multireg) {
      if (c) vfvm_destroy(c);
      *status = c ? VFVM_ERR_INPUT : st;
      delete b;
      return nullptr;
    }
    b->ctx.push_back(c);
    b->ns = c->ns;
    b->offsets[i + 1] = b->offsets[i] + (int64_t)c->N * c->ns;
  }
  std::vector<int> order(ninst);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return b->ctx[a]->N > b->ctx[c]->N; });
  if (b->order.upload(order) != cudaSuccess || b->U.alloc(b->offsets[ninst]) != cudaSuccess ||
      b->Uold.alloc(b->offsets[ninst]) != cudaSuccess || b->queue.alloc(1) != cudaSuccess ||
      b->failed.alloc(1) != cudaSuccess || b->outs.alloc(sizeof(NewtonOut) * ninst) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&b->e0) != cudaSuccess || cudaEventCreate(&b->e1) != cudaSuccess) {
    *status = VFVM_ERR_CUDA;
    delete b;
    return nullptr;
  }
  *status = VFVM_OK;
  return b;
}

extern "C" void vfvm_batch_destroy(vfvm_batch* b) {
  if (!b) return;
  if (b->stream) cudaStreamSynchronize(b->stream);
  delete b;
}

extern "C" int vfvm_batch_set_instance(vfvm_batch* b, int32_t inst, const double* params, int32_t nparams,
                                       const double* nodedata, int32_t nnodedata) {
  if (!b || inst < 0 || inst >= b->ninst) return VFVM_ERR_INPUT;
  vfvm_ctx* c = b->ctx[inst];
  int rc = VFVM_OK;
  if (params && (rc = vfvm_set_params(c, params, nparams))) return rc;
  if (nodedata && (rc = set_nodedata(c, nodedata, nnodedata))) return rc;
  b->desc_precision = -1;  // descriptors are rebuilt before the next solve
  if (b->sweep) b->sweep->valid = false;
  return VFVM_OK;
}

extern "C" int vfvm_batch_info(vfvm_batch* b, int64_t out[7]) {
  if (!b || !out) return VFVM_ERR_INPUT;
  out[0] = b->ninst;
  out[1] = b->offsets[b->ninst];
  out[2] = b->tuned_ctas;
  out[3] = b->last_graphed ? 1 : 0;
  out[4] = b->last_engine;
  out[5] = b->shared_grid ? 1 : 0;
  out[6] = b->last_launches;
  return VFVM_OK;
}

extern "C" int vfvm_batch_offsets(vfvm_batch* b, int64_t* offsets) {
  if (!b || !offsets) return VFVM_ERR_INPUT;
  std::copy(b->offsets.begin(), b->offsets.end(), offsets);
  return VFVM_OK;
}

namespace {

int batch_run(vfvm_batch* b, const vfvm_control* ctl, int ctas, double time, double tstep, double lambda, float* ms,
              const double* guess = nullptr, const double* fallback = nullptr) {
  if (ctl->krylov != VFVM_KRYLOV_BICGSTAB) return VFVM_ERR_INPUT;  // batched solves run BiCGStab only
  if (ctl->precon == VFVM_PRECON_BLOCK_ILU0)
    for (auto* c : b->ctx)
      if (c->ncolors > kMaxBlockIluColors) return VFVM_ERR_INPUT;
  return dispatch_physics(b->phys, [&](auto ph) { return batch_run_t<decltype(ph)>(b, ctl, ctas, time, tstep, lambda, guess, fallback, ms);
  });
}

// Device inputs written on the legacy default stream before the call (the
// default stream of most frameworks) are complete before the batch reads them.
cudaError_t wait_legacy_stream(vfvm_batch* b) {
  cudaError_t e = cudaEventRecord(b->e0, cudaStreamLegacy);
  return e == cudaSuccess ? cudaStreamWaitEvent(b->stream, b->e0, 0) : e;
}

int batch_ctas(vfvm_batch* b, const vfvm_control* ctl) {
  if (ctl->team_ctas > 0) return ctl->team_ctas;
  if (b->tuned_ctas > 0 && b->tuned_engine == 0) return b->tuned_ctas;
  return 2;
}

int batch_results(vfvm_batch* b, vfvm_history* hist, float ms, int32_t* from_guess = nullptr) {
  std::vector<NewtonOut> outs(b->ninst);
  VFVM_CUDA(cudaMemcpy(outs.data(), b->outs.p, sizeof(NewtonOut) * b->ninst, cudaMemcpyDeviceToHost));
  int worst = VFVM_OK;
  for (int i = 0; i < b->ninst; ++i) {
    if (from_guess) from_guess[i] = outs[i].from_guess;
    if (outs[i].status != VFVM_OK && worst == VFVM_OK) worst = outs[i].status;
    if (hist) {
      std::memset(&hist[i], 0, sizeof(vfvm_history));
      hist[i].nnewton = outs[i].nnewton;
      hist[i].nlin = outs[i].nlin;
      hist[i].status = outs[i].status;
      hist[i].updatenorm = outs[i].updnorm;
      hist[i].resnorm = outs[i].resnorm;
      hist[i].time_ms = ms;
    }
  }
  return worst;
}

}  // namespace

extern "C" int vfvm_batch_load_device(vfvm_batch* b, const double* params_dev, int32_t nparams,
                                      const double* nodedata_dev, int32_t nnodedata) {
  if (!b) return VFVM_ERR_INPUT;
  vfvm_ctx* c0 = b->ctx[0];
  if (params_dev && (nparams < physics_nparams(c0->phys) || nparams < 1)) return VFVM_ERR_INPUT;
  if (nodedata_dev && (nnodedata != c0->nnd || nnodedata < 1)) return VFVM_ERR_INPUT;
  for (auto* c : b->ctx) {
    if (params_dev && nparams != c->nparams) return VFVM_ERR_INPUT;  // the parameter count stays
    if (nodedata_dev && !c->nodedata.own) return VFVM_ERR_INPUT;
  }
  VFVM_CUDA(wait_legacy_stream(b));
  const size_t pb = (size_t)nparams * sizeof(double);
  int64_t off = 0;
  for (int i = 0; i < b->ninst; ++i) {
    vfvm_ctx* c = b->ctx[i];
    if (params_dev)
      VFVM_CUDA(cudaMemcpyAsync(c->params.p, params_dev + (size_t)i * nparams, pb, cudaMemcpyDeviceToDevice, b->stream));
    if (nodedata_dev) {
      const size_t nb = (size_t)c->N * nnodedata;
      VFVM_CUDA(cudaMemcpyAsync(c->nodedata.p, nodedata_dev + off, nb * sizeof(double), cudaMemcpyDeviceToDevice,
                                b->stream));
      off += (int64_t)nb;
    }
  }
  b->desc_precision = -1;
  if (SweepHost* h = b->sweep) {
    // the sweep engine's packed copies have the same system-major layout: refill them in one copy each
    const bool pfit = !params_dev || (size_t)b->ninst * pb == h->params.n;
    const bool nfit = !nodedata_dev || (size_t)off * sizeof(double) == h->nodedata.n;
    if (h->valid && pfit && nfit) {
      if (params_dev)
        VFVM_CUDA(cudaMemcpyAsync(h->params.p, params_dev, h->params.n, cudaMemcpyDeviceToDevice, b->stream));
      if (nodedata_dev)
        VFVM_CUDA(cudaMemcpyAsync(h->nodedata.p, nodedata_dev, h->nodedata.n, cudaMemcpyDeviceToDevice, b->stream));
    } else {
      h->valid = false;
    }
  }
  VFVM_CUDA(cudaStreamSynchronize(b->stream));
  return VFVM_OK;
}

extern "C" int vfvm_batch_solve_device(vfvm_batch* b, const vfvm_control* ctl, const double* inival_dev,
                                       double* U_dev, double time, double tstep, double lambda, vfvm_history* hist) {
  if (!b || !ctl || !inival_dev || !U_dev) return VFVM_ERR_INPUT;
  const size_t n = (size_t)b->offsets[b->ninst];
  VFVM_CUDA(wait_legacy_stream(b));
  VFVM_CUDA(cudaMemcpyAsync(b->U.p, inival_dev, n * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
  VFVM_CUDA(cudaMemcpyAsync(b->Uold.p, inival_dev, n * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
  float ms = 0;
  int rc = batch_run(b, ctl, batch_ctas(b, ctl), time, tstep, lambda, &ms);
  if (rc) return rc;
  VFVM_CUDA(cudaMemcpyAsync(U_dev, b->U.p, n * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
  VFVM_CUDA(cudaStreamSynchronize(b->stream));
  return batch_results(b, hist, ms);
}

// Guarded start: Newton from guess_dev while every iteration reduces the FP64
// residual, else plain Newton from inival_dev; from_guess[i] (optional) = 1
// where the result was reached from the guess.
extern "C" int vfvm_batch_solve_guarded_device(vfvm_batch* b, const vfvm_control* ctl, const double* guess_dev,
                                               const double* inival_dev, double* U_dev, double time, double tstep,
                                               double lambda, vfvm_history* hist, int32_t* from_guess) {
  if (!b || !ctl || !guess_dev || !inival_dev || !U_dev) return VFVM_ERR_INPUT;
  const size_t n = (size_t)b->offsets[b->ninst];
  VFVM_CUDA(wait_legacy_stream(b));
  VFVM_CUDA(cudaMemcpyAsync(b->U.p, inival_dev, n * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
  VFVM_CUDA(cudaMemcpyAsync(b->Uold.p, inival_dev, n * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
  float ms = 0;
  int rc = batch_run(b, ctl, batch_ctas(b, ctl), time, tstep, lambda, &ms, guess_dev, inival_dev);
  if (rc) return rc;
  VFVM_CUDA(cudaMemcpyAsync(U_dev, b->U.p, n * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
  VFVM_CUDA(cudaStreamSynchronize(b->stream));
  return batch_results(b, hist, ms, from_guess);
}

extern "C" int vfvm_batch_solve(vfvm_batch* b, const vfvm_control* ctl, const double* inival, double* U, double time,
                                double tstep, double lambda, vfvm_history* hist) {
  if (!b || !ctl || !inival || !U) return VFVM_ERR_INPUT;
  const size_t n = (size_t)b->offsets[b->ninst];
  VFVM_CUDA(cudaMemcpyAsync(b->U.p, inival, n * sizeof(double), cudaMemcpyHostToDevice, b->stream));
  VFVM_CUDA(cudaMemcpyAsync(b->Uold.p, b->U.p, n * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
  float ms = 0;
  int rc = batch_run(b, ctl, batch_ctas(b, ctl), time, tstep, lambda, &ms);
  if (rc) return rc;
  VFVM_CUDA(cudaMemcpyAsync(U, b->U.p, n * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  VFVM_CUDA(cudaStreamSynchronize(b->stream));
  return batch_results(b, hist, ms);
}

// Autotuner: times the batched solve from inival (device) for each candidate
// number of CTAs per system and keeps the fastest for later solves of this batch.
extern "C" int vfvm_batch_tune(vfvm_batch* b, const vfvm_control* ctl, const double* inival_dev, int32_t* best_ctas,
                               float* times_ms, int32_t ncand, const int32_t* candidates) {
  if (!b || !ctl || !inival_dev || ncand < 1 || !candidates) return VFVM_ERR_INPUT;
  // a control no candidate can run (batched solves are BiCGStab only) is an
  // input error, not "no candidate fits"
  if (ctl->krylov != VFVM_KRYLOV_BICGSTAB) return VFVM_ERR_INPUT;
  const size_t n = (size_t)b->offsets[b->ninst];
  float best = 1e30f;
  int bestc = -1, failed_rc = VFVM_ERR_INPUT;
  VFVM_CUDA(wait_legacy_stream(b));
  // the candidates are CTAs per system (team engine) or blocks per system (sweep
  // engine), passed as the control's team_ctas
  vfvm_control c = *ctl;
  for (int k = 0; k < ncand; ++k) {
    VFVM_CUDA(cudaMemcpyAsync(b->U.p, inival_dev, n * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
    VFVM_CUDA(cudaMemcpyAsync(b->Uold.p, inival_dev, n * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
    float ms = 0;
    c.team_ctas = candidates[k];
    int rc = batch_run(b, &c, candidates[k], 0.0, INFINITY, 0.0, &ms);
    if (rc == VFVM_ERR_INPUT) { if (times_ms) times_ms[k] = -1.0f; continue; }  // does not fit the device
    if (rc) return rc;
    if (times_ms) times_ms[k] = ms;
    const int res = batch_results(b, nullptr, ms);
    if (res != VFVM_OK) { failed_rc = res; continue; }
    if (ms < best) { best = ms; bestc = candidates[k]; }
  }
  // no candidate solved the batch: keep the previous setting and say why
  // (VFVM_ERR_INPUT: none fits the device; otherwise the solve's own status)
  if (bestc < 0) return failed_rc;
  b->tuned_ctas = bestc;
  b->tuned_engine = b->last_engine;
  if (best_ctas) *best_ctas = bestc;
  return VFVM_OK;
}
