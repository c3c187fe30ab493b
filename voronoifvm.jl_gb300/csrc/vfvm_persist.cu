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
  for (int i = 0; i < ninst; ++i) {
    int st = 0;
    vfvm_ctx* c = vfvm_create(&grids[i], &phys[i], &st);
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

extern "C" int vfvm_batch_offsets(vfvm_batch* b, int64_t* offsets) {
  if (!b || !offsets) return VFVM_ERR_INPUT;
  std::copy(b->offsets.begin(), b->offsets.end(), offsets);
  return VFVM_OK;
}

namespace {

int batch_run(vfvm_batch* b, const vfvm_control* ctl, int ctas, double time, double tstep, double lambda, float* ms) {
  if (ctl->precon == VFVM_PRECON_BLOCK_ILU0)
    for (auto* c : b->ctx)
      if (c->ncolors > kMaxBlockIluColors) return VFVM_ERR_INPUT;
  return dispatch_physics(b->phys, [&](auto ph) { return batch_run_t<decltype(ph)>(b, ctl, ctas, time, tstep, lambda, ms); });
}

int batch_ctas(vfvm_batch* b, const vfvm_control* ctl) {
  if (ctl->team_ctas > 0) return ctl->team_ctas;
  if (b->tuned_ctas > 0) return b->tuned_ctas;
  return 2;
}

int batch_results(vfvm_batch* b, vfvm_history* hist, float ms) {
  std::vector<NewtonOut> outs(b->ninst);
  VFVM_CUDA(cudaMemcpy(outs.data(), b->outs.p, sizeof(NewtonOut) * b->ninst, cudaMemcpyDeviceToHost));
  int worst = VFVM_OK;
  for (int i = 0; i < b->ninst; ++i) {
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

extern "C" int vfvm_batch_solve_device(vfvm_batch* b, const vfvm_control* ctl, const double* inival_dev,
                                       double* U_dev, double time, double tstep, double lambda, vfvm_history* hist) {
  if (!b || !ctl || !inival_dev || !U_dev) return VFVM_ERR_INPUT;
  const size_t n = (size_t)b->offsets[b->ninst];
  VFVM_CUDA(cudaMemcpyAsync(b->U.p, inival_dev, n * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
  VFVM_CUDA(cudaMemcpyAsync(b->Uold.p, inival_dev, n * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
  float ms = 0;
  int rc = batch_run(b, ctl, batch_ctas(b, ctl), time, tstep, lambda, &ms);
  if (rc) return rc;
  VFVM_CUDA(cudaMemcpyAsync(U_dev, b->U.p, n * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
  VFVM_CUDA(cudaStreamSynchronize(b->stream));
  return batch_results(b, hist, ms);
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
  const size_t n = (size_t)b->offsets[b->ninst];
  float best = 1e30f;
  int bestc = candidates[0];
  for (int k = 0; k < ncand; ++k) {
    VFVM_CUDA(cudaMemcpyAsync(b->U.p, inival_dev, n * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
    VFVM_CUDA(cudaMemcpyAsync(b->Uold.p, inival_dev, n * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
    float ms = 0;
    int rc = batch_run(b, ctl, candidates[k], 0.0, INFINITY, 0.0, &ms);
    if (rc == VFVM_ERR_INPUT) { if (times_ms) times_ms[k] = -1.0f; continue; }  // does not fit the device
    if (rc) return rc;
    if (times_ms) times_ms[k] = ms;
    if (batch_results(b, nullptr, ms) == VFVM_OK && ms < best) { best = ms; bestc = candidates[k]; }
  }
  b->tuned_ctas = bestc;
  if (best_ctas) *best_ctas = bestc;
  return VFVM_OK;
}
