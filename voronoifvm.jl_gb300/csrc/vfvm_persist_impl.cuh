// Host side of the persistent Newton engine (one system per cooperative launch)
// and of the batched solver (many systems of uneven size in one cooperative
// launch, a group of CTAs per system, largest systems first).
#pragma once
#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>
#include "vfvm_newton_team.cuh"
#include "vfvm_persist.cuh"

namespace vfvm {

// coarse: include the context's selected coarse stage (not with block Jacobi)
template <class Ph, typename KT>
NewtonData<Ph, KT> make_newton_data(vfvm_ctx* c, double* U, double* Uold, bool coarse) {
  Workspace* w = c->ws;
  KVecs<KT>& k = *reinterpret_cast<KVecs<KT>*>(std::is_same<KT, double>::value ? (void*)&w->k64 : (void*)&w->k32);
  KT* J = std::is_same<KT, double>::value ? (KT*)c->J.p : (KT*)c->Jf.p;
  NewtonData<Ph, KT> nd;
  nd.t = c->tables();
  nd.U = U;
  nd.Uold = Uold;
  nd.F = c->F.p;
  nd.J = J;
  nd.bw = k.b.p;
  nd.dirdof = c->dirichlet_dof.p;
  nd.kd.N = c->N;
  nd.kd.rowptr = c->browptr.p;
  nd.kd.col = c->bcol.p;
  nd.kd.A = J;
  nd.kd.diag = c->diag.p;
  nd.kd.dinv = k.dinv.p;
  nd.kd.b = k.b.p;
  nd.kd.x = k.x.p;
  nd.kd.r = k.r.p; nd.kd.r0 = k.r0.p; nd.kd.p = k.p.p; nd.kd.v = k.v.p; nd.kd.s = k.s.p; nd.kd.t = k.t.p;
  nd.il.ncolors = c->ncolors;
  nd.il.color_ptr = c->color_ptr.p;
  nd.il.color_nodes = c->color_nodes.p;
  nd.il.node_color = w->node_color.p;
  nd.il.lower_ptr = c->lower_ptr.p;
  nd.il.lower_slots = c->lower_slots.p;
  nd.il.ilu = k.ilu.p;
  nd.il.y = k.sh.p;
  nd.nvals = c->nnzb * (int64_t)c->ns * c->ns;
  nd.kd.cd = coarse ? c->coarse_data() : CoarseData{};
  return nd;
}

inline int sm_count() {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  return sms;
}

template <class Ph, typename KT, int PRECON>
int persistent_launch(vfvm_ctx* c, const vfvm_control* ctl, const PersistRunHost& rh, vfvm_history* hist,
                             float* ms) {
  Workspace* w = c->ws;
  auto kern = newton_persistent_kernel<Ph, KT, PRECON>;
  NewtonData<Ph, KT> nd = make_newton_data<Ph, KT>(c, c->U.p, c->Uold.p, PRECON != VFVM_PRECON_JACOBI);
  const size_t smem = nd.kd.cd.nc ? coarse_smem_bytes(nd.kd.cd.nc) : 0;
  VFVM_CUDA(cudaFuncSetAttribute((const void*)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  VFVM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kPersistThreads, smem));
  const int sms = sm_count();
  if (per_sm < 1 || sms < 1) return VFVM_ERR_CUDA;
  int grid = sms * std::min(per_sm, 2);
  if (ctl->team_ctas > 0) grid = std::min(ctl->team_ctas, sms * per_sm);
  const int need = (int)((c->N + kPersistThreads - 1) / kPersistThreads);
  grid = std::max(1, std::min(grid, need));
  if (w->pbar.n < 8) VFVM_CUDA(w->pbar.alloc(8));
  if (w->ppartials.n < (size_t)2 * grid * 8) VFVM_CUDA(w->ppartials.alloc((size_t)2 * grid * 8));
  if (w->pout.n < sizeof(NewtonOut)) VFVM_CUDA(w->pout.alloc(sizeof(NewtonOut)));
  VFVM_CUDA(cudaMemsetAsync(w->pbar.p, 0, 8 * sizeof(unsigned), c->stream));
  DevControl dc = make_devcontrol(*ctl);
  GridSync gs{w->pbar.p, w->ppartials.p};
  PersistRun run{rh.nsteps, rh.time, 1.0 / rh.tstep, rh.lambda, rh.t0, rh.dt};
  NewtonOut* out = reinterpret_cast<NewtonOut*>(w->pout.p);
  void* args[] = {&nd, &dc, &gs, &run, &out};
  VFVM_CUDA(cudaEventRecord(w->ev0, c->stream));
  VFVM_CUDA(cudaLaunchCooperativeKernel((void*)kern, dim3(grid), dim3(kPersistThreads), args, smem, c->stream));
  VFVM_CUDA(cudaEventRecord(w->ev1, c->stream));
  NewtonOut h;
  VFVM_CUDA(cudaMemcpyAsync(&h, out, sizeof(NewtonOut), cudaMemcpyDeviceToHost, c->stream));
  VFVM_CUDA(cudaStreamSynchronize(c->stream));
  float t = 0;
  VFVM_CUDA(cudaEventElapsedTime(&t, w->ev0, w->ev1));
  if (ms) *ms = t;
  if (hist) {
    std::memset(hist, 0, sizeof(*hist));
    hist->nnewton = h.nnewton;
    hist->nlin = h.nlin;
    hist->nsteps = h.nsteps;
    hist->status = h.status;
    hist->updatenorm = h.updnorm;
    hist->resnorm = h.resnorm;
    hist->time_ms = t;
  }
  // mirror into the device-state block read by the graph-engine helpers
  w->st_host->status = h.status;
  w->st_host->nnewton = h.nnewton;
  w->st_host->nlin = h.nlin;
  w->st_host->updnorm = h.updnorm;
  w->st_host->resnorm = h.resnorm;
  return h.status;
}

template <class Ph>
int persistent_solve_t(vfvm_ctx* c, const vfvm_control* ctl, const PersistRunHost& run, vfvm_history* hist, float* ms) {
  const bool f64 = ctl->precision == VFVM_PRECISION_FP64;
  switch (ctl->precon) {
    case VFVM_PRECON_JACOBI:
      return f64 ? persistent_launch<Ph, double, VFVM_PRECON_JACOBI>(c, ctl, run, hist, ms)
                 : persistent_launch<Ph, float, VFVM_PRECON_JACOBI>(c, ctl, run, hist, ms);
    case VFVM_PRECON_ILU0:
      return f64 ? persistent_launch<Ph, double, VFVM_PRECON_ILU0>(c, ctl, run, hist, ms)
                 : persistent_launch<Ph, float, VFVM_PRECON_ILU0>(c, ctl, run, hist, ms);
    default:
      return f64 ? persistent_launch<Ph, double, VFVM_PRECON_BLOCK_ILU0>(c, ctl, run, hist, ms)
                 : persistent_launch<Ph, float, VFVM_PRECON_BLOCK_ILU0>(c, ctl, run, hist, ms);
  }
}

}  // namespace vfvm


namespace vfvm {

template <class Ph, typename KT, int PRECON>
int batch_launch(vfvm_batch* b, const vfvm_control* ctl, int ctas_per_system, double time, double tstep,
                 double lambda, const double* guess, const double* fallback, float* ms) {
  auto kern = newton_batch_kernel<Ph, KT, PRECON>;
  const size_t smem = b->desc_coarse_nc ? coarse_smem_bytes(b->desc_coarse_nc) : 0;
  VFVM_CUDA(cudaFuncSetAttribute((const void*)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  VFVM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kPersistThreads, smem));
  const int sms = sm_count();
  if (per_sm < 1 || sms < 1) return VFVM_ERR_CUDA;
  const int G = std::max(1, ctas_per_system);
  const int total = sms * std::min(per_sm, 4);
  int ngroups = std::max(1, total / G);
  ngroups = std::min(ngroups, b->ninst);
  const int grid = ngroups * G;
  if (grid > sms * per_sm) return VFVM_ERR_INPUT;
  // per-group barrier words and partials
  if (b->bars.n < (size_t)8 * ngroups) VFVM_CUDA(b->bars.alloc((size_t)8 * ngroups));
  if (b->partials.n < (size_t)2 * G * 8 * ngroups) VFVM_CUDA(b->partials.alloc((size_t)2 * G * 8 * ngroups));
  if (b->slots.n < (size_t)ngroups) VFVM_CUDA(b->slots.alloc(ngroups));
  std::vector<BatchSync> hs(ngroups);
  for (int g = 0; g < ngroups; ++g)
    hs[g] = BatchSync{GridSync{b->bars.p + 8 * (size_t)g, b->partials.p + (size_t)2 * G * 8 * g}, b->slots.p + g};
  if (b->syncs.n < sizeof(BatchSync) * ngroups) VFVM_CUDA(b->syncs.alloc(sizeof(BatchSync) * ngroups));
  VFVM_CUDA(cudaMemcpy(b->syncs.p, hs.data(), sizeof(BatchSync) * ngroups, cudaMemcpyHostToDevice));
  const NewtonData<Ph, KT>* insts = reinterpret_cast<const NewtonData<Ph, KT>*>(b->desc.p);
  const int* order = b->order.p;
  DevControl dc = make_devcontrol(*ctl);
  const BatchSync* groups = reinterpret_cast<const BatchSync*>(b->syncs.p);
  unsigned* queue = b->queue.p;
  NewtonOut* outs = reinterpret_cast<NewtonOut*>(b->outs.p);
  int* failed = b->failed.p;
  int ninst = b->ninst;
  double tinv = 1.0 / tstep;
  int gsz = G;
  const double* ubase = b->U.p;
  void* args[] = {&insts, &ninst, &order, &dc, &groups, &gsz, &queue, &time, &tinv, &lambda, &outs, &failed,
                  &guess, &fallback, &ubase};
  // The solve is one captured graph: scheduler resets + the persistent
  // cooperative launch.  Each call captures it again and updates the cached
  // executable graph in place (kernel arguments change between calls).
  auto enqueue = [&]() -> cudaError_t {
    cudaError_t e = cudaMemsetAsync(b->bars.p, 0, 8 * sizeof(unsigned) * ngroups, b->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->queue.p, 0, sizeof(unsigned), b->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->failed.p, 0, sizeof(int), b->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->outs.p, 0, sizeof(NewtonOut) * b->ninst, b->stream);
    if (e == cudaSuccess)
      e = cudaLaunchCooperativeKernel((void*)kern, dim3(grid), dim3(kPersistThreads), args, smem, b->stream);
    return e;
  };
  bool graphed = false;
  if (b->use_graph) {
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      const cudaError_t e1 = enqueue();
      e = cudaStreamEndCapture(b->stream, &g);
      if (e1 != cudaSuccess) e = e1;
    }
    if (e == cudaSuccess && g) {
      if (b->exec) {
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(b->exec, g, &info) != cudaSuccess) {
          cudaGetLastError();
          cudaGraphExecDestroy(b->exec);
          b->exec = nullptr;
        }
      }
      if (!b->exec && cudaGraphInstantiate(&b->exec, g, 0) != cudaSuccess) b->exec = nullptr;
      graphed = b->exec != nullptr;
    }
    if (g) cudaGraphDestroy(g);
    if (!graphed) {  // capture of the cooperative launch refused: launch directly from now on
      cudaGetLastError();
      b->use_graph = false;
    }
  }
  VFVM_CUDA(cudaEventRecord(b->e0, b->stream));
  if (graphed) VFVM_CUDA(cudaGraphLaunch(b->exec, b->stream));
  else VFVM_CUDA(enqueue());
  VFVM_CUDA(cudaEventRecord(b->e1, b->stream));
  VFVM_CUDA(cudaStreamSynchronize(b->stream));
  b->last_graphed = graphed;
  if (ms) VFVM_CUDA(cudaEventElapsedTime(ms, b->e0, b->e1));
  int hfailed = 0;
  VFVM_CUDA(cudaMemcpy(&hfailed, failed, sizeof(int), cudaMemcpyDeviceToHost));
  return hfailed ? VFVM_ERR_TIMEOUT : VFVM_OK;
}

// instance descriptors for a precision and coarse-stage size (0: none)
template <class Ph, typename KT>
int batch_prepare(vfvm_batch* b, int precision, int coarse) {
  if (b->desc_precision == precision && b->desc_coarse == coarse) return VFVM_OK;
  std::vector<NewtonData<Ph, KT>> d(b->ninst);
  int maxnc = 0;
  for (int i = 0; i < b->ninst; ++i) {
    int rc = ensure_workspace(b->ctx[i], precision);
    if (rc) return rc;
    if ((rc = ensure_coarse(b->ctx[i], coarse))) return rc;
    d[i] = make_newton_data<Ph, KT>(b->ctx[i], b->U.p + b->offsets[i], b->Uold.p + b->offsets[i], coarse > 0);
    maxnc = std::max(maxnc, d[i].kd.cd.nc);
  }
  VFVM_CUDA(b->desc.alloc(sizeof(NewtonData<Ph, KT>) * b->ninst));
  VFVM_CUDA(cudaMemcpy(b->desc.p, d.data(), sizeof(NewtonData<Ph, KT>) * b->ninst, cudaMemcpyHostToDevice));
  b->desc_precision = precision;
  b->desc_coarse = coarse;
  b->desc_coarse_nc = maxnc;
  return VFVM_OK;
}

template <class Ph>
int batch_run_t(vfvm_batch* b, const vfvm_control* ctl, int ctas, double time, double tstep, double lambda,
                const double* guess, const double* fallback, float* ms) {
  const bool f64 = ctl->precision == VFVM_PRECISION_FP64;
  const bool jac = ctl->precon == VFVM_PRECON_JACOBI;
  const int coarse = ctl->precon == VFVM_PRECON_JACOBI ? 0 : ctl->coarse;
  int rc = f64 ? batch_prepare<Ph, double>(b, ctl->precision, coarse)
               : batch_prepare<Ph, float>(b, ctl->precision, coarse);
  if (rc) return rc;
  (void)jac;
  switch (ctl->precon) {
    case VFVM_PRECON_JACOBI:
      return f64 ? batch_launch<Ph, double, VFVM_PRECON_JACOBI>(b, ctl, ctas, time, tstep, lambda, guess, fallback, ms)
                 : batch_launch<Ph, float, VFVM_PRECON_JACOBI>(b, ctl, ctas, time, tstep, lambda, guess, fallback, ms);
    case VFVM_PRECON_ILU0:
      return f64 ? batch_launch<Ph, double, VFVM_PRECON_ILU0>(b, ctl, ctas, time, tstep, lambda, guess, fallback, ms)
                 : batch_launch<Ph, float, VFVM_PRECON_ILU0>(b, ctl, ctas, time, tstep, lambda, guess, fallback, ms);
    default:
      return f64 ? batch_launch<Ph, double, VFVM_PRECON_BLOCK_ILU0>(b, ctl, ctas, time, tstep, lambda, guess, fallback, ms)
                 : batch_launch<Ph, float, VFVM_PRECON_BLOCK_ILU0>(b, ctl, ctas, time, tstep, lambda, guess, fallback, ms);
  }
}

}  // namespace vfvm
