// Host side of the persistent Newton engine (one system per cooperative launch)
// and of the batched solver (many systems of uneven size in one cooperative
// launch, a group of CTAs per system, largest systems first).
#pragma once
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <vector>
#include "vfvm_newton_team.cuh"
#include "vfvm_persist.cuh"
#include "vfvm_sweep.cuh"

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
  nd.kd.ew = c->ell_w;
  nd.kd.ell_col = c->ell_col.p;
  nd.kd.ell_slot = c->ell_slot.p;
  nd.kd.ell_val = k.ell_val.p;
  nd.il.lw = c->lo_w;
  nd.il.uw = c->up_w;
  nd.il.lo_node = c->lo_node.p;
  nd.il.lo_slot = c->lo_slot.p;
  nd.il.up_node = c->up_node.p;
  nd.il.up_slot = c->up_slot.p;
  nd.il.lo_val = k.lo_val.p;
  nd.il.up_val = k.up_val.p;
  nd.nvals = c->nnzb * (int64_t)c->ns * c->ns;
  nd.kd.cd = coarse ? c->coarse_data() : CoarseData{};
  nd.kd.gv = k.gv.p;
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
  if (ctl->krylov == VFVM_KRYLOV_GMRES) {
    KVecs<KT>& k = *reinterpret_cast<KVecs<KT>*>(std::is_same<KT, double>::value ? (void*)&w->k64 : (void*)&w->k32);
    const size_t need = (size_t)(ctl->gmres_restart + 1) * c->N * c->ns;
    if (k.gv.n < need) VFVM_CUDA(k.gv.alloc(need));
  }
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

template <class Ph, typename KT>
int persistent_solve_kt(vfvm_ctx* c, const vfvm_control* ctl, const PersistRunHost& run, vfvm_history* hist,
                        float* ms) {
  switch (ctl->precon) {
    case VFVM_PRECON_JACOBI: return persistent_launch<Ph, KT, VFVM_PRECON_JACOBI>(c, ctl, run, hist, ms);
    case VFVM_PRECON_ILU0: return persistent_launch<Ph, KT, VFVM_PRECON_ILU0>(c, ctl, run, hist, ms);
    default: return persistent_launch<Ph, KT, VFVM_PRECON_BLOCK_ILU0>(c, ctl, run, hist, ms);
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

// ---------------------------------------------------------------------------
// Sweep engine host side: contiguous per-system arrays, the Newton graph with
// conditional WHILE nodes (built once per precision / coarse size), one launch
// per solve.
// ---------------------------------------------------------------------------

// leaves of a graph (nodes without dependents): where the next node attaches
inline cudaError_t graph_leaves(cudaGraph_t g, std::vector<cudaGraphNode_t>& leaves) {
  size_t nn = 0;
  cudaError_t e = cudaGraphGetNodes(g, nullptr, &nn);
  if (e != cudaSuccess) return e;
  std::vector<cudaGraphNode_t> nodes(nn);
  if ((e = cudaGraphGetNodes(g, nodes.data(), &nn)) != cudaSuccess) return e;
  leaves.clear();
  for (auto nd : nodes) {
    size_t out = 0;
    if ((e = cudaGraphNodeGetDependentNodes(nd, nullptr, nullptr, &out)) != cudaSuccess) return e;
    if (out == 0) leaves.push_back(nd);
  }
  return cudaSuccess;
}

// appends a conditional WHILE node after the leaves of g; returns its body graph
inline cudaError_t add_while(cudaGraph_t g, cudaGraphConditionalHandle h, cudaGraphNode_t* node, cudaGraph_t* body) {
  std::vector<cudaGraphNode_t> leaves;
  cudaError_t e = graph_leaves(g, leaves);
  if (e != cudaSuccess) return e;
  cudaGraphNodeParams wp = {};
  wp.type = cudaGraphNodeTypeConditional;
  wp.conditional.handle = h;
  wp.conditional.type = cudaGraphCondTypeWhile;
  wp.conditional.size = 1;
  if ((e = cudaGraphAddNode(node, g, leaves.data(), nullptr, leaves.size(), &wp)) != cudaSuccess) return e;
  *body = wp.conditional.phGraph_out[0];
  return cudaSuccess;
}

// grid of the BiCGStab iteration kernels: bpi blocks per system, striding over
// the list of systems still iterating (about four waves of blocks when full)
template <class Ph, typename KT>
dim3 sweep_list_grid(const SweepArgs<Ph, KT>&) {
  return dim3(4 * 152 * 8);  // 1D: the kernels spread these blocks over the systems still iterating
}

template <class Ph, typename KT>
void sweep_apply(const SweepArgs<Ph, KT>& a, dim3 grid, int which, cudaStream_t s) {
  const int ul = which == 0 ? 0 : 1;  // the first application (Newton head) has no list yet
  for (int c = 0; c < a.ncolors; ++c) sw_ilu_fwd_kernel<Ph, KT><<<grid, kSweepThreads, 0, s>>>(a, c, which, ul);
  for (int c = a.ncolors - 1; c >= 0; --c) sw_ilu_bwd_kernel<Ph, KT><<<grid, kSweepThreads, 0, s>>>(a, c, which, ul);
  if (a.cd0.nc) {  // the prolongation is fused into the next kernel (kstart, alpha, omega)
    sw_coarse_restrict_kernel<Ph, KT><<<grid, kSweepThreads, 0, s>>>(a, which, ul);
    sw_coarse_matvec_kernel<Ph, KT><<<grid, kSweepThreads, 0, s>>>(a, ul);
  }
}

// kernel sequences of the sweep engine (captured into the graph, or launched
// eagerly with host-side loop control for per-kernel profiling)
template <class Ph, typename KT>
void sweep_newton_head(const SweepArgs<Ph, KT>& a, cudaStream_t s) {
  const dim3 grid(a.bpi, a.S);
  sw_restart_kernel<Ph, KT><<<grid, kSweepThreads, 0, s>>>(a);
  sw_assemble_kernel<Ph, KT><<<grid, kSweepThreads, 0, s>>>(a);
  sw_prep_kernel<Ph, KT><<<grid, kSweepThreads, 0, s>>>(a);
  sw_ilu_copy_kernel<Ph, KT><<<grid, kSweepThreads, 0, s>>>(a);
  for (int c = 0; c < a.ncolors; ++c) sw_ilu_factor_kernel<Ph, KT><<<grid, kSweepThreads, 0, s>>>(a, c);
  sw_pack_kernel<Ph, KT><<<grid, kSweepThreads, 0, s>>>(a);
  if (a.cd0.nc) {
    sw_galerkin_kernel<Ph, KT><<<grid, kSweepThreads, 0, s>>>(a);
    sw_galerkin2_kernel<Ph, KT><<<grid, kSweepThreads, 0, s>>>(a);
    sw_coarse_invert_kernel<Ph, KT><<<a.S, 1024, coarse_smem_bytes(a.cd0.nc), s>>>(a);
  }
  sweep_apply<Ph, KT>(a, grid, 0, s);  // r = M^-1 b
  sw_kstart_kernel<Ph, KT><<<grid, kSweepThreads, 0, s>>>(a);
}

template <class Ph, typename KT>
void sweep_krylov_iteration(const SweepArgs<Ph, KT>& a, cudaStream_t s) {
  const dim3 grid = sweep_list_grid(a);
  sw_p_kernel<Ph, KT><<<grid, kSweepThreads, 0, s>>>(a);
  sw_spmv_kernel<Ph, KT><<<grid, kSweepThreads, 0, s>>>(a, 1);
  sweep_apply<Ph, KT>(a, grid, 1, s);
  sw_alpha_kernel<Ph, KT><<<grid, kSweepThreads, 0, s>>>(a);
  sw_s_kernel<Ph, KT><<<grid, kSweepThreads, 0, s>>>(a);
  sw_spmv_kernel<Ph, KT><<<grid, kSweepThreads, 0, s>>>(a, 2);
  sweep_apply<Ph, KT>(a, grid, 2, s);
  sw_omega_kernel<Ph, KT><<<grid, kSweepThreads, 0, s>>>(a);
  sw_xr_kernel<Ph, KT><<<grid, kSweepThreads, 0, s>>>(a);
}

template <class Ph, typename KT>
int sweep_build_graph(SweepHost& h, const SweepArgs<Ph, KT>& a, cudaStream_t s) {
  if (h.exec) { cudaGraphExecDestroy(h.exec); h.exec = nullptr; }
  if (h.graph) { cudaGraphDestroy(h.graph); h.graph = nullptr; }
  cudaGraph_t g;
  VFVM_CUDA(cudaGraphCreate(&g, 0));
  h.graph = g;
  cudaGraphConditionalHandle ncond, kcond;
  VFVM_CUDA(cudaGraphConditionalHandleCreate(&ncond, g, 0, 0));
  VFVM_CUDA(cudaGraphConditionalHandleCreate(&kcond, g, 0, 0));
  const dim3 grid(a.bpi, a.S);
  cudaGraph_t cap;
  // prologue: start values, Dirichlet values, state; Newton condition
  VFVM_CUDA(cudaStreamBeginCaptureToGraph(s, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  sw_init_kernel<Ph, KT><<<grid, kSweepThreads, 0, s>>>(a);
  sw_cond_kernel<<<1, 1024, 0, s>>>(a.st, a.S, 1, ncond, a.klist, a.kcount, a.runs, a.call);
  VFVM_CUDA(cudaStreamEndCapture(s, &cap));
  cudaGraphNode_t wnode, knode;
  cudaGraph_t body, kbody;
  VFVM_CUDA(add_while(g, ncond, &wnode, &body));
  // Newton body up to the Krylov loop
  VFVM_CUDA(cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  sweep_newton_head<Ph, KT>(a, s);
  sw_cond_kernel<<<1, 1024, 0, s>>>(a.st, a.S, 0, kcond, a.klist, a.kcount, a.runs, a.call);
  VFVM_CUDA(cudaStreamEndCapture(s, &cap));
  VFVM_CUDA(add_while(body, kcond, &knode, &kbody));
  // one BiCGStab iteration of every active system
  VFVM_CUDA(cudaStreamBeginCaptureToGraph(s, kbody, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  sweep_krylov_iteration<Ph, KT>(a, s);
  sw_cond_kernel<<<1, 1024, 0, s>>>(a.st, a.S, 0, kcond, a.klist, a.kcount, a.runs, a.call);
  VFVM_CUDA(cudaStreamEndCapture(s, &cap));
  // Newton update after the Krylov loop, next Newton condition
  VFVM_CUDA(cudaStreamBeginCaptureToGraph(s, body, &knode, nullptr, 1, cudaStreamCaptureModeThreadLocal));
  sw_update_kernel<Ph, KT><<<grid, kSweepThreads, 0, s>>>(a);
  sw_cond_kernel<<<1, 1024, 0, s>>>(a.st, a.S, 1, ncond, a.klist, a.kcount, a.runs, a.call);
  VFVM_CUDA(cudaStreamEndCapture(s, &cap));
  VFVM_CUDA(cudaGetLastError());
  VFVM_CUDA(cudaGraphInstantiate(&h.exec, g, 0));
  h.args.assign(reinterpret_cast<const char*>(&a), reinterpret_cast<const char*>(&a) + sizeof(a));
  return VFVM_OK;
}

// Eager variant for per-kernel profiling (VFVM_SWEEP_EAGER=1): the same kernel
// sequence, loops controlled on the host from the state records.
template <class Ph, typename KT>
int sweep_eager(const SweepArgs<Ph, KT>& a, cudaStream_t s) {
  const dim3 grid(a.bpi, a.S);
  std::vector<SweepState> st(a.S);
  std::vector<int> list;
  int started = 0;  // systems that entered the current BiCGStab loop
  SweepCall call;
  VFVM_CUDA(cudaMemcpyAsync(&call, a.call, sizeof(SweepCall), cudaMemcpyDeviceToHost, s));
  auto any = [&](int which, bool& out) -> int {
    VFVM_CUDA(cudaMemcpyAsync(st.data(), a.st, sizeof(SweepState) * a.S, cudaMemcpyDeviceToHost, s));
    VFVM_CUDA(cudaStreamSynchronize(s));
    out = false;
    list.clear();
    for (int i = 0; i < a.S; ++i) {
      const auto& x = st[i];
      out = out || (which == 0 ? x.kactive != 0 : (x.nactive || x.restart));
      if (x.kactive) list.push_back(i);
    }
    // the batch-level inexact Newton rule (sw_cond_kernel)
    if (which == 1) started = 0;
    if (which == 0) {
      if (started == 0) started = (int)list.size();
      if ((int)list.size() <= call.ctl.batch_tail && 10 * (int)list.size() <= started) out = false;
    }
    if (which == 0) {  // the compact list the iteration kernels stride over
      const int cnt = (int)list.size();
      VFVM_CUDA(cudaMemcpyAsync(a.kcount, &cnt, sizeof(int), cudaMemcpyHostToDevice, s));
      if (cnt) VFVM_CUDA(cudaMemcpyAsync(a.klist, list.data(), sizeof(int) * cnt, cudaMemcpyHostToDevice, s));
      VFVM_CUDA(cudaStreamSynchronize(s));
    }
    return VFVM_OK;
  };
  sw_init_kernel<Ph, KT><<<grid, kSweepThreads, 0, s>>>(a);
  bool nact = false, kact = false;
  int rc = any(1, nact);
  for (int guard = 0; !rc && nact && guard < 100000; ++guard) {
    sweep_newton_head<Ph, KT>(a, s);
    if ((rc = any(0, kact))) break;
    for (int k = 0; kact && k < 1000000; ++k) {
      sweep_krylov_iteration<Ph, KT>(a, s);
      if ((rc = any(0, kact))) break;
    }
    sw_update_kernel<Ph, KT><<<grid, kSweepThreads, 0, s>>>(a);
    if (!rc) rc = any(1, nact);
  }
  return rc;
}

// bpi_req: blocks per system (0: chosen from the system size; the autotuner
// passes its candidates here)
template <class Ph, typename KT>
int sweep_run(vfvm_batch* b, const vfvm_control* ctl, int bpi_req, double time, double tstep, double lambda,
              const double* guess, const double* fallback, float* ms) {
  constexpr int NS = Ph::NS, B = NS * NS;
  vfvm_ctx* c0 = b->ctx[0];
  const int S = b->ninst, N = c0->N;
  const int64_t n = (int64_t)N * NS, nb = c0->nnzb;
  int rc = ensure_workspace(c0, ctl->precision);
  if (rc) return rc;
  if ((rc = ensure_coarse(c0, ctl->coarse))) return rc;
  if (!b->sweep) b->sweep = new SweepHost;
  SweepHost& h = *b->sweep;
  const int nc = c0->coarse ? c0->coarse->nc : 0;
  const int bpi = bpi_req > 0 ? std::min(bpi_req, kSweepMaxBpi)
                              : std::max(1, std::min(64, (N + kSweepThreads * 4 - 1) / (kSweepThreads * 4)));
  if (h.precision != ctl->precision || h.coarse != ctl->coarse || h.bpi != bpi || !h.exec) {
    auto take = [](DBuf<char>& d, size_t bytes) { return d.n == bytes ? cudaSuccess : d.alloc(bytes); };
    const size_t kt = sizeof(KT);
    const int np = std::max(1, c0->nparams), nnd = c0->nnd;
    VFVM_CUDA(take(h.F, (size_t)S * n * 8));
    VFVM_CUDA(take(h.J, (size_t)S * nb * B * kt));
    VFVM_CUDA(take(h.ilu, (size_t)S * nb * B * kt));
    VFVM_CUDA(take(h.dinv, (size_t)S * N * B * kt));
    VFVM_CUDA(take(h.ell, (size_t)S * c0->ell_w * N * B * kt));
    VFVM_CUDA(take(h.lo, (size_t)S * std::max(c0->lo_w, 1) * N * B * kt));
    VFVM_CUDA(take(h.up, (size_t)S * std::max(c0->up_w, 1) * N * B * kt));
    VFVM_CUDA(take(h.vecs, (size_t)9 * S * n * kt));
    VFVM_CUDA(take(h.params, (size_t)S * np * 8));
    VFVM_CUDA(take(h.nodedata, (size_t)S * std::max<int64_t>(1, (int64_t)N * nnd) * 8));
    VFVM_CUDA(take(h.cA, (size_t)S * std::max(1, nc * nc) * 4));
    VFVM_CUDA(take(h.crc, (size_t)S * std::max(1, nc) * 4));
    VFVM_CUDA(take(h.czc, (size_t)S * std::max(1, nc) * 4));
    VFVM_CUDA(take(h.st, (size_t)S * sizeof(SweepState)));
    VFVM_CUDA(take(h.partials, (size_t)S * kSweepMaxBpi * 8 * 8));
    VFVM_CUDA(take(h.tickets, (size_t)S * 4));
    VFVM_CUDA(take(h.call, sizeof(SweepCall)));
    VFVM_CUDA(take(h.klist, (size_t)(S + 1) * 4));
    VFVM_CUDA(take(h.runs, 4 * sizeof(unsigned)));
    VFVM_CUDA(cudaMemset(h.tickets.p, 0, (size_t)S * 4));
    VFVM_CUDA(cudaMemset(h.st.p, 0, (size_t)S * sizeof(SweepState)));
    VFVM_CUDA(cudaMemset(h.vecs.p, 0, (size_t)9 * S * n * kt));
    VFVM_CUDA(cudaFuncSetAttribute((const void*)sw_coarse_invert_kernel<Ph, KT>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)coarse_smem_bytes(kCoarseMax)));
    SweepArgs<Ph, KT> a;
    a.t = c0->tables();
    a.S = S; a.N = N; a.nb = (int)nb; a.bpi = bpi; a.n = n;
    a.U = b->U.p; a.Uold = b->Uold.p; a.F = reinterpret_cast<double*>(h.F.p);
    a.params = reinterpret_cast<const double*>(h.params.p); a.np = np;
    a.nodedata = reinterpret_cast<const double*>(h.nodedata.p);
    a.dirdof = c0->dirichlet_dof.p;
    a.J = reinterpret_cast<KT*>(h.J.p); a.ilu = reinterpret_cast<KT*>(h.ilu.p);
    a.dinv = reinterpret_cast<KT*>(h.dinv.p); a.ell_val = reinterpret_cast<KT*>(h.ell.p);
    a.lo_val = reinterpret_cast<KT*>(h.lo.p); a.up_val = reinterpret_cast<KT*>(h.up.p);
    KT* vb = reinterpret_cast<KT*>(h.vecs.p);
    KT** vv[] = {&a.b, &a.x, &a.r, &a.r0, &a.p, &a.v, &a.s, &a.t2, &a.y};
    for (int k = 0; k < 9; ++k) *vv[k] = vb + (int64_t)k * S * n;
    // shared index tables (value pointers are per system, set in the kernels)
    NewtonData<Ph, KT> nd = make_newton_data<Ph, KT>(c0, b->U.p, b->Uold.p, nc > 0);
    a.kd0 = nd.kd;
    a.il0 = nd.il;
    a.cd0 = nd.kd.cd;
    a.cd0.A = reinterpret_cast<float*>(h.cA.p);
    a.cd0.rc = reinterpret_cast<float*>(h.crc.p);
    a.cd0.zc = reinterpret_cast<float*>(h.czc.p);
    a.st = reinterpret_cast<SweepState*>(h.st.p);
    a.partials = reinterpret_cast<double*>(h.partials.p);
    a.tickets = reinterpret_cast<unsigned*>(h.tickets.p);
    a.call = reinterpret_cast<const SweepCall*>(h.call.p);
    a.ncolors = c0->ncolors;
    a.klist = reinterpret_cast<int*>(h.klist.p);
    a.kcount = reinterpret_cast<int*>(h.klist.p) + S;
    a.runs = reinterpret_cast<unsigned*>(h.runs.p);
    if ((rc = sweep_build_graph<Ph, KT>(h, a, b->stream))) return rc;
    h.precision = ctl->precision;
    h.coarse = ctl->coarse;
    h.bpi = bpi;
    h.valid = false;
  }
  if (!h.valid) {  // gather every system's parameters and node data
    const int np = std::max(1, c0->nparams), nnd = c0->nnd;
    for (int i = 0; i < S; ++i) {
      VFVM_CUDA(cudaMemcpyAsync(h.params.p + (size_t)i * np * 8, b->ctx[i]->params.p, (size_t)np * 8,
                                cudaMemcpyDeviceToDevice, b->stream));
      if (nnd)
        VFVM_CUDA(cudaMemcpyAsync(h.nodedata.p + (size_t)i * N * nnd * 8, b->ctx[i]->nodedata.p,
                                  (size_t)N * nnd * 8, cudaMemcpyDeviceToDevice, b->stream));
    }
    h.valid = true;
  }
  SweepCall call{};
  call.ctl = make_devcontrol(*ctl);
  call.time = time;
  call.tstepinv = 1.0 / tstep;
  call.lambda = lambda;
  call.start = guess ? guess : b->U.p;
  call.fallback = guess ? fallback : nullptr;
  call.guard = guess ? 1 : 0;
  VFVM_CUDA(cudaMemcpyAsync(h.call.p, &call, sizeof(call), cudaMemcpyHostToDevice, b->stream));
  VFVM_CUDA(cudaMemsetAsync(h.runs.p, 0, 4 * sizeof(unsigned), b->stream));
  VFVM_CUDA(cudaEventRecord(b->e0, b->stream));
  const char* eager = std::getenv("VFVM_SWEEP_EAGER");
  if (eager && eager[0] == '1') {
    SweepArgs<Ph, KT> a;
    std::memcpy(&a, h.args.data(), sizeof(a));
    if ((rc = sweep_eager<Ph, KT>(a, b->stream))) return rc;
  } else {
    VFVM_CUDA(cudaGraphLaunch(h.exec, b->stream));
  }
  VFVM_CUDA(cudaEventRecord(b->e1, b->stream));
  std::vector<SweepState> st(S);
  VFVM_CUDA(cudaMemcpyAsync(st.data(), h.st.p, (size_t)S * sizeof(SweepState), cudaMemcpyDeviceToHost, b->stream));
  VFVM_CUDA(cudaStreamSynchronize(b->stream));
  if (ms) VFVM_CUDA(cudaEventElapsedTime(ms, b->e0, b->e1));
  {  // kernels launched by the graph: prologue 2, per Newton body head + 3, per BiCGStab body iteration
    unsigned runs[2] = {0, 0};
    VFVM_CUDA(cudaMemcpy(runs, h.runs.p, sizeof(runs), cudaMemcpyDeviceToHost));
    const int64_t C = c0->ncolors, co = nc > 0 ? 1 : 0;
    const int64_t NB = runs[1] > 0 ? (int64_t)runs[1] - 1 : 0, KB = (int64_t)runs[0] - NB;
    const int64_t head = 3 + 1 + C + 1 + 3 * co + 2 * C + 2 * co + 1;   // restart .. kstart
    const int64_t iter = 2 + 2 * (2 * C + 2 * co) + 1 + 1 + 1 + 1 + 1;  // p, spmv x2, applies, alpha, s, omega, xr, cond
    b->last_launches = 2 + NB * (head + 3) + KB * iter;
  }
  std::vector<NewtonOut> outs(S);
  for (int i = 0; i < S; ++i) {
    outs[i] = NewtonOut{st[i].status, st[i].nnewton, st[i].nlin, 0, st[i].updnorm, st[i].resnorm,
                        st[i].from_guess, 0};
    if (st[i].nactive || st[i].restart) outs[i].status = VFVM_ERR_CONVERGENCE;
  }
  VFVM_CUDA(cudaMemcpy(b->outs.p, outs.data(), sizeof(NewtonOut) * S, cudaMemcpyHostToDevice));
  b->last_graphed = true;
  b->last_engine = 1;
  return VFVM_OK;
}

template <class Ph, typename KT>
int batch_run_kt(vfvm_batch* b, const vfvm_control* ctl, int ctas, double time, double tstep, double lambda,
                 const double* guess, const double* fallback, float* ms) {
  // shared-grid batches with ILU0 run on the sweep engine unless the persistent engine is asked for
  if (b->shared_grid && ctl->precon == VFVM_PRECON_ILU0 && ctl->engine != VFVM_ENGINE_PERSISTENT &&
      !b->ctx[0]->has_legacy && !b->ctx[0]->multireg) {
    // blocks per system: the control's team_ctas, else the autotuned value, else automatic
    const int bpi = ctl->team_ctas > 0 ? ctas : b->tuned_engine == 1 ? b->tuned_ctas : 0;
    return sweep_run<Ph, KT>(b, ctl, bpi, time, tstep, lambda, guess, fallback, ms);
  }
  b->last_engine = 0;
  b->last_launches = 1;
  const int coarse = ctl->precon == VFVM_PRECON_JACOBI ? 0 : ctl->coarse;
  int rc = batch_prepare<Ph, KT>(b, ctl->precision, coarse);
  if (rc) return rc;
  switch (ctl->precon) {
    case VFVM_PRECON_JACOBI:
      return batch_launch<Ph, KT, VFVM_PRECON_JACOBI>(b, ctl, ctas, time, tstep, lambda, guess, fallback, ms);
    case VFVM_PRECON_ILU0:
      return batch_launch<Ph, KT, VFVM_PRECON_ILU0>(b, ctl, ctas, time, tstep, lambda, guess, fallback, ms);
    default:
      return batch_launch<Ph, KT, VFVM_PRECON_BLOCK_ILU0>(b, ctl, ctas, time, tstep, lambda, guess, fallback, ms);
  }
}

}  // namespace vfvm
