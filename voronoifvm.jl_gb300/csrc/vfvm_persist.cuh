// Declarations of the persistent engine and batched solver templates.  Their
// definitions (vfvm_persist_impl.cuh) are instantiated once per physics in
// separate objects (vfvm_persist_inst.cu, compiled with -DVFVM_INST_PHYS=... and
// -DVFVM_INST_KT=double|float) so the heavy kernels build in parallel.
#pragma once
#include <vector>
#include "vfvm_solver.cuh"

namespace vfvm {
// device memory and the captured graph of the sweep engine (vfvm_sweep.cuh)
struct SweepHost {
  int precision = -1, coarse = -1, bpi = -1;
  bool valid = false;                 // false after vfvm_batch_set_instance: parameters are re-gathered
  DBuf<char> F, J, ilu, dinv, ell, lo, up, vecs, params, nodedata, cA, crc, czc, st, partials, tickets, call, klist,
      runs;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<char> args;             // the kernel arguments the graph was built with
  ~SweepHost() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
  }
};
}  // namespace vfvm

struct vfvm_batch {
  // systems of one physics, packed unknowns, instance descriptors, scheduling state
  int ninst = 0, phys = 0, ns = 1;
  std::vector<vfvm_ctx*> ctx;
  std::vector<int64_t> offsets;  // dof offsets, ninst+1
  vfvm::DBuf<double> U, Uold;
  vfvm::DBuf<char> desc;               // NewtonData array of the current precision and coarse stage
  int desc_precision = -1, desc_coarse = 0, desc_coarse_nc = 0;
  vfvm::DBuf<int> order;
  vfvm::DBuf<unsigned> bars;
  vfvm::DBuf<double> partials;
  vfvm::DBuf<int> slots;
  vfvm::DBuf<char> syncs;
  vfvm::DBuf<unsigned> queue;
  vfvm::DBuf<char> outs;
  vfvm::DBuf<int> failed;
  cudaStream_t stream = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int tuned_ctas = 0;                // autotuned CTAs per system (team engine) or blocks per system (sweep)
  int tuned_engine = -1;             // engine the tuned value belongs to
  cudaGraphExec_t exec = nullptr;  // the captured solve (resets + persistent launch)
  bool use_graph = true, last_graphed = false;
  bool shared_grid = false;          // all systems are clones of ctx[0] (one grid)
  vfvm::SweepHost* sweep = nullptr;  // sweep engine state (shared-grid batches)
  int last_engine = 0;               // 0 persistent teams, 1 sweep
  int64_t last_launches = 0;         // kernels launched by the last solve
  ~vfvm_batch() {
    delete sweep;
    if (exec) cudaGraphExecDestroy(exec);
    // clones hold views of the first context's grid tables: destroy it last
    for (size_t i = ctx.size(); i-- > 0;) vfvm_destroy(ctx[i]);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace vfvm {
// one precision (KT = double: FP64 form, float: mixed form); instantiated per
// (physics, precision) pair in vfvm_persist_inst.cu
template <class Ph, typename KT>
int persistent_solve_kt(vfvm_ctx* c, const vfvm_control* ctl, const PersistRunHost& run, vfvm_history* hist, float* ms);
template <class Ph, typename KT>
int batch_run_kt(vfvm_batch* b, const vfvm_control* ctl, int ctas, double time, double tstep, double lambda,
                 const double* guess, const double* fallback, float* ms);

template <class Ph>
int persistent_solve_t(vfvm_ctx* c, const vfvm_control* ctl, const PersistRunHost& run, vfvm_history* hist, float* ms) {
  return ctl->precision == VFVM_PRECISION_FP64 ? persistent_solve_kt<Ph, double>(c, ctl, run, hist, ms)
                                               : persistent_solve_kt<Ph, float>(c, ctl, run, hist, ms);
}
template <class Ph>
int batch_run_t(vfvm_batch* b, const vfvm_control* ctl, int ctas, double time, double tstep, double lambda,
                const double* guess, const double* fallback, float* ms) {
  return ctl->precision == VFVM_PRECISION_FP64
             ? batch_run_kt<Ph, double>(b, ctl, ctas, time, tstep, lambda, guess, fallback, ms)
             : batch_run_kt<Ph, float>(b, ctl, ctas, time, tstep, lambda, guess, fallback, ms);
}
}  // namespace vfvm
