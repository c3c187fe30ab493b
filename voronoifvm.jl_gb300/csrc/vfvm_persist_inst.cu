// Explicit instantiation of the persistent engine and batched solver for one
// physics, selected at compile time with -DVFVM_INST_PHYS=<functor type>
// (build.py compiles this file once per registered physics, in parallel).
#include "vfvm_persist_impl.cuh"

#ifndef VFVM_INST_PHYS
#error "compile with -DVFVM_INST_PHYS=vfvm::Phys..."
#endif

namespace vfvm {
template int persistent_solve_t<VFVM_INST_PHYS>(vfvm_ctx*, const vfvm_control*, const PersistRunHost&, vfvm_history*,
                                                float*);
template int batch_run_t<VFVM_INST_PHYS>(vfvm_batch*, const vfvm_control*, int, double, double, double, const double*,
                                         const double*, float*);
}  // namespace vfvm
