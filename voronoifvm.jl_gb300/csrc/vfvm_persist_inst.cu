// Explicit instantiation of the persistent engine and batched solver for one
// physics and one precision, selected at compile time with
// -DVFVM_INST_PHYS=<functor type> -DVFVM_INST_KT=<double|float> (build.py
// compiles this file once per pair, in parallel).
#include "vfvm_persist_impl.cuh"

#if !defined(VFVM_INST_PHYS) || !defined(VFVM_INST_KT)
#error "compile with -DVFVM_INST_PHYS=vfvm::Phys... -DVFVM_INST_KT=double|float"
#endif

namespace vfvm {
template int persistent_solve_kt<VFVM_INST_PHYS, VFVM_INST_KT>(vfvm_ctx*, const vfvm_control*, const PersistRunHost&,
                                                               vfvm_history*, float*);
template int batch_run_kt<VFVM_INST_PHYS, VFVM_INST_KT>(vfvm_batch*, const vfvm_control*, int, double, double, double,
                                                        const double*, const double*, float*);
}  // namespace vfvm
