// Contexts that share a grid: many systems on one grid (parameter sweeps,
// training-data generation) reuse one set of device tables.
#include <algorithm>
#include <cstring>
#include "vfvm_context.cuh"
#include "vfvm_physics.cuh"

namespace vfvm {

#define CLONE_CUDA(call)                                                                           \
  do {                                                                                             \
    cudaError_t _e = (call);                                                                       \
    if (_e != cudaSuccess) {                                                                       \
      fprintf(stderr, "vfvm clone_context: %s (%s:%d)\n", cudaGetErrorString(_e), __FILE__, __LINE__); \
      *status = VFVM_ERR_CUDA;                                                                     \
      delete c;                                                                                    \
      return nullptr;                                                                              \
    }                                                                                              \
  } while (0)

vfvm_ctx* clone_context(const vfvm_ctx* b, const vfvm_physics_desc* ph, int* status) {
  *status = VFVM_ERR_INPUT;
  if (!b || !ph || ph->physics_id != b->phys) return nullptr;
  if (ph->nparams < physics_nparams(ph->physics_id) || (ph->nparams > 0 && !ph->params)) return nullptr;
  if (ph->nnodedata < physics_nnodedata(ph->physics_id) || (ph->nnodedata > 0 && !ph->nodedata)) return nullptr;
  if (ph->nnodedata != b->nnd) return nullptr;
  vfvm_ctx* c = new vfvm_ctx;
  c->dim = b->dim; c->N = b->N; c->ncells = b->ncells; c->nbf = b->nbf; c->ns = b->ns; c->phys = b->phys; c->E = b->E;
  c->nregions = b->nregions; c->nbregions = b->nbregions; c->single_region = b->single_region;
  c->multireg = b->multireg; c->nnd = b->nnd; c->device = b->device;
  c->nnzb = b->nnzb; c->nnz = b->nnz; c->ncolors = b->ncolors; c->h_color_ptr = b->h_color_ptr;
  c->grid_base = b->grid_base ? b->grid_base : b;
  CLONE_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  // shared grid tables
  c->coord.view(b->coord); c->node_fac.view(b->node_fac); c->slot_fac.view(b->slot_fac); c->slot_facf.view(b->slot_facf);
  c->nitem_fac.view(b->nitem_fac); c->sitem_fac.view(b->sitem_fac); c->bn_fac.view(b->bn_fac);
  c->browptr.view(b->browptr); c->bcol.view(b->bcol); c->diag.view(b->diag);
  c->nitem_ptr.view(b->nitem_ptr); c->nitem_reg.view(b->nitem_reg); c->sitem_ptr.view(b->sitem_ptr);
  c->sitem_reg.view(b->sitem_reg); c->bn_ptr.view(b->bn_ptr); c->bn_reg.view(b->bn_reg);
  c->dirichlet_dof.view(b->dirichlet_dof); c->pmap.view(b->pmap);
  c->sbe_ptr.view(b->sbe_ptr); c->sbe_reg.view(b->sbe_reg); c->sbe_fac.view(b->sbe_fac);
  c->color_nodes.view(b->color_nodes); c->color_ptr.view(b->color_ptr);
  c->lower_ptr.view(b->lower_ptr); c->lower_slots.view(b->lower_slots);
  c->ell_w = b->ell_w; c->lo_w = b->lo_w; c->up_w = b->up_w;
  c->ell_col.view(b->ell_col); c->ell_slot.view(b->ell_slot); c->lo_node.view(b->lo_node);
  c->lo_slot.view(b->lo_slot); c->up_node.view(b->up_node); c->up_slot.view(b->up_slot);
  c->ntiles = b->ntiles; c->tile_nodes = b->tile_nodes; c->tile_maxloc = b->tile_maxloc;
  c->tile_maxedges = b->tile_maxedges; c->tile_threads = b->tile_threads; c->tile_edge_evals = b->tile_edge_evals;
  c->tile_ptr.view(b->tile_ptr); c->tile_nown.view(b->tile_nown); c->tile_eptr.view(b->tile_eptr);
  c->tile_lnodes.view(b->tile_lnodes); c->tile_edge_ab.view(b->tile_edge_ab); c->tile_edge_fac.view(b->tile_edge_fac);
  c->tile_edge_facf.view(b->tile_edge_facf); c->slot_le.view(b->slot_le);
  c->species_masked = b->species_masked; c->h_reg_spec = b->h_reg_spec; c->h_node_spec = b->h_node_spec;
  c->reg_spec.view(b->reg_spec); c->node_spec.view(b->node_spec); c->outflow_node.view(b->outflow_node);
  // own physics data; the legacy boundary data must match the base's structure
  c->h_params.assign(ph->params, ph->params + ph->nparams);
  c->nparams = ph->nparams;
  std::vector<double> pp(c->h_params);
  if (pp.empty()) pp.push_back(0.0);
  CLONE_CUDA(c->params.upload(pp));
  if (c->nnd > 0) {
    std::vector<double> nd(ph->nodedata, ph->nodedata + (size_t)c->N * c->nnd);
    CLONE_CUDA(c->nodedata.upload(nd));
  }
  std::vector<double> bf((size_t)c->ns * c->nbregions, 0.0), bv(bf.size(), 0.0);
  if (ph->nbregions > 0 && ph->bfactors && ph->bvalues) {
    for (int r = 0; r < std::min(ph->nbregions, c->nbregions); ++r)
      for (int i = 0; i < c->ns; ++i) {
        bf[i + (size_t)c->ns * r] = ph->bfactors[i + (size_t)c->ns * r];
        bv[i + (size_t)c->ns * r] = ph->bvalues[i + (size_t)c->ns * r];
      }
  }
  for (size_t i = 0; i < bf.size(); ++i) if (bf[i] != 0.0 || bv[i] != 0.0) c->has_legacy = true;
  if (c->has_legacy != b->has_legacy) { *status = VFVM_ERR_INPUT; delete c; return nullptr; }
  CLONE_CUDA(c->bfactors.upload(bf));
  CLONE_CUDA(c->bvalues.upload(bv));
  const size_t n = (size_t)c->N * c->ns;
  CLONE_CUDA(c->U.alloc(n));
  CLONE_CUDA(c->Uold.alloc(n));
  CLONE_CUDA(c->F.alloc(n));
  CLONE_CUDA(c->J.alloc((size_t)c->nnzb * c->ns * c->ns));
  CLONE_CUDA(c->errflag.alloc(4));
  CLONE_CUDA(cudaMemset(c->errflag.p, 0, 4 * sizeof(int)));
  *status = VFVM_OK;
  return c;
}

int set_nodedata(vfvm_ctx* c, const double* data, int nnd) {
  if (!c || nnd != c->nnd || (nnd > 0 && !data)) return VFVM_ERR_INPUT;
  if (nnd == 0) return VFVM_OK;
  if (!c->nodedata.own) return VFVM_ERR_INPUT;
  VFVM_CUDA(cudaMemcpyAsync(c->nodedata.p, data, (size_t)c->N * nnd * sizeof(double), cudaMemcpyHostToDevice,
                            c->stream));
  VFVM_CUDA(cudaStreamSynchronize(c->stream));
  return VFVM_OK;
}

}  // namespace vfvm

extern "C" int vfvm_set_nodedata(vfvm_ctx* c, const double* data, int32_t nnodedata) {
  return vfvm::set_nodedata(c, data, nnodedata);
}
