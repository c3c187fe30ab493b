// Host side of the coarse-grid correction: aggregation of the nodes into the
// boxes of a coarse tensor grid over the bounding box, and the lists that the
// device Galerkin product P^T A P gathers over.
#include <algorithm>
#include <cmath>
#include <numeric>
#include "vfvm_context.cuh"

static_assert(vfvm::kCoarseMax == VFVM_COARSE_MAX, "coarse size limit of the C ABI");

namespace vfvm {

namespace {

// boxes per axis with prod(nb) <= nagg_target, proportional to the extents
void choose_boxes(const std::vector<double>& ext, int nagg_target, int nb[3]) {
  const int dim = (int)ext.size();
  double vol = 1.0;
  int active = 0;
  for (double e : ext) if (e > 0) { vol *= e; ++active; }
  for (int a = 0; a < 3; ++a) nb[a] = 1;
  if (active == 0) return;
  const double s = std::pow((double)nagg_target / vol, 1.0 / active);
  for (int a = 0; a < dim; ++a) nb[a] = ext[a] > 0 ? std::max(1, (int)std::floor(ext[a] * s + 1e-9)) : 1;
  auto prod = [&]() { return (long long)nb[0] * nb[1] * nb[2]; };
  while (prod() > nagg_target) {
    int big = 0;
    for (int a = 1; a < dim; ++a) if (nb[a] > nb[big]) big = a;
    if (nb[big] == 1) break;
    --nb[big];
  }
}

}  // namespace

int ensure_coarse(vfvm_ctx* c, int target) {
  c->coarse = nullptr;
  if (target <= 0) return VFVM_OK;
  if (target > kCoarseMax) return VFVM_ERR_INPUT;
  auto it = c->coarse_spaces.find(target);
  if (it != c->coarse_spaces.end()) {
    c->coarse = it->second;
    return VFVM_OK;
  }
  auto* cs = new CoarseSpace;
  c->coarse_spaces[target] = cs;
  cs->target = target;
  const int ns = c->ns, N = c->N;
  if (c->grid_base) {
    vfvm_ctx* base = const_cast<vfvm_ctx*>(c->grid_base);
    CoarseSpace* keep = base->coarse;  // the base's selection is left as it was
    int rc = ensure_coarse(base, target);
    const CoarseSpace* bs = base->coarse;
    base->coarse = keep;
    if (rc) return rc;
    cs->nagg = bs->nagg; cs->nc = bs->nc; cs->npairs = bs->npairs;
    cs->agg_of_node.view(bs->agg_of_node); cs->agg_ptr.view(bs->agg_ptr); cs->agg_nodes.view(bs->agg_nodes);
    cs->pair_ptr.view(bs->pair_ptr); cs->pair_ij.view(bs->pair_ij); cs->pair_slot.view(bs->pair_slot);
    cs->pair_row.view(bs->pair_row);
  } else {
    const int dim = c->dim;
    std::vector<double> lo(dim, 1e300), hi(dim, -1e300);
    for (int K = 0; K < N; ++K)
      for (int a = 0; a < dim; ++a) {
        lo[a] = std::min(lo[a], c->h_coord[(size_t)K * dim + a]);
        hi[a] = std::max(hi[a], c->h_coord[(size_t)K * dim + a]);
      }
    std::vector<double> ext(dim);
    for (int a = 0; a < dim; ++a) ext[a] = hi[a] - lo[a];
    int nb[3];
    choose_boxes(ext, std::max(1, target / ns), nb);
    // box of every node, then compact the non-empty boxes into aggregates
    std::vector<int> box(N);
    for (int K = 0; K < N; ++K) {
      int id = 0, stride = 1;
      for (int a = 0; a < dim; ++a) {
        int ia = ext[a] > 0 ? (int)std::floor((c->h_coord[(size_t)K * dim + a] - lo[a]) / ext[a] * nb[a]) : 0;
        ia = std::min(std::max(ia, 0), nb[a] - 1);
        id += ia * stride;
        stride *= nb[a];
      }
      box[K] = id;
    }
    std::vector<int> remap((size_t)nb[0] * nb[1] * nb[2], -1);
    int nagg = 0;
    for (int K = 0; K < N; ++K) if (remap[box[K]] < 0) remap[box[K]] = 0;
    for (auto& r : remap) if (r == 0) r = nagg++;
    std::vector<int> agg(N);
    for (int K = 0; K < N; ++K) agg[K] = remap[box[K]];
    std::vector<int> aptr(nagg + 1, 0), anodes(N);
    for (int K = 0; K < N; ++K) ++aptr[agg[K] + 1];
    for (int I = 0; I < nagg; ++I) aptr[I + 1] += aptr[I];
    {
      std::vector<int> fill(aptr.begin(), aptr.end() - 1);
      for (int K = 0; K < N; ++K) anodes[fill[agg[K]]++] = K;
    }
    // block slots grouped by (aggregate of row, aggregate of column)
    const int64_t nnzb = c->nnzb;
    std::vector<int64_t> key(nnzb);
    std::vector<int> rowof(nnzb);
    for (int K = 0; K < N; ++K)
      for (int s = c->h_browptr[K]; s < c->h_browptr[K + 1]; ++s) {
        key[s] = (int64_t)agg[K] * nagg + agg[c->h_bcol[s]];
        rowof[s] = K;
      }
    std::vector<int> order(nnzb);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return key[a] < key[b]; });
    std::vector<int> pptr, pij, pslot(nnzb), prow(nnzb);
    for (int64_t q = 0; q < nnzb; ++q) {
      const int s = order[q];
      if (q == 0 || key[s] != key[order[q - 1]]) {
        pptr.push_back((int)q);
        pij.push_back((int)key[s]);
      }
      pslot[q] = s;
      prow[q] = rowof[s];
    }
    pptr.push_back((int)nnzb);
    cs->nagg = nagg;
    cs->nc = nagg * ns;
    cs->npairs = (int)pij.size();
    if (cs->nc > kCoarseMax) return VFVM_ERR_INPUT;
    VFVM_CUDA(cs->agg_of_node.upload(agg));
    VFVM_CUDA(cs->agg_ptr.upload(aptr));
    VFVM_CUDA(cs->agg_nodes.upload(anodes));
    VFVM_CUDA(cs->pair_ptr.upload(pptr));
    VFVM_CUDA(cs->pair_ij.upload(pij));
    VFVM_CUDA(cs->pair_slot.upload(pslot));
    VFVM_CUDA(cs->pair_row.upload(prow));
  }
  VFVM_CUDA(cs->A.alloc((size_t)cs->nc * cs->nc));
  VFVM_CUDA(cs->rc.alloc(cs->nc));
  VFVM_CUDA(cs->zc.alloc(cs->nc));
  VFVM_CUDA(cudaMemset(cs->A.p, 0, (size_t)cs->nc * cs->nc * sizeof(float)));
  VFVM_CUDA(cudaMemset(cs->rc.p, 0, cs->nc * sizeof(float)));
  VFVM_CUDA(cudaMemset(cs->zc.p, 0, cs->nc * sizeof(float)));
  c->coarse = cs;
  return VFVM_OK;
}

}  // namespace vfvm

vfvm::CoarseData vfvm_ctx::coarse_data() const {
  vfvm::CoarseData d;
  if (!coarse || coarse->nc == 0) return d;
  d.nagg = coarse->nagg;
  d.nc = coarse->nc;
  d.npairs = coarse->npairs;
  d.dirdof = dirichlet_dof.p;
  d.agg_of_node = coarse->agg_of_node.p;
  d.agg_ptr = coarse->agg_ptr.p;
  d.agg_nodes = coarse->agg_nodes.p;
  d.pair_ptr = coarse->pair_ptr.p;
  d.pair_ij = coarse->pair_ij.p;
  d.pair_slot = coarse->pair_slot.p;
  d.pair_row = coarse->pair_row.p;
  d.A = coarse->A.p;
  d.rc = coarse->rc.p;
  d.zc = coarse->zc.p;
  return d;
}
