// Node tiles of the edge-once assembly, built on the host once per grid.
//
// The reference's edge loop (assemble_edges, src/vfvm_assembly.jl:128-200)
// evaluates every edge flux once and adds it to both end nodes.  On the GPU the
// tiled kernel keeps that property inside a tile: a CTA owns a compact set of
// nodes, stages their unknowns (and those of the halo) in shared memory,
// evaluates each edge with an owned endpoint once and lets every owned node
// gather its edges' results in the reference's edge order.  Only edges that
// cross a tile boundary are evaluated twice (once per owning tile).
//
// Tiles are runs of the Z-order (Morton) curve through the node coordinates:
// compact for structured and unstructured grids alike, with no mesh
// partitioner.  Inside a tile the owned nodes and the halo are sorted by node
// index, so the unknowns of a tile are read as runs of consecutive nodes.
#include <algorithm>
#include <cstdio>
#include <numeric>
#include "vfvm_context.cuh"

namespace vfvm {

namespace {

// nodes per tile: the tile's edge results must fit in shared memory next to its
// staged unknowns (about 2.3 E/N edges per node in 2D, 5-9 in 3D)
int tile_size(int dim, int ns) {
  if (dim <= 2) return ns <= 2 ? 256 : 128;
  return ns <= 1 ? 256 : (ns == 2 ? 128 : 64);
}

uint64_t spread2(uint64_t v) {  // 32 bits -> even bit positions
  v &= 0xffffffffull;
  v = (v | (v << 16)) & 0x0000ffff0000ffffull;
  v = (v | (v << 8)) & 0x00ff00ff00ff00ffull;
  v = (v | (v << 4)) & 0x0f0f0f0f0f0f0f0full;
  v = (v | (v << 2)) & 0x3333333333333333ull;
  v = (v | (v << 1)) & 0x5555555555555555ull;
  return v;
}
uint64_t spread3(uint64_t v) {  // 21 bits -> every third bit position
  v &= 0x1fffffull;
  v = (v | (v << 32)) & 0x001f00000000ffffull;
  v = (v | (v << 16)) & 0x001f0000ff0000ffull;
  v = (v | (v << 8)) & 0x100f00f00f00f00full;
  v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
  v = (v | (v << 2)) & 0x1249249249249249ull;
  return v;
}

}  // namespace

int plan_tiles(const TileInput& in, TilePlan& out) {
  out = TilePlan{};
  const int N = in.N, dim = in.dim;
  const int T = tile_size(dim, in.ns);

  // Z-order keys of the quantised coordinates
  double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  for (int d = 0; d < dim; ++d) {
    lo[d] = hi[d] = in.coord[d];
    for (int k = 1; k < N; ++k) {
      const double x = in.coord[(size_t)k * dim + d];
      lo[d] = std::min(lo[d], x);
      hi[d] = std::max(hi[d], x);
    }
  }
  const int bits = dim == 1 ? 62 : (dim == 2 ? 31 : 21);
  const double qmax = (double)((1ull << bits) - 1);
  std::vector<uint64_t> key(N);
  for (int k = 0; k < N; ++k) {
    uint64_t q[3] = {0, 0, 0};
    for (int d = 0; d < dim; ++d) {
      const double w = hi[d] - lo[d];
      const double r = w > 0 ? (in.coord[(size_t)k * dim + d] - lo[d]) / w : 0.0;
      q[d] = (uint64_t)(std::min(std::max(r, 0.0), 1.0) * qmax);
    }
    key[k] = dim == 1 ? q[0] : (dim == 2 ? spread2(q[0]) | (spread2(q[1]) << 1)
                                         : spread3(q[0]) | (spread3(q[1]) << 1) | (spread3(q[2]) << 2));
  }
  std::vector<int> order(N);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return key[a] < key[b]; });

  const int ntiles = (N + T - 1) / T;
  std::vector<int> tile_of(N);
  for (int i = 0; i < N; ++i) tile_of[order[i]] = i / T;

  TilePlan& P = out;
  P.tile_ptr.assign(1, 0);
  P.tile_eptr.assign(1, 0);
  P.slot_le.assign(in.nnzb, 0);
  std::vector<int> loc(N, -1), own, halo;
  for (int t = 0; t < ntiles; ++t) {
    own.assign(order.begin() + (size_t)t * T, order.begin() + std::min<size_t>((size_t)(t + 1) * T, N));
    std::sort(own.begin(), own.end());
    halo.clear();
    for (int K : own)
      for (int s = in.browptr[K]; s < in.browptr[K + 1]; ++s) {
        const int M = in.bcol[s];
        if (tile_of[M] != t) halo.push_back(M);
      }
    std::sort(halo.begin(), halo.end());
    halo.erase(std::unique(halo.begin(), halo.end()), halo.end());
    const int nloc = (int)(own.size() + halo.size());
    if (nloc > 65535) { out = TilePlan{}; return VFVM_OK; }  // 16-bit local indices: no tiles
    const int base = (int)P.lnodes.size();
    P.lnodes.insert(P.lnodes.end(), own.begin(), own.end());
    P.lnodes.insert(P.lnodes.end(), halo.begin(), halo.end());
    for (int l = 0; l < nloc; ++l) loc[P.lnodes[base + l]] = l;
    int ne = 0;
    for (int K : own) {
      const int dg = in.diag[K];
      for (int s = in.browptr[K]; s < in.browptr[K + 1]; ++s) {
        if (s == dg) continue;
        const int M = in.bcol[s];
        const bool owned = tile_of[M] == t;
        if (owned && M < K) continue;  // created with M's row (owned rows are visited in node order)
        if (ne >= 65535) { out = TilePlan{}; return VFVM_OK; }
        const int a = std::min(K, M), b = std::max(K, M);
        P.edge_ab.push_back((unsigned)loc[a] | ((unsigned)loc[b] << 16));
        P.edge_fac.push_back(in.slot_fac[s]);
        P.slot_le[s] = (uint16_t)ne;
        if (owned) {  // the same edge in M's row
          const int* rb = in.bcol + in.browptr[M];
          const int* re = in.bcol + in.browptr[M + 1];
          const int* it = std::lower_bound(rb, re, K);
          if (it == re || *it != K) {
            fprintf(stderr, "vfvm: unsymmetric block pattern at nodes %d, %d\n", K, M);
            out = TilePlan{};
            return VFVM_ERR_INPUT;
          }
          P.slot_le[in.browptr[M] + (it - rb)] = (uint16_t)ne;
        }
        ++ne;
      }
    }
    for (int l = 0; l < nloc; ++l) loc[P.lnodes[base + l]] = -1;
    P.tile_ptr.push_back((int)P.lnodes.size());
    P.tile_nown.push_back((int)own.size());
    P.tile_eptr.push_back((int)P.edge_ab.size());
    P.maxloc = std::max(P.maxloc, nloc);
    P.maxedges = std::max(P.maxedges, ne);
  }
  P.ntiles = ntiles;
  P.tile_nodes = T;
  return VFVM_OK;
}

int build_assembly_tiles(vfvm_ctx* c, const std::vector<double>& slot_fac) {
  c->ntiles = 0;
  if (c->multireg) return VFVM_OK;  // multi-region grids keep the node-centric kernel
  TileInput in{c->N, c->dim, c->ns, c->nnzb, c->h_coord.data(), c->h_browptr.data(), c->h_bcol.data(),
               c->h_diag.data(), slot_fac.data()};
  TilePlan P;
  const int rc = plan_tiles(in, P);
  if (rc != VFVM_OK || P.ntiles == 0) return rc;
  std::vector<float> efacf(P.edge_fac.begin(), P.edge_fac.end());
  cudaError_t e;
  if ((e = c->tile_ptr.upload(P.tile_ptr)) != cudaSuccess || (e = c->tile_nown.upload(P.tile_nown)) != cudaSuccess ||
      (e = c->tile_eptr.upload(P.tile_eptr)) != cudaSuccess || (e = c->tile_lnodes.upload(P.lnodes)) != cudaSuccess ||
      (e = c->tile_edge_ab.upload(P.edge_ab)) != cudaSuccess || (e = c->tile_edge_fac.upload(P.edge_fac)) != cudaSuccess ||
      (e = c->tile_edge_facf.upload(efacf)) != cudaSuccess || (e = c->slot_le.upload(P.slot_le)) != cudaSuccess) {
    fprintf(stderr, "vfvm: tile tables: %s\n", cudaGetErrorString(e));
    return VFVM_ERR_CUDA;
  }
  c->ntiles = P.ntiles;
  c->tile_nodes = P.tile_nodes;
  c->tile_threads = 256;  // all threads evaluate edges; the first tile_nodes also gather nodes
  c->tile_maxloc = P.maxloc;
  c->tile_maxedges = P.maxedges;
  c->tile_edge_evals = (int64_t)P.edge_ab.size();
  return VFVM_OK;
}

}  // namespace vfvm

vfvm::TileTables vfvm_ctx::tile_tables() const {
  vfvm::TileTables t;
  t.ntiles = ntiles;
  t.maxloc = tile_maxloc;
  t.maxedges = tile_maxedges;
  t.tile_ptr = tile_ptr.p;
  t.tile_nown = tile_nown.p;
  t.tile_eptr = tile_eptr.p;
  t.lnodes = tile_lnodes.p;
  t.edge_ab = tile_edge_ab.p;
  t.edge_fac = tile_edge_fac.p;
  t.edge_facf = tile_edge_facf.p;
  t.slot_le = slot_le.p;
  return t;
}
