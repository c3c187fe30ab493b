// Context: device-resident tables and work buffers of one system.
#pragma once
#include <map>
#include <vector>
#include <string>
#include "vfvm_coarse.cuh"
#include "vfvm_common.cuh"

namespace vfvm {

// Device buffer that frees itself.
template <class T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  bool own = true;  // false: a view of another context's buffer (shared grid tables)
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  ~DBuf() { release(); }
  void release() { if (p && own) cudaFree(p); p = nullptr; n = 0; own = true; }
  void view(const DBuf& o) { release(); p = o.p; n = o.n; own = false; }
  cudaError_t alloc(size_t count) {
    release();
    n = count;
    if (count == 0) return cudaSuccess;
    return cudaMalloc(&p, count * sizeof(T));
  }
  cudaError_t upload(const std::vector<T>& h) {
    cudaError_t e = alloc(h.size());
    if (e != cudaSuccess || h.empty()) return e;
    return cudaMemcpy(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
  }
};

// Tables handed to the assembly kernels by value.
struct AsmTables {
  int N, ns, dim;
  const double* coord;        // N x dim, node-major
  const int* browptr;         // N+1 block-row pointers
  const int* bcol;            // block columns (node index), sorted per row
  const int* diag;            // slot of the diagonal block per row
  // single-region fast path
  int region;                 // the single cell region
  const double* node_fac;     // N
  const double* slot_fac;     // per slot: edge factor (0 at the diagonal)
  const float* slot_facf;     // the same in FP32 (mixed-form Jacobian)
  // multi-region path (nullptr otherwise)
  const int* nitem_ptr; const int* nitem_reg; const double* nitem_fac;
  const int* sitem_ptr; const int* sitem_reg; const double* sitem_fac;
  // boundary-node items grouped by node (bface order within a node)
  const int* bn_ptr; const int* bn_reg; const double* bn_fac;
  // boundary-edge items (edges of boundary faces, per boundary region) grouped by
  // Jacobian slot: both slots of an edge list its items; nullptr when the
  // physics has no bflux
  const int* sbe_ptr; const int* sbe_reg; const double* sbe_fac;
  // physics data
  const double* params;
  const double* nodedata; int nnd;
  const double* bfactors; const double* bvalues; int nbregions; int has_legacy;
  // species restricted to regions (nullptr: every species on every node):
  // reg_spec[ireg-1] = bit mask of the species enabled in cell region ireg,
  // node_spec[K] = bit mask of the species of node K
  const unsigned* reg_spec; const unsigned* node_spec;
  // nodes on an outflow boundary region (physics with boutflow; nullptr: none)
  const uint8_t* outflow_node;
};

// Node tiles of the edge-once assembly (vfvm_tiles.cu builds them, the tiled
// kernel in vfvm_assembly.cu reads them).  Tile t owns a compact set of nodes
// (a run of the Z-order curve through the node coordinates); its local node
// list is the owned nodes followed by the halo (neighbours owned by other
// tiles).  Its edge list holds every edge with an owned endpoint once: edges
// between two owned nodes once, edges to the halo once per tile that owns an
// endpoint.  slot_le maps every off-diagonal Jacobian slot of an owned row to
// the local index of its edge.
struct TileTables {
  int ntiles, maxloc, maxedges;
  const int* tile_ptr;             // ntiles+1 offsets into lnodes
  const int* tile_nown;            // owned nodes per tile (the first entries of its lnodes)
  const int* tile_eptr;            // ntiles+1 offsets into the edge arrays
  const int* lnodes;               // local node lists (global node ids)
  const unsigned* edge_ab;         // local endpoints: first | second << 16 (low -> high node index)
  const double* edge_fac;          // edge form factor
  const float* edge_facf;          // the same in FP32 (mixed-form partials)
  const unsigned short* slot_le;   // nnzb: local edge index of an off-diagonal slot
};

// Shared-memory layout of one tile (byte offsets), identical on host and device.
struct TileSmem {
  size_t lnodes, uv, us, ef, ja, jb, nf, nj, total;
};
template <int NS, typename P>
VFVM_HD TileSmem tile_smem_layout(int maxloc, int maxedges) {
  auto up = [](size_t b) { return (b + 15) & ~(size_t)15; };
  TileSmem L;
  L.lnodes = 0;
  L.uv = up((size_t)maxloc * 4);
  L.us = up(L.uv + (size_t)maxloc * NS * 8);
  const size_t us_bytes = std::is_same<P, double>::value ? 0 : (size_t)maxloc * NS * sizeof(P);
  L.ef = up(L.us + us_bytes);
  L.ja = up(L.ef + (size_t)maxedges * NS * 8);
  L.jb = up(L.ja + (size_t)maxedges * NS * NS * sizeof(P));
  L.nf = up(L.jb + (size_t)maxedges * NS * NS * sizeof(P));  // node terms of the owned nodes
  L.nj = up(L.nf + (size_t)maxloc * NS * 8);
  L.total = up(L.nj + (size_t)maxloc * NS * NS * sizeof(P));
  return L;
}

struct Workspace;  // Krylov / Newton work buffers (vfvm_solver.cu)

// Aggregation tables of the coarse-grid correction (vfvm_coarse.cuh), built for
// a target number of coarse unknowns; contexts on a shared grid view the
// tables of the first one and own only the matrix and vectors.
struct CoarseSpace {
  int target = 0, nagg = 0, nc = 0, npairs = 0;
  DBuf<int> agg_of_node, agg_ptr, agg_nodes, pair_ptr, pair_ij, pair_slot, pair_row;
  DBuf<float> A, rc, zc;
};

}  // namespace vfvm

struct vfvm_ctx {
  int dim = 0, N = 0, ncells = 0, nbf = 0, ns = 1, phys = 0, E = 0;
  int nregions = 1, nbregions = 0, single_region = 1;
  bool multireg = false;
  int nparams = 0, nnd = 0;
  bool has_legacy = false;
  int device = 0;
  cudaStream_t stream = nullptr;

  // host tables
  std::vector<double> h_coord;              // N x dim node-major
  std::vector<int> h_browptr, h_bcol, h_diag;
  std::vector<int> h_edgenodes;             // 2E (lo, hi)
  std::vector<double> h_edgefac, h_nodevol; // summed over regions
  std::vector<double> h_params;
  int64_t nnzb = 0;

  // device tables
  vfvm::DBuf<double> coord, node_fac, slot_fac, nitem_fac, sitem_fac, bn_fac, params, nodedata, bfactors, bvalues;
  vfvm::DBuf<float> slot_facf;
  vfvm::DBuf<int> browptr, bcol, diag, nitem_ptr, nitem_reg, sitem_ptr, sitem_reg, bn_ptr, bn_reg;
  vfvm::DBuf<uint8_t> dirichlet_dof;       // 1 where a Dirichlet penalty acts on the dof
  vfvm::DBuf<int> sbe_ptr, sbe_reg;         // boundary-edge items per slot (physics with bflux)
  vfvm::DBuf<double> sbe_fac;
  // species restricted to regions (enable_species! / enable_boundary_species!);
  // such contexts take the multi-region paths (multireg is set)
  bool species_masked = false;
  std::vector<unsigned> h_reg_spec, h_node_spec;
  vfvm::DBuf<unsigned> reg_spec, node_spec;
  vfvm::DBuf<uint8_t> outflow_node;         // 1 on the nodes of outflow boundary regions (boutflow)

  // scalar (reference) pattern
  int64_t nnz = 0;
  std::vector<int64_t> h_rowptr;
  std::vector<int32_t> h_colind;
  vfvm::DBuf<int64_t> pmap;                 // scalar entry -> BSR value index

  // multicolour ordering (ILU0)
  int ncolors = 0;
  std::vector<int> h_color_ptr;             // ncolors+1
  vfvm::DBuf<int> color_nodes;              // nodes sorted by (colour, index)
  vfvm::DBuf<int> color_ptr;                // device copy of h_color_ptr
  vfvm::DBuf<int> lower_ptr, lower_slots;   // per node: lower-colour slots in factorization order
  // ELL (fixed-width, column-major, -1 padded) copies for the Krylov solve:
  // matrix rows by node (ell_*: node index, block slot), ILU0 lower/upper
  // couplings by position in colour order (lo_*/up_*: neighbour node, block slot)
  int ell_w = 0, lo_w = 0, up_w = 0;
  vfvm::DBuf<int> ell_col, ell_slot, lo_node, lo_slot, up_node, up_slot;

  // node tiles of the edge-once assembly (single-region grids; ntiles = 0: none)
  int ntiles = 0, tile_nodes = 0, tile_maxloc = 0, tile_maxedges = 0, tile_threads = 0;
  int64_t tile_edge_evals = 0;              // edges evaluated per assembly (cross-tile edges twice)
  vfvm::DBuf<int> tile_ptr, tile_nown, tile_eptr, tile_lnodes;
  vfvm::DBuf<unsigned> tile_edge_ab;
  vfvm::DBuf<double> tile_edge_fac;
  vfvm::DBuf<float> tile_edge_facf;
  vfvm::DBuf<uint16_t> slot_le;

  // assembly buffers
  vfvm::DBuf<double> U, Uold, F, J;         // J: nnzb*ns*ns
  vfvm::DBuf<float> Jf;
  vfvm::DBuf<int> errflag;

  vfvm::Workspace* ws = nullptr;
  vfvm::CoarseSpace* coarse = nullptr;     // coarse-grid correction in use (nullptr: none)
  std::map<int, vfvm::CoarseSpace*> coarse_spaces;  // built on first use, by target size
  const vfvm_ctx* grid_base = nullptr;     // clones: the context whose grid tables they view

  vfvm::AsmTables tables() const;
  vfvm::TileTables tile_tables() const;
  // the coarse stage's device view (nc == 0 when it is off)
  vfvm::CoarseData coarse_data() const;
};

namespace vfvm {
// assembly launches (vfvm_assembly.cu)
// tv: device pointer to {time, 1/tstep, lambda}
int launch_assemble(vfvm_ctx* c, const double* U, const double* Uold, const double* tv, double* F, double* J,
                    float* Jf, cudaStream_t s);
int launch_init_dirichlet(vfvm_ctx* c, double* U, const double* tv, cudaStream_t s);
int launch_pattern_gather(vfvm_ctx* c, const double* J, double* out, cudaStream_t s);
// node tiles of the edge-once assembly (vfvm_tiles.cu): plan_tiles is the
// host-only planner (ntiles = 0 where the grid does not suit tiles),
// build_assembly_tiles plans from the context's host tables and uploads
struct TileInput {
  int N, dim, ns;
  int64_t nnzb;
  const double* coord;       // N x dim, node-major
  const int* browptr;        // N+1
  const int* bcol;           // nnzb, sorted per row
  const int* diag;           // N
  const double* slot_fac;    // nnzb: edge factor per off-diagonal slot
};
struct TilePlan {
  int ntiles = 0, tile_nodes = 0, maxloc = 0, maxedges = 0;
  std::vector<int> tile_ptr, tile_nown, tile_eptr, lnodes;
  std::vector<unsigned> edge_ab;
  std::vector<double> edge_fac;
  std::vector<uint16_t> slot_le;
};
int plan_tiles(const TileInput& in, TilePlan& out);
int build_assembly_tiles(vfvm_ctx* c, const std::vector<double>& slot_fac);
// per-physics launch attributes of the tiled assembly (shared memory above the
// default limit); called once per context, outside any stream capture
int prepare_tiled_assembly(vfvm_ctx* c);
void destroy_workspace(Workspace* w);
// A context on the same grid as `base` with other physics data: grid tables are
// shared views of base's device buffers (base must outlive the clone); unknowns,
// Jacobian, parameters, node data and legacy boundary data are its own.
vfvm_ctx* clone_context(const vfvm_ctx* base, const vfvm_physics_desc* ph, int* status);
// replace the per-node physics data (nnodes x nnodedata values, host)
int set_nodedata(vfvm_ctx* c, const double* data, int nnd);
// select the coarse space for about `target` coarse unknowns (0: none), building
// it on first use.  Clones view the tables of their grid_base (built first).
int ensure_coarse(vfvm_ctx* c, int target);
}  // namespace vfvm
