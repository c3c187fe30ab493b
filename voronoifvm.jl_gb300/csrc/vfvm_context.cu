// Context creation: grid tables, edgewise form factors, Jacobian block pattern,
// boundary items, structural masks, multicolour ordering; upload to the device.
//
// Host-side setup mirrors what SystemState(sys) + update_grid_edgewise! do once
// per system in the reference (src/vfvm_state.jl:99-157,
// src/vfvm_system.jl:690-755).  It runs once per context; the per-Newton-step
// work is all on the device.
#include <algorithm>
#include <cstring>
#include <limits>
#include <map>
#include <numeric>
#include <random>
#include "vfvm_context.cuh"
#include "vfvm_physics.cuh"

using namespace vfvm;

namespace {

// Local edges of a simplex: edge e joins local nodes en[e][0], en[e][1].
// Triangle: edge e is opposite local node e.  Tetrahedron: pairs in lexicographic
// order.  The Voronoi formulas below only need a consistent edge <-> node-pair map.
const int kTriEdges[3][2] = {{1, 2}, {2, 0}, {0, 1}};
const int kTetEdges[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};

inline double dist2(const double* a, const double* b, int dim) {
  double s = 0;
  for (int c = 0; c < dim; ++c) { double d = a[c] - b[c]; s += d * d; }
  return s;
}

constexpr double kPi = 3.141592653589793;

// First coordinate (r) of a triangle's circumcenter: the published formula
// relative to vertex a (J. R. Shewchuk, "Lecture Notes on Geometric Robustness").
double tri_circumcenter_r(const double* a, const double* b, const double* c) {
  const double xba = b[0] - a[0], yba = b[1] - a[1], xca = c[0] - a[0], yca = c[1] - a[1];
  const double balength = xba * xba + yba * yba, calength = xca * xca + yca * yca;
  const double denominator = 0.5 / (xba * yca - yba * xca);
  return a[0] + (yca * balength - yba * calength) * denominator;
}

// Voronoi node volumes and edge weights sigma_kl / h_kl of one simplex
// (src/vfvm_formfactors.jl:12-23, :64-100, :163-235) in the grid's coordinate
// system (VFVM_COORD_*):
// * polar / spherical 1D (:25-62): the shell volumes between the cell's inner
//   radius r0, its midpoint and its outer radius r1, and the circle / sphere
//   surface at the midpoint over r1 - r0; as in the reference, the inner part
//   goes to the cell's first node, the outer to its second (cells run outwards
//   on the grids of simplexgrid);
// * cylindrical 2D (:102-161): the Cartesian contributions, each node's part of
//   the Voronoi cell times 2 pi the mean radius of its triangle (node, edge
//   midpoint, circumcenter), each edge weight times 2 pi the mean radius of the
//   Voronoi face (edge midpoint, circumcenter).
void simplex_factors(int dim, int csys, const double* const* x, double* nodef, double* edgef) {
  if (dim == 1 && csys != VFVM_COORD_CARTESIAN) {
    double r0 = x[0][0], r1 = x[1][0];
    if (r1 < r0) std::swap(r0, r1);
    const double rhalf = 0.5 * (r1 + r0);
    if (csys == VFVM_COORD_POLAR1D) {
      nodef[0] = kPi * (rhalf * rhalf - r0 * r0);
      nodef[1] = kPi * (r1 * r1 - rhalf * rhalf);
      edgef[0] = 2.0 * kPi * rhalf / (r1 - r0);
    } else {
      nodef[0] = kPi * (rhalf * rhalf * rhalf - r0 * r0 * r0) * 4.0 / 3.0;
      nodef[1] = kPi * (r1 * r1 * r1 - rhalf * rhalf * rhalf) * 4.0 / 3.0;
      edgef[0] = 4.0 * kPi * (rhalf * rhalf) / (r1 - r0);
    }
    return;
  }
  if (dim == 1) {
    double h = std::fabs(x[1][0] - x[0][0]);
    nodef[0] = nodef[1] = 0.5 * h;
    edgef[0] = 1.0 / h;
    return;
  }
  if (dim == 2) {
    double l2[3];
    for (int e = 0; e < 3; ++e) l2[e] = dist2(x[kTriEdges[e][0]], x[kTriEdges[e][1]], 2);
    // twice the area from two edge vectors
    double ax = x[kTriEdges[2][0]][0] - x[kTriEdges[2][1]][0], ay = x[kTriEdges[2][0]][1] - x[kTriEdges[2][1]][1];
    double bx = x[kTriEdges[1][0]][0] - x[kTriEdges[1][1]][0], by = x[kTriEdges[1][0]][1] - x[kTriEdges[1][1]][1];
    double area = std::fabs(0.5 * (ax * by - bx * ay));
    double inv8a = 0.125 / area;
    for (int i = 0; i < 3; ++i) nodef[i] = 0.0;
    if (csys == VFVM_COORD_CYLINDRICAL2D) {
      const double rcc = tri_circumcenter_r(x[0], x[1], x[2]);
      for (int e = 0; e < 3; ++e) {
        const int a0 = kTriEdges[e][0], a1 = kTriEdges[e][1];
        edgef[e] = (l2[(e + 1) % 3] + l2[(e + 2) % 3] - l2[e]) * inv8a;
        const double emid = 0.5 * (x[a0][0] + x[a1][0]);
        const double cyl0 = 2.0 * kPi * (x[a0][0] + rcc + emid) / 3.0;
        const double cyl1 = 2.0 * kPi * (x[a1][0] + rcc + emid) / 3.0;
        nodef[a0] += edgef[e] * l2[e] * 0.25 * cyl0;
        nodef[a1] += edgef[e] * l2[e] * 0.25 * cyl1;
      }
      for (int e = 0; e < 3; ++e) {
        const double rmid = (rcc + 0.5 * (x[kTriEdges[e][0]][0] + x[kTriEdges[e][1]][0])) / 2.0;
        edgef[e] *= 2.0 * kPi * rmid;
      }
      return;
    }
    for (int e = 0; e < 3; ++e) {
      // half the cotangent of the angle opposite edge e
      edgef[e] = (l2[(e + 1) % 3] + l2[(e + 2) % 3] - l2[e]) * inv8a;
      double q = 0.25 * edgef[e] * l2[e];
      nodef[kTriEdges[e][0]] += q;
      nodef[kTriEdges[e][1]] += q;
    }
    return;
  }
  // tetrahedron: face-based formula of WIAS/pdelib as used by the reference
  double l2[6];
  for (int e = 0; e < 6; ++e) l2[e] = dist2(x[kTetEdges[e][0]], x[kTetEdges[e][1]], 3);
  double a[3], b[3], c[3];
  for (int k = 0; k < 3; ++k) { a[k] = x[1][k] - x[0][k]; b[k] = x[2][k] - x[0][k]; c[k] = x[3][k] - x[0][k]; }
  double det = a[0] * (b[1] * c[2] - c[1] * b[2]) + b[0] * (c[1] * a[2] - a[1] * c[2]) + c[0] * (a[1] * b[2] - b[1] * a[2]);
  double vol6 = std::fabs(det);
  double w = 96.0 * vol6;  // 96 * 6 * volume
  // for each face (opposite local node v): its three edges and, for each of them,
  // the tetrahedron edge opposite to it
  static const int face_e[4][3] = {{4, 5, 3}, {5, 2, 1}, {4, 0, 2}, {0, 3, 1}};
  static const int opp_e[4][3] = {{1, 0, 2}, {0, 3, 4}, {1, 5, 3}, {5, 2, 4}};
  double ef[6] = {0, 0, 0, 0, 0, 0};
  for (int v = 0; v < 4; ++v) {
    const int e1 = face_e[v][0], e2 = face_e[v][1], e3 = face_e[v][2];
    double h1 = l2[e1] * (l2[e2] + l2[e3] - l2[e1]);
    double h2 = l2[e2] * (l2[e3] + l2[e1] - l2[e2]);
    double h3 = l2[e3] * (l2[e1] + l2[e2] - l2[e3]);
    double vf = (h1 * l2[opp_e[v][0]] + h2 * l2[opp_e[v][1]] + h3 * l2[opp_e[v][2]] - 2.0 * l2[e1] * l2[e2] * l2[e3]) /
                (w * (h1 + h2 + h3));
    ef[e1] += h1 * vf;
    ef[e2] += h2 * vf;
    ef[e3] += h3 * vf;
  }
  for (int i = 0; i < 4; ++i) nodef[i] = 0.0;
  for (int e = 0; e < 6; ++e) {
    nodef[kTetEdges[e][0]] += ef[e];
    nodef[kTetEdges[e][1]] += ef[e];
    edgef[e] = 6.0 * ef[e] / l2[e];
  }
}

// Boundary face node factors (src/vfvm_formfactors.jl:244-332): a point (1,
// or the circle 2 pi r / the sphere 4 pi r^2 at its radius), a segment (half
// its length each, or in cylindrical coordinates pi (r_node + r_mid) l / 2, the
// surface of revolution of its half), a triangle.
void bface_factors(int dim, int csys, const double* const* x, double* nodef) {
  if (dim == 1) {
    const double r = x[0][0];
    nodef[0] = csys == VFVM_COORD_POLAR1D ? 2.0 * kPi * r : csys == VFVM_COORD_SPHERICAL1D ? 4.0 * kPi * (r * r) : 1.0;
    return;
  }
  if (dim == 2 && csys == VFVM_COORD_CYLINDRICAL2D) {
    const double r1 = x[0][0], r2 = x[1][0], dr = r1 - r2, dz = x[0][1] - x[1][1];
    const double rmid = (r1 + r2) / 2.0, l = std::sqrt(dr * dr + dz * dz);
    nodef[0] = kPi * (r1 + rmid) * l / 2.0;
    nodef[1] = kPi * (r2 + rmid) * l / 2.0;
    return;
  }
  if (dim == 2) {
    double h = std::sqrt(dist2(x[0], x[1], 2));
    nodef[0] = nodef[1] = 0.5 * h;
    return;
  }
  double l2[3];
  for (int e = 0; e < 3; ++e) l2[e] = dist2(x[kTriEdges[e][0]], x[kTriEdges[e][1]], 3);
  double g[3];
  for (int e = 0; e < 3; ++e) g[e] = (l2[(e + 1) % 3] + l2[(e + 2) % 3] - l2[e]) * l2[e];
  double area = 0.25 * std::sqrt(g[0] + g[1] + g[2]);
  double s = 1.0 / (8.0 * area);
  for (int i = 0; i < 3; ++i) nodef[i] = 0.0;
  for (int e = 0; e < 3; ++e) {
    double q = 0.25 * g[e] * s;
    nodef[kTriEdges[e][0]] += q;
    nodef[kTriEdges[e][1]] += q;
  }
}

// Edge factors of the edges of a boundary face (the bfacefactors! edge
// parameters, src/vfvm_formfactors.jl:263-274 for a segment, :293-332 for a
// triangle): 1 / length for a segment; half the cotangent of the opposite angle
// for a triangle, local edge e opposite local node e.
// In cylindrical coordinates the reference sets no edge parameter for a
// boundary segment (its zero-initialised bfaceedgefactors, src/vfvm_system.jl:652).
void bface_edge_factors(int dim, int csys, const double* const* x, double* edgef) {
  if (dim == 2) {
    edgef[0] = csys == VFVM_COORD_CYLINDRICAL2D ? 0.0 : 1.0 / std::sqrt(dist2(x[0], x[1], 2));
    return;
  }
  double l2[3];
  for (int e = 0; e < 3; ++e) l2[e] = dist2(x[kTriEdges[e][0]], x[kTriEdges[e][1]], 3);
  double g[3];
  for (int e = 0; e < 3; ++e) g[e] = (l2[(e + 1) % 3] + l2[(e + 2) % 3] - l2[e]) * l2[e];
  double area = 0.25 * std::sqrt(g[0] + g[1] + g[2]);
  double s = 1.0 / (8.0 * area);
  for (int e = 0; e < 3; ++e) edgef[e] = g[e] * s / l2[e];
}

struct RegFac { int reg; double fac; };

inline void add_regfac(std::vector<RegFac>& v, int reg, double f) {
  for (auto& r : v) if (r.reg == reg) { r.fac += f; return; }
  v.push_back({reg, f});
  std::sort(v.begin(), v.end(), [](const RegFac& a, const RegFac& b) { return a.reg < b.reg; });
}

// Host-side evaluation of the physics on duals at random states to find which
// local Jacobian entries can ever be nonzero (structural masks).
template <class Ph>
void probe_t(const Ph& ph0, const double* params, int dim, const std::vector<int>& cregs, const std::vector<int>& bregs,
             std::vector<uint8_t>& nm, std::vector<uint8_t>& em, std::vector<uint8_t>& bm) {
  constexpr int NS = Ph::NS;
  Ph ph = ph0;
  ph.load(params);
  nm.assign(NS * NS, 0); em.assign(NS * 2 * NS, 0); bm.assign(NS * NS, 0);
  std::mt19937_64 rng(1234);
  std::uniform_real_distribution<double> U(0.1, 1.1), X(0.0, 1.0);
  double dK[4] = {1.3, 1.3, 1.3, 1.3}, dL[4] = {0.7, 0.7, 0.7, 0.7};
  for (int sample = 0; sample < 6; ++sample) {
    double x[3] = {X(rng), X(rng), X(rng)}, y[3] = {X(rng), X(rng), X(rng)};
    for (int reg : cregs) {
      NodeItem ni{0, reg, x, 0.5, 0.5, dK};
      Dual<NS> u[NS], r[NS], s[NS];
      for (int i = 0; i < NS; ++i) { u[i] = dseed<NS, double>(U(rng), i); r[i] = dconst<NS, double>(0); s[i] = dconst<NS, double>(0); }
      if (Ph::has_reaction) ph.reaction(r, u, ni);
      if (Ph::has_storage) ph.storage(s, u, ni);
      for (int i = 0; i < NS; ++i)
        for (int j = 0; j < NS; ++j)
          if (r[i].d[j] != 0.0 || s[i].d[j] != 0.0) nm[i * NS + j] = 1;
      EdgeItem ei{0, 1, reg, x, y, 0.5, 0.5, dK, dL};
      Dual<2 * NS> uk[NS], ul[NS], f[NS];
      for (int i = 0; i < NS; ++i) {
        uk[i] = dseed<2 * NS, double>(U(rng), i);
        ul[i] = dseed<2 * NS, double>(U(rng), NS + i);
        f[i] = dconst<2 * NS, double>(0);
      }
      ph.flux(f, uk, ul, ei);
      for (int i = 0; i < NS; ++i)
        for (int j = 0; j < 2 * NS; ++j)
          if (f[i].d[j] != 0.0) em[i * 2 * NS + j] = 1;
      if (Ph::has_boutflow) {  // the flux's entries, on the edges at an outflow node
        for (int node = 1; node <= 2; ++node) {
          EdgeItem eo = ei;
          eo.outflownode = node;
          for (int i = 0; i < NS; ++i) f[i] = dconst<2 * NS, double>(0);
          ph.boutflow(f, uk, ul, eo);
          for (int i = 0; i < NS; ++i)
            for (int j = 0; j < 2 * NS; ++j)
              if (f[i].d[j] != 0.0) em[i * 2 * NS + j] = 1;
        }
      }
      if (Ph::has_edgereaction) {  // the same four entries per species pair as a flux
        for (int i = 0; i < NS; ++i) f[i] = dconst<2 * NS, double>(0);
        ph.edgereaction(f, uk, ul, ei);
        for (int i = 0; i < NS; ++i)
          for (int j = 0; j < 2 * NS; ++j)
            if (f[i].d[j] != 0.0) em[i * 2 * NS + j] = 1;
      }
    }
    for (int reg : bregs) {
      double dv[NS];
      BNodeItem bi{0, reg, x, 0.5, 0.5, 1.0, kDirichlet, dv};
      Dual<NS> u[NS], yb[NS], sb[NS];
      for (int i = 0; i < NS; ++i) {
        u[i] = dseed<NS, double>(U(rng), i);
        yb[i] = dconst<NS, double>(0);
        sb[i] = dconst<NS, double>(0);
      }
      if (Ph::has_breaction) ph.breaction(yb, u, bi);
      if (Ph::has_bstorage) ph.bstorage(sb, u, bi);
      for (int i = 0; i < NS; ++i)
        for (int j = 0; j < NS; ++j)
          if (yb[i].d[j] != 0.0 || sb[i].d[j] != 0.0) bm[i * NS + j] = 1;
    }
  }
}

// Structural mask of bflux on boundary region reg: which partials d f_i /
// d u_first,j and d f_i / d u_second,j can be nonzero (NS x 2NS).
template <class Ph>
void probe_bflux_t(const Ph& ph0, const double* params, int reg, std::vector<uint8_t>& out) {
  constexpr int NS = Ph::NS;
  Ph ph = ph0;
  ph.load(params);
  out.assign(NS * 2 * NS, 0);
  if (!Ph::has_bflux) return;
  std::mt19937_64 rng(4321);
  std::uniform_real_distribution<double> U(0.1, 1.1), X(0.0, 1.0);
  for (int sample = 0; sample < 6; ++sample) {
    double x[3] = {X(rng), X(rng), X(rng)}, y[3] = {X(rng), X(rng), X(rng)};
    BEdgeItem be{0, 1, reg, x, y, 0.5, 0.5};
    Dual<2 * NS> uk[NS], ul[NS], f[NS];
    for (int i = 0; i < NS; ++i) {
      uk[i] = dseed<2 * NS, double>(U(rng), i);
      ul[i] = dseed<2 * NS, double>(U(rng), NS + i);
      f[i] = dconst<2 * NS, double>(0);
    }
    ph.bflux(f, uk, ul, be);
    for (int i = 0; i < NS; ++i)
      for (int j = 0; j < 2 * NS; ++j)
        if (f[i].d[j] != 0.0) out[i * 2 * NS + j] = 1;
  }
}

// Structural mask of the boundary-node terms (breaction, bstorage) on boundary
// region reg: which partials d y_i / d u_j can be nonzero (NS x NS).  Per
// region, since the reference creates an entry only where a term's partial is
// nonzero (_addnz, src/vfvm_assembly.jl:318-407): a coupling that a physics
// makes on one boundary region gives no entries at the nodes of the others.
template <class Ph>
void probe_bnode_t(const Ph& ph0, const double* params, int reg, std::vector<uint8_t>& out) {
  constexpr int NS = Ph::NS;
  Ph ph = ph0;
  ph.load(params);
  out.assign(NS * NS, 0);
  if (!Ph::has_breaction && !Ph::has_bstorage) return;
  std::mt19937_64 rng(2468);
  std::uniform_real_distribution<double> U(0.1, 1.1), X(0.0, 1.0);
  for (int sample = 0; sample < 6; ++sample) {
    double x[3] = {X(rng), X(rng), X(rng)}, dv[NS];
    BNodeItem bi{0, reg, x, 0.5, 0.5, 1.0, kDirichlet, dv};
    Dual<NS> u[NS], yb[NS], sb[NS];
    for (int i = 0; i < NS; ++i) {
      u[i] = dseed<NS, double>(U(rng), i);
      yb[i] = dconst<NS, double>(0);
      sb[i] = dconst<NS, double>(0);
    }
    if (Ph::has_breaction) ph.breaction(yb, u, bi);
    if (Ph::has_bstorage) ph.bstorage(sb, u, bi);
    for (int i = 0; i < NS; ++i)
      for (int j = 0; j < NS; ++j)
        if (yb[i].d[j] != 0.0 || sb[i].d[j] != 0.0) out[i * NS + j] = 1;
  }
}

// Dirichlet species of a boundary region according to breaction (the
// dirichlet_value capture of _initialize_dirichlet!).
template <class Ph>
void dirichlet_species_t(const Ph& ph0, const double* params, int reg, int ns, uint8_t* out) {
  constexpr int NS = Ph::NS;
  Ph ph = ph0;
  ph.load(params);
  double dv[NS], u[NS], y[NS], x[3] = {0.25, 0.25, 0.25};
  for (int i = 0; i < NS; ++i) { dv[i] = std::numeric_limits<double>::infinity(); u[i] = 0.5; y[i] = 0; }
  BNodeItem bi{0, reg, x, 0.0, 0.0, 1.0, kDirichlet, dv};
  if (Ph::has_breaction) ph.breaction(y, u, bi);
  for (int i = 0; i < ns && i < NS; ++i) out[i] = std::isinf(dv[i]) ? 0 : 1;
}

}  // namespace

AsmTables vfvm_ctx::tables() const {
  AsmTables t;
  t.N = N; t.ns = ns; t.dim = dim;
  t.coord = coord.p; t.browptr = browptr.p; t.bcol = bcol.p; t.diag = diag.p;
  t.region = single_region;
  t.node_fac = node_fac.p; t.slot_fac = slot_fac.p; t.slot_facf = slot_facf.p;
  t.nitem_ptr = multireg ? nitem_ptr.p : nullptr; t.nitem_reg = nitem_reg.p; t.nitem_fac = nitem_fac.p;
  t.sitem_ptr = multireg ? sitem_ptr.p : nullptr; t.sitem_reg = sitem_reg.p; t.sitem_fac = sitem_fac.p;
  t.bn_ptr = bn_ptr.p; t.bn_reg = bn_reg.p; t.bn_fac = bn_fac.p;
  t.sbe_ptr = sbe_ptr.n ? sbe_ptr.p : nullptr; t.sbe_reg = sbe_reg.p; t.sbe_fac = sbe_fac.p;
  t.params = params.p; t.nodedata = nodedata.p; t.nnd = nnd;
  t.bfactors = bfactors.p; t.bvalues = bvalues.p; t.nbregions = nbregions; t.has_legacy = has_legacy ? 1 : 0;
  t.reg_spec = species_masked ? reg_spec.p : nullptr;
  t.node_spec = species_masked ? node_spec.p : nullptr;
  t.outflow_node = outflow_node.n ? outflow_node.p : nullptr;
  return t;
}

#define SETUP_CUDA(call)                       \
  do {                                         \
    cudaError_t _e = (call);                   \
    if (_e != cudaSuccess) {                   \
      fprintf(stderr, "vfvm_create: %s (%s:%d)\n", cudaGetErrorString(_e), __FILE__, __LINE__); \
      *status = VFVM_ERR_CUDA;                 \
      delete c;                                \
      return nullptr;                          \
    }                                          \
  } while (0)

extern "C" void vfvm_control_default(vfvm_control* c) {
  std::memset(c, 0, sizeof(*c));
  c->abstol = 1.0e-10; c->reltol = 1.0e-10; c->maxiters = 100;
  c->tol_round = 1.0e-10; c->tol_mono = 1.0e-3;
  c->damp_initial = 1.0; c->damp_growth = 1.2; c->max_round = 1000;
  c->is_linear = 0; c->updatecontrol = 1;
  c->reltol_linear = 1.0e-4; c->abstol_linear = 0.0; c->maxiters_linear = 100;
  c->krylov = VFVM_KRYLOV_BICGSTAB; c->precon = VFVM_PRECON_ILU0; c->precision = VFVM_PRECISION_FP64;
  c->gmres_restart = 30;
  c->dt = 0.1; c->dt_min = 1.0e-3; c->dt_max = 1.0; c->dt_grow = 1.2; c->dt_decrease = 0.5;
  c->dp = 1.0; c->dp_min = 1.0e-3; c->dp_max = 1.0; c->dp_grow = 1.0; c->dp_decrease = 0.5;
  c->du_opt = 0.1; c->du_max_factor = 1.2;
  c->num_final_steps = 5; c->force_first_step = 0; c->handle_exceptions = 0; c->store_all = 1;
  c->engine = VFVM_ENGINE_AUTO; c->team_ctas = 0; c->coarse = 0;
}

extern "C" vfvm_ctx* vfvm_create(const vfvm_grid* g, const vfvm_physics_desc* ph, int* status) {
  int dummy;
  if (!status) status = &dummy;
  *status = VFVM_ERR_INPUT;
  if (!g || !ph || g->dim < 1 || g->dim > 3 || g->nnodes < 2 || g->ncells < 1 || !g->coord || !g->cellnodes ||
      !g->cellregions || (g->nbfaces > 0 && (!g->bfacenodes || !g->bfaceregions)))
    return nullptr;
  const int ns = physics_nspec(ph->physics_id);
  if (ns == 0) return nullptr;
  if (ph->nparams < physics_nparams(ph->physics_id) || (ph->nparams > 0 && !ph->params)) return nullptr;
  if (ph->nnodedata < physics_nnodedata(ph->physics_id) || (ph->nnodedata > 0 && !ph->nodedata)) return nullptr;
  {
    std::vector<double> p(ph->params, ph->params + ph->nparams);
    p.resize(16, 0.0);
    if (!dispatch_physics(ph->physics_id, [&](auto phy) { return decltype(phy)::valid(g->dim, p.data()) ? 1 : 0; }))
      return nullptr;
  }
  const int dim = g->dim, N = g->nnodes, nc = g->ncells, nbf = g->nbfaces, nvc = dim + 1;
  // the coordinate systems with form factors: Cartesian in every dimension,
  // polar and spherical in 1D, cylindrical in 2D
  const int csys = g->coordsystem;
  if (!(csys == VFVM_COORD_CARTESIAN || (dim == 1 && (csys == VFVM_COORD_POLAR1D || csys == VFVM_COORD_SPHERICAL1D)) ||
        (dim == 2 && csys == VFVM_COORD_CYLINDRICAL2D)))
    return nullptr;
  // index validation: every table entry must address an existing node/region
  for (int64_t i = 0; i < (int64_t)nvc * nc; ++i) if (g->cellnodes[i] < 0 || g->cellnodes[i] >= N) return nullptr;
  for (int64_t i = 0; i < (int64_t)dim * nbf; ++i) if (g->bfacenodes[i] < 0 || g->bfacenodes[i] >= N) return nullptr;
  for (int i = 0; i < nc; ++i) if (g->cellregions[i] < 1) return nullptr;
  for (int i = 0; i < nbf; ++i) if (g->bfaceregions[i] < 1) return nullptr;

  vfvm_ctx* c = new vfvm_ctx;
  c->dim = dim; c->N = N; c->ncells = nc; c->nbf = nbf; c->ns = ns; c->phys = ph->physics_id;
  SETUP_CUDA(cudaGetDevice(&c->device));
  SETUP_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));

  c->h_coord.resize((size_t)N * dim);
  for (int k = 0; k < N; ++k)
    for (int d = 0; d < dim; ++d) c->h_coord[(size_t)k * dim + d] = g->coord[d + (size_t)dim * k];

  // --- edges: (lo, hi) node pairs, numbered lexicographically
  const int nle = dim == 1 ? 1 : (dim == 2 ? 3 : 6);
  auto ledge = [&](int e, int k) { return dim == 1 ? k : (dim == 2 ? kTriEdges[e][k] : kTetEdges[e][k]); };
  std::vector<int64_t> keys((size_t)nc * nle);
  for (int cell = 0; cell < nc; ++cell)
    for (int e = 0; e < nle; ++e) {
      int a = g->cellnodes[ledge(e, 0) + (size_t)nvc * cell], b = g->cellnodes[ledge(e, 1) + (size_t)nvc * cell];
      if (a > b) std::swap(a, b);
      keys[(size_t)cell * nle + e] = (int64_t)a * N + b;
    }
  std::vector<int64_t> ukeys(keys);
  std::sort(ukeys.begin(), ukeys.end());
  ukeys.erase(std::unique(ukeys.begin(), ukeys.end()), ukeys.end());
  const int E = (int)ukeys.size();
  c->E = E;
  c->h_edgenodes.resize(2 * (size_t)E);
  for (int e = 0; e < E; ++e) { c->h_edgenodes[2 * e] = (int)(ukeys[e] / N); c->h_edgenodes[2 * e + 1] = (int)(ukeys[e] % N); }

  // --- edgewise form factors per (node, region) and (edge, region)
  int maxreg = 1;
  for (int i = 0; i < nc; ++i) maxreg = std::max(maxreg, g->cellregions[i]);
  c->nregions = maxreg;
  c->single_region = g->cellregions[0];
  c->multireg = false;
  for (int i = 1; i < nc; ++i) if (g->cellregions[i] != c->single_region) { c->multireg = true; break; }

  // --- species restricted to regions (enable_species! / enable_boundary_species!,
  // src/vfvm_system.jl:433-513): the species mask of every cell region and, from
  // the cells and boundary faces containing it, of every node (node_dof)
  if (ph->ncellregions_species > 0 || ph->nbregions_species > 0) {
    if (ns > 32 || ph->ncellregions_species < 0 || ph->nbregions_species < 0 ||
        (ph->ncellregions_species > 0 && !ph->region_species) ||
        (ph->nbregions_species > 0 && !ph->bregion_species)) {
      *status = VFVM_ERR_INPUT;
      delete c;
      return nullptr;
    }
    const unsigned all = ns == 32 ? ~0u : (1u << ns) - 1u;
    auto mask_of = [&](const int32_t* tab, int ncols, int reg) {
      unsigned m = 0;
      if (reg >= 1 && reg <= ncols)
        for (int i = 0; i < ns; ++i)
          if (tab[i + (size_t)ns * (reg - 1)]) m |= 1u << i;
      return m;
    };
    c->h_reg_spec.assign(maxreg, 0u);
    for (int r = 1; r <= maxreg; ++r) c->h_reg_spec[r - 1] = mask_of(ph->region_species, ph->ncellregions_species, r);
    unsigned bulk = 0, bnd = 0;  // a species is a bulk or a boundary species, not both
    for (int r = 1; r <= ph->ncellregions_species; ++r) bulk |= mask_of(ph->region_species, ph->ncellregions_species, r);
    for (int r = 1; r <= ph->nbregions_species; ++r) bnd |= mask_of(ph->bregion_species, ph->nbregions_species, r);
    c->h_node_spec.assign(N, 0u);
    for (int cell = 0; cell < nc; ++cell) {
      const unsigned m = c->h_reg_spec[g->cellregions[cell] - 1];
      for (int v = 0; v < nvc; ++v) c->h_node_spec[g->cellnodes[v + (size_t)nvc * cell]] |= m;
    }
    for (int b = 0; b < nbf; ++b) {
      const unsigned m = mask_of(ph->bregion_species, ph->nbregions_species, g->bfaceregions[b]);
      for (int v = 0; v < dim; ++v) c->h_node_spec[g->bfacenodes[v + (size_t)dim * b]] |= m;
    }
    bool any = false, masked = false;
    for (int k = 0; k < N; ++k) { any = any || c->h_node_spec[k] != 0; masked = masked || c->h_node_spec[k] != all; }
    for (int cell = 0; cell < nc; ++cell) masked = masked || c->h_reg_spec[g->cellregions[cell] - 1] != all;
    if ((bulk & bnd) != 0 || !any) {  // the reference's DomainError / "No species enabled"
      *status = VFVM_ERR_INPUT;
      delete c;
      return nullptr;
    }
    if (masked) {
      c->species_masked = true;
      c->multireg = true;  // the node-centric kernel with per-item regions applies the masks
    } else {
      c->h_reg_spec.clear();
      c->h_node_spec.clear();
    }
  }
  std::vector<std::vector<RegFac>> nfac(N), efac(E);
  {
    const double* xs[4];
    double nf[4], ef[6];
    for (int cell = 0; cell < nc; ++cell) {
      for (int v = 0; v < nvc; ++v) xs[v] = &c->h_coord[(size_t)g->cellnodes[v + (size_t)nvc * cell] * dim];
      simplex_factors(dim, csys, xs, nf, ef);
      const int reg = g->cellregions[cell];
      for (int v = 0; v < nvc; ++v) add_regfac(nfac[g->cellnodes[v + (size_t)nvc * cell]], reg, nf[v]);
      for (int e = 0; e < nle; ++e) {
        int eid = (int)(std::lower_bound(ukeys.begin(), ukeys.end(), keys[(size_t)cell * nle + e]) - ukeys.begin());
        add_regfac(efac[eid], reg, ef[e]);
      }
    }
  }
  c->h_nodevol.assign(N, 0.0);
  c->h_edgefac.assign(E, 0.0);
  for (int k = 0; k < N; ++k) for (auto& r : nfac[k]) c->h_nodevol[k] += r.fac;
  for (int e = 0; e < E; ++e) for (auto& r : efac[e]) c->h_edgefac[e] += r.fac;

  // --- block pattern: row K = {K} u neighbours(K), sorted
  std::vector<int> deg(N, 1);
  for (int e = 0; e < E; ++e) { deg[c->h_edgenodes[2 * e]]++; deg[c->h_edgenodes[2 * e + 1]]++; }
  c->h_browptr.assign(N + 1, 0);
  for (int k = 0; k < N; ++k) c->h_browptr[k + 1] = c->h_browptr[k] + deg[k];
  c->nnzb = c->h_browptr[N];
  if (c->nnzb >= (int64_t)std::numeric_limits<int>::max() / (ns * ns)) { *status = VFVM_ERR_INPUT; delete c; return nullptr; }
  c->h_bcol.assign(c->nnzb, 0);
  std::vector<int> slot_edge(c->nnzb, -1);
  {
    std::vector<int> fill(c->h_browptr.begin(), c->h_browptr.end() - 1);
    for (int k = 0; k < N; ++k) c->h_bcol[fill[k]++] = k;
    for (int e = 0; e < E; ++e) {
      int a = c->h_edgenodes[2 * e], b = c->h_edgenodes[2 * e + 1];
      slot_edge[fill[a]] = e; c->h_bcol[fill[a]++] = b;
      slot_edge[fill[b]] = e; c->h_bcol[fill[b]++] = a;
    }
    std::vector<std::pair<int, int>> tmp;
    for (int k = 0; k < N; ++k) {
      tmp.clear();
      for (int s = c->h_browptr[k]; s < c->h_browptr[k + 1]; ++s) tmp.push_back({c->h_bcol[s], slot_edge[s]});
      std::sort(tmp.begin(), tmp.end());
      for (size_t i = 0; i < tmp.size(); ++i) { c->h_bcol[c->h_browptr[k] + i] = tmp[i].first; slot_edge[c->h_browptr[k] + i] = tmp[i].second; }
    }
  }
  c->h_diag.assign(N, 0);
  for (int k = 0; k < N; ++k)
    for (int s = c->h_browptr[k]; s < c->h_browptr[k + 1]; ++s)
      if (c->h_bcol[s] == k) c->h_diag[k] = s;

  std::vector<double> node_fac(N, 0.0), slot_fac(c->nnzb, 0.0);
  std::vector<int> nitem_ptr, nitem_reg, sitem_ptr, sitem_reg;
  std::vector<double> nitem_fac, sitem_fac;
  if (!c->multireg) {
    for (int k = 0; k < N; ++k) node_fac[k] = nfac[k].empty() ? 0.0 : nfac[k][0].fac;
    for (int64_t s = 0; s < c->nnzb; ++s) slot_fac[s] = slot_edge[s] >= 0 ? c->h_edgefac[slot_edge[s]] : 0.0;
  } else {
    nitem_ptr.push_back(0);
    for (int k = 0; k < N; ++k) {
      for (auto& r : nfac[k]) { nitem_reg.push_back(r.reg); nitem_fac.push_back(r.fac); }
      nitem_ptr.push_back((int)nitem_reg.size());
    }
    sitem_ptr.push_back(0);
    for (int64_t s = 0; s < c->nnzb; ++s) {
      if (slot_edge[s] >= 0)
        for (auto& r : efac[slot_edge[s]]) { sitem_reg.push_back(r.reg); sitem_fac.push_back(r.fac); }
      sitem_ptr.push_back((int)sitem_reg.size());
    }
  }

  // --- boundary-node items grouped by node, bface order inside a node
  const int nbn = dim;  // nodes per boundary face
  std::vector<int> bn_ptr(N + 1, 0), bn_reg((size_t)nbf * nbn);
  std::vector<double> bn_fac((size_t)nbf * nbn);
  {
    std::vector<int> cnt(N, 0);
    for (int64_t i = 0; i < (int64_t)nbf * nbn; ++i) cnt[g->bfacenodes[i]]++;
    for (int k = 0; k < N; ++k) bn_ptr[k + 1] = bn_ptr[k] + cnt[k];
    std::vector<int> fill(bn_ptr.begin(), bn_ptr.end() - 1);
    const double* xs[3];
    double bf[3];
    int maxbreg = 0;
    for (int b = 0; b < nbf; ++b) {
      for (int v = 0; v < nbn; ++v) xs[v] = &c->h_coord[(size_t)g->bfacenodes[v + (size_t)nbn * b] * dim];
      bface_factors(dim, csys, xs, bf);
      maxbreg = std::max(maxbreg, g->bfaceregions[b]);
      for (int v = 0; v < nbn; ++v) {
        int k = g->bfacenodes[v + (size_t)nbn * b];
        bn_reg[fill[k]] = g->bfaceregions[b];
        bn_fac[fill[k]] = bf[v];
        fill[k]++;
      }
    }
    c->nbregions = std::max(maxbreg, ph->nbregions);
  }

  // --- boundary-edge items (physics with bflux): the edges of the boundary
  // faces with their face edge factors, summed per (edge, boundary region) and
  // listed under both Jacobian slots of the edge (assemble_bedges,
  // src/vfvm_assembly.jl:444-510; factors src/vfvm_formfactors.jl:263-332)
  const bool has_bflux = dispatch_physics(c->phys, [](auto phy) { return decltype(phy)::has_bflux ? 1 : 0; }) == 1;
  std::vector<int> sbe_ptr, sbe_reg;
  std::vector<double> sbe_fac;
  std::map<int, std::vector<uint8_t>> bem_of_reg;  // structural bflux mask per boundary region
  if (has_bflux && dim >= 2 && nbf > 0) {
    std::map<int64_t, std::vector<RegFac>> be;  // key: lo * N + hi
    const double* xs[3];
    double ef[3];
    const int nle_b = dim == 2 ? 1 : 3;
    for (int b = 0; b < nbf; ++b) {
      for (int v = 0; v < nbn; ++v) xs[v] = &c->h_coord[(size_t)g->bfacenodes[v + (size_t)nbn * b] * dim];
      bface_edge_factors(dim, csys, xs, ef);
      for (int e = 0; e < nle_b; ++e) {
        int a = g->bfacenodes[(dim == 2 ? 0 : kTriEdges[e][0]) + (size_t)nbn * b];
        int bb = g->bfacenodes[(dim == 2 ? 1 : kTriEdges[e][1]) + (size_t)nbn * b];
        if (a > bb) std::swap(a, bb);
        add_regfac(be[(int64_t)a * N + bb], g->bfaceregions[b], ef[e]);
      }
    }
    sbe_ptr.assign(c->nnzb + 1, 0);
    int64_t found = 0;
    for (int k = 0; k < N; ++k)
      for (int s = c->h_browptr[k]; s < c->h_browptr[k + 1]; ++s) {
        const int m = c->h_bcol[s];
        if (m != k) {
          auto it = be.find((int64_t)std::min(k, m) * N + std::max(k, m));
          if (it != be.end()) {
            ++found;
            for (auto& r : it->second) { sbe_reg.push_back(r.reg); sbe_fac.push_back(r.fac); }
          }
        }
        sbe_ptr[s + 1] = (int)sbe_reg.size();
      }
    if (found != 2 * (int64_t)be.size()) {  // every boundary-face edge is an edge of the cells
      fprintf(stderr, "vfvm_create: boundary-face edges that are not cell edges\n");
      *status = VFVM_ERR_INPUT;
      delete c;
      return nullptr;
    }
    std::vector<double> p(ph->params, ph->params + ph->nparams);
    p.resize(16, 0.0);
    for (int b = 0; b < nbf; ++b) {
      const int reg = g->bfaceregions[b];
      if (!bem_of_reg.count(reg))
        dispatch_physics(c->phys, [&](auto phy) { probe_bflux_t(phy, p.data(), reg, bem_of_reg[reg]); return 0; });
    }
  }

  // --- outflow nodes: the nodes of the boundary faces in the physics'
  // outflowboundaries (update_grid!, src/vfvm_system.jl:660-673)
  std::vector<uint8_t> outflow_h;
  if (dispatch_physics(c->phys, [](auto phy) { return decltype(phy)::has_boutflow ? 1 : 0; }) == 1) {
    std::vector<double> p(ph->params, ph->params + ph->nparams);
    p.resize(16, 0.0);
    outflow_h.assign(N, 0);
    for (int b = 0; b < nbf; ++b) {
      const int reg = g->bfaceregions[b];
      const bool out = dispatch_physics(c->phys, [&](auto phy) {
        return decltype(phy)::outflow_region(p.data(), reg) ? 1 : 0; }) == 1;
      if (out)
        for (int v = 0; v < nbn; ++v) outflow_h[g->bfacenodes[v + (size_t)nbn * b]] = 1;
    }
  }

  // --- legacy boundary data (boundary_dirichlet!(sys, ispec, ireg, val) etc.)
  std::vector<double> bfac_h((size_t)ns * c->nbregions, 0.0), bval_h((size_t)ns * c->nbregions, 0.0);
  if (ph->nbregions > 0 && ph->bfactors && ph->bvalues) {
    for (int r = 0; r < ph->nbregions; ++r)
      for (int i = 0; i < ns; ++i) {
        bfac_h[i + (size_t)ns * r] = ph->bfactors[i + (size_t)ns * r];
        bval_h[i + (size_t)ns * r] = ph->bvalues[i + (size_t)ns * r];
      }
    for (size_t i = 0; i < bfac_h.size(); ++i) if (bfac_h[i] != 0.0 || bval_h[i] != 0.0) c->has_legacy = true;
  }

  // --- structural masks -> scalar pattern (the entries the reference creates)
  c->h_params.assign(ph->params, ph->params + ph->nparams);
  c->nparams = ph->nparams;
  std::vector<uint8_t> nm, em, bm;  // bm: boundary terms over all regions (the pattern uses the per-region masks)
  std::vector<int> cregs;
  for (int i = 0; i < nc; ++i) cregs.push_back(g->cellregions[i]);
  std::sort(cregs.begin(), cregs.end());
  cregs.erase(std::unique(cregs.begin(), cregs.end()), cregs.end());
  std::vector<int> bregs(bn_reg);
  std::sort(bregs.begin(), bregs.end());
  bregs.erase(std::unique(bregs.begin(), bregs.end()), bregs.end());
  {
    std::vector<double> p(c->h_params);
    p.resize(16, 0.0);
    dispatch_physics(c->phys, [&](auto phy) { probe_t(phy, p.data(), dim, cregs, bregs, nm, em, bm); return 0; });
  }
  std::map<int, std::vector<uint8_t>> bnm_of_reg;  // boundary-node terms, per boundary region
  {
    std::vector<double> p(c->h_params);
    p.resize(16, 0.0);
    for (int reg : bregs)
      dispatch_physics(c->phys, [&](auto phy) { probe_bnode_t(phy, p.data(), reg, bnm_of_reg[reg]); return 0; });
  }
  std::vector<uint8_t> dir_dof((size_t)N * ns, 0);
  {
    std::vector<double> p(c->h_params);
    p.resize(16, 0.0);
    std::vector<uint8_t> regdir((size_t)(c->nbregions + 1) * ns, 0);
    for (int reg : bregs)
      dispatch_physics(c->phys, [&](auto phy) { dirichlet_species_t(phy, p.data(), reg, ns, &regdir[(size_t)reg * ns]); return 0; });
    for (int k = 0; k < N; ++k)
      for (int it = bn_ptr[k]; it < bn_ptr[k + 1]; ++it) {
        int reg = bn_reg[it];
        for (int i = 0; i < ns; ++i) {
          bool d = regdir[(size_t)reg * ns + i] != 0;
          if (c->has_legacy && reg - 1 < c->nbregions && bfac_h[i + (size_t)ns * (reg - 1)] == kDirichlet) d = true;
          if (d) dir_dof[(size_t)k * ns + i] = 1;
        }
      }
  }
  {
    const int n = N * ns;
    c->h_rowptr.assign(n + 1, 0);
    c->h_colind.clear();
    std::vector<int64_t> pmap;
    for (int k = 0; k < N; ++k) {
      bool bnode = bn_ptr[k + 1] > bn_ptr[k];
      // species whose legacy boundary factor is nonzero in a region of this node
      std::vector<uint8_t> legdiag(ns, 0);
      if (c->has_legacy)
        for (int it = bn_ptr[k]; it < bn_ptr[k + 1]; ++it)
          for (int i = 0; i < ns; ++i)
            if (bn_reg[it] - 1 < c->nbregions && bfac_h[i + (size_t)ns * (bn_reg[it] - 1)] != 0.0) legdiag[i] = 1;
      // species restricted to regions: entry (i, j) of a term exists only when
      // both species belong to the term's region (cell terms) or node (boundary
      // terms; a boundary edge: its first node), src/vfvm_assemblydata.jl:245-470
      const bool msk = c->species_masked;
      auto pair_in = [](unsigned m, int i, int j) { return ((m >> i) & 1u) && ((m >> j) & 1u); };
      auto node_items_allow = [&](int i, int j) {
        if (!msk) return true;
        for (int it = nitem_ptr[k]; it < nitem_ptr[k + 1]; ++it)
          if (pair_in(c->h_reg_spec[nitem_reg[it] - 1], i, j)) return true;
        return false;
      };
      auto slot_items_allow = [&](int s, int i, int j) {
        if (!msk) return true;
        for (int it = sitem_ptr[s]; it < sitem_ptr[s + 1]; ++it)
          if (pair_in(c->h_reg_spec[sitem_reg[it] - 1], i, j)) return true;
        return false;
      };
      auto edges_allow = [&](int i, int j) {  // some incident edge carries (i, j)
        if (!msk) return true;
        for (int s2 = c->h_browptr[k]; s2 < c->h_browptr[k + 1]; ++s2)
          if (c->h_bcol[s2] != k && slot_items_allow(s2, i, j)) return true;
        return false;
      };
      const unsigned kspec = msk ? c->h_node_spec[k] : ~0u;
      // boundary-edge (bflux) partials of this row: per slot, and summed into the diagonal
      auto bflux_on = [&](int s, bool first_col, int i, int j) {
        if (sbe_ptr.empty()) return false;
        if (msk && !pair_in(c->h_node_spec[std::min(k, c->h_bcol[s])], i, j)) return false;
        for (int it = sbe_ptr[s]; it < sbe_ptr[s + 1]; ++it) {
          const auto& mk = bem_of_reg[sbe_reg[it]];
          if (mk[i * 2 * ns + (first_col ? 0 : ns) + j]) return true;
        }
        return false;
      };
      for (int i = 0; i < ns; ++i) {
        for (int s = c->h_browptr[k]; s < c->h_browptr[k + 1]; ++s) {
          int m = c->h_bcol[s];
          for (int j = 0; j < ns; ++j) {
            bool on;
            if (m == k) {
              on = (nm[i * ns + j] && node_items_allow(i, j)) ||
                   ((em[i * 2 * ns + j] || em[i * 2 * ns + ns + j]) && edges_allow(i, j));
              if (bnode) {
                bool bterm = false;  // a boundary-node term of one of this node's boundary regions
                for (int it = bn_ptr[k]; !bterm && it < bn_ptr[k + 1]; ++it) bterm = bnm_of_reg[bn_reg[it]][i * ns + j] != 0;
                on = on || (bterm && pair_in(kspec, i, j));
                if (i == j && legdiag[i]) on = true;
              }
              // a species the node does not carry: F += U - Uold, unit diagonal
              if (i == j && msk && !((kspec >> i) & 1u)) on = true;
              for (int s2 = c->h_browptr[k]; !on && s2 < c->h_browptr[k + 1]; ++s2) {
                const int m2 = c->h_bcol[s2];
                if (m2 != k) on = bflux_on(s2, k < m2, i, j);  // d f / d u_K of K's boundary edges
              }
            } else if (k < m) {  // k first: d f / d u_second
              on = (em[i * 2 * ns + ns + j] && slot_items_allow(s, i, j)) || bflux_on(s, false, i, j);
            } else {             // k second: d f / d u_first
              on = (em[i * 2 * ns + j] && slot_items_allow(s, i, j)) || bflux_on(s, true, i, j);
            }
            if (on) {
              c->h_colind.push_back(m * ns + j);
              pmap.push_back((int64_t)s * ns * ns + i * ns + j);
            }
          }
        }
        c->h_rowptr[(size_t)k * ns + i + 1] = (int64_t)c->h_colind.size();
      }
    }
    c->nnz = (int64_t)c->h_colind.size();
    SETUP_CUDA(c->pmap.upload(pmap));
  }

  // --- greedy multicolouring of the node graph (ILU0 ordering)
  {
    std::vector<int> color(N, -1), mark;
    int ncol = 0;
    for (int k = 0; k < N; ++k) {
      mark.assign(ncol + 1, 0);
      for (int s = c->h_browptr[k]; s < c->h_browptr[k + 1]; ++s) {
        int m = c->h_bcol[s];
        if (m != k && color[m] >= 0) mark[color[m]] = 1;
      }
      int col = 0;
      while (col < ncol && mark[col]) ++col;
      color[k] = col;
      ncol = std::max(ncol, col + 1);
    }
    c->ncolors = ncol;
    c->h_color_ptr.assign(ncol + 1, 0);
    for (int k = 0; k < N; ++k) c->h_color_ptr[color[k] + 1]++;
    for (int q = 0; q < ncol; ++q) c->h_color_ptr[q + 1] += c->h_color_ptr[q];
    std::vector<int> cn(N), fill(c->h_color_ptr.begin(), c->h_color_ptr.end() - 1);
    for (int k = 0; k < N; ++k) cn[fill[color[k]]++] = k;
    SETUP_CUDA(c->color_nodes.upload(cn));
    SETUP_CUDA(c->color_ptr.upload(c->h_color_ptr));
    // lower slots per node in factorization order (colour, then node index)
    std::vector<int> lptr(N + 1, 0), lslots;
    std::vector<std::pair<int64_t, int>> tmp;
    for (int k = 0; k < N; ++k) {
      tmp.clear();
      for (int s = c->h_browptr[k]; s < c->h_browptr[k + 1]; ++s) {
        int m = c->h_bcol[s];
        if (m != k && color[m] < color[k]) tmp.push_back({(int64_t)color[m] * N + m, s});
      }
      std::sort(tmp.begin(), tmp.end());
      for (auto& t : tmp) lslots.push_back(t.second);
      lptr[k + 1] = (int)lslots.size();
    }
    SETUP_CUDA(c->lower_ptr.upload(lptr));
    SETUP_CUDA(c->lower_slots.upload(lslots));
    // ELL copies for the Krylov solve (fixed width, entry w of row r at w*N + r,
    // padding -1): the matrix by node, and the ILU0 lower/upper couplings by
    // position in colour order.  One thread per row then issues all of a row's
    // loads at once instead of walking pointer chains.
    int W = 0, LW = 0, UW = 0;
    for (int k = 0; k < N; ++k) {
      W = std::max(W, c->h_browptr[k + 1] - c->h_browptr[k]);
      LW = std::max(LW, lptr[k + 1] - lptr[k]);
    }
    std::vector<int> upcount(N, 0);
    for (int k = 0; k < N; ++k)
      for (int s = c->h_browptr[k]; s < c->h_browptr[k + 1]; ++s)
        if (color[c->h_bcol[s]] > color[k]) ++upcount[k];
    for (int k = 0; k < N; ++k) UW = std::max(UW, upcount[k]);
    c->ell_w = W; c->lo_w = LW; c->up_w = UW;
    std::vector<int> ecol((size_t)W * N, -1), eslot((size_t)W * N, -1);
    for (int k = 0; k < N; ++k)
      for (int s = c->h_browptr[k], w = 0; s < c->h_browptr[k + 1]; ++s, ++w) {
        ecol[(size_t)w * N + k] = c->h_bcol[s];
        eslot[(size_t)w * N + k] = s;
      }
    std::vector<int> lnode((size_t)std::max(LW, 1) * N, -1), lslot((size_t)std::max(LW, 1) * N, -1);
    std::vector<int> unode((size_t)std::max(UW, 1) * N, -1), uslot((size_t)std::max(UW, 1) * N, -1);
    for (int pos = 0; pos < N; ++pos) {
      const int k = cn[pos];
      for (int q = lptr[k], w = 0; q < lptr[k + 1]; ++q, ++w) {
        lslot[(size_t)w * N + pos] = lslots[q];
        lnode[(size_t)w * N + pos] = c->h_bcol[lslots[q]];
      }
      int w = 0;
      for (int s = c->h_browptr[k]; s < c->h_browptr[k + 1]; ++s)
        if (color[c->h_bcol[s]] > color[k]) {
          uslot[(size_t)w * N + pos] = s;
          unode[(size_t)w * N + pos] = c->h_bcol[s];
          ++w;
        }
    }
    SETUP_CUDA(c->ell_col.upload(ecol));
    SETUP_CUDA(c->ell_slot.upload(eslot));
    SETUP_CUDA(c->lo_node.upload(lnode));
    SETUP_CUDA(c->lo_slot.upload(lslot));
    SETUP_CUDA(c->up_node.upload(unode));
    SETUP_CUDA(c->up_slot.upload(uslot));
  }

  // --- upload
  std::vector<double> nd;
  c->nnd = ph->nnodedata;
  if (c->nnd > 0) nd.assign(ph->nodedata, ph->nodedata + (size_t)N * c->nnd);
  std::vector<double> pp(c->h_params);
  if (pp.empty()) pp.push_back(0.0);
  SETUP_CUDA(c->coord.upload(c->h_coord));
  SETUP_CUDA(c->browptr.upload(c->h_browptr));
  SETUP_CUDA(c->bcol.upload(c->h_bcol));
  SETUP_CUDA(c->diag.upload(c->h_diag));
  SETUP_CUDA(c->node_fac.upload(node_fac));
  SETUP_CUDA(c->slot_fac.upload(slot_fac));
  {
    std::vector<float> sf(slot_fac.begin(), slot_fac.end());
    SETUP_CUDA(c->slot_facf.upload(sf));
  }
  if (c->multireg) {
    SETUP_CUDA(c->nitem_ptr.upload(nitem_ptr));
    SETUP_CUDA(c->nitem_reg.upload(nitem_reg));
    SETUP_CUDA(c->nitem_fac.upload(nitem_fac));
    SETUP_CUDA(c->sitem_ptr.upload(sitem_ptr));
    SETUP_CUDA(c->sitem_reg.upload(sitem_reg));
    SETUP_CUDA(c->sitem_fac.upload(sitem_fac));
  }
  SETUP_CUDA(c->bn_ptr.upload(bn_ptr));
  SETUP_CUDA(c->bn_reg.upload(bn_reg));
  SETUP_CUDA(c->bn_fac.upload(bn_fac));
  SETUP_CUDA(c->params.upload(pp));
  SETUP_CUDA(c->nodedata.upload(nd));
  SETUP_CUDA(c->bfactors.upload(bfac_h));
  SETUP_CUDA(c->bvalues.upload(bval_h));
  if (c->species_masked) {
    SETUP_CUDA(c->reg_spec.upload(c->h_reg_spec));
    SETUP_CUDA(c->node_spec.upload(c->h_node_spec));
  }
  if (!outflow_h.empty()) SETUP_CUDA(c->outflow_node.upload(outflow_h));
  SETUP_CUDA(c->dirichlet_dof.upload(dir_dof));
  if (!sbe_ptr.empty()) {
    SETUP_CUDA(c->sbe_ptr.upload(sbe_ptr));
    SETUP_CUDA(c->sbe_reg.upload(sbe_reg));
    SETUP_CUDA(c->sbe_fac.upload(sbe_fac));
  }
  const size_t n = (size_t)N * ns;
  SETUP_CUDA(c->U.alloc(n));
  SETUP_CUDA(c->Uold.alloc(n));
  SETUP_CUDA(c->F.alloc(n));
  SETUP_CUDA(c->J.alloc((size_t)c->nnzb * ns * ns));
  SETUP_CUDA(c->errflag.alloc(4));
  SETUP_CUDA(cudaMemset(c->errflag.p, 0, 4 * sizeof(int)));
  {
    int rc = build_assembly_tiles(c, slot_fac);
    if (rc == VFVM_OK) rc = prepare_tiled_assembly(c);
    if (rc != VFVM_OK) { *status = rc; delete c; return nullptr; }
  }
  *status = VFVM_OK;
  return c;
}

extern "C" void vfvm_destroy(vfvm_ctx* c) {
  if (!c) return;
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->ws) destroy_workspace(c->ws);
  for (auto& kv : c->coarse_spaces) delete kv.second;
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

extern "C" int vfvm_info(vfvm_ctx* c, int64_t out[8]) {
  if (!c || !out) return VFVM_ERR_INPUT;
  out[0] = c->ns; out[1] = c->N; out[2] = c->E; out[3] = c->nnz; out[4] = c->nnzb; out[5] = c->ncolors;
  out[6] = c->dim; out[7] = c->multireg ? 1 : 0;
  return VFVM_OK;
}

extern "C" int vfvm_pattern(vfvm_ctx* c, int64_t* rowptr, int32_t* colind) {
  if (!c) return VFVM_ERR_INPUT;
  if (rowptr) std::copy(c->h_rowptr.begin(), c->h_rowptr.end(), rowptr);
  if (colind) std::copy(c->h_colind.begin(), c->h_colind.end(), colind);
  return VFVM_OK;
}

extern "C" int vfvm_geometry(vfvm_ctx* c, double* nodevol, double* edgefac, int32_t* edgenodes) {
  if (!c) return VFVM_ERR_INPUT;
  if (nodevol) std::copy(c->h_nodevol.begin(), c->h_nodevol.end(), nodevol);
  if (edgefac) std::copy(c->h_edgefac.begin(), c->h_edgefac.end(), edgefac);
  if (edgenodes) std::copy(c->h_edgenodes.begin(), c->h_edgenodes.end(), edgenodes);
  return VFVM_OK;
}

extern "C" int vfvm_set_params(vfvm_ctx* c, const double* params, int32_t nparams) {
  if (!c || nparams < physics_nparams(c->phys) || (nparams > 0 && !params)) return VFVM_ERR_INPUT;
  c->h_params.assign(params, params + nparams);
  std::vector<double> pp(c->h_params);
  if (pp.empty()) pp.push_back(0.0);
  if (pp.size() > c->params.n) VFVM_CUDA(c->params.alloc(pp.size()));
  VFVM_CUDA(cudaMemcpyAsync(c->params.p, pp.data(), pp.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  VFVM_CUDA(cudaStreamSynchronize(c->stream));
  c->nparams = nparams;
  return VFVM_OK;
}

extern "C" void* vfvm_stream(vfvm_ctx* c) { return c ? (void*)c->stream : nullptr; }
