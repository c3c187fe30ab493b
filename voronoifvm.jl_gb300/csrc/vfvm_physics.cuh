// Device physics functors.
//
// The reference passes Julia closures flux!/reaction!/storage!/source!/
// breaction! (src/vfvm_physics.jl:67-182) and differentiates them with
// ForwardDiff.  Closures cannot cross a C ABI, so each physics used by this
// library is a registered functor, selected by VFVM_PHYS_* id plus a parameter
// block.  Every callback is a template over the number type so the same code
// runs on plain doubles (residual-only evaluation, Dirichlet initialisation)
// and on Dual<N,P> (residual + Jacobian).
//
// Conventions: f, u are arrays of NS species; flux gets the first-node values
// uK and the second-node values uL of an edge (the reference's u[ispec,1] and
// u[ispec,2]).
#pragma once
#include "vfvm_common.cuh"

namespace vfvm {

struct PhysBase {
  static constexpr bool has_reaction = false, has_storage = false, has_source = false, has_breaction = false;
  // boundary callbacks beyond breaction: bflux (boundary edges), bstorage, bsource
  // (src/vfvm_physics.jl:82-180)
  static constexpr bool has_bflux = false, has_bstorage = false, has_bsource = false;
  // edgereaction (src/vfvm_physics.jl:67-182): an edge term added to both end nodes
  static constexpr bool has_edgereaction = false;
  // boutflow (src/vfvm_physics.jl:148-160): an edge term on the edges with a node
  // on an outflow boundary region, added to that node's residual
  static constexpr bool has_boutflow = false;
  template <class T> VFVM_HD void boutflow(T*, const T*, const T*, const EdgeItem&) const {}
  static bool outflow_region(const double*, int) { return false; }  // outflowboundaries
  template <class T> VFVM_HD void reaction(T*, const T*, const NodeItem&) const {}
  template <class T> VFVM_HD void edgereaction(T*, const T*, const T*, const EdgeItem&) const {}
  template <class T> VFVM_HD void storage(T*, const T*, const NodeItem&) const {}
  VFVM_HD void source(double*, const NodeItem&) const {}
  template <class T> VFVM_HD void breaction(T*, const T*, const BNodeItem&) const {}
  template <class T> VFVM_HD void bflux(T*, const T*, const T*, const BEdgeItem&) const {}
  template <class T> VFVM_HD void bstorage(T*, const T*, const BNodeItem&) const {}
  VFVM_HD void bsource(double*, const BNodeItem&) const {}
  // whether the parameter block suits grids of this dimension (checked once by vfvm_create)
  static bool valid(int, const double*) { return true; }
  // parameters with derivatives (the reference's nparams / parameters(u)): the
  // first NPD entries of the parameter block; a physics with NPD > 0 is a
  // template over the parameter type PT with `rebind<PT>` and `seed(k)`
  static constexpr int NPD = 0;
};

// examples/Example105_NonlinearPoisson1D.jl:41-60;  params: eps
struct PhysEx105 : PhysBase {
  static constexpr int NS = 1;
  static constexpr bool has_reaction = true, has_source = true;
  double eps;
  VFVM_HD void load(const double* p) { eps = p[0]; }
  template <class T> VFVM_HD void flux(T* f, const T* uK, const T* uL, const EdgeItem&) const { f[0] = (uK[0] - uL[0]) * eps; }
  template <class T> VFVM_HD void reaction(T* f, const T* u, const NodeItem&) const { f[0] = exp(u[0]) - exp(-u[0]); }
  VFVM_HD void source(double* f, const NodeItem& n) const { f[0] = (n.x[0] <= 0.5) ? 1.0 : -1.0; }
};

// examples/Example106_NonlinearDiffusion1D.jl:58-68;  params: m
struct PhysEx106 : PhysBase {
  static constexpr int NS = 1;
  static constexpr bool has_storage = true;
  double m;
  VFVM_HD void load(const double* p) { m = p[0]; }
  template <class T> VFVM_HD void flux(T* f, const T* uK, const T* uL, const EdgeItem&) const { f[0] = pow(uK[0], m) - pow(uL[0], m); }
  template <class T> VFVM_HD void storage(T* f, const T* u, const NodeItem&) const { f[0] = u[0]; }
};

// examples/Example110_ReactionDiffusion1D_TwoSpecies.jl:40-64;  params: eps1, eps2
struct PhysEx110 : PhysBase {
  static constexpr int NS = 2;
  static constexpr bool has_reaction = true, has_storage = true, has_source = true;
  double e1, e2;
  VFVM_HD void load(const double* p) { e1 = p[0]; e2 = p[1]; }
  template <class T> VFVM_HD void flux(T* f, const T* uK, const T* uL, const EdgeItem&) const {
    f[0] = (uK[0] - uL[0]) * e1 * (0.01 + uK[1] + uL[1]);
    f[1] = (uK[1] - uL[1]) * e2 * (0.01 + uK[0] + uL[0]);
  }
  template <class T> VFVM_HD void reaction(T* f, const T* u, const NodeItem&) const { T r = u[0] * u[1]; f[0] = r; f[1] = -r; }
  template <class T> VFVM_HD void storage(T* f, const T* u, const NodeItem&) const { f[0] = u[0]; f[1] = u[1]; }
  VFVM_HD void source(double* f, const NodeItem& n) const { f[0] = 1.0e-4 * (0.01 + n.x[0]); f[1] = 1.0e-4 * (0.01 + 1.0 - n.x[0]); }
};

// examples/Example160_UnipolarDriftDiffusion1D.jl:52-84 (sedan flux, species phi, c);  params: eps, z, V
struct PhysEx160 : PhysBase {
  static constexpr int NS = 2;
  static constexpr bool has_reaction = true, has_storage = true, has_breaction = true;
  double eps, z, V;
  VFVM_HD void load(const double* p) { eps = p[0]; z = p[1]; V = p[2]; }
  template <class T> VFVM_HD void flux(T* f, const T* uK, const T* uL, const EdgeItem&) const {
    f[0] = (uK[0] - uL[0]) * eps;
    const double eps_reg = 1.0e-10;
    T mu1 = -log1p(dmax(-uK[1], -1.0 + eps_reg));
    T mu2 = -log1p(dmax(-uL[1], -1.0 + eps_reg));
    T bp, bm;
    fbernoulli_pm((uK[0] - uL[0]) * (2.0 * z) + (mu1 - mu2), bp, bm);
    f[1] = bm * uK[1] - bp * uL[1];
  }
  template <class T> VFVM_HD void reaction(T* f, const T* u, const NodeItem&) const { f[0] = (1.0 - 2.0 * u[1]) * z; f[1] = u[1] * 0.0; }
  template <class T> VFVM_HD void storage(T* f, const T* u, const NodeItem&) const { f[0] = u[0] * 0.0; f[1] = u[1]; }
  template <class T> VFVM_HD void breaction(T* f, const T* u, const BNodeItem& b) const {
    const double Vt = ramp(b.time, 0.0, 1.0e-2, 0.0, V);
    boundary_dirichlet(f, u, b, 0, 1, Vt);
    boundary_dirichlet(f, u, b, 0, 2, 0.0);
    boundary_dirichlet(f, u, b, 1, 2, 0.5);
  }
};

// examples/Example207_NonlinearPoisson2D.jl:36-50;  params: eps
struct PhysEx207 : PhysBase {
  static constexpr int NS = 1;
  static constexpr bool has_reaction = true, has_storage = true, has_source = true;
  double eps;
  VFVM_HD void load(const double* p) { eps = p[0]; }
  template <class T> VFVM_HD void flux(T* f, const T* uK, const T* uL, const EdgeItem&) const { f[0] = (sq(uK[0]) - sq(uL[0])) * eps; }
  template <class T> VFVM_HD void reaction(T* f, const T* u, const NodeItem&) const { f[0] = sq(u[0]); }
  template <class T> VFVM_HD void storage(T* f, const T* u, const NodeItem&) const { f[0] = u[0]; }
  VFVM_HD void source(double* f, const NodeItem& n) const {
    const double x1 = n.x[0] - 0.5, x2 = n.x[1] - 0.5;
    f[0] = ::exp(-20.0 * (x1 * x1 + x2 * x2));
  }
};

// examples/Example301_Laplace3D.jl:15-24
struct PhysEx301 : PhysBase {
  static constexpr int NS = 1;
  static constexpr bool has_source = true;
  VFVM_HD void load(const double*) {}
  template <class T> VFVM_HD void flux(T* f, const T* uK, const T* uL, const EdgeItem&) const { f[0] = uK[0] - uL[0]; }
  VFVM_HD void source(double* f, const NodeItem& n) const { f[0] = n.x[0] * ::sin(5.0 * n.x[1]) * ::exp(n.x[2]); }
};

// examples/Example440_ParallelState.jl:16-25;  params: influx
struct PhysEx440 : PhysBase {
  static constexpr int NS = 1;
  static constexpr bool has_breaction = true;
  double influx;
  VFVM_HD void load(const double* p) { influx = p[0]; }
  template <class T> VFVM_HD void flux(T* f, const T* uK, const T* uL, const EdgeItem&) const { f[0] = sq(uK[0]) - sq(uL[0]); }
  template <class T> VFVM_HD void breaction(T* f, const T* u, const BNodeItem& b) const {
    boundary_dirichlet(f, u, b, 0, 1, 0.1);
    if (b.region == 2) f[0] = f[0] - influx;  // boundary_neumann!, src/vfvm_physics.jl:533
  }
};

// test/test030_cachesol.jl:10-18
struct PhysLaplaceDir : PhysBase {
  static constexpr int NS = 1;
  static constexpr bool has_breaction = true;
  VFVM_HD void load(const double*) {}
  template <class T> VFVM_HD void flux(T* f, const T* uK, const T* uL, const EdgeItem&) const { f[0] = uK[0] - uL[0]; }
  template <class T> VFVM_HD void breaction(T* f, const T* u, const BNodeItem& b) const {
    boundary_dirichlet(f, u, b, 0, 1, 0.0);
    boundary_dirichlet(f, u, b, 0, 2, 1.0);
  }
};

// Workload 1: -div(grad u) + u^3 = 1, u = 0 on every boundary region.
struct PhysNLPoisson : PhysBase {
  static constexpr int NS = 1;
  static constexpr bool has_reaction = true, has_breaction = true;
  VFVM_HD void load(const double*) {}
  template <class T> VFVM_HD void flux(T* f, const T* uK, const T* uL, const EdgeItem&) const { f[0] = uK[0] - uL[0]; }
  template <class T> VFVM_HD void reaction(T* f, const T* u, const NodeItem&) const { f[0] = cube(u[0]) - 1.0; }
  template <class T> VFVM_HD void breaction(T* f, const T* u, const BNodeItem& b) const { boundary_dirichlet(f, u, b, 0, b.region, 0.0); }
};

// Workload 2: porous medium u_t - div(grad u^2) = 0, homogeneous Neumann.
struct PhysPorous : PhysBase {
  static constexpr int NS = 1;
  static constexpr bool has_storage = true;
  VFVM_HD void load(const double*) {}
  template <class T> VFVM_HD void flux(T* f, const T* uK, const T* uL, const EdgeItem&) const { f[0] = sq(uK[0]) - sq(uL[0]); }
  template <class T> VFVM_HD void storage(T* f, const T* u, const NodeItem&) const { f[0] = u[0]; }
};

// Workload 3: bipolar drift-diffusion in density variables (psi, n, p), scaled
// units (thermal voltage 1, intrinsic density 1):
//   flux_psi = lambda2 (psi_K - psi_L)
//   flux_n   = mu_n (B(psi_K - psi_L) n_K - B(psi_L - psi_K) n_L)
//   flux_p   = mu_p (B(psi_L - psi_K) p_K - B(psi_K - psi_L) p_L)
//   reaction_psi = n - p - C(x),  reaction_n = reaction_p = R,
//   R = (n p - 1) / (tau_p (n + 1) + tau_n (p + 1))          (SRH)
//   C = +doping for x < 0.5, -doping otherwise;
//   ohmic contacts: region 4 (x = 0) at bias 0, region 2 (x = 1) at bias V*lambda.
// params: lambda2, mu_n, mu_p, tau_n, tau_p, doping, V
struct PhysBipolar : PhysBase {
  static constexpr int NS = 3;
  static constexpr bool has_reaction = true, has_breaction = true;
  double lambda2, mun, mup, taun, taup, doping, V;
  VFVM_HD void load(const double* p) { lambda2 = p[0]; mun = p[1]; mup = p[2]; taun = p[3]; taup = p[4]; doping = p[5]; V = p[6]; }
  VFVM_HD double C(const double* x) const { return x[0] < 0.5 ? doping : -doping; }
  template <class T> VFVM_HD void flux(T* f, const T* uK, const T* uL, const EdgeItem&) const {
    T dpsi = uK[0] - uL[0];
    f[0] = dpsi * lambda2;
    T bp, bm;
    fbernoulli_pm(dpsi, bp, bm);
    f[1] = (bp * uK[1] - bm * uL[1]) * mun;
    f[2] = (bm * uK[2] - bp * uL[2]) * mup;
  }
  template <class T> VFVM_HD void reaction(T* f, const T* u, const NodeItem& n) const {
    f[0] = u[1] - u[2] - C(n.x);
    T r = (u[1] * u[2] - 1.0) / ((u[1] + 1.0) * taup + (u[2] + 1.0) * taun);
    f[1] = r; f[2] = r;
  }
  template <class T> VFVM_HD void breaction(T* f, const T* u, const BNodeItem& b) const {
    if (b.region != 2 && b.region != 4) return;
    const double c = C(b.x);
    const double nn = 0.5 * c + ::sqrt(0.25 * c * c + 1.0);
    const double pp = 1.0 / nn;
    const double bias = (b.region == 2) ? V * b.lambda : 0.0;
    const double psi = ::asinh(0.5 * c) + bias;
    boundary_dirichlet(f, u, b, 0, b.region, psi);
    boundary_dirichlet(f, u, b, 1, b.region, nn);
    boundary_dirichlet(f, u, b, 2, b.region, pp);
  }
};

// Workload 4: two-species reaction-diffusion,
//   flux_i = D_i (u_i,K - u_i,L);  f1 = k (u1 - u2^2), f2 = -k (u1 - u2^2);
//   Dirichlet: region 4 (x = 0): u1 = 1, u2 = 0;  region 2 (x = 1): u1 = 0, u2 = 1.
// params: D1, D2, k
struct PhysRD2 : PhysBase {
  static constexpr int NS = 2;
  static constexpr bool has_reaction = true, has_breaction = true;
  double D1, D2, k;
  VFVM_HD void load(const double* p) { D1 = p[0]; D2 = p[1]; k = p[2]; }
  template <class T> VFVM_HD void flux(T* f, const T* uK, const T* uL, const EdgeItem&) const {
    f[0] = (uK[0] - uL[0]) * D1;
    f[1] = (uK[1] - uL[1]) * D2;
  }
  template <class T> VFVM_HD void reaction(T* f, const T* u, const NodeItem&) const {
    T r = (u[0] - sq(u[1])) * k;
    f[0] = r; f[1] = -r;
  }
  template <class T> VFVM_HD void breaction(T* f, const T* u, const BNodeItem& b) const {
    boundary_dirichlet(f, u, b, 0, 4, 1.0);
    boundary_dirichlet(f, u, b, 1, 4, 0.0);
    boundary_dirichlet(f, u, b, 0, 2, 0.0);
    boundary_dirichlet(f, u, b, 1, 2, 1.0);
  }
};

// Workload 5: -div(kappa grad u) + exp(u) = f, u = 0 on every boundary; node data
// kappa, edge coefficient = arithmetic mean of the two node values.  params: f
struct PhysKappaExp : PhysBase {
  static constexpr int NS = 1;
  static constexpr bool has_reaction = true, has_source = true, has_breaction = true;
  double fsrc;
  VFVM_HD void load(const double* p) { fsrc = p[0]; }
  template <class T> VFVM_HD void flux(T* f, const T* uK, const T* uL, const EdgeItem& e) const {
    f[0] = (uK[0] - uL[0]) * (0.5 * (e.dataK[0] + e.dataL[0]));
  }
  template <class T> VFVM_HD void reaction(T* f, const T* u, const NodeItem&) const { f[0] = exp(u[0]); }
  VFVM_HD void source(double* f, const NodeItem&) const { f[0] = fsrc; }
  template <class T> VFVM_HD void breaction(T* f, const T* u, const BNodeItem& b) const { boundary_dirichlet(f, u, b, 0, b.region, 0.0); }
};

// Heat equation with a conducting surface layer on boundary region breg (the
// single-species form of examples/Example311_HeatEquation_BoundaryDiffusion.jl):
//   u_t - div(eps grad u) = 0 in the domain (storage u, flux eps (u_K - u_L));
//   on region breg: surface diffusion along the boundary edges (bflux
//   eps_s (u_K - u_L)), surface capacity (bstorage c_s u), heat loss k u^3
//   (breaction) and a heat source q0 exp(-20 ((x-1/2)^2 + (y-1/2)^2)) (bsource);
//   the other boundary regions are insulated.  Grids of dimension 2 or 3.
// params: eps, eps_s, c_s, k, q0, breg
struct PhysSurfaceHeat : PhysBase {
  static constexpr int NS = 1;
  static constexpr bool has_storage = true, has_breaction = true, has_bflux = true, has_bstorage = true,
                        has_bsource = true;
  double eps, eps_s, c_s, k, q0;
  int breg;
  VFVM_HD void load(const double* p) { eps = p[0]; eps_s = p[1]; c_s = p[2]; k = p[3]; q0 = p[4]; breg = (int)p[5]; }
  template <class T> VFVM_HD void flux(T* f, const T* uK, const T* uL, const EdgeItem&) const { f[0] = (uK[0] - uL[0]) * eps; }
  template <class T> VFVM_HD void storage(T* f, const T* u, const NodeItem&) const { f[0] = u[0]; }
  template <class T> VFVM_HD void bflux(T* f, const T* uK, const T* uL, const BEdgeItem& e) const {
    if (e.region == breg) f[0] = (uK[0] - uL[0]) * eps_s;
  }
  template <class T> VFVM_HD void bstorage(T* f, const T* u, const BNodeItem& b) const {
    if (b.region == breg) f[0] = u[0] * c_s;
  }
  template <class T> VFVM_HD void breaction(T* f, const T* u, const BNodeItem& b) const {
    if (b.region == breg) f[0] = cube(u[0]) * k;
  }
  VFVM_HD void bsource(double* f, const BNodeItem& b) const {
    if (b.region == breg) {
      const double x1 = b.x[0] - 0.5, x2 = b.x[1] - 0.5;
      f[0] = q0 * ::exp(-20.0 * (x1 * x1 + x2 * x2));
    }
  }
};

// A bulk species and a boundary species (examples/Example230_BoundaryFlux.jl):
// species 1: -d u'' + k u = c (flux, reaction, source); species 2 on boundary
// region breg: -d_b v'' + k_b(y) v = c_b(y) along the boundary (bflux,
// breaction, bsource), k_b = kmax, c_b = 0 where y <= 1/2, k_b = 0, c_b = cmax
// elsewhere.  The bulk callbacks carry the same law for species 2 in the first
// coordinate, so a 1D grid with species 2 enabled as a bulk species solves the
// example's reference line problem (the example's node-index switch of k and c
// at the middle node equals the coordinate switch at 1/2).  Species 2 is
// meant to be restricted to breg (enable_boundary_species!) on grids of
// dimension 2, and breg = 0 on the 1D grid.
// params: d, k, c, d_b, kmax, cmax, breg
struct PhysBoundarySpecies : PhysBase {
  static constexpr int NS = 2;
  static constexpr bool has_reaction = true, has_source = true, has_breaction = true, has_bflux = true,
                        has_bsource = true;
  double d, k, c, db, kmax, cmax;
  int breg;
  VFVM_HD void load(const double* p) { d = p[0]; k = p[1]; c = p[2]; db = p[3]; kmax = p[4]; cmax = p[5]; breg = (int)p[6]; }
  // the boundary callbacks read the second coordinate: boundary region breg needs dim >= 2
  static bool valid(int dim, const double* p) { return dim >= 2 || (int)p[6] == 0; }
  VFVM_HD double kb(double s) const { return s <= 0.5 ? kmax : 0.0; }
  VFVM_HD double cb(double s) const { return s <= 0.5 ? 0.0 : cmax; }
  template <class T> VFVM_HD void flux(T* f, const T* uK, const T* uL, const EdgeItem&) const {
    f[0] = (uK[0] - uL[0]) * d;
    f[1] = (uK[1] - uL[1]) * db;
  }
  template <class T> VFVM_HD void reaction(T* f, const T* u, const NodeItem& n) const {
    f[0] = u[0] * k;
    f[1] = u[1] * kb(n.x[0]);
  }
  VFVM_HD void source(double* f, const NodeItem& n) const { f[0] = c; f[1] = cb(n.x[0]); }
  template <class T> VFVM_HD void bflux(T* f, const T* uK, const T* uL, const BEdgeItem& e) const {
    if (e.region == breg) f[1] = (uK[1] - uL[1]) * db;
  }
  template <class T> VFVM_HD void breaction(T* f, const T* u, const BNodeItem& b) const {
    if (b.region == breg) f[1] = u[1] * kb(b.x[1]);
  }
  VFVM_HD void bsource(double* f, const BNodeItem& b) const {
    if (b.region == breg) f[1] = cb(b.x[1]);
  }
};

// examples/DevEx002_EdgeReaction.jl:49-104 (case :compare_max): u_t - div grad u
// = 1 with u = 0 on every boundary region (1-6), the unit source given as
// mode 0: a node reaction -1; mode 1: an edge reaction -h^2/(2 dim), h the
// edge length; mode 2: an edge reaction -(x_K - x_L)^2 / 2.
// params: mode, dim
struct PhysEdgeReaction : PhysBase {
  static constexpr int NS = 1;
  static constexpr bool has_reaction = true, has_storage = true, has_breaction = true, has_edgereaction = true;
  int mode, dim;
  VFVM_HD void load(const double* p) { mode = (int)p[0]; dim = (int)p[1]; }
  static bool valid(int d, const double* p) { return (int)p[1] == d && p[0] >= 0.0 && p[0] <= 2.0; }
  template <class T> VFVM_HD void flux(T* f, const T* uK, const T* uL, const EdgeItem&) const { f[0] = uK[0] - uL[0]; }
  template <class T> VFVM_HD void storage(T* f, const T* u, const NodeItem&) const { f[0] = u[0]; }
  // constant terms are written as u * 0 + value so that T may be a dual number
  template <class T> VFVM_HD void reaction(T* f, const T* u, const NodeItem&) const {
    if (mode == 0) f[0] = u[0] * 0.0 + (-1.0);
  }
  template <class T> VFVM_HD void edgereaction(T* f, const T* uK, const T*, const EdgeItem& e) const {
    if (mode == 1) {
      double s = 0.0;
      for (int d = 0; d < dim; ++d) s += (e.xK[d] - e.xL[d]) * (e.xK[d] - e.xL[d]);
      const double h = sqrt(s);  // meas(edge)
      f[0] = uK[0] * 0.0 + (-1.0 * (h * h) / (2 * dim));
    } else if (mode == 2) {
      const double dp = e.xK[0] - e.xL[0];
      f[0] = uK[0] * 0.0 + (-dp * dp / 2);
    }
  }
  template <class T> VFVM_HD void breaction(T* f, const T* u, const BNodeItem& b) const {
    for (int r = 1; r <= 6; ++r) boundary_dirichlet(f, u, b, 0, r, 0.0);
  }
};

// The callbacks of examples/Example206_JouleHeat.jl:63-92 (phi, T): flux
// kappa(y_T) (phi_K - phi_L), lambda (T_K - T_L); edge reaction (Joule heat)
// -kappa(y_T) (phi_K - phi_L)^2 on T; storage c T; phi = -10 on boundary
// region 1, +10 on region 2; Robin 0.5 T - T0 for T on regions 1-4.  kappa(T)
// = kappa0 exp(alpha (T - T0)) is evaluated at the output value y_T, which is
// still 0 where the example reads it (the example's own form).
// params: kappa0, alpha, T0, lambda, c
struct PhysJouleHeat : PhysBase {
  static constexpr int NS = 2;
  static constexpr bool has_storage = true, has_breaction = true, has_edgereaction = true;
  double kappa0, alpha, T0, lam, c;
  VFVM_HD void load(const double* p) { kappa0 = p[0]; alpha = p[1]; T0 = p[2]; lam = p[3]; c = p[4]; }
  template <class T> VFVM_HD T kappa(const T& t) const { return exp((t - T0) * alpha) * kappa0; }
  template <class T> VFVM_HD void flux(T* f, const T* uK, const T* uL, const EdgeItem&) const {
    f[0] = kappa(f[1]) * (uK[0] - uL[0]);
    f[1] = (uK[1] - uL[1]) * lam;
  }
  template <class T> VFVM_HD void edgereaction(T* f, const T* uK, const T* uL, const EdgeItem&) const {
    const T d = uK[0] - uL[0];
    f[1] = kappa(f[1]) * (-1.0) * d * d;
  }
  template <class T> VFVM_HD void storage(T* f, const T* u, const NodeItem&) const { f[1] = u[1] * c; }
  template <class T> VFVM_HD void breaction(T* f, const T* u, const BNodeItem& b) const {
    boundary_dirichlet(f, u, b, 0, 1, -10.0);
    boundary_dirichlet(f, u, b, 0, 2, 10.0);
    for (int r = 1; r <= 4; ++r)
      if (b.region == r) f[1] = f[1] + (u[1] * 0.5 - T0);  // boundary_robin!: y += factor u - value
  }
};

// examples/Example161_BipolarDriftDiffusionCurrent.jl:85-151: quasi-Fermi
// potentials phi_n, phi_p and the electrostatic potential psi (species 1-3),
// densities n = exp(zn (phi_n - psi + En)), p = exp(zp (phi_p - psi + Ep)),
// zn = -1, zp = 1; doping Cn / Ca / -Cp in cell regions 1 / 2 / 3;
// Scharfetter-Gummel fluxes through fbernoulli_pm; recombination
// (1 + 1/(n+p)) n p (1 - exp(phi_n - phi_p)); Dirichlet values on boundary
// regions 1 and 2, the latter shifted by the bias scanProtocol(t) (:54-66).
// params: Cn, Cp, Ca, En, Ep, mu_n, mu_p, lambda, tPrecond, tRamp, tExt, Vprecond, VExt, DirichletVal
struct PhysEx161 : PhysBase {
  static constexpr int NS = 3;
  static constexpr bool has_reaction = true, has_storage = true, has_breaction = true;
  double Cn, Cp, Ca, En, Ep, mun, mup, lambda, tPrecond, tRamp, tExt, Vprecond, VExt, DirichletVal;
  static constexpr double zn = -1.0, zp = 1.0;
  VFVM_HD void load(const double* p) {
    Cn = p[0]; Cp = p[1]; Ca = p[2]; En = p[3]; Ep = p[4]; mun = p[5]; mup = p[6]; lambda = p[7];
    tPrecond = p[8]; tRamp = p[9]; tExt = p[10]; Vprecond = p[11]; VExt = p[12]; DirichletVal = p[13];
  }
  VFVM_HD double scan(double t) const {
    const double tEnd = tPrecond + tRamp + tExt;
    if (0.0 <= t && t <= tPrecond) return Vprecond;
    if (tPrecond <= t && t <= tPrecond + tRamp) return Vprecond - (Vprecond - VExt) / tRamp * (t - tPrecond);
    if (tPrecond + tRamp <= t && t <= tEnd) return VExt;
    return 0.0;
  }
  template <class T> VFVM_HD void reaction(T* f, const T* u, const NodeItem& n) const {
    const T nn = vexp(zn * (u[0] - u[2] + En));
    const T np = vexp(zp * (u[1] - u[2] + Ep));
    const double C = n.region == 1 ? Cn : (n.region == 2 ? Ca : (n.region == 3 ? -Cp : 0.0));
    f[2] = -(C + zn * nn + zp * np);
    const T recomb = (1.0 + 1.0 / (nn + np)) * (nn * np * (1.0 - vexp(u[0] - u[1])));
    f[0] = zn * recomb;
    f[1] = zp * recomb;
  }
  template <class T> VFVM_HD void flux(T* f, const T* uK, const T* uL, const EdgeItem&) const {
    f[2] = -(lambda * lambda) * (uL[2] - uK[2]);
    T bp, bm;
    fbernoulli_pm(-(uL[2] - uK[2]), bp, bm);
    const T nn1 = vexp(zn * (uK[0] - uK[2] + En)), np1 = vexp(zp * (uK[1] - uK[2] + Ep));
    const T nn2 = vexp(zn * (uL[0] - uL[2] + En)), np2 = vexp(zp * (uL[1] - uL[2] + Ep));
    f[0] = -zn * mun * (bm * nn2 - bp * nn1);
    f[1] = -zp * mup * (bp * np2 - bm * np1);
  }
  template <class T> VFVM_HD void storage(T* f, const T* u, const NodeItem&) const {
    f[0] = zn * vexp(zn * (u[0] - u[2] + En));
    f[1] = zp * vexp(zp * (u[1] - u[2] + Ep));
  }
  template <class T> VFVM_HD void breaction(T* f, const T* u, const BNodeItem& b) const {
    const double s = scan(b.time);
    boundary_dirichlet(f, u, b, 0, 1, 0.0);
    boundary_dirichlet(f, u, b, 1, 1, 0.0);
    boundary_dirichlet(f, u, b, 2, 1, 0.5 * (En + Ep) + asinh(Cn / (2 * sqrt(::exp(-(En - Ep))))));
    boundary_dirichlet(f, u, b, 0, 2, DirichletVal + s);
    boundary_dirichlet(f, u, b, 1, 2, DirichletVal + s);
    boundary_dirichlet(f, u, b, 2, 2, 0.5 * (En + Ep) + asinh(-Cp / (2 * sqrt(::exp(-(En - Ep))))) + DirichletVal + s);
  }
};

// The system of TestFunctionFactory (src/vfvm_testfunctions.jl:38-50): flux
// u_K - u_L, storage u; its Dirichlet values come through the legacy
// boundary data (T = 0 and 1 on the chosen boundary regions).
struct PhysTestFunction : PhysBase {
  static constexpr int NS = 1;
  static constexpr bool has_storage = true;
  VFVM_HD void load(const double*) {}
  template <class T> VFVM_HD void flux(T* f, const T* uK, const T* uL, const EdgeItem&) const { f[0] = uK[0] - uL[0]; }
  template <class T> VFVM_HD void storage(T* f, const T* u, const NodeItem&) const { f[0] = u[0]; }
};

// examples/Example430_ParameterDerivativesStationary.jl:146-166 (runh): flux
// (1 + p) (u_K^2 - u_L^2), reaction p u^5, u = 0 on boundary region 1 and u = p
// on region 3, with p the parameter whose derivatives dF/dp the assembly
// provides (the reference's parameters(u)[1], nparams = 1).  PT is double for
// the ordinary assembly and a dual number of width one for dF/dp.
// params: p
template <class PT>
struct PhysEx430T : PhysBase {
  static constexpr int NS = 1;
  static constexpr int NPD = 1;
  static constexpr bool has_reaction = true, has_breaction = true;
  template <class Q> using rebind = PhysEx430T<Q>;
  PT p;
  VFVM_HD void load(const double* q) { p = pconst<PT>(q[0]); }
  VFVM_HD void seed(int k) {
    if constexpr (!std::is_same<PT, double>::value) p.d[0] = k == 0 ? 1.0 : 0.0;
  }
  template <class T> VFVM_HD void flux(T* f, const T* uK, const T* uL, const EdgeItem&) const {
    f[0] = (1.0 + p) * (uK[0] * uK[0] - uL[0] * uL[0]);
  }
  template <class T> VFVM_HD void reaction(T* f, const T* u, const NodeItem&) const {
    const T u2 = u[0] * u[0];
    f[0] = p * (u2 * u2 * u[0]);
  }
  template <class T> VFVM_HD void breaction(T* f, const T* u, const BNodeItem& b) const {
    boundary_dirichlet(f, u, b, 0, 1, 0.0);
    boundary_dirichlet(f, u, b, 0, 3, p);
  }
};
using PhysEx430 = PhysEx430T<double>;

// The flow-and-transport system of the reference's outflow example
// (pluto-examples/outflow.jl): pressure p and concentration c, Darcy velocity
// v_h = k (p_K - p_L), flux (v_h, D (B(-v_h/D) c_K - B(v_h/D) c_L)) through
// fbernoulli_pm(v_h / D); inflow v_in (Neumann) and c = c_in on boundary region
// G_in, p = 0 on G_out; the outflow term -v_h c_out on the edges with a node on
// G_out (c_out: that node's c).
// params: k, v_in, c_in, D, G_in, G_out
struct PhysOutflow : PhysBase {
  static constexpr int NS = 2;
  static constexpr bool has_breaction = true, has_boutflow = true;
  double k, v_in, c_in, D;
  int gin, gout;
  VFVM_HD void load(const double* p) { k = p[0]; v_in = p[1]; c_in = p[2]; D = p[3]; gin = (int)p[4]; gout = (int)p[5]; }
  static bool outflow_region(const double* p, int reg) { return reg == (int)p[5]; }
  template <class T> VFVM_HD void flux(T* f, const T* uK, const T* uL, const EdgeItem&) const {
    const T vh = (uK[0] - uL[0]) * k;
    f[0] = vh;
    T bp, bm;
    fbernoulli_pm(vh / D, bp, bm);
    f[1] = (bm * uK[1] - bp * uL[1]) * D;
  }
  template <class T> VFVM_HD void breaction(T* f, const T* u, const BNodeItem& b) const {
    if (b.region == gin) f[0] = f[0] - v_in;  // boundary_neumann!
    boundary_dirichlet(f, u, b, 0, gout, 0.0);
    boundary_dirichlet(f, u, b, 1, gin, c_in);
  }
  template <class T> VFVM_HD void boutflow(T* f, const T* uK, const T* uL, const EdgeItem& e) const {
    const T vh = (uK[0] - uL[0]) * k;
    f[1] = -(vh * (e.outflownode == 1 ? uK[1] : uL[1]));
  }
};

// examples/Example210_NonlinearPoisson2D_Reaction.jl:24-46: two species with
// flux eps (u_K - u_L), reaction k (u1 - u2) and k (u2 - u1), source
// exp(-20 ((x-1/2)^2 + (y-1/2)^2)) for species 1, storage u; no-flux boundary.
// params: eps, k
struct PhysEx210 : PhysBase {
  static constexpr int NS = 2;
  static constexpr bool has_reaction = true, has_storage = true, has_source = true;
  double eps, k;
  VFVM_HD void load(const double* p) { eps = p[0]; k = p[1]; }
  template <class T> VFVM_HD void flux(T* f, const T* uK, const T* uL, const EdgeItem&) const {
    f[0] = (uK[0] - uL[0]) * eps;
    f[1] = (uK[1] - uL[1]) * eps;
  }
  template <class T> VFVM_HD void reaction(T* f, const T* u, const NodeItem&) const {
    f[0] = (u[0] - u[1]) * k;
    f[1] = (u[1] - u[0]) * k;
  }
  template <class T> VFVM_HD void storage(T* f, const T* u, const NodeItem&) const { f[0] = u[0]; f[1] = u[1]; }
  VFVM_HD void source(double* f, const NodeItem& n) const {
    const double x1 = n.x[0] - 0.5, x2 = n.x[1] - 0.5;
    f[0] = ::exp(-20.0 * (x1 * x1 + x2 * x2));
  }
};

// examples/Example102_StationaryConvectionDiffusion1D.jl:40-78: -(D u' - v u)' =
// 0 with the example's three fluxes, vh = project(edge, v) = (x_L - x_K) v
// (src/vfvm_geometryitems.jl:634-640, v along the first coordinate):
// flux 0 exponential: D B(-vh/D) u_K - D B(vh/D) u_L with the example's own
//   B(x) = x / (exp(x) - 1), B = 1 where |x| < nextfloat(eps);
// flux 1 upwind: D (u_K - u_L) + vh u_K if vh > 0, else + vh u_L;
// flux 2 central: D (u_K - u_L) + vh (u_K + u_L) / 2.
// params: D, v, flux
struct PhysEx102 : PhysBase {
  static constexpr int NS = 1;
  double D, v;
  int mode;
  VFVM_HD void load(const double* p) { D = p[0]; v = p[1]; mode = (int)p[2]; }
  VFVM_HD static double bern(double x) {
    return fabs(x) < 0x1.0000000000001p-52 ? 1.0 : x / (::exp(x) - 1.0);
  }
  template <class T> VFVM_HD void flux(T* f, const T* uK, const T* uL, const EdgeItem& e) const {
    const double vh = (e.xL[0] - e.xK[0]) * v;
    if (mode == 0) {
      const double bplus = D * bern(vh / D), bminus = D * bern(-vh / D);
      f[0] = uK[0] * bminus - uL[0] * bplus;
    } else if (mode == 1) {
      f[0] = (uK[0] - uL[0]) * D + (vh > 0.0 ? uK[0] : uL[0]) * vh;
    } else {
      f[0] = (uK[0] - uL[0]) * D + (uK[0] + uL[0]) * vh / 2.0;
    }
  }
};

// examples/Example107_NonlinearStorage1D.jl:44-64: flux u_K - u_L, storage
// (eps + u)^(1/m).
// params: m, eps
struct PhysEx107 : PhysBase {
  static constexpr int NS = 1;
  static constexpr bool has_storage = true;
  double m, eps;
  VFVM_HD void load(const double* p) { m = p[0]; eps = p[1]; }
  template <class T> VFVM_HD void flux(T* f, const T* uK, const T* uL, const EdgeItem&) const { f[0] = uK[0] - uL[0]; }
  template <class T> VFVM_HD void storage(T* f, const T* u, const NodeItem&) const { f[0] = vpow(u[0] + eps, 1.0 / m); }
};

// examples/Example115_HeterogeneousCatalysis1D.jl:113-176: species A, B in the
// bulk (flux D_A, D_B; storage u; source exp(-100 (x - 1/2)^2) for A), species
// C a boundary species on region iCat; there, with R_AC = kp_AC u_A (1 - u_C) -
// km_AC u_C and R_BC = kp_BC u_B (1 - u_C) - km_BC u_C, the boundary reactions
// S R_AC, S R_BC, -R_BC - R_AC and the boundary storage u_C.
// params: D_A, D_B, kp_AC, km_AC, kp_BC, km_BC, S, iCat
struct PhysEx115 : PhysBase {
  static constexpr int NS = 3;
  static constexpr bool has_storage = true, has_source = true, has_breaction = true, has_bstorage = true;
  double DA, DB, kpAC, kmAC, kpBC, kmBC, S;
  int icat;
  VFVM_HD void load(const double* p) {
    DA = p[0]; DB = p[1]; kpAC = p[2]; kmAC = p[3]; kpBC = p[4]; kmBC = p[5]; S = p[6]; icat = (int)p[7];
  }
  template <class T> VFVM_HD void flux(T* f, const T* uK, const T* uL, const EdgeItem&) const {
    f[0] = (uK[0] - uL[0]) * DA;
    f[1] = (uK[1] - uL[1]) * DB;
  }
  template <class T> VFVM_HD void storage(T* f, const T* u, const NodeItem&) const { f[0] = u[0]; f[1] = u[1]; }
  VFVM_HD void source(double* f, const NodeItem& n) const {
    const double x1 = n.x[0] - 0.5;
    f[0] = ::exp(-100.0 * (x1 * x1));
  }
  template <class T> VFVM_HD void breaction(T* f, const T* u, const BNodeItem& b) const {
    if (b.region != icat) return;
    const T rac = kpAC * u[0] * (1.0 - u[2]) - kmAC * u[2];
    const T rbc = kpBC * u[1] * (1.0 - u[2]) - kmBC * u[2];
    f[0] = S * rac;
    f[1] = S * rbc;
    f[2] = -rbc - rac;
  }
  template <class T> VFVM_HD void bstorage(T* f, const T* u, const BNodeItem& b) const {
    if (b.region == icat) f[2] = u[2];
  }
};

// examples/Example215_NonlinearPoisson2D_BoundaryReaction.jl:27-50: two
// species, flux eps (u_K - u_L), storage u, and on boundary region 2 the
// reactions k (u1 - u2), k (u2 - u1).
// params: eps, k
struct PhysEx215 : PhysBase {
  static constexpr int NS = 2;
  static constexpr bool has_storage = true, has_breaction = true;
  double eps, k;
  VFVM_HD void load(const double* p) { eps = p[0]; k = p[1]; }
  template <class T> VFVM_HD void flux(T* f, const T* uK, const T* uL, const EdgeItem&) const {
    f[0] = (uK[0] - uL[0]) * eps;
    f[1] = (uK[1] - uL[1]) * eps;
  }
  template <class T> VFVM_HD void storage(T* f, const T* u, const NodeItem&) const { f[0] = u[0]; f[1] = u[1]; }
  template <class T> VFVM_HD void breaction(T* f, const T* u, const BNodeItem& b) const {
    if (b.region != 2) return;
    f[0] = (u[0] - u[1]) * k;
    f[1] = (u[1] - u[0]) * k;
  }
};

// examples/Example220_NonlinearPoisson2D_BoundarySpecies.jl:23-57: bulk species
// 1, 2 (flux eps (u_K - u_L), storage u, source exp(-20 ((x-1/2)^2 + (y-1/2)^2))
// for species 1) and species 3 on boundary region 2 with the boundary storage u3
// and the reactions k (u1 - u3), k (u3 - u1) + k (u3 - u2), k (u2 - u3) there.
// params: k, eps
struct PhysEx220 : PhysBase {
  static constexpr int NS = 3;
  static constexpr bool has_storage = true, has_source = true, has_breaction = true, has_bstorage = true;
  double k, eps;
  VFVM_HD void load(const double* p) { k = p[0]; eps = p[1]; }
  static bool valid(int dim, const double*) { return dim >= 2; }
  template <class T> VFVM_HD void flux(T* f, const T* uK, const T* uL, const EdgeItem&) const {
    f[0] = (uK[0] - uL[0]) * eps;
    f[1] = (uK[1] - uL[1]) * eps;
  }
  template <class T> VFVM_HD void storage(T* f, const T* u, const NodeItem&) const { f[0] = u[0]; f[1] = u[1]; }
  VFVM_HD void source(double* f, const NodeItem& n) const {
    const double x1 = n.x[0] - 0.5, x2 = n.x[1] - 0.5;
    f[0] = ::exp(-20.0 * (x1 * x1 + x2 * x2));
  }
  template <class T> VFVM_HD void breaction(T* f, const T* u, const BNodeItem& b) const {
    if (b.region != 2) return;
    f[0] = (u[0] - u[2]) * k;
    f[2] = (u[2] - u[0]) * k + (u[2] - u[1]) * k;
    f[1] = (u[1] - u[2]) * k;
  }
  template <class T> VFVM_HD void bstorage(T* f, const T* u, const BNodeItem& b) const {
    if (b.region == 2) f[2] = u[2];
  }
};

// examples/Example203_CoordinateSystems.jl:14-17 and its sources: flux u_K -
// u_L, the constant source f (1 for the disk, cylinder and ball, 0 for the ring,
// cylinder shell and spherical shell); the coordinate system is the grid's.
// params: f
struct PhysEx203 : PhysBase {
  static constexpr int NS = 1;
  static constexpr bool has_source = true;
  double f0;
  VFVM_HD void load(const double* p) { f0 = p[0]; }
  template <class T> VFVM_HD void flux(T* f, const T* uK, const T* uL, const EdgeItem&) const { f[0] = uK[0] - uL[0]; }
  VFVM_HD void source(double* f, const NodeItem&) const { f[0] = f0; }
};

inline int physics_nspec(int id) {
  switch (id) {
    case VFVM_PHYS_EX105: case VFVM_PHYS_EX106: case VFVM_PHYS_EX207: case VFVM_PHYS_EX301:
    case VFVM_PHYS_EX440: case VFVM_PHYS_LAPLACE_DIRICHLET: case VFVM_PHYS_NLPOISSON:
    case VFVM_PHYS_POROUS: case VFVM_PHYS_KAPPA_EXP: case VFVM_PHYS_SURFACE_HEAT:
    case VFVM_PHYS_EDGE_REACTION: case VFVM_PHYS_TESTFUNCTION: case VFVM_PHYS_EX430: case VFVM_PHYS_EX102:
    case VFVM_PHYS_EX107: case VFVM_PHYS_EX203: return 1;
    case VFVM_PHYS_EX110: case VFVM_PHYS_EX160: case VFVM_PHYS_RD2: case VFVM_PHYS_BOUNDARY_SPECIES:
    case VFVM_PHYS_JOULE_HEAT: case VFVM_PHYS_OUTFLOW: case VFVM_PHYS_EX210: case VFVM_PHYS_EX215: return 2;
    case VFVM_PHYS_BIPOLAR: case VFVM_PHYS_EX161: case VFVM_PHYS_EX115: case VFVM_PHYS_EX220: return 3;
  }
  return 0;
}
inline int physics_nparams(int id) {
  switch (id) {
    case VFVM_PHYS_EX105: case VFVM_PHYS_EX106: case VFVM_PHYS_EX207: case VFVM_PHYS_EX440:
    case VFVM_PHYS_KAPPA_EXP: return 1;
    case VFVM_PHYS_EX110: return 2;
    case VFVM_PHYS_EX160: case VFVM_PHYS_RD2: return 3;
    case VFVM_PHYS_BIPOLAR: return 7;
    case VFVM_PHYS_SURFACE_HEAT: return 6;
    case VFVM_PHYS_BOUNDARY_SPECIES: return 7;
    case VFVM_PHYS_EDGE_REACTION: return 2;
    case VFVM_PHYS_JOULE_HEAT: return 5;
    case VFVM_PHYS_EX161: return 14;
    case VFVM_PHYS_EX430: return 1;
    case VFVM_PHYS_OUTFLOW: return 6;
    case VFVM_PHYS_EX210: return 2;
    case VFVM_PHYS_EX102: return 3;
    case VFVM_PHYS_EX107: return 2;
    case VFVM_PHYS_EX115: return 8;
    case VFVM_PHYS_EX215: return 2;
    case VFVM_PHYS_EX220: return 2;
    case VFVM_PHYS_EX203: return 1;
  }
  return 0;
}
inline int physics_nnodedata(int id) { return id == VFVM_PHYS_KAPPA_EXP ? 1 : 0; }

// Calls fn(PhysType{}) for the physics id (host-side dispatch to templated launches).
template <class Fn>
int dispatch_physics(int id, Fn&& fn) {
  switch (id) {
    case VFVM_PHYS_EX105: return fn(PhysEx105{});
    case VFVM_PHYS_EX106: return fn(PhysEx106{});
    case VFVM_PHYS_EX110: return fn(PhysEx110{});
    case VFVM_PHYS_EX160: return fn(PhysEx160{});
    case VFVM_PHYS_EX207: return fn(PhysEx207{});
    case VFVM_PHYS_EX301: return fn(PhysEx301{});
    case VFVM_PHYS_EX440: return fn(PhysEx440{});
    case VFVM_PHYS_LAPLACE_DIRICHLET: return fn(PhysLaplaceDir{});
    case VFVM_PHYS_NLPOISSON: return fn(PhysNLPoisson{});
    case VFVM_PHYS_POROUS: return fn(PhysPorous{});
    case VFVM_PHYS_BIPOLAR: return fn(PhysBipolar{});
    case VFVM_PHYS_RD2: return fn(PhysRD2{});
    case VFVM_PHYS_KAPPA_EXP: return fn(PhysKappaExp{});
    case VFVM_PHYS_SURFACE_HEAT: return fn(PhysSurfaceHeat{});
    case VFVM_PHYS_BOUNDARY_SPECIES: return fn(PhysBoundarySpecies{});
    case VFVM_PHYS_EDGE_REACTION: return fn(PhysEdgeReaction{});
    case VFVM_PHYS_JOULE_HEAT: return fn(PhysJouleHeat{});
    case VFVM_PHYS_EX161: return fn(PhysEx161{});
    case VFVM_PHYS_TESTFUNCTION: return fn(PhysTestFunction{});
    case VFVM_PHYS_EX430: return fn(PhysEx430{});
    case VFVM_PHYS_OUTFLOW: return fn(PhysOutflow{});
    case VFVM_PHYS_EX210: return fn(PhysEx210{});
    case VFVM_PHYS_EX102: return fn(PhysEx102{});
    case VFVM_PHYS_EX107: return fn(PhysEx107{});
    case VFVM_PHYS_EX115: return fn(PhysEx115{});
    case VFVM_PHYS_EX215: return fn(PhysEx215{});
    case VFVM_PHYS_EX220: return fn(PhysEx220{});
    case VFVM_PHYS_EX203: return fn(PhysEx203{});
  }
  return VFVM_ERR_INPUT;
}

}  // namespace vfvm
