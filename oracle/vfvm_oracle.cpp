// VoronoiFVM.jl assembly oracle -- TEST INFRASTRUCTURE ONLY.
//
// A plain CPU (FP64) restatement of the reference's edgewise assembly path, used
// by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg as the
// checker.  Nothing in the shipped package links or calls this file.
//
// What it restates (paths relative to the reference project):
//   cellfactors! (Edge1D, Triangle2D, Tetrahedron3D)   src/vfvm_formfactors.jl:12-23,64-100,163-235
//     (Polar1D, Spherical1D, Cylindrical2D)            src/vfvm_formfactors.jl:25-62,102-161
//   bfacefactors! (Vertex0D, Edge1D, Triangle2D)        src/vfvm_formfactors.jl:244-332
//   edgewise factor accumulation                       src/vfvm_system.jl:712-754
//   Dirichlet constant 1e30                            src/vfvm_system.jl:329
//   _initialize_dirichlet!                             src/vfvm_system.jl:947-1003
//   eval_and_assemble (single partition)               src/vfvm_assembly.jl:520-570
//   assemble_nodes / assemble_edges / assemble_bnodes  src/vfvm_assembly.jl:38-126,128-200,318-442
//   assemble_bedges (bflux on boundary-face edges)     src/vfvm_assembly.jl:444-510
//   cellwise assembly data (per-cell node/edge factors) src/vfvm_assemblydata.jl:126-208
//   _addnz (skip exact zeros, NaN is an error)         src/vfvm_assembly.jl:21-28
//   assemble_res_jac (Node, BNode, Edge)               src/vfvm_assemblydata.jl:245-302,350-382
//   ResJacEvaluator: forward-mode AD, full chunk       src/vfvm_physics.jl:421-452
//   boundary_dirichlet!/boundary_neumann!              src/vfvm_physics.jl:487-494,533
//   fbernoulli_pm / bernoulli_horner                   src/vfvm_functions.jl:1-90
// The physics callbacks restate the user functions of the reference examples
// they are named after, and the benchmark workloads (documented per physics).
//
// Jacobian pattern: a candidate CSR (node + neighbour blocks, all species) with a
// per-entry "present" flag set exactly when the reference would create the entry
// (a nonzero contribution, _addnz).  Only present entries are reported.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <limits>

namespace {

const double kDirichlet = 1.0e30;

// ---------------------------------------------------------------- dual numbers
template <int N>
struct Dual {
  double v;
  double d[N];
};
template <int N> inline Dual<N> mk(double v) { Dual<N> r; r.v = v; for (int i = 0; i < N; ++i) r.d[i] = 0; return r; }
template <int N> inline double val(const Dual<N>& a) { return a.v; }
inline double val(double a) { return a; }
template <int N> inline Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) { Dual<N> r; r.v = a.v + b.v; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i]; return r; }
template <int N> inline Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) { Dual<N> r; r.v = a.v - b.v; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i]; return r; }
template <int N> inline Dual<N> operator-(const Dual<N>& a) { Dual<N> r; r.v = -a.v; for (int i = 0; i < N; ++i) r.d[i] = -a.d[i]; return r; }
template <int N> inline Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) { Dual<N> r; r.v = a.v * b.v; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i]; return r; }
template <int N> inline Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = a.v / b.v; double ib = 1.0 / (b.v * b.v);
  for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] * b.v - a.v * b.d[i]) * ib;
  return r;
}
template <int N> inline Dual<N> operator+(const Dual<N>& a, double b) { Dual<N> r = a; r.v += b; return r; }
template <int N> inline Dual<N> operator+(double b, const Dual<N>& a) { Dual<N> r = a; r.v += b; return r; }
template <int N> inline Dual<N> operator-(const Dual<N>& a, double b) { Dual<N> r = a; r.v -= b; return r; }
template <int N> inline Dual<N> operator-(double b, const Dual<N>& a) { Dual<N> r; r.v = b - a.v; for (int i = 0; i < N; ++i) r.d[i] = -a.d[i]; return r; }
template <int N> inline Dual<N> operator*(const Dual<N>& a, double b) { Dual<N> r; r.v = a.v * b; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b; return r; }
template <int N> inline Dual<N> operator*(double b, const Dual<N>& a) { return a * b; }
template <int N> inline Dual<N> operator/(const Dual<N>& a, double b) { Dual<N> r; r.v = a.v / b; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] / b; return r; }
template <int N> inline Dual<N> operator/(double a, const Dual<N>& b) { return mk<N>(a) / b; }
template <int N> inline Dual<N> exp(const Dual<N>& a) { Dual<N> r; r.v = std::exp(a.v); for (int i = 0; i < N; ++i) r.d[i] = r.v * a.d[i]; return r; }
template <int N> inline Dual<N> expm1(const Dual<N>& a) { Dual<N> r; r.v = std::expm1(a.v); double e = std::exp(a.v); for (int i = 0; i < N; ++i) r.d[i] = e * a.d[i]; return r; }
template <int N> inline Dual<N> log(const Dual<N>& a) { Dual<N> r; r.v = std::log(a.v); for (int i = 0; i < N; ++i) r.d[i] = a.d[i] / a.v; return r; }
template <int N> inline Dual<N> log1p(const Dual<N>& a) { Dual<N> r; r.v = std::log1p(a.v); for (int i = 0; i < N; ++i) r.d[i] = a.d[i] / (1.0 + a.v); return r; }
// x^p for real p (ForwardDiff: p*x^(p-1)*dx)
template <int N> inline Dual<N> pow(const Dual<N>& a, double p) { Dual<N> r; r.v = std::pow(a.v, p); double dp = p * std::pow(a.v, p - 1); for (int i = 0; i < N; ++i) r.d[i] = dp * a.d[i]; return r; }
template <int N> inline Dual<N> sq(const Dual<N>& a) { return a * a; }
template <int N> inline Dual<N> cube(const Dual<N>& a) { Dual<N> r; r.v = a.v * a.v * a.v; double dp = 3 * a.v * a.v; for (int i = 0; i < N; ++i) r.d[i] = dp * a.d[i]; return r; }
template <int N> inline Dual<N> dmax(const Dual<N>& a, double b) { return a.v >= b ? a : mk<N>(b); }
inline double sq(double a) { return a * a; }
inline double cube(double a) { return a * a * a; }
inline double dmax(double a, double b) { return std::max(a, b); }
using std::exp; using std::expm1; using std::log; using std::log1p; using std::pow;

// Bernoulli function, src/vfvm_functions.jl:2-31,78-90
const double c1 = 1.0 / 47900160.0, c2 = -1.0 / 1209600.0, c3 = 1.0 / 30240.0,
             c4 = -1.0 / 720.0, c5 = 1.0 / 12.0, c6 = -1.0 / 2.0;
template <class T> inline T bernoulli_horner(const T& x) {
  T y = x * c1;
  y = x * y;
  y = x * (c2 + y);
  y = x * y;
  y = x * (c3 + y);
  y = x * y;
  y = x * (c4 + y);
  y = x * y;
  y = x * (c5 + y);
  y = x * (c6 + y);
  return 1.0 + y;
}
template <class T> inline void fbernoulli_pm(const T& x, T& bp, T& bm) {
  double xv = val(x);
  if (xv < -50.0) { bp = -x; bm = x * 0.0; }
  else if (xv > 50.0) { bp = x * 0.0; bm = x; }
  else if (std::fabs(xv) < 0.25) { bp = bernoulli_horner(x); bm = x + bp; }
  else { bp = x / expm1(x); bm = x + bp; }
}
template <class T> inline T fbernoulli(const T& x) {
  double xv = val(x);
  if (xv < -50.0) return -x;
  if (xv > 50.0) return x * 0.0;
  if (std::fabs(xv) < 0.25) return bernoulli_horner(x);
  return x / expm1(x);
}

// ramp(t; dt, du), src/vfvm_physics.jl:516-525
inline double ramp(double t, double t0, double t1, double u0, double u1) {
  if (t < t0) return u0;
  if (t < t1) return u0 + (u1 - u0) * (t - t0) / (t1 - t0);
  return u1;
}

// ---------------------------------------------------------------- geometry items
struct NodeInfo { int index, region; const double* x; double time, lambda; const double* ndata; };
struct EdgeInfo {
  int K, L, region; const double* xK; const double* xL; double time, lambda; const double* ndataK; const double* ndataL;
  int outflownode = 0;  // outflownode(edge): 1 or 2 on edges with a node on an outflow boundary
};
struct BNodeInfo { int index, region; const double* x; double time, lambda, fac, Dirichlet; double* dirichlet_value; };
struct BEdgeInfo { int K, L, region; const double* xK; const double* xL; double time, lambda; };

// boundary_dirichlet!(y,u,bnode,ispec,ireg,val), src/vfvm_physics.jl:487-494
template <class T> inline void boundary_dirichlet(T* y, const T* u, BNodeInfo& b, int ispec, int ireg, double v) {
  if (b.region == ireg) {
    y[ispec] = y[ispec] + b.Dirichlet * (u[ispec] - v);
    b.dirichlet_value[ispec] = v;
  }
}
// a Dirichlet value given by a parameter (a dual number carrying d/dp)
template <int N> inline void boundary_dirichlet(Dual<N>* y, const Dual<N>* u, BNodeInfo& b, int ispec, int ireg,
                                                const Dual<N>& v) {
  if (b.region == ireg) {
    y[ispec] = y[ispec] + b.Dirichlet * (u[ispec] - v);
    b.dirichlet_value[ispec] = v.v;
  }
}

// ---------------------------------------------------------------- physics
// Physics ids follow include/vfvm_gb300.h (VFVM_PHYS_*).
struct PhysParams { const double* p; int np; };

// Boundary callbacks beyond breaction (bflux, bstorage, bsource): absent unless a
// physics defines them.
struct OBase {
  static const bool has_bflux = false, has_bstorage = false, has_bsource = false, has_edgereaction = false;
  static const bool has_boutflow = false;
  template <class T> void boutflow(T*, const T*, const T*, const EdgeInfo&) const {}
  bool outflow_region(int) const { return false; }
  template <class T> void edgereaction(T*, const T*, const T*, const EdgeInfo&) const {}
  template <class T> void bflux(T*, const T*, const T*, const BEdgeInfo&) const {}
  template <class T> void bstorage(T*, const T*, BNodeInfo&) const {}
  void bsource(double*, BNodeInfo&) const {}
};

// Each physics: NS, has_* flags, templated callbacks.
struct PhysEx105 : OBase {  // examples/Example105_NonlinearPoisson1D.jl:41-60
  static const int NS = 1; double eps;
  static const bool has_reaction = true, has_storage = false, has_source = true, has_breaction = false;
  template <class T> void flux(T* f, const T* uK, const T* uL, const EdgeInfo&) const { f[0] = eps * (uK[0] - uL[0]); }
  template <class T> void reaction(T* f, const T* u, const NodeInfo&) const { f[0] = exp(u[0]) - exp(-u[0]); }
  template <class T> void storage(T*, const T*, const NodeInfo&) const {}
  void source(double* f, const NodeInfo& n) const { f[0] = (n.x[0] <= 0.5) ? 1.0 : -1.0; }
  template <class T> void breaction(T*, const T*, BNodeInfo&) const {}
};
struct PhysEx106 : OBase {  // examples/Example106_NonlinearDiffusion1D.jl:58-68
  static const int NS = 1; double m;
  static const bool has_reaction = false, has_storage = true, has_source = false, has_breaction = false;
  template <class T> void flux(T* f, const T* uK, const T* uL, const EdgeInfo&) const { f[0] = pow(uK[0], m) - pow(uL[0], m); }
  template <class T> void reaction(T*, const T*, const NodeInfo&) const {}
  template <class T> void storage(T* f, const T* u, const NodeInfo&) const { f[0] = u[0]; }
  void source(double*, const NodeInfo&) const {}
  template <class T> void breaction(T*, const T*, BNodeInfo&) const {}
};
struct PhysEx110 : OBase {  // examples/Example110_ReactionDiffusion1D_TwoSpecies.jl:40-64
  static const int NS = 2; double eps1, eps2;
  static const bool has_reaction = true, has_storage = true, has_source = true, has_breaction = false;
  template <class T> void flux(T* f, const T* uK, const T* uL, const EdgeInfo&) const {
    f[0] = eps1 * (uK[0] - uL[0]) * (0.01 + uK[1] + uL[1]);
    f[1] = eps2 * (uK[1] - uL[1]) * (0.01 + uK[0] + uL[0]);
  }
  template <class T> void reaction(T* f, const T* u, const NodeInfo&) const { f[0] = u[0] * u[1]; f[1] = -(u[0] * u[1]); }
  template <class T> void storage(T* f, const T* u, const NodeInfo&) const { f[0] = u[0]; f[1] = u[1]; }
  void source(double* f, const NodeInfo& n) const { f[0] = 1.0e-4 * (0.01 + n.x[0]); f[1] = 1.0e-4 * (0.01 + 1.0 - n.x[0]); }
  template <class T> void breaction(T*, const T*, BNodeInfo&) const {}
};
struct PhysEx160 : OBase {  // examples/Example160_UnipolarDriftDiffusion1D.jl:52-84 (sedan flux; iphi=1, ic=2)
  static const int NS = 2; double eps, z, V;
  static const bool has_reaction = true, has_storage = true, has_source = false, has_breaction = true;
  template <class T> void flux(T* f, const T* uK, const T* uL, const EdgeInfo&) const {
    f[0] = eps * (uK[0] - uL[0]);
    const double eps_reg = 1.0e-10;
    T mu1 = -log1p(dmax(-uK[1], -1.0 + eps_reg));
    T mu2 = -log1p(dmax(-uL[1], -1.0 + eps_reg));
    T bp, bm;
    fbernoulli_pm(z * 2.0 * (uK[0] - uL[0]) + (mu1 - mu2), bp, bm);
    f[1] = bm * uK[1] - bp * uL[1];
  }
  template <class T> void reaction(T* f, const T* u, const NodeInfo&) const { f[0] = z * (1.0 - 2.0 * u[1]); f[1] = u[1] * 0.0; }
  template <class T> void storage(T* f, const T* u, const NodeInfo&) const { f[0] = u[0] * 0.0; f[1] = u[1]; }
  void source(double*, const NodeInfo&) const {}
  template <class T> void breaction(T* f, const T* u, BNodeInfo& b) const {
    double Vt = ramp(b.time, 0.0, 1.0e-2, 0.0, V);
    boundary_dirichlet(f, u, b, 0, 1, Vt);
    boundary_dirichlet(f, u, b, 0, 2, 0.0);
    boundary_dirichlet(f, u, b, 1, 2, 0.5);
  }
};
struct PhysEx207 : OBase {  // examples/Example207_NonlinearPoisson2D.jl:36-50
  static const int NS = 1; double eps;
  static const bool has_reaction = true, has_storage = true, has_source = true, has_breaction = false;
  template <class T> void flux(T* f, const T* uK, const T* uL, const EdgeInfo&) const { f[0] = eps * (sq(uK[0]) - sq(uL[0])); }
  template <class T> void reaction(T* f, const T* u, const NodeInfo&) const { f[0] = sq(u[0]); }
  template <class T> void storage(T* f, const T* u, const NodeInfo&) const { f[0] = u[0]; }
  void source(double* f, const NodeInfo& n) const { double x1 = n.x[0] - 0.5, x2 = n.x[1] - 0.5; f[0] = std::exp(-20.0 * (x1 * x1 + x2 * x2)); }
  template <class T> void breaction(T*, const T*, BNodeInfo&) const {}
};
struct PhysEx301 : OBase {  // examples/Example301_Laplace3D.jl:15-24
  static const int NS = 1;
  static const bool has_reaction = false, has_storage = false, has_source = true, has_breaction = false;
  template <class T> void flux(T* f, const T* uK, const T* uL, const EdgeInfo&) const { f[0] = uK[0] - uL[0]; }
  template <class T> void reaction(T*, const T*, const NodeInfo&) const {}
  template <class T> void storage(T*, const T*, const NodeInfo&) const {}
  void source(double* f, const NodeInfo& n) const { f[0] = n.x[0] * std::sin(5.0 * n.x[1]) * std::exp(n.x[2]); }
  template <class T> void breaction(T*, const T*, BNodeInfo&) const {}
};
struct PhysEx440 : OBase {  // examples/Example440_ParallelState.jl:16-25
  static const int NS = 1; double influx;
  static const bool has_reaction = false, has_storage = false, has_source = false, has_breaction = true;
  template <class T> void flux(T* f, const T* uK, const T* uL, const EdgeInfo&) const { f[0] = sq(uK[0]) - sq(uL[0]); }
  template <class T> void reaction(T*, const T*, const NodeInfo&) const {}
  template <class T> void storage(T*, const T*, const NodeInfo&) const {}
  void source(double*, const NodeInfo&) const {}
  template <class T> void breaction(T* f, const T* u, BNodeInfo& b) const {
    boundary_dirichlet(f, u, b, 0, 1, 0.1);
    if (b.region == 2) f[0] = f[0] - influx;  // boundary_neumann!, src/vfvm_physics.jl:533
  }
};
struct PhysLaplaceDir : OBase {  // test/test030_cachesol.jl:10-18
  static const int NS = 1;
  static const bool has_reaction = false, has_storage = false, has_source = false, has_breaction = true;
  template <class T> void flux(T* f, const T* uK, const T* uL, const EdgeInfo&) const { f[0] = uK[0] - uL[0]; }
  template <class T> void reaction(T*, const T*, const NodeInfo&) const {}
  template <class T> void storage(T*, const T*, const NodeInfo&) const {}
  void source(double*, const NodeInfo&) const {}
  template <class T> void breaction(T* f, const T* u, BNodeInfo& b) const {
    boundary_dirichlet(f, u, b, 0, 1, 0.0);
    boundary_dirichlet(f, u, b, 0, 2, 1.0);
  }
};
// Benchmark workload 1: -div(grad u) + u^3 = 1, u = 0 on every boundary region.
struct PhysNLPoisson : OBase {
  static const int NS = 1;
  static const bool has_reaction = true, has_storage = false, has_source = false, has_breaction = true;
  template <class T> void flux(T* f, const T* uK, const T* uL, const EdgeInfo&) const { f[0] = uK[0] - uL[0]; }
  template <class T> void reaction(T* f, const T* u, const NodeInfo&) const { f[0] = cube(u[0]) - 1.0; }
  template <class T> void storage(T*, const T*, const NodeInfo&) const {}
  void source(double*, const NodeInfo&) const {}
  template <class T> void breaction(T* f, const T* u, BNodeInfo& b) const { boundary_dirichlet(f, u, b, 0, b.region, 0.0); }
};
// Benchmark workload 2: porous medium u_t - div(grad u^2) = 0, homogeneous Neumann.
struct PhysPorous : OBase {
  static const int NS = 1;
  static const bool has_reaction = false, has_storage = true, has_source = false, has_breaction = false;
  template <class T> void flux(T* f, const T* uK, const T* uL, const EdgeInfo&) const { f[0] = sq(uK[0]) - sq(uL[0]); }
  template <class T> void reaction(T*, const T*, const NodeInfo&) const {}
  template <class T> void storage(T* f, const T* u, const NodeInfo&) const { f[0] = u[0]; }
  void source(double*, const NodeInfo&) const {}
  template <class T> void breaction(T*, const T*, BNodeInfo&) const {}
};
// Benchmark workload 3: bipolar drift-diffusion in density variables (psi, n, p),
// scaled units (thermal voltage 1, intrinsic density 1).
//   flux_psi = lambda2 (psi_K - psi_L)
//   flux_n   = mu_n (B(psi_K - psi_L) n_K - B(psi_L - psi_K) n_L)
//   flux_p   = mu_p (B(psi_L - psi_K) p_K - B(psi_K - psi_L) p_L)
//   reaction_psi = n - p - C(x),  reaction_n = reaction_p = R,
//   R = (n p - 1) / (tau_p (n + 1) + tau_n (p + 1))         (SRH)
//   C = +doping for x < 0.5, -doping otherwise
//   ohmic contacts: region 4 (x = 0) at bias 0, region 2 (x = 1) at bias V*lambda_embed
// params: lambda2, mu_n, mu_p, tau_n, tau_p, doping, V
struct PhysBipolar : OBase {
  static const int NS = 3; double lambda2, mun, mup, taun, taup, doping, V;
  static const bool has_reaction = true, has_storage = false, has_source = false, has_breaction = true;
  double C(const double* x) const { return x[0] < 0.5 ? doping : -doping; }
  template <class T> void flux(T* f, const T* uK, const T* uL, const EdgeInfo&) const {
    f[0] = lambda2 * (uK[0] - uL[0]);
    T bp, bm;
    fbernoulli_pm(uK[0] - uL[0], bp, bm);
    f[1] = mun * (bp * uK[1] - bm * uL[1]);
    f[2] = mup * (bm * uK[2] - bp * uL[2]);
  }
  template <class T> void reaction(T* f, const T* u, const NodeInfo& n) const {
    f[0] = u[1] - u[2] - C(n.x);
    T r = (u[1] * u[2] - 1.0) / (taup * (u[1] + 1.0) + taun * (u[2] + 1.0));
    f[1] = r; f[2] = r;
  }
  template <class T> void storage(T*, const T*, const NodeInfo&) const {}
  void source(double*, const NodeInfo&) const {}
  template <class T> void breaction(T* f, const T* u, BNodeInfo& b) const {
    if (b.region != 2 && b.region != 4) return;
    double c = C(b.x);
    double nn = 0.5 * c + std::sqrt(0.25 * c * c + 1.0);
    double pp = 1.0 / nn;
    double bias = (b.region == 2) ? V * b.lambda : 0.0;
    double psi = std::asinh(0.5 * c) + bias;
    boundary_dirichlet(f, u, b, 0, b.region, psi);
    boundary_dirichlet(f, u, b, 1, b.region, nn);
    boundary_dirichlet(f, u, b, 2, b.region, pp);
  }
};
// Benchmark workload 4: two-species reaction-diffusion
//   flux_i = D_i (u_i,K - u_i,L);  f1 = k (u1 - u2^2), f2 = -k (u1 - u2^2)
//   Dirichlet: region 4 (x = 0): u1 = 1, u2 = 0;  region 2 (x = 1): u1 = 0, u2 = 1
// params: D1, D2, k
struct PhysRD2 : OBase {
  static const int NS = 2; double D1, D2, k;
  static const bool has_reaction = true, has_storage = false, has_source = false, has_breaction = true;
  template <class T> void flux(T* f, const T* uK, const T* uL, const EdgeInfo&) const {
    f[0] = D1 * (uK[0] - uL[0]);
    f[1] = D2 * (uK[1] - uL[1]);
  }
  template <class T> void reaction(T* f, const T* u, const NodeInfo&) const {
    T r = k * (u[0] - sq(u[1]));
    f[0] = r; f[1] = -r;
  }
  template <class T> void storage(T*, const T*, const NodeInfo&) const {}
  void source(double*, const NodeInfo&) const {}
  template <class T> void breaction(T* f, const T* u, BNodeInfo& b) const {
    boundary_dirichlet(f, u, b, 0, 4, 1.0);
    boundary_dirichlet(f, u, b, 1, 4, 0.0);
    boundary_dirichlet(f, u, b, 0, 2, 0.0);
    boundary_dirichlet(f, u, b, 1, 2, 1.0);
  }
};
// Benchmark workload 5: -div(kappa grad u) + exp(u) = f, u = 0 on every boundary;
// node data: kappa; edge coefficient = arithmetic mean of the two node values.
// params: f
struct PhysKappaExp : OBase {
  static const int NS = 1; double fsrc;
  static const bool has_reaction = true, has_storage = false, has_source = true, has_breaction = true;
  template <class T> void flux(T* f, const T* uK, const T* uL, const EdgeInfo& e) const {
    double kap = 0.5 * (e.ndataK[0] + e.ndataL[0]);
    f[0] = kap * (uK[0] - uL[0]);
  }
  template <class T> void reaction(T* f, const T* u, const NodeInfo&) const { f[0] = exp(u[0]); }
  template <class T> void storage(T*, const T*, const NodeInfo&) const {}
  void source(double* f, const NodeInfo&) const { f[0] = fsrc; }
  template <class T> void breaction(T* f, const T* u, BNodeInfo& b) const { boundary_dirichlet(f, u, b, 0, b.region, 0.0); }
};

// Heat equation with a conducting surface layer on boundary region breg, the
// single-species form of examples/Example311_HeatEquation_BoundaryDiffusion.jl
// (flux, bflux, breaction, bsource, bstorage, storage at :40-76 there):
// storage u, flux eps (uK - uL); on breg: bflux eps_s (uK - uL), bstorage c_s u,
// breaction k u^3, bsource q0 exp(-20 ((x-1/2)^2 + (y-1/2)^2)).
struct PhysSurfaceHeat : OBase {
  static const int NS = 1;
  static const bool has_reaction = false, has_storage = true, has_source = false, has_breaction = true;
  static const bool has_bflux = true, has_bstorage = true, has_bsource = true;
  double eps, eps_s, c_s, k, q0; int breg;
  template <class T> void flux(T* f, const T* uK, const T* uL, const EdgeInfo&) const { f[0] = eps * (uK[0] - uL[0]); }
  template <class T> void reaction(T*, const T*, const NodeInfo&) const {}
  template <class T> void storage(T* f, const T* u, const NodeInfo&) const { f[0] = u[0]; }
  void source(double*, const NodeInfo&) const {}
  template <class T> void breaction(T* f, const T* u, BNodeInfo& b) const { if (b.region == breg) f[0] = k * cube(u[0]); }
  template <class T> void bflux(T* f, const T* uK, const T* uL, const BEdgeInfo& e) const {
    if (e.region == breg) f[0] = eps_s * (uK[0] - uL[0]);
  }
  template <class T> void bstorage(T* f, const T* u, BNodeInfo& b) const { if (b.region == breg) f[0] = c_s * u[0]; }
  void bsource(double* f, BNodeInfo& b) const {
    if (b.region == breg) {
      double x1 = b.x[0] - 0.5, x2 = b.x[1] - 0.5;
      f[0] = q0 * std::exp(-20.0 * (x1 * x1 + x2 * x2));
    }
  }
};

// examples/Example230_BoundaryFlux.jl:58-165: species 1 is the 2D bulk species
// (flux2D!, reaction2D!, source2D!, :106-121), species 2 the boundary species
// on region breg (bflux!, breaction!, bsource!, :123-165; the switch at
// bnode.coord[2] <= 0.5).  The bulk callbacks of species 2 restate the 1D line
// problem (flux!, reaction!, source!, :58-71); its node-index switch of k1 and
// c1 at length_x_half is the switch at x <= 1/2 for the example's even n.
struct PhysBoundarySpecies : OBase {
  static const int NS = 2;
  static const bool has_reaction = true, has_storage = false, has_source = true, has_breaction = true;
  static const bool has_bflux = true, has_bstorage = false, has_bsource = true;
  double d, k, c, db, kmax, cmax; int breg;
  double kb(double s) const { return s <= 0.5 ? kmax : 0.0; }
  double cb(double s) const { return s <= 0.5 ? 0.0 : cmax; }
  template <class T> void flux(T* f, const T* uK, const T* uL, const EdgeInfo&) const {
    f[0] = d * (uK[0] - uL[0]);
    f[1] = db * (uK[1] - uL[1]);
  }
  template <class T> void reaction(T* f, const T* u, const NodeInfo& n) const {
    f[0] = k * u[0];
    f[1] = kb(n.x[0]) * u[1];
  }
  template <class T> void storage(T*, const T*, const NodeInfo&) const {}
  void source(double* f, const NodeInfo& n) const { f[0] = c; f[1] = cb(n.x[0]); }
  template <class T> void breaction(T* f, const T* u, BNodeInfo& b) const { if (b.region == breg) f[1] = kb(b.x[1]) * u[1]; }
  template <class T> void bflux(T* f, const T* uK, const T* uL, const BEdgeInfo& e) const {
    if (e.region == breg) f[1] = db * (uK[1] - uL[1]);
  }
  void bsource(double* f, BNodeInfo& b) const { if (b.region == breg) f[1] = cb(b.x[1]); }
};

// examples/DevEx002_EdgeReaction.jl:49-104 (case :compare_max): storage u, flux
// u_K - u_L, u = 0 on boundary regions 1-6 (bcondition!), and the unit source as
// reaction! (mode 0: -1), edgereaction! (mode 1: -meas(edge)^2 / (2 dim)) or
// edgereaction2! (mode 2: -(phi_K - phi_L)^2 / 2, phi the first coordinate).
struct PhysEdgeReaction : OBase {
  static const int NS = 1;
  static const bool has_reaction = true, has_storage = true, has_source = false, has_breaction = true;
  static const bool has_edgereaction = true;
  int mode = 0, dim = 1;
  template <class T> void flux(T* f, const T* uK, const T* uL, const EdgeInfo&) const { f[0] = uK[0] - uL[0]; }
  template <class T> void storage(T* f, const T* u, const NodeInfo&) const { f[0] = u[0]; }
  template <class T> void reaction(T* f, const T* u, const NodeInfo&) const { if (mode == 0) f[0] = u[0] * 0.0 + (-1.0); }
  void source(double*, const NodeInfo&) const {}
  template <class T> void edgereaction(T* f, const T* uK, const T*, const EdgeInfo& e) const {
    if (mode == 1) {
      double s = 0.0;
      for (int k = 0; k < dim; ++k) s += (e.xK[k] - e.xL[k]) * (e.xK[k] - e.xL[k]);
      double h = std::sqrt(s);
      f[0] = uK[0] * 0.0 + (-1.0 * (h * h) / (2 * dim));
    } else if (mode == 2) {
      double dp = e.xK[0] - e.xL[0];
      f[0] = uK[0] * 0.0 + (-dp * dp / 2);
    }
  }
  template <class T> void breaction(T* f, const T* u, BNodeInfo& b) const {
    for (int r = 1; r <= 6; ++r) boundary_dirichlet(f, u, b, 0, r, 0.0);
  }
};

// examples/Example206_JouleHeat.jl:63-92: storage!, flux!, jouleheat! (the edge
// reaction) and bcondition! (boundary_dirichlet! for phi on regions 1, 2;
// boundary_robin! y += 0.5 T - T0 for T on regions 1-4, src/vfvm_physics.jl:551).
// kappa is evaluated at y[iT], still 0 where the example reads it.
struct PhysJouleHeat : OBase {
  static const int NS = 2;
  static const bool has_reaction = false, has_storage = true, has_source = false, has_breaction = true;
  static const bool has_edgereaction = true;
  double kappa0, alpha, T0, lam, c;
  template <class T> T kappa(const T& t) const { return kappa0 * exp(alpha * (t - T0)); }
  template <class T> void flux(T* f, const T* uK, const T* uL, const EdgeInfo&) const {
    f[0] = kappa(f[1]) * (uK[0] - uL[0]);
    f[1] = lam * (uK[1] - uL[1]);
  }
  template <class T> void edgereaction(T* f, const T* uK, const T* uL, const EdgeInfo&) const {
    f[1] = kappa(f[1]) * (-1.0) * (uK[0] - uL[0]) * (uK[0] - uL[0]);  // -kappa * d * d
  }
  template <class T> void reaction(T*, const T*, const NodeInfo&) const {}
  template <class T> void storage(T* f, const T* u, const NodeInfo&) const { f[1] = c * u[1]; }
  void source(double*, const NodeInfo&) const {}
  template <class T> void breaction(T* f, const T* u, BNodeInfo& b) const {
    boundary_dirichlet(f, u, b, 0, 1, -10.0);
    boundary_dirichlet(f, u, b, 0, 2, 10.0);
    for (int r = 1; r <= 4; ++r)
      if (b.region == r) f[1] = f[1] + (0.5 * u[1] - T0);
  }
};

// examples/Example161_BipolarDriftDiffusionCurrent.jl:85-151: quasi-Fermi
// potentials phi_n, phi_p and the electrostatic potential psi (species 1-3),
// densities n = exp(zn (phi_n - psi + En)), p = exp(zp (phi_p - psi + Ep)) with
// zn = -1, zp = 1; doping Cn / Ca / -Cp in cell regions 1 / 2 / 3; Scharfetter-
// Gummel fluxes through fbernoulli_pm; the bias scanProtocol(t) (:54-66) on
// boundary region 2.
// params: Cn, Cp, Ca, En, Ep, mun, mup, lambda, tPrecond, tRamp, tExt, Vprecond, VExt, DirichletVal
struct PhysEx161 : OBase {
  static const int NS = 3;
  static const bool has_reaction = true, has_storage = true, has_source = false, has_breaction = true;
  double Cn, Cp, Ca, En, Ep, mun, mup, lambda, tPrecond, tRamp, tExt, Vprecond, VExt, DirichletVal;
  static constexpr double zn = -1.0, zp = 1.0;
  double scan(double t) const {
    const double tEnd = tPrecond + tRamp + tExt;
    if (0.0 <= t && t <= tPrecond) return Vprecond;
    if (tPrecond <= t && t <= tPrecond + tRamp) return Vprecond - (Vprecond - VExt) / tRamp * (t - tPrecond);
    if (tPrecond + tRamp <= t && t <= tEnd) return VExt;
    return 0.0;
  }
  template <class T> void reaction(T* f, const T* u, const NodeInfo& n) const {
    T nn = exp(zn * (u[0] - u[2] + En));
    T np = exp(zp * (u[1] - u[2] + Ep));
    double C = n.region == 1 ? Cn : (n.region == 2 ? Ca : (n.region == 3 ? -Cp : 0.0));
    f[2] = -(C + zn * nn + zp * np);
    const double r0 = 1.0;
    T recomb = (r0 + 1.0 / (nn + np)) * (nn * np * (1.0 - exp(u[0] - u[1])));
    f[0] = zn * recomb;
    f[1] = zp * recomb;
  }
  template <class T> void flux(T* f, const T* uK, const T* uL, const EdgeInfo&) const {
    f[2] = -(lambda * lambda) * (uL[2] - uK[2]);
    T bp, bm;
    fbernoulli_pm(-(uL[2] - uK[2]), bp, bm);
    T nn1 = exp(zn * (uK[0] - uK[2] + En)), np1 = exp(zp * (uK[1] - uK[2] + Ep));
    T nn2 = exp(zn * (uL[0] - uL[2] + En)), np2 = exp(zp * (uL[1] - uL[2] + Ep));
    f[0] = -zn * mun * (bm * nn2 - bp * nn1);
    f[1] = -zp * mup * (bp * np2 - bm * np1);
  }
  template <class T> void storage(T* f, const T* u, const NodeInfo&) const {
    f[0] = zn * exp(zn * (u[0] - u[2] + En));
    f[1] = zp * exp(zp * (u[1] - u[2] + Ep));
  }
  void source(double*, const NodeInfo&) const {}
  template <class T> void breaction(T* f, const T* u, BNodeInfo& b) const {
    const double s = scan(b.time);
    boundary_dirichlet(f, u, b, 0, 1, 0.0);
    boundary_dirichlet(f, u, b, 1, 1, 0.0);
    boundary_dirichlet(f, u, b, 2, 1, 0.5 * (En + Ep) + std::asinh(Cn / (2 * std::sqrt(std::exp(-(En - Ep))))));
    boundary_dirichlet(f, u, b, 0, 2, DirichletVal + s);
    boundary_dirichlet(f, u, b, 1, 2, DirichletVal + s);
    boundary_dirichlet(f, u, b, 2, 2,
                       0.5 * (En + Ep) + std::asinh(-Cp / (2 * std::sqrt(std::exp(-(En - Ep))))) + DirichletVal + s);
  }
};

// examples/Example430_ParameterDerivativesStationary.jl:146-166 (runh, fluxh!,
// rh!, bch!): flux (1 + p)(u_K^2 - u_L^2), reaction p u^5, u = 0 on boundary
// region 1 and u = p on region 3, p = parameters(u)[1].  PT = double for the
// assembly, Dual<1> (seeded) for the parameter derivatives.
template <class PT>
struct PhysEx430T : OBase {
  static const int NS = 1;
  static const bool has_reaction = true, has_storage = false, has_source = false, has_breaction = true;
  PT p;
  template <class T> void flux(T* f, const T* uK, const T* uL, const EdgeInfo&) const {
    f[0] = (1.0 + p) * (uK[0] * uK[0] - uL[0] * uL[0]);
  }
  template <class T> void reaction(T* f, const T* u, const NodeInfo&) const {
    T u2 = u[0] * u[0];
    f[0] = p * (u2 * u2 * u[0]);
  }
  template <class T> void storage(T*, const T*, const NodeInfo&) const {}
  void source(double*, const NodeInfo&) const {}
  template <class T> void breaction(T* f, const T* u, BNodeInfo& b) const {
    boundary_dirichlet(f, u, b, 0, 1, 0.0);
    boundary_dirichlet(f, u, b, 0, 3, p);
  }
};

// pluto-examples/outflow.jl: darcyvelo, flux, bcondition and boutflow of
// FlowTransportData (p species 1, c species 2); outflowboundaries = [G_out].
struct PhysOutflow : OBase {
  static const int NS = 2;
  static const bool has_reaction = false, has_storage = false, has_source = false, has_breaction = true;
  static const bool has_boutflow = true;
  double k, v_in, c_in, D; int gin, gout;
  bool outflow_region(int reg) const { return reg == gout; }
  template <class T> T darcyvelo(const T* uK, const T* uL) const { return k * (uK[0] - uL[0]); }
  template <class T> void flux(T* f, const T* uK, const T* uL, const EdgeInfo&) const {
    T vh = darcyvelo(uK, uL);
    f[0] = vh;
    T bp, bm;
    fbernoulli_pm(vh / D, bp, bm);
    f[1] = D * (bm * uK[1] - bp * uL[1]);
  }
  template <class T> void reaction(T*, const T*, const NodeInfo&) const {}
  template <class T> void storage(T*, const T*, const NodeInfo&) const {}
  void source(double*, const NodeInfo&) const {}
  template <class T> void breaction(T* f, const T* u, BNodeInfo& b) const {
    if (b.region == gin) f[0] = f[0] - v_in;  // boundary_neumann!, src/vfvm_physics.jl:532
    boundary_dirichlet(f, u, b, 0, gout, 0.0);
    boundary_dirichlet(f, u, b, 1, gin, c_in);
  }
  template <class T> void boutflow(T* f, const T* uK, const T* uL, const EdgeInfo& e) const {
    f[1] = -(darcyvelo(uK, uL) * (e.outflownode == 1 ? uK[1] : uL[1]));
  }
};

// examples/Example210_NonlinearPoisson2D_Reaction.jl:24-46: two species,
// flux eps (u_K - u_L) each, reaction k (u1 - u2) / k (u2 - u1), source
// exp(-20 ((x-1/2)^2 + (y-1/2)^2)) for species 1, storage u.
struct PhysEx210 : OBase {
  static const int NS = 2;
  static const bool has_reaction = true, has_storage = true, has_source = true, has_breaction = false;
  double eps, k;
  template <class T> void flux(T* f, const T* uK, const T* uL, const EdgeInfo&) const {
    f[0] = eps * (uK[0] - uL[0]);
    f[1] = eps * (uK[1] - uL[1]);
  }
  template <class T> void reaction(T* f, const T* u, const NodeInfo&) const {
    f[0] = k * (u[0] - u[1]);
    f[1] = k * (u[1] - u[0]);
  }
  template <class T> void storage(T* f, const T* u, const NodeInfo&) const { f[0] = u[0]; f[1] = u[1]; }
  void source(double* f, const NodeInfo& n) const {
    const double x1 = n.x[0] - 0.5, x2 = n.x[1] - 0.5;
    f[0] = std::exp(-20.0 * (x1 * x1 + x2 * x2));
  }
  template <class T> void breaction(T*, const T*, BNodeInfo&) const {}
};

// examples/Example102_StationaryConvectionDiffusion1D.jl:40-78: the example's
// exponential (mode 0), upwind (1) and central (2) fluxes with vh =
// project(edge, v) (src/vfvm_geometryitems.jl:634-640) and its own
// bernoulli(x) = x / (exp(x) - 1), 1 where |x| < nextfloat(eps).
struct PhysEx102 : OBase {
  static const int NS = 1;
  static const bool has_reaction = false, has_storage = false, has_source = false, has_breaction = false;
  double D, v; int mode;
  static double bernoulli(double x) {
    if (std::fabs(x) < std::nextafter(std::numeric_limits<double>::epsilon(), 1.0)) return 1.0;
    return x / (std::exp(x) - 1.0);
  }
  template <class T> void flux(T* f, const T* uK, const T* uL, const EdgeInfo& e) const {
    const double vh = (e.xL[0] - e.xK[0]) * v;
    if (mode == 0) {
      const double Bplus = D * bernoulli(vh / D), Bminus = D * bernoulli(-vh / D);
      f[0] = Bminus * uK[0] - Bplus * uL[0];
    } else if (mode == 1) {
      const T fdiff = D * (uK[0] - uL[0]);
      f[0] = vh > 0 ? fdiff + vh * uK[0] : fdiff + vh * uL[0];
    } else {
      f[0] = D * (uK[0] - uL[0]) + vh * (uK[0] + uL[0]) / 2.0;
    }
  }
  template <class T> void reaction(T*, const T*, const NodeInfo&) const {}
  template <class T> void storage(T*, const T*, const NodeInfo&) const {}
  void source(double*, const NodeInfo&) const {}
  template <class T> void breaction(T*, const T*, BNodeInfo&) const {}
};

// examples/Example107_NonlinearStorage1D.jl:44-64: flux u_K - u_L, storage (eps + u)^(1/m).
struct PhysEx107 : OBase {
  static const int NS = 1;
  static const bool has_reaction = false, has_storage = true, has_source = false, has_breaction = false;
  double m, eps;
  template <class T> void flux(T* f, const T* uK, const T* uL, const EdgeInfo&) const { f[0] = uK[0] - uL[0]; }
  template <class T> void storage(T* f, const T* u, const NodeInfo&) const { f[0] = pow(eps + u[0], 1.0 / m); }
  template <class T> void reaction(T*, const T*, const NodeInfo&) const {}
  void source(double*, const NodeInfo&) const {}
  template <class T> void breaction(T*, const T*, BNodeInfo&) const {}
};

// examples/Example115_HeterogeneousCatalysis1D.jl:113-176: A, B in the bulk,
// C on boundary region iCat; R_AC, R_BC mass-action rates with the free-site
// factor (1 - u_C); breaction S R_AC, S R_BC, -R_BC - R_AC; bstorage u_C.
struct PhysEx115 : OBase {
  static const int NS = 3;
  static const bool has_reaction = false, has_storage = true, has_source = true, has_breaction = true;
  static const bool has_bstorage = true;
  double D_A, D_B, kp_AC, km_AC, kp_BC, km_BC, S; int iCat;
  template <class T> T R_AC(const T& uA, const T& uC) const { return kp_AC * uA * (1.0 - uC) - km_AC * uC; }
  template <class T> T R_BC(const T& uB, const T& uC) const { return kp_BC * uB * (1.0 - uC) - km_BC * uC; }
  template <class T> void flux(T* f, const T* uK, const T* uL, const EdgeInfo&) const {
    f[0] = D_A * (uK[0] - uL[0]);
    f[1] = D_B * (uK[1] - uL[1]);
  }
  template <class T> void storage(T* f, const T* u, const NodeInfo&) const { f[0] = u[0]; f[1] = u[1]; }
  template <class T> void reaction(T*, const T*, const NodeInfo&) const {}
  void source(double* f, const NodeInfo& n) const { double x1 = n.x[0] - 0.5; f[0] = std::exp(-100.0 * (x1 * x1)); }
  template <class T> void breaction(T* f, const T* u, BNodeInfo& b) const {
    if (b.region == iCat) {
      f[0] = S * R_AC(u[0], u[2]);
      f[1] = S * R_BC(u[1], u[2]);
      f[2] = -R_BC(u[1], u[2]) - R_AC(u[0], u[2]);
    }
  }
  template <class T> void bstorage(T* f, const T* u, BNodeInfo& b) const { if (b.region == iCat) f[2] = u[2]; }
};

// examples/Example215_NonlinearPoisson2D_BoundaryReaction.jl:27-50: two
// species, flux eps, storage u, breaction k_react (u1 - u2) / (u2 - u1) on region 2.
struct PhysEx215 : OBase {
  static const int NS = 2;
  static const bool has_reaction = false, has_storage = true, has_source = false, has_breaction = true;
  double eps, k_react;
  template <class T> void flux(T* f, const T* uK, const T* uL, const EdgeInfo&) const {
    f[0] = eps * (uK[0] - uL[0]);
    f[1] = eps * (uK[1] - uL[1]);
  }
  template <class T> void storage(T* f, const T* u, const NodeInfo&) const { f[0] = u[0]; f[1] = u[1]; }
  template <class T> void reaction(T*, const T*, const NodeInfo&) const {}
  void source(double*, const NodeInfo&) const {}
  template <class T> void breaction(T* f, const T* u, BNodeInfo& b) const {
    if (b.region == 2) {
      f[0] = k_react * (u[0] - u[1]);
      f[1] = k_react * (u[1] - u[0]);
    }
  }
};

// examples/Example220_NonlinearPoisson2D_BoundarySpecies.jl:23-57: bulk
// species 1, 2 and boundary species 3 on region 2 (bstorage u3, breaction
// k (u1 - u3), k (u3 - u1) + k (u3 - u2), k (u2 - u3)); source for species 1.
struct PhysEx220 : OBase {
  static const int NS = 3;
  static const bool has_reaction = false, has_storage = true, has_source = true, has_breaction = true;
  static const bool has_bstorage = true;
  double k, eps;
  template <class T> void flux(T* f, const T* uK, const T* uL, const EdgeInfo&) const {
    f[0] = eps * (uK[0] - uL[0]);
    f[1] = eps * (uK[1] - uL[1]);
  }
  template <class T> void storage(T* f, const T* u, const NodeInfo&) const { f[0] = u[0]; f[1] = u[1]; }
  template <class T> void reaction(T*, const T*, const NodeInfo&) const {}
  void source(double* f, const NodeInfo& n) const {
    double x1 = n.x[0] - 0.5, x2 = n.x[1] - 0.5;
    f[0] = std::exp(-20.0 * (x1 * x1 + x2 * x2));
  }
  template <class T> void breaction(T* f, const T* u, BNodeInfo& b) const {
    if (b.region == 2) {
      f[0] = k * (u[0] - u[2]);
      f[2] = k * (u[2] - u[0]) + k * (u[2] - u[1]);
      f[1] = k * (u[1] - u[2]);
    }
  }
  template <class T> void bstorage(T* f, const T* u, BNodeInfo& b) const { if (b.region == 2) f[2] = u[2]; }
};

// examples/Example203_CoordinateSystems.jl: flux u_K - u_L (:14-17) and the
// constant source of each case (1.0 or 0.0).
struct PhysEx203 : OBase {
  static const int NS = 1;
  static const bool has_reaction = false, has_storage = false, has_source = true, has_breaction = false;
  double f0;
  template <class T> void flux(T* f, const T* uK, const T* uL, const EdgeInfo&) const { f[0] = uK[0] - uL[0]; }
  template <class T> void reaction(T*, const T*, const NodeInfo&) const {}
  template <class T> void storage(T*, const T*, const NodeInfo&) const {}
  void source(double* f, const NodeInfo&) const { f[0] = f0; }
  template <class T> void breaction(T*, const T*, BNodeInfo&) const {}
};

// The physics of TestFunctionFactory (src/vfvm_testfunctions.jl:38-50): flux
// u_K - u_L, storage u; Dirichlet data through the legacy boundary factors.
struct PhysTestFunction : OBase {
  static const int NS = 1;
  static const bool has_reaction = false, has_storage = true, has_source = false, has_breaction = false;
  template <class T> void flux(T* f, const T* uK, const T* uL, const EdgeInfo&) const { f[0] = uK[0] - uL[0]; }
  template <class T> void storage(T* f, const T* u, const NodeInfo&) const { f[0] = u[0]; }
  template <class T> void reaction(T*, const T*, const NodeInfo&) const {}
  void source(double*, const NodeInfo&) const {}
  template <class T> void breaction(T*, const T*, BNodeInfo&) const {}
};

// ---------------------------------------------------------------- system
struct Oracle {
  int dim = 0, N = 0, ncells = 0, nbf = 0, ns = 1, phys = 0, nregions = 1, nbregions = 0, nnd = 0;
  int csys = 0;                    // coordinate system: 0 Cartesian, 1 Polar1D, 2 Spherical1D, 3 Cylindrical2D
  std::vector<double> coord;       // dim x N
  std::vector<int> cellnodes, cellregions, bfacenodes, bfaceregions;
  std::vector<double> params, ndata;
  std::vector<double> bfactors, bvalues;  // legacy BC: ns x nbregions
  bool has_legacy = false;
  // edges
  int E = 0;
  std::vector<int> edgenodes;      // 2 x E
  std::vector<int> celledges;      // nedges_per_cell x ncells
  // edgewise factors: per node/edge, list of (region, fac) sorted by region
  std::vector<std::vector<std::pair<int, double>>> nodefac, edgefac;
  std::vector<double> bfacenodefac;  // dim x nbf  (nodes per bface = dim)
  // candidate CSR over dofs
  std::vector<int64_t> rowptr;
  std::vector<int> colind;
  std::vector<double> vals;
  std::vector<uint8_t> present;
  int nerr = 0;
  // assembly = :cellwise (the reference's default, src/vfvm_system.jl:220):
  // node and edge terms per cell with the cell's own factors
  bool cellwise = false;
  // species restricted to regions (enable_species!, enable_boundary_species!,
  // src/vfvm_system.jl:433-513): species bit masks per cell region and per node
  // (node_dof); masked = false: every species on every node
  bool masked = false;
  std::vector<unsigned> reg_spec, node_spec;
  // outflow nodes (outflownoderegions, src/vfvm_system.jl:660-673): nodes of the
  // boundary faces in outflowboundaries
  std::vector<uint8_t> outflow;
};

inline int nn_bface(int dim) { return dim; }  // nodes per boundary face: Vertex0D 1, Edge1D 2, Triangle2D 3

// local_celledgenodes: Edge1D (1,2); Triangle2D edges opposite node 1,2,3;
// Tetrahedron3D [1 2; 1 3; 1 4; 2 3; 2 4; 3 4] (0-based below)
const int tri_en[3][2] = {{1, 2}, {2, 0}, {0, 1}};
const int tet_en[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};

const double kPi = 3.141592653589793;  // Julia's pi as a Float64

// tricircumcenter! (ExtendableGrids, an unvendored dependency): the circumcenter
// of the triangle a, b, c by the published formula relative to a (Shewchuk).
void tricircumcenter(double* cc, const double* a, const double* b, const double* c) {
  double xba = b[0] - a[0], yba = b[1] - a[1], xca = c[0] - a[0], yca = c[1] - a[1];
  double balength = xba * xba + yba * yba, calength = xca * xca + yca * yca;
  double denominator = 0.5 / (xba * yca - yba * xca);
  cc[0] = a[0] + (yca * balength - yba * calength) * denominator;
  cc[1] = a[1] + (xba * calength - xca * balength) * denominator;
}

// cellfactors!, src/vfvm_formfactors.jl:12-23 (Edge1D), :25-62 (Edge1D Polar1D,
// Spherical1D), :64-100 (Triangle2D), :102-161 (Triangle2D Cylindrical2D),
// :163-235 (Tetrahedron3D)
void cellfactors(int dim, int csys, const double* coord, const int* n, double* npar, double* epar) {
  if (dim == 1 && (csys == 1 || csys == 2)) {
    double r0 = coord[n[0]], r1 = coord[n[1]];
    if (r1 < r0) { r0 = coord[n[1]]; r1 = coord[n[0]]; }
    double rhalf = 0.5 * (r1 + r0);
    if (csys == 1) {
      npar[0] = kPi * (rhalf * rhalf - r0 * r0);
      npar[1] = kPi * (r1 * r1 - rhalf * rhalf);
      epar[0] = 2.0 * kPi * rhalf / (r1 - r0);
    } else {
      npar[0] = kPi * (rhalf * rhalf * rhalf - r0 * r0 * r0) * 4.0 / 3.0;
      npar[1] = kPi * (r1 * r1 * r1 - rhalf * rhalf * rhalf) * 4.0 / 3.0;
      epar[0] = 4.0 * kPi * (rhalf * rhalf) / (r1 - r0);
    }
  } else if (dim == 2 && csys == 3) {
    double V[2][3];
    for (int i = 0; i < 3; ++i)
      for (int c = 0; c < 2; ++c) V[c][i] = coord[c + 2 * n[tri_en[i][0]]] - coord[c + 2 * n[tri_en[i][1]]];
    double det = V[0][2] * V[1][1] - V[0][1] * V[1][2];
    double vol = std::fabs(0.5 * det), ivol = 1.0 / vol;
    double dd[3];
    for (int i = 0; i < 3; ++i) dd[i] = V[0][i] * V[0][i] + V[1][i] * V[1][i];
    double emid[3];
    for (int i = 0; i < 3; ++i) emid[i] = 0.5 * (coord[2 * n[tri_en[i][0]]] + coord[2 * n[tri_en[i][1]]]);
    double cc[2];
    tricircumcenter(cc, coord + 2 * n[0], coord + 2 * n[1], coord + 2 * n[2]);
    double rcc = cc[0];
    epar[0] = (dd[1] + dd[2] - dd[0]) * 0.125 * ivol;
    epar[1] = (dd[2] + dd[0] - dd[1]) * 0.125 * ivol;
    epar[2] = (dd[0] + dd[1] - dd[2]) * 0.125 * ivol;
    npar[0] = npar[1] = npar[2] = 0.0;
    for (int i = 0; i < 3; ++i) {
      double r1 = coord[2 * n[tri_en[i][0]]], r2 = coord[2 * n[tri_en[i][1]]];
      double cylfac1 = 2 * kPi * (r1 + rcc + emid[i]) / 3;
      double cylfac2 = 2 * kPi * (r2 + rcc + emid[i]) / 3;
      npar[tri_en[i][0]] += epar[i] * dd[i] * 0.25 * cylfac1;
      npar[tri_en[i][1]] += epar[i] * dd[i] * 0.25 * cylfac2;
    }
    for (int i = 0; i < 3; ++i) {
      double rmid = (rcc + emid[i]) / 2;
      epar[i] *= 2 * kPi * rmid;
    }
  } else if (dim == 1) {
    double d = std::fabs(coord[n[1]] - coord[n[0]]);
    npar[0] = d / 2; npar[1] = d / 2; epar[0] = 1 / d;
  } else if (dim == 2) {
    double V[2][3];
    for (int i = 0; i < 3; ++i)
      for (int c = 0; c < 2; ++c) V[c][i] = coord[c + 2 * n[tri_en[i][0]]] - coord[c + 2 * n[tri_en[i][1]]];
    double det = V[0][2] * V[1][1] - V[0][1] * V[1][2];
    double vol = std::fabs(0.5 * det), ivol = 1.0 / vol;
    double dd[3];
    for (int i = 0; i < 3; ++i) dd[i] = V[0][i] * V[0][i] + V[1][i] * V[1][i];
    epar[0] = (dd[1] + dd[2] - dd[0]) * 0.125 * ivol;
    epar[1] = (dd[2] + dd[0] - dd[1]) * 0.125 * ivol;
    epar[2] = (dd[0] + dd[1] - dd[2]) * 0.125 * ivol;
    npar[0] = npar[1] = npar[2] = 0.0;
    for (int i = 0; i < 3; ++i) {
      npar[tri_en[i][0]] += epar[i] * dd[i] * 0.25;
      npar[tri_en[i][1]] += epar[i] * dd[i] * 0.25;
    }
  } else {
    const int pi1[4] = {4, 5, 4, 0}, pi2[4] = {5, 2, 0, 3}, pi3[4] = {3, 1, 2, 1};
    const int po1[4] = {1, 0, 1, 5}, po2[4] = {0, 3, 5, 2}, po3[4] = {2, 4, 3, 4};
    double dd[6];
    for (int i = 0; i < 6; ++i) {
      int p1 = n[tet_en[i][0]], p2 = n[tet_en[i][1]];
      double dx = coord[3 * p1] - coord[3 * p2], dy = coord[3 * p1 + 1] - coord[3 * p2 + 1], dz = coord[3 * p1 + 2] - coord[3 * p2 + 2];
      dd[i] = dx * dx + dy * dy + dz * dz;
    }
    for (int i = 0; i < 6; ++i) epar[i] = 0;
    const double* c0 = coord + 3 * n[0];
    double x1 = coord[3 * n[1]] - c0[0], y1 = coord[3 * n[1] + 1] - c0[1], z1 = coord[3 * n[1] + 2] - c0[2];
    double x2 = coord[3 * n[2]] - c0[0], y2 = coord[3 * n[2] + 1] - c0[1], z2 = coord[3 * n[2] + 2] - c0[2];
    double x3 = coord[3 * n[3]] - c0[0], y3 = coord[3 * n[3] + 1] - c0[1], z3 = coord[3 * n[3] + 2] - c0[2];
    double det = (x1 * (y2 * z3 - y3 * z2) + x2 * (y3 * z1 - y1 * z3) + x3 * (y1 * z2 - y2 * z1));
    if (det < 0) det = -det;
    double vol = det / 6;
    double vv = 96 * 6 * vol;
    for (int i = 0; i < 4; ++i) {
      npar[i] = 0.0;
      int i1 = pi1[i], i2 = pi2[i], i3 = pi3[i];
      double h1 = dd[i1] * (dd[i2] + dd[i3] - dd[i1]);
      double h2 = dd[i2] * (dd[i3] + dd[i1] - dd[i2]);
      double h3 = dd[i3] * (dd[i1] + dd[i2] - dd[i3]);
      double df = h1 + h2 + h3;
      double vf = (h1 * dd[po1[i]] + h2 * dd[po2[i]] + h3 * dd[po3[i]] - 2 * dd[i1] * dd[i2] * dd[i3]) / (vv * df);
      epar[i1] += h1 * vf;
      epar[i2] += h2 * vf;
      epar[i3] += h3 * vf;
    }
    for (int i = 0; i < 6; ++i) {
      npar[tet_en[i][0]] += epar[i];
      npar[tet_en[i][1]] += epar[i];
      epar[i] = 6 * epar[i] / dd[i];
    }
  }
}

// bfacefactors!, src/vfvm_formfactors.jl:244-247 (Vertex0D), :249-261 (Vertex0D
// Polar1D, Spherical1D), :263-274 (Edge1D), :276-291 (Edge1D Cylindrical2D: no
// edge parameter, which stays 0 as in the reference's zeroed array), :293-332 (Triangle2D)
void bfacefactors(int dim, int csys, const double* coord, const int* n, double* npar, double* epar) {
  if (dim == 1) {
    double r = coord[n[0]];
    npar[0] = csys == 1 ? 2 * kPi * r : csys == 2 ? 4 * kPi * (r * r) : 1.0;
  } else if (dim == 2 && csys == 3) {
    double r1 = coord[2 * n[0]], r2 = coord[2 * n[1]], z1 = coord[2 * n[0] + 1], z2 = coord[2 * n[1] + 1];
    double dr = r1 - r2, rmid = (r1 + r2) / 2, dz = z1 - z2;
    double l = std::sqrt(dr * dr + dz * dz);
    npar[0] = kPi * (r1 + rmid) * l / 2;
    npar[1] = kPi * (r2 + rmid) * l / 2;
    epar[0] = 0.0;
  } else if (dim == 2) {
    double dx = coord[2 * n[0]] - coord[2 * n[1]], dy = coord[2 * n[0] + 1] - coord[2 * n[1] + 1];
    double d = std::sqrt(dx * dx + dy * dy);
    npar[0] = d / 2; npar[1] = d / 2; epar[0] = 1 / d;
  } else {
    double e[3] = {0, 0, 0};
    for (int j = 0; j < 3; ++j) {
      double d = coord[j + 3 * n[tri_en[0][0]]] - coord[j + 3 * n[tri_en[0][1]]]; e[0] += d * d;
      d = coord[j + 3 * n[tri_en[1][0]]] - coord[j + 3 * n[tri_en[1][1]]]; e[1] += d * d;
      d = coord[j + 3 * n[tri_en[2][0]]] - coord[j + 3 * n[tri_en[2][1]]]; e[2] += d * d;
    }
    double dd[3] = {e[0], e[1], e[2]};
    e[0] = (dd[1] + dd[2] - dd[0]) * dd[0];
    e[1] = (dd[2] + dd[0] - dd[1]) * dd[1];
    e[2] = (dd[0] + dd[1] - dd[2]) * dd[2];
    double vol = std::sqrt(e[0] + e[1] + e[2]) * 0.25;
    double d = 1.0 / (8 * vol);
    npar[0] = npar[1] = npar[2] = 0.0;
    for (int i = 0; i < 3; ++i) {
      npar[tri_en[i][0]] += e[i] * d * 0.25;
      npar[tri_en[i][1]] += e[i] * d * 0.25;
    }
    epar[0] = e[0] * d / dd[0];
    epar[1] = e[1] * d / dd[1];
    epar[2] = e[2] * d / dd[2];
  }
}

void add_factor(std::vector<std::pair<int, double>>& v, int reg, double f) {
  for (auto& p : v)
    if (p.first == reg) { p.second += f; return; }
  v.emplace_back(reg, f);
  std::sort(v.begin(), v.end(), [](const std::pair<int, double>& a, const std::pair<int, double>& b) { return a.first < b.first; });
}

// update_grid_edgewise!, src/vfvm_system.jl:690-755
void setup(Oracle& o) {
  const int d = o.dim;
  const int nen = d == 1 ? 1 : (d == 2 ? 3 : 6);
  const int nnc = d + 1;
  // global edges (lo, hi), numbered lexicographically
  std::vector<int64_t> keys;
  keys.reserve((size_t)o.ncells * nen);
  auto ledge = [&](int i, int k) -> int { return d == 1 ? k : (d == 2 ? tri_en[i][k] : tet_en[i][k]); };
  for (int c = 0; c < o.ncells; ++c)
    for (int i = 0; i < nen; ++i) {
      int a = o.cellnodes[ledge(i, 0) + nnc * c], b = o.cellnodes[ledge(i, 1) + nnc * c];
      if (a > b) std::swap(a, b);
      keys.push_back((int64_t)a * o.N + b);
    }
  std::vector<int64_t> uk = keys;
  std::sort(uk.begin(), uk.end());
  uk.erase(std::unique(uk.begin(), uk.end()), uk.end());
  o.E = (int)uk.size();
  o.edgenodes.resize(2 * o.E);
  for (int e = 0; e < o.E; ++e) { o.edgenodes[2 * e] = (int)(uk[e] / o.N); o.edgenodes[2 * e + 1] = (int)(uk[e] % o.N); }
  o.celledges.resize((size_t)nen * o.ncells);
  for (size_t i = 0; i < keys.size(); ++i) o.celledges[i] = (int)(std::lower_bound(uk.begin(), uk.end(), keys[i]) - uk.begin());
  // factors
  o.nodefac.assign(o.N, {});
  o.edgefac.assign(o.E, {});
  double npar[4], epar[6];
  for (int c = 0; c < o.ncells; ++c) {
    cellfactors(d, o.csys, o.coord.data(), &o.cellnodes[nnc * c], npar, epar);
    int ireg = o.cellregions[c];
    for (int i = 0; i < nnc; ++i) add_factor(o.nodefac[o.cellnodes[i + nnc * c]], ireg, npar[i]);
    for (int i = 0; i < nen; ++i) add_factor(o.edgefac[o.celledges[i + nen * c]], ireg, epar[i]);
  }
  const int nbn = nn_bface(d);
  o.bfacenodefac.assign((size_t)nbn * o.nbf, 0.0);
  for (int b = 0; b < o.nbf; ++b) bfacefactors(d, o.csys, o.coord.data(), &o.bfacenodes[nbn * b], &o.bfacenodefac[nbn * b], epar);
  // candidate CSR: rows (K,i), columns (M,j) for M in {K} u neighbours(K)
  std::vector<std::vector<int>> nb(o.N);
  for (int e = 0; e < o.E; ++e) { nb[o.edgenodes[2 * e]].push_back(o.edgenodes[2 * e + 1]); nb[o.edgenodes[2 * e + 1]].push_back(o.edgenodes[2 * e]); }
  const int ns = o.ns;
  const int64_t n = (int64_t)o.N * ns;
  o.rowptr.assign(n + 1, 0);
  o.colind.clear();
  for (int K = 0; K < o.N; ++K) {
    nb[K].push_back(K);
    std::sort(nb[K].begin(), nb[K].end());
    for (int i = 0; i < ns; ++i) {
      for (int M : nb[K])
        for (int j = 0; j < ns; ++j) o.colind.push_back(M * ns + j);
      o.rowptr[(int64_t)K * ns + i + 1] = (int64_t)o.colind.size();
    }
  }
  o.vals.assign(o.colind.size(), 0.0);
  o.present.assign(o.colind.size(), 0);
}

// _addnz, src/vfvm_assembly.jl:21-28
inline void addnz(Oracle& o, int64_t i, int64_t j, double v, double fac) {
  if (std::isnan(v)) { o.nerr++; return; }
  if (v != 0.0) {
    int64_t lo = o.rowptr[i], hi = o.rowptr[i + 1];
    const int* p = std::lower_bound(o.colind.data() + lo, o.colind.data() + hi, (int)j);
    int64_t k = p - o.colind.data();
    o.vals[k] += v * fac;
    o.present[k] = 1;
  }
}

template <class P>
int assemble_t(Oracle& o, const P& ph, const double* U, const double* Uold, double time, double tstep, double lambda, double* F) {
  const int NS = P::NS;
  const int64_t n = (int64_t)o.N * NS;
  std::fill(F, F + n, 0.0);                       // F .= 0
  std::fill(o.vals.begin(), o.vals.end(), 0.0);   // zero!(matrix)
  o.nerr = 0;
  const double tstepinv = 1.0 / tstep;
  const int d = o.dim;
  const double* nd = o.ndata.empty() ? nullptr : o.ndata.data();
  // one node term: fac * (reaction - source + (storage - old storage) / tstep)
  // isregionspecies / isnodespecies masks of assemble_res_jac (src/vfvm_assemblydata.jl:245-470)
  auto region_mask = [&](int reg) { return o.masked ? o.reg_spec[reg - 1] : ~0u; };
  auto node_mask = [&](int K) { return o.masked ? o.node_spec[K] : ~0u; };
  auto node_term = [&](int K, int reg, double fac) {
    const unsigned m = region_mask(reg);
    NodeInfo ni{K, reg, &o.coord[d * K], time, lambda, nd ? nd + (size_t)o.nnd * K : nullptr};
    double src[NS] = {0}, oldstor[NS] = {0};
    Dual<NS> u[NS], rr[NS], rs[NS];
    for (int i = 0; i < NS; ++i) { u[i] = mk<NS>(U[K * NS + i]); u[i].d[i] = 1.0; rr[i] = mk<NS>(0); rs[i] = mk<NS>(0); }
    if (P::has_source) ph.source(src, ni);
    if (P::has_reaction) ph.reaction(rr, u, ni);
    if (P::has_storage) {
      ph.storage(rs, u, ni);
      double uo[NS];
      for (int i = 0; i < NS; ++i) uo[i] = Uold[K * NS + i];
      ph.storage(oldstor, uo, ni);
    }
    for (int i = 0; i < NS; ++i) {
      if (!((m >> i) & 1u)) continue;
      F[K * NS + i] += fac * (rr[i].v - src[i] + (rs[i].v - oldstor[i]) * tstepinv);
      for (int j = 0; j < NS; ++j)
        if ((m >> j) & 1u) addnz(o, (int64_t)K * NS + i, (int64_t)K * NS + j, rr[i].d[j] + rs[i].d[j] * tstepinv, fac);
    }
  };
  // one edge term: flux (bflux on boundary edges) between K (first) and L, scattered 4-way
  auto edge_term = [&](int K, int L, int reg, double fac, bool boundary) {
    const unsigned m = boundary ? node_mask(K) : region_mask(reg);
    Dual<2 * NS> uK[NS], uL[NS], f[NS];
    for (int i = 0; i < NS; ++i) {
      uK[i] = mk<2 * NS>(U[K * NS + i]); uK[i].d[i] = 1.0;
      uL[i] = mk<2 * NS>(U[L * NS + i]); uL[i].d[NS + i] = 1.0;
      f[i] = mk<2 * NS>(0);
    }
    if (boundary) {
      BEdgeInfo be{K, L, reg, &o.coord[d * K], &o.coord[d * L], time, lambda};
      ph.bflux(f, uK, uL, be);
    } else {
      EdgeInfo ei{K, L, reg, &o.coord[d * K], &o.coord[d * L], time, lambda,
                  nd ? nd + (size_t)o.nnd * K : nullptr, nd ? nd + (size_t)o.nnd * L : nullptr};
      ph.flux(f, uK, uL, ei);
    }
    for (int i = 0; i < NS; ++i) {
      if (!((m >> i) & 1u)) continue;
      double v = fac * f[i].v;
      F[K * NS + i] += v;
      F[L * NS + i] += -v;
      for (int j = 0; j < NS; ++j) {
        if (!((m >> j) & 1u)) continue;
        int64_t iK = (int64_t)K * NS + i, iL = (int64_t)L * NS + i, jK = (int64_t)K * NS + j, jL = (int64_t)L * NS + j;
        addnz(o, iK, jK, +f[i].d[j], fac);
        addnz(o, iL, jK, -f[i].d[j], fac);
        addnz(o, iK, jL, +f[i].d[NS + j], fac);
        addnz(o, iL, jL, -f[i].d[NS + j], fac);
      }
    }
    // boutflow, src/vfvm_assembly.jl:239-313: on edges with a node on an outflow
    // boundary (outflownode!: the second node if both are), +fac r to the first
    // node if it is an outflow node, -fac r to the second if it is
    if (P::has_boutflow && !boundary && !o.outflow.empty() && (o.outflow[K] || o.outflow[L])) {
      Dual<2 * NS> r[NS];
      for (int i = 0; i < NS; ++i) r[i] = mk<2 * NS>(0);
      EdgeInfo ei{K, L, reg, &o.coord[d * K], &o.coord[d * L], time, lambda,
                  nd ? nd + (size_t)o.nnd * K : nullptr, nd ? nd + (size_t)o.nnd * L : nullptr};
      ei.outflownode = o.outflow[L] ? 2 : 1;
      ph.boutflow(r, uK, uL, ei);
      for (int i = 0; i < NS; ++i) {
        if (!((m >> i) & 1u)) continue;
        double v = fac * r[i].v;
        if (o.outflow[K]) F[K * NS + i] += v;
        if (o.outflow[L]) F[L * NS + i] += -v;
        for (int j = 0; j < NS; ++j) {
          if (!((m >> j) & 1u)) continue;
          int64_t iK = (int64_t)K * NS + i, iL = (int64_t)L * NS + i, jK = (int64_t)K * NS + j, jL = (int64_t)L * NS + j;
          if (o.outflow[K]) {
            addnz(o, iK, jK, +r[i].d[j], fac);
            addnz(o, iK, jL, r[i].d[NS + j], fac);
          }
          if (o.outflow[L]) {
            addnz(o, iL, jK, -r[i].d[j], fac);
            addnz(o, iL, jL, -r[i].d[NS + j], fac);
          }
        }
      }
    }
    // edgereaction, src/vfvm_assembly.jl:202-238: fac * r to both end nodes,
    // Jacobian entries with the signs placed there
    if (P::has_edgereaction && !boundary) {
      Dual<2 * NS> r[NS];
      for (int i = 0; i < NS; ++i) r[i] = mk<2 * NS>(0);
      EdgeInfo ei{K, L, reg, &o.coord[d * K], &o.coord[d * L], time, lambda,
                  nd ? nd + (size_t)o.nnd * K : nullptr, nd ? nd + (size_t)o.nnd * L : nullptr};
      ph.edgereaction(r, uK, uL, ei);
      for (int i = 0; i < NS; ++i) {
        if (!((m >> i) & 1u)) continue;
        double v = fac * r[i].v;
        F[K * NS + i] += v;
        F[L * NS + i] += v;
        for (int j = 0; j < NS; ++j) {
          if (!((m >> j) & 1u)) continue;
          int64_t iK = (int64_t)K * NS + i, iL = (int64_t)L * NS + i, jK = (int64_t)K * NS + j, jL = (int64_t)L * NS + j;
          addnz(o, iK, jK, +r[i].d[j], fac);
          addnz(o, iL, jK, -r[i].d[j], fac);
          addnz(o, iK, jL, -r[i].d[NS + j], fac);
          addnz(o, iL, jL, +r[i].d[NS + j], fac);
        }
      }
    }
  };
  if (!o.cellwise) {
    // assemble_nodes, src/vfvm_assembly.jl:38-126 (edgewise: per node and region)
    for (int K = 0; K < o.N; ++K)
      for (auto& rf : o.nodefac[K]) node_term(K, rf.first, rf.second);
    // assemble_edges, src/vfvm_assembly.jl:128-200 (edgewise: per edge and region)
    for (int e = 0; e < o.E; ++e)
      for (auto& rf : o.edgefac[e]) edge_term(o.edgenodes[2 * e], o.edgenodes[2 * e + 1], rf.first, rf.second, false);
  } else {
    // the same loops over the cells (CellwiseAssemblyData, src/vfvm_assemblydata.jl:126-136,181-208):
    // every cell node and every cell edge with the cell's own factor; edge
    // orientation from the global edge (low -> high node index)
    const int nnc = d + 1, nen = d == 1 ? 1 : (d == 2 ? 3 : 6);
    double npar[4], epar[6];
    for (int c = 0; c < o.ncells; ++c) {
      cellfactors(d, o.csys, o.coord.data(), &o.cellnodes[nnc * c], npar, epar);
      for (int i = 0; i < nnc; ++i) node_term(o.cellnodes[i + nnc * c], o.cellregions[c], npar[i]);
    }
    for (int c = 0; c < o.ncells; ++c) {
      cellfactors(d, o.csys, o.coord.data(), &o.cellnodes[nnc * c], npar, epar);
      for (int i = 0; i < nen; ++i) {
        const int e = o.celledges[i + nen * c];
        edge_term(o.edgenodes[2 * e], o.edgenodes[2 * e + 1], o.cellregions[c], epar[i], false);
      }
    }
  }
  // assemble_bnodes, src/vfvm_assembly.jl:318-407
  const int nbn = nn_bface(d);
  double dval[NS];
  for (int b = 0; b < o.nbf; ++b) {
    for (int ib = 0; ib < nbn; ++ib) {
      int K = o.bfacenodes[ib + nbn * b];
      int reg = o.bfaceregions[b];
      double fac = o.bfacenodefac[ib + nbn * b];
      double Dir = kDirichlet;
      if (o.has_legacy && reg - 1 < o.nbregions) {
        Dir = kDirichlet / fac;
        for (int i = 0; i < NS; ++i) {
          double bf = o.bfactors[i + NS * (reg - 1)], bv = o.bvalues[i + NS * (reg - 1)];
          if (bf == kDirichlet) {
            F[K * NS + i] += bf * (U[K * NS + i] - bv);
            addnz(o, (int64_t)K * NS + i, (int64_t)K * NS + i, bf, 1.0);
          } else {
            F[K * NS + i] += fac * (bf * U[K * NS + i] - bv);
            addnz(o, (int64_t)K * NS + i, (int64_t)K * NS + i, bf, fac);
          }
        }
      }
      BNodeInfo bi{K, reg, &o.coord[d * K], time, lambda, fac, Dir, dval};
      Dual<NS> u[NS], y[NS];
      double bsrc[NS] = {0};
      for (int i = 0; i < NS; ++i) { u[i] = mk<NS>(U[K * NS + i]); u[i].d[i] = 1.0; y[i] = mk<NS>(0); }
      if (P::has_bsource) ph.bsource(bsrc, bi);
      if (P::has_breaction) ph.breaction(y, u, bi);
      const unsigned nm = node_mask(K);
      for (int i = 0; i < NS; ++i) {
        if (!((nm >> i) & 1u)) continue;
        F[K * NS + i] += fac * (y[i].v - bsrc[i]);
        for (int j = 0; j < NS; ++j)
          if ((nm >> j) & 1u) addnz(o, (int64_t)K * NS + i, (int64_t)K * NS + j, y[i].d[j], fac);
      }
      // bstorage, src/vfvm_assembly.jl:409-440
      if (P::has_bstorage) {
        Dual<NS> sb[NS];
        double uo[NS], so[NS] = {0};
        for (int i = 0; i < NS; ++i) { sb[i] = mk<NS>(0); uo[i] = Uold[K * NS + i]; }
        ph.bstorage(sb, u, bi);
        ph.bstorage(so, uo, bi);
        for (int i = 0; i < NS; ++i) {
          if (!((nm >> i) & 1u)) continue;
          F[K * NS + i] += fac * (sb[i].v - so[i]) * tstepinv;
          for (int j = 0; j < NS; ++j)
            if ((nm >> j) & 1u) addnz(o, (int64_t)K * NS + i, (int64_t)K * NS + j, sb[i].d[j], fac * tstepinv);
        }
      }
    }
  }
  // assemble_bedges, src/vfvm_assembly.jl:444-510: the edges of every boundary
  // face with the face's edge factors (boundary data are always per face),
  // oriented low -> high node index
  if (P::has_bflux && d >= 2) {
    double npar[3], epar[3];
    const int nle = d == 2 ? 1 : 3;
    for (int b = 0; b < o.nbf; ++b) {
      const int* bn = &o.bfacenodes[nbn * b];
      bfacefactors(d, o.csys, o.coord.data(), bn, npar, epar);
      for (int i = 0; i < nle; ++i) {
        int K = d == 2 ? bn[0] : bn[tri_en[i][0]], L = d == 2 ? bn[1] : bn[tri_en[i][1]];
        if (K > L) std::swap(K, L);
        edge_term(K, L, o.bfaceregions[b], epar[i], true);
      }
    }
  }
  // _eval_and_assemble_inactive_species, src/vfvm_system.jl:1012-1026: the
  // species a node does not carry get F += U - Uold and a unit diagonal
  if (o.masked)
    for (int K = 0; K < o.N; ++K)
      for (int i = 0; i < NS; ++i)
        if (!((o.node_spec[K] >> i) & 1u)) {
          F[K * NS + i] += U[K * NS + i] - Uold[K * NS + i];
          addnz(o, (int64_t)K * NS + i, (int64_t)K * NS + i, 1.0, 1.0);
        }
  return o.nerr ? 2 : 0;
}

// _initialize_dirichlet!, src/vfvm_system.jl:947-1003
template <class P>
void init_dirichlet_t(Oracle& o, const P& ph, double* U, double time, double lambda) {
  const int NS = P::NS;
  const int d = o.dim, nbn = nn_bface(d);
  for (int b = 0; b < o.nbf; ++b)
    for (int ib = 0; ib < nbn; ++ib) {
      int K = o.bfacenodes[ib + nbn * b];
      int reg = o.bfaceregions[b];
      double dval[NS];
      for (int i = 0; i < NS; ++i) dval[i] = std::numeric_limits<double>::infinity();
      BNodeInfo bi{K, reg, &o.coord[d * K], time, lambda, o.bfacenodefac[ib + nbn * b], kDirichlet, dval};
      double u[NS], y[NS];
      for (int i = 0; i < NS; ++i) { u[i] = U[K * NS + i]; y[i] = 0.0; }
      if (P::has_breaction) ph.breaction(y, u, bi);
      for (int i = 0; i < NS; ++i) {
        if (!std::isinf(dval[i])) U[K * NS + i] = dval[i];
        if (o.has_legacy && reg - 1 < o.nbregions) {
          double bf = o.bfactors[i + NS * (reg - 1)];
          if (std::fabs(bf - kDirichlet) <= 1.4901161193847656e-8 * std::max(std::fabs(bf), kDirichlet))
            U[K * NS + i] = o.bvalues[i + NS * (reg - 1)];
        }
      }
    }
  // _initialize_inactive_dof!, src/vfvm_system.jl:1030-1042
  if (o.masked)
    for (int K = 0; K < o.N; ++K)
      for (int i = 0; i < NS; ++i)
        if (!((o.node_spec[K] >> i) & 1u)) U[K * NS + i] = 0.0;
}

// Test-function integrals (src/vfvm_testfunctions.jl:210-380): per species
// out[0] I_flux = sum fac flux(U) (T_K - T_L) over edge items, out[1] I_react =
// sum fac reaction(U) T_K and out[2] I_src = sum fac source T_K over node
// items, out[3] / out[4] the storage of U / Uold, out[5] the edge reaction
// with T_K + T_L.  Items as in the assembly mode (edgewise: per node/edge and
// region; cellwise: per cell).
template <class P>
void integrate_t(Oracle& o, const P& ph, const double* T, const double* U, const double* Uold, double* out) {
  const int NS = P::NS, d = o.dim;
  for (int k = 0; k < 6 * NS; ++k) out[k] = 0.0;
  const double* nd = o.ndata.empty() ? nullptr : o.ndata.data();
  auto node_item = [&](int K, int reg, double fac) {
    NodeInfo ni{K, reg, &o.coord[d * K], 0.0, 1.0, nd ? nd + (size_t)o.nnd * K : nullptr};
    double y[NS], u[NS], uo[NS];
    for (int i = 0; i < NS; ++i) { u[i] = U[K * NS + i]; uo[i] = Uold[K * NS + i]; }
    for (int i = 0; i < NS; ++i) y[i] = 0.0;
    if (P::has_reaction) ph.reaction(y, u, ni);
    for (int i = 0; i < NS; ++i) out[1 * NS + i] += fac * y[i] * T[K];
    for (int i = 0; i < NS; ++i) y[i] = 0.0;
    if (P::has_source) ph.source(y, ni);
    for (int i = 0; i < NS; ++i) out[2 * NS + i] += fac * y[i] * T[K];
    for (int i = 0; i < NS; ++i) y[i] = 0.0;
    if (P::has_storage) ph.storage(y, u, ni);
    for (int i = 0; i < NS; ++i) out[3 * NS + i] += fac * y[i] * T[K];
    for (int i = 0; i < NS; ++i) y[i] = 0.0;
    if (P::has_storage) ph.storage(y, uo, ni);
    for (int i = 0; i < NS; ++i) out[4 * NS + i] += fac * y[i] * T[K];
  };
  auto edge_item = [&](int K, int L, int reg, double fac) {
    EdgeInfo ei{K, L, reg, &o.coord[d * K], &o.coord[d * L], 0.0, 1.0,
                nd ? nd + (size_t)o.nnd * K : nullptr, nd ? nd + (size_t)o.nnd * L : nullptr};
    double y[NS], uK[NS], uL[NS];
    for (int i = 0; i < NS; ++i) { uK[i] = U[K * NS + i]; uL[i] = U[L * NS + i]; y[i] = 0.0; }
    ph.flux(y, uK, uL, ei);
    for (int i = 0; i < NS; ++i) out[0 * NS + i] += fac * y[i] * (T[K] - T[L]);
    if (P::has_edgereaction) {
      for (int i = 0; i < NS; ++i) y[i] = 0.0;
      ph.edgereaction(y, uK, uL, ei);
      for (int i = 0; i < NS; ++i) out[5 * NS + i] += fac * y[i] * (T[K] + T[L]);
    }
  };
  if (!o.cellwise) {
    for (int K = 0; K < o.N; ++K)
      for (auto& rf : o.nodefac[K]) node_item(K, rf.first, rf.second);
    for (int e = 0; e < o.E; ++e)
      for (auto& rf : o.edgefac[e]) edge_item(o.edgenodes[2 * e], o.edgenodes[2 * e + 1], rf.first, rf.second);
  } else {
    const int nnc = d + 1, nen = d == 1 ? 1 : (d == 2 ? 3 : 6);
    double npar[4], epar[6];
    for (int c = 0; c < o.ncells; ++c) {
      cellfactors(d, o.csys, o.coord.data(), &o.cellnodes[nnc * c], npar, epar);
      for (int i = 0; i < nnc; ++i) node_item(o.cellnodes[i + nnc * c], o.cellregions[c], npar[i]);
    }
    for (int c = 0; c < o.ncells; ++c) {
      cellfactors(d, o.csys, o.coord.data(), &o.cellnodes[nnc * c], npar, epar);
      for (int i = 0; i < nen; ++i) {
        const int e = o.celledges[i + nen * c];
        edge_item(o.edgenodes[2 * e], o.edgenodes[2 * e + 1], o.cellregions[c], epar[i]);
      }
    }
  }
}

// mass_matrix, src/vfvm_diffeq_interface.jl:60-112: the storage Jacobian at
// U = 0 (node items: storage with the node factor; boundary items: bstorage
// with the boundary factor), with the species masks of assemble_res_jac.
template <class P>
void mass_t(Oracle& o, const P& ph) {
  const int NS = P::NS, d = o.dim;
  std::fill(o.vals.begin(), o.vals.end(), 0.0);
  std::fill(o.present.begin(), o.present.end(), 0);
  Dual<NS> u[NS], s[NS];
  for (int i = 0; i < NS; ++i) { u[i] = mk<NS>(0.0); u[i].d[i] = 1.0; }
  const double* nd = o.ndata.empty() ? nullptr : o.ndata.data();
  auto node_item = [&](int K, int reg, double fac) {
    if (!P::has_storage) return;
    const unsigned m = o.masked ? o.reg_spec[reg - 1] : ~0u;
    NodeInfo ni{K, reg, &o.coord[d * K], 0.0, 0.0, nd ? nd + (size_t)o.nnd * K : nullptr};
    for (int i = 0; i < NS; ++i) s[i] = mk<NS>(0);
    ph.storage(s, u, ni);
    for (int i = 0; i < NS; ++i)
      for (int j = 0; j < NS; ++j)
        if (((m >> i) & 1u) && ((m >> j) & 1u)) addnz(o, (int64_t)K * NS + i, (int64_t)K * NS + j, s[i].d[j], fac);
  };
  if (!o.cellwise) {
    for (int K = 0; K < o.N; ++K)
      for (auto& rf : o.nodefac[K]) node_item(K, rf.first, rf.second);
  } else {
    const int nnc = d + 1;
    double npar[4], epar[6];
    for (int c = 0; c < o.ncells; ++c) {
      cellfactors(d, o.csys, o.coord.data(), &o.cellnodes[nnc * c], npar, epar);
      for (int i = 0; i < nnc; ++i) node_item(o.cellnodes[i + nnc * c], o.cellregions[c], npar[i]);
    }
  }
  if (P::has_bstorage) {
    const int nbn = nn_bface(d);
    for (int b = 0; b < o.nbf; ++b)
      for (int ib = 0; ib < nbn; ++ib) {
        const int K = o.bfacenodes[ib + nbn * b];
        const double fac = o.bfacenodefac[ib + nbn * b];
        const unsigned m = o.masked ? o.node_spec[K] : ~0u;
        BNodeInfo bi{K, o.bfaceregions[b], &o.coord[d * K], 0.0, 0.0, fac, kDirichlet, nullptr};
        for (int i = 0; i < NS; ++i) s[i] = mk<NS>(0);
        ph.bstorage(s, u, bi);
        for (int i = 0; i < NS; ++i)
          for (int j = 0; j < NS; ++j)
            if (((m >> i) & 1u) && ((m >> j) & 1u)) addnz(o, (int64_t)K * NS + i, (int64_t)K * NS + j, s[i].d[j], fac);
      }
  }
}

// Parameter derivatives dudp (src/vfvm_assembly.jl: asm_param of the node terms
// :116-120, edges :194-198, edge reactions :232-236, breaction :403-405, bstorage
// :434-436, boundary edges :497-501): the unknowns as constants, the physics'
// parameter seeded (PD: the physics with Dual<1> parameters).
template <class PD>
void dparams_t(Oracle& o, const PD& ph, const double* U, double time, double tstep, double lambda, double* out) {
  const int NS = PD::NS, d = o.dim;
  const int64_t n = (int64_t)o.N * NS;
  std::fill(out, out + n, 0.0);
  const double tstepinv = 1.0 / tstep;
  const double* nd = o.ndata.empty() ? nullptr : o.ndata.data();
  auto region_mask = [&](int reg) { return o.masked ? o.reg_spec[reg - 1] : ~0u; };
  auto node_mask = [&](int K) { return o.masked ? o.node_spec[K] : ~0u; };
  auto cst = [&](int K, Dual<1>* u) { for (int i = 0; i < NS; ++i) u[i] = mk<1>(U[K * NS + i]); };
  auto node_item = [&](int K, int reg, double fac) {
    const unsigned m = region_mask(reg);
    NodeInfo ni{K, reg, &o.coord[d * K], time, lambda, nd ? nd + (size_t)o.nnd * K : nullptr};
    Dual<1> u[NS], r[NS], st[NS];
    cst(K, u);
    for (int i = 0; i < NS; ++i) { r[i] = mk<1>(0); st[i] = mk<1>(0); }
    if (PD::has_reaction) ph.reaction(r, u, ni);
    if (PD::has_storage) ph.storage(st, u, ni);
    for (int i = 0; i < NS; ++i)
      if ((m >> i) & 1u) out[K * NS + i] += (r[i].d[0] + st[i].d[0] * tstepinv) * fac;
  };
  auto edge_item = [&](int K, int L, int reg, double fac, bool boundary) {
    const unsigned m = boundary ? node_mask(K) : region_mask(reg);
    Dual<1> uK[NS], uL[NS], f[NS];
    cst(K, uK);
    cst(L, uL);
    for (int i = 0; i < NS; ++i) f[i] = mk<1>(0);
    if (boundary) {
      BEdgeInfo be{K, L, reg, &o.coord[d * K], &o.coord[d * L], time, lambda};
      ph.bflux(f, uK, uL, be);
    } else {
      EdgeInfo ei{K, L, reg, &o.coord[d * K], &o.coord[d * L], time, lambda,
                  nd ? nd + (size_t)o.nnd * K : nullptr, nd ? nd + (size_t)o.nnd * L : nullptr};
      ph.flux(f, uK, uL, ei);
    }
    for (int i = 0; i < NS; ++i)
      if ((m >> i) & 1u) {
        out[K * NS + i] += fac * f[i].d[0];
        out[L * NS + i] -= fac * f[i].d[0];
      }
    if (PD::has_edgereaction && !boundary) {
      EdgeInfo ei{K, L, reg, &o.coord[d * K], &o.coord[d * L], time, lambda,
                  nd ? nd + (size_t)o.nnd * K : nullptr, nd ? nd + (size_t)o.nnd * L : nullptr};
      for (int i = 0; i < NS; ++i) f[i] = mk<1>(0);
      ph.edgereaction(f, uK, uL, ei);
      for (int i = 0; i < NS; ++i)
        if ((m >> i) & 1u) {
          out[K * NS + i] += fac * f[i].d[0];
          out[L * NS + i] += fac * f[i].d[0];
        }
    }
  };
  if (!o.cellwise) {
    for (int K = 0; K < o.N; ++K)
      for (auto& rf : o.nodefac[K]) node_item(K, rf.first, rf.second);
    for (int e = 0; e < o.E; ++e)
      for (auto& rf : o.edgefac[e]) edge_item(o.edgenodes[2 * e], o.edgenodes[2 * e + 1], rf.first, rf.second, false);
  } else {
    const int nnc = d + 1, nen = d == 1 ? 1 : (d == 2 ? 3 : 6);
    double npar[4], epar[6];
    for (int c = 0; c < o.ncells; ++c) {
      cellfactors(d, o.csys, o.coord.data(), &o.cellnodes[nnc * c], npar, epar);
      for (int i = 0; i < nnc; ++i) node_item(o.cellnodes[i + nnc * c], o.cellregions[c], npar[i]);
    }
    for (int c = 0; c < o.ncells; ++c) {
      cellfactors(d, o.csys, o.coord.data(), &o.cellnodes[nnc * c], npar, epar);
      for (int i = 0; i < nen; ++i) {
        const int e = o.celledges[i + nen * c];
        edge_item(o.edgenodes[2 * e], o.edgenodes[2 * e + 1], o.cellregions[c], epar[i], false);
      }
    }
  }
  const int nbn = nn_bface(d);
  for (int b = 0; b < o.nbf; ++b)
    for (int ib = 0; ib < nbn; ++ib) {
      const int K = o.bfacenodes[ib + nbn * b];
      const int reg = o.bfaceregions[b];
      const double fac = o.bfacenodefac[ib + nbn * b];
      const unsigned m = node_mask(K);
      double dval[NS];
      const double Dir = (o.has_legacy && reg - 1 < o.nbregions) ? kDirichlet / fac : kDirichlet;
      BNodeInfo bi{K, reg, &o.coord[d * K], time, lambda, fac, Dir, dval};
      Dual<1> u[NS], y[NS], sb[NS];
      cst(K, u);
      for (int i = 0; i < NS; ++i) { y[i] = mk<1>(0); sb[i] = mk<1>(0); }
      if (PD::has_breaction) ph.breaction(y, u, bi);
      if (PD::has_bstorage) ph.bstorage(sb, u, bi);
      for (int i = 0; i < NS; ++i)
        if ((m >> i) & 1u) out[K * NS + i] += y[i].d[0] * fac + sb[i].d[0] * fac * tstepinv;
    }
  if (PD::has_bflux && d >= 2) {
    double npar[3], epar[3];
    const int nle = d == 2 ? 1 : 3;
    for (int b = 0; b < o.nbf; ++b) {
      const int* bn = &o.bfacenodes[nbn * b];
      bfacefactors(d, o.csys, o.coord.data(), bn, npar, epar);
      for (int i = 0; i < nle; ++i) {
        int K = d == 2 ? bn[0] : bn[tri_en[i][0]], L = d == 2 ? bn[1] : bn[tri_en[i][1]];
        if (K > L) std::swap(K, L);
        edge_item(K, L, o.bfaceregions[b], epar[i], true);
      }
    }
  }
}

// Derivatives of the steady test-function current of species s,
// m = sum_edges fac flux_s (T_K - T_L) + sum_nodes fac (reaction_s - source_s) T_K
// (+ edge reaction with T_K + T_L): du = dm/dU (n values), from the node and edge
// terms on duals.
template <class P>
void integrate_grad_t(Oracle& o, const P& ph, const double* T, const double* U, int s, double* du) {
  const int NS = P::NS, d = o.dim;
  std::fill(du, du + (int64_t)o.N * NS, 0.0);
  const double* nd = o.ndata.empty() ? nullptr : o.ndata.data();
  auto node_item = [&](int K, int reg, double fac) {
    if (!P::has_reaction) return;
    NodeInfo ni{K, reg, &o.coord[d * K], 0.0, 1.0, nd ? nd + (size_t)o.nnd * K : nullptr};
    Dual<NS> u[NS], r[NS];
    for (int i = 0; i < NS; ++i) { u[i] = mk<NS>(U[K * NS + i]); u[i].d[i] = 1.0; r[i] = mk<NS>(0); }
    ph.reaction(r, u, ni);
    for (int j = 0; j < NS; ++j) du[K * NS + j] += fac * r[s].d[j] * T[K];
  };
  auto edge_item = [&](int K, int L, int reg, double fac) {
    EdgeInfo ei{K, L, reg, &o.coord[d * K], &o.coord[d * L], 0.0, 1.0,
                nd ? nd + (size_t)o.nnd * K : nullptr, nd ? nd + (size_t)o.nnd * L : nullptr};
    Dual<2 * NS> uK[NS], uL[NS], f[NS];
    for (int i = 0; i < NS; ++i) {
      uK[i] = mk<2 * NS>(U[K * NS + i]); uK[i].d[i] = 1.0;
      uL[i] = mk<2 * NS>(U[L * NS + i]); uL[i].d[NS + i] = 1.0;
      f[i] = mk<2 * NS>(0);
    }
    ph.flux(f, uK, uL, ei);
    for (int j = 0; j < NS; ++j) {
      du[K * NS + j] += fac * f[s].d[j] * (T[K] - T[L]);
      du[L * NS + j] += fac * f[s].d[NS + j] * (T[K] - T[L]);
    }
    if (P::has_edgereaction) {
      for (int i = 0; i < NS; ++i) f[i] = mk<2 * NS>(0);
      ph.edgereaction(f, uK, uL, ei);
      for (int j = 0; j < NS; ++j) {
        du[K * NS + j] += fac * f[s].d[j] * (T[K] + T[L]);
        du[L * NS + j] += fac * f[s].d[NS + j] * (T[K] + T[L]);
      }
    }
  };
  for (int K = 0; K < o.N; ++K)
    for (auto& rf : o.nodefac[K]) node_item(K, rf.first, rf.second);
  for (int e = 0; e < o.E; ++e)
    for (auto& rf : o.edgefac[e]) edge_item(o.edgenodes[2 * e], o.edgenodes[2 * e + 1], rf.first, rf.second);
}

// d m / d p of the same current at fixed U (the physics with Dual<1> parameters)
template <class PD>
double integrate_dp_t(Oracle& o, const PD& ph, const double* T, const double* U, int s) {
  const int NS = PD::NS, d = o.dim;
  const double* nd = o.ndata.empty() ? nullptr : o.ndata.data();
  double acc = 0.0;
  for (int K = 0; K < o.N; ++K)
    for (auto& rf : o.nodefac[K]) {
      NodeInfo ni{K, rf.first, &o.coord[d * K], 0.0, 1.0, nd ? nd + (size_t)o.nnd * K : nullptr};
      Dual<1> u[NS], r[NS];
      for (int i = 0; i < NS; ++i) { u[i] = mk<1>(U[K * NS + i]); r[i] = mk<1>(0); }
      if (PD::has_reaction) ph.reaction(r, u, ni);
      acc += rf.second * r[s].d[0] * T[K];
    }
  for (int e = 0; e < o.E; ++e)
    for (auto& rf : o.edgefac[e]) {
      const int K = o.edgenodes[2 * e], L = o.edgenodes[2 * e + 1];
      EdgeInfo ei{K, L, rf.first, &o.coord[d * K], &o.coord[d * L], 0.0, 1.0,
                  nd ? nd + (size_t)o.nnd * K : nullptr, nd ? nd + (size_t)o.nnd * L : nullptr};
      Dual<1> uK[NS], uL[NS], f[NS];
      for (int i = 0; i < NS; ++i) { uK[i] = mk<1>(U[K * NS + i]); uL[i] = mk<1>(U[L * NS + i]); f[i] = mk<1>(0); }
      ph.flux(f, uK, uL, ei);
      acc += rf.second * f[s].d[0] * (T[K] - T[L]);
    }
  return acc;
}

template <class F>
int dispatch(const Oracle& o, F&& fn) {
  const double* p = o.params.data();
  auto P = [&](int i) { return i < (int)o.params.size() ? p[i] : 0.0; };
  switch (o.phys) {
    case 1: { PhysEx105 ph; ph.eps = P(0); return fn(ph); }
    case 2: { PhysEx106 ph; ph.m = P(0); return fn(ph); }
    case 3: { PhysEx110 ph; ph.eps1 = P(0); ph.eps2 = P(1); return fn(ph); }
    case 4: { PhysEx160 ph; ph.eps = P(0); ph.z = P(1); ph.V = P(2); return fn(ph); }
    case 5: { PhysEx207 ph; ph.eps = P(0); return fn(ph); }
    case 6: { PhysEx301 ph; return fn(ph); }
    case 7: { PhysEx440 ph; ph.influx = P(0); return fn(ph); }
    case 8: { PhysLaplaceDir ph; return fn(ph); }
    case 11: { PhysNLPoisson ph; return fn(ph); }
    case 12: { PhysPorous ph; return fn(ph); }
    case 13: { PhysBipolar ph; ph.lambda2 = P(0); ph.mun = P(1); ph.mup = P(2); ph.taun = P(3); ph.taup = P(4); ph.doping = P(5); ph.V = P(6); return fn(ph); }
    case 14: { PhysRD2 ph; ph.D1 = P(0); ph.D2 = P(1); ph.k = P(2); return fn(ph); }
    case 15: { PhysKappaExp ph; ph.fsrc = P(0); return fn(ph); }
    case 16: { PhysSurfaceHeat ph; ph.eps = P(0); ph.eps_s = P(1); ph.c_s = P(2); ph.k = P(3); ph.q0 = P(4); ph.breg = (int)P(5); return fn(ph); }
    case 20: {
      PhysEx161 ph;
      ph.Cn = P(0); ph.Cp = P(1); ph.Ca = P(2); ph.En = P(3); ph.Ep = P(4); ph.mun = P(5); ph.mup = P(6);
      ph.lambda = P(7); ph.tPrecond = P(8); ph.tRamp = P(9); ph.tExt = P(10); ph.Vprecond = P(11); ph.VExt = P(12);
      ph.DirichletVal = P(13);
      return fn(ph);
    }
    case 21: { PhysTestFunction ph; return fn(ph); }
    case 22: { PhysEx430T<double> ph; ph.p = P(0); return fn(ph); }
    case 24: { PhysEx210 ph; ph.eps = P(0); ph.k = P(1); return fn(ph); }
    case 25: { PhysEx102 ph; ph.D = P(0); ph.v = P(1); ph.mode = (int)P(2); return fn(ph); }
    case 26: { PhysEx107 ph; ph.m = P(0); ph.eps = P(1); return fn(ph); }
    case 27: {
      PhysEx115 ph;
      ph.D_A = P(0); ph.D_B = P(1); ph.kp_AC = P(2); ph.km_AC = P(3); ph.kp_BC = P(4); ph.km_BC = P(5); ph.S = P(6);
      ph.iCat = (int)P(7);
      return fn(ph);
    }
    case 28: { PhysEx215 ph; ph.eps = P(0); ph.k_react = P(1); return fn(ph); }
    case 29: { PhysEx220 ph; ph.k = P(0); ph.eps = P(1); return fn(ph); }
    case 30: { PhysEx203 ph; ph.f0 = P(0); return fn(ph); }
    case 23: {
      PhysOutflow ph;
      ph.k = P(0); ph.v_in = P(1); ph.c_in = P(2); ph.D = P(3); ph.gin = (int)P(4); ph.gout = (int)P(5);
      return fn(ph);
    }
    case 18: { PhysEdgeReaction ph; ph.mode = (int)P(0); ph.dim = (int)P(1); return fn(ph); }
    case 19: { PhysJouleHeat ph; ph.kappa0 = P(0); ph.alpha = P(1); ph.T0 = P(2); ph.lam = P(3); ph.c = P(4); return fn(ph); }
    case 17: { PhysBoundarySpecies ph; ph.d = P(0); ph.k = P(1); ph.c = P(2); ph.db = P(3); ph.kmax = P(4); ph.cmax = P(5); ph.breg = (int)P(6); return fn(ph); }
  }
  return -1;
}

int nspec_of(int phys) {
  switch (phys) {
    case 3: case 4: case 14: case 17: case 19: case 23: case 24: case 28: return 2;
    case 13: case 20: case 27: case 29: return 3;
    case 1: case 2: case 5: case 6: case 7: case 8: case 11: case 12: case 15: case 16: case 18: case 21: case 22:
    case 25: case 26: case 30: return 1;
  }
  return 0;
}

}  // namespace

extern "C" {

void* oracle_create(int dim, int nnodes, const double* coord, int ncells, const int* cellnodes, const int* cellregions,
                    int nbfaces, const int* bfacenodes, const int* bfaceregions, int physics_id,
                    const double* params, int nparams, const double* nodedata, int nnodedata,
                    const double* bfactors, const double* bvalues, int nbregions, int coordsystem) {
  int ns = nspec_of(physics_id);
  if (ns == 0 || dim < 1 || dim > 3) return nullptr;
  if (!(coordsystem == 0 || (dim == 1 && (coordsystem == 1 || coordsystem == 2)) || (dim == 2 && coordsystem == 3)))
    return nullptr;
  Oracle* o = new Oracle;
  o->dim = dim; o->N = nnodes; o->ncells = ncells; o->nbf = nbfaces; o->ns = ns; o->phys = physics_id;
  o->csys = coordsystem;
  o->coord.assign(coord, coord + (size_t)dim * nnodes);
  o->cellnodes.assign(cellnodes, cellnodes + (size_t)(dim + 1) * ncells);
  o->cellregions.assign(cellregions, cellregions + ncells);
  o->bfacenodes.assign(bfacenodes, bfacenodes + (size_t)dim * nbfaces);
  o->bfaceregions.assign(bfaceregions, bfaceregions + nbfaces);
  if (nparams > 0) o->params.assign(params, params + nparams);
  o->nnd = nnodedata;
  if (nnodedata > 0) o->ndata.assign(nodedata, nodedata + (size_t)nnodedata * nnodes);
  o->nbregions = nbregions;
  if (bfactors && bvalues && nbregions > 0) {
    o->bfactors.assign(bfactors, bfactors + (size_t)ns * nbregions);
    o->bvalues.assign(bvalues, bvalues + (size_t)ns * nbregions);
    for (size_t i = 0; i < o->bfactors.size(); ++i)
      if (o->bfactors[i] != 0.0 || o->bvalues[i] != 0.0) o->has_legacy = true;
  }
  setup(*o);
  dispatch(*o, [&](const auto& ph) {
    if (!std::decay_t<decltype(ph)>::has_boutflow) return 0;
    o->outflow.assign(o->N, 0);
    for (int b = 0; b < o->nbf; ++b)
      if (ph.outflow_region(o->bfaceregions[b]))
        for (int v = 0; v < nn_bface(o->dim); ++v) o->outflow[o->bfacenodes[v + nn_bface(o->dim) * b]] = 1;
    return 0;
  });
  return o;
}

void oracle_destroy(void* h) { delete static_cast<Oracle*>(h); }

// assembly = :cellwise (1) or :edgewise (0, the default here)
void oracle_set_cellwise(void* h, int cellwise) { static_cast<Oracle*>(h)->cellwise = cellwise != 0; }

// enable_species!(sys, ispec, regions) / enable_boundary_species!(sys, ispec,
// bregions) (src/vfvm_system.jl:433-513): region_species (ns x ncreg,
// column-major) and bregion_species (ns x nbreg) nonzero where enabled; a node
// carries the species of the cells and boundary faces containing it.  Returns
// 0, or -1 for a species that is both a bulk and a boundary species, or for no
// species at all (the reference's DomainError and "No species enabled").
int oracle_set_species(void* h, int ncreg, const int* region_species, int nbreg, const int* bregion_species) {
  Oracle* o = static_cast<Oracle*>(h);
  const int ns = o->ns, d = o->dim;
  int maxreg = 1;
  for (int c = 0; c < o->ncells; ++c) maxreg = std::max(maxreg, o->cellregions[c]);
  auto mask = [&](const int* tab, int ncols, int reg) {
    unsigned m = 0;
    if (reg >= 1 && reg <= ncols)
      for (int i = 0; i < ns; ++i)
        if (tab[i + ns * (reg - 1)]) m |= 1u << i;
    return m;
  };
  unsigned bulk = 0, bnd = 0;
  for (int r = 1; r <= ncreg; ++r) bulk |= mask(region_species, ncreg, r);
  for (int r = 1; r <= nbreg; ++r) bnd |= mask(bregion_species, nbreg, r);
  o->reg_spec.assign(maxreg, 0u);
  for (int r = 1; r <= maxreg; ++r) o->reg_spec[r - 1] = mask(region_species, ncreg, r);
  o->node_spec.assign(o->N, 0u);
  for (int c = 0; c < o->ncells; ++c)
    for (int v = 0; v <= d; ++v) o->node_spec[o->cellnodes[v + (d + 1) * c]] |= o->reg_spec[o->cellregions[c] - 1];
  for (int b = 0; b < o->nbf; ++b)
    for (int v = 0; v < d; ++v) o->node_spec[o->bfacenodes[v + d * b]] |= mask(bregion_species, nbreg, o->bfaceregions[b]);
  bool any = false;
  for (int K = 0; K < o->N; ++K) any = any || o->node_spec[K] != 0;
  o->masked = true;
  return ((bulk & bnd) != 0 || !any) ? -1 : 0;
}

int oracle_nspec(void* h) { return static_cast<Oracle*>(h)->ns; }
int oracle_nedges(void* h) { return static_cast<Oracle*>(h)->E; }
int64_t oracle_ncandidates(void* h) { return (int64_t) static_cast<Oracle*>(h)->colind.size(); }

// Node volumes (sum over regions) and edge factors (sum over regions), for geometry tests.
void oracle_factors(void* h, double* nodevol, double* edgefac, int* edgenodes) {
  Oracle* o = static_cast<Oracle*>(h);
  for (int K = 0; K < o->N; ++K) { double s = 0; for (auto& p : o->nodefac[K]) s += p.second; nodevol[K] = s; }
  for (int e = 0; e < o->E; ++e) {
    double s = 0; for (auto& p : o->edgefac[e]) s += p.second; edgefac[e] = s;
    edgenodes[2 * e] = o->edgenodes[2 * e]; edgenodes[2 * e + 1] = o->edgenodes[2 * e + 1];
  }
}

void oracle_bfacefactors(void* h, double* out) {
  Oracle* o = static_cast<Oracle*>(h);
  std::copy(o->bfacenodefac.begin(), o->bfacenodefac.end(), out);
}

// Evaluate F and J at U (Uold for storage).  keep_pattern != 0 keeps entries created
// by earlier calls on this handle (ExtendableSparse keeps them across Newton steps).
int oracle_assemble(void* h, const double* U, const double* Uold, double time, double tstep, double lambda,
                    double* F, int keep_pattern) {
  Oracle* o = static_cast<Oracle*>(h);
  if (!keep_pattern) std::fill(o->present.begin(), o->present.end(), 0);
  return dispatch(*o, [&](const auto& ph) { return assemble_t(*o, ph, U, Uold, time, tstep, lambda, F); });
}

// Copy the present entries of the last assembly as CSR (rowptr n+1, colind, vals).  Returns nnz.
int64_t oracle_csr(void* h, int64_t* rowptr, int* colind, double* vals) {
  Oracle* o = static_cast<Oracle*>(h);
  int64_t n = (int64_t)o->N * o->ns, k = 0;
  if (rowptr) rowptr[0] = 0;
  for (int64_t i = 0; i < n; ++i) {
    for (int64_t p = o->rowptr[i]; p < o->rowptr[i + 1]; ++p)
      if (o->present[p]) {
        if (colind) colind[k] = o->colind[p];
        if (vals) vals[k] = o->vals[p];
        ++k;
      }
    if (rowptr) rowptr[i + 1] = k;
  }
  return k;
}

// Test-function integrals of U (Uold for the old storage): out = 6 x nspec,
// see integrate_t
void oracle_integrate(void* h, const double* T, const double* U, const double* Uold, double* out) {
  Oracle* o = static_cast<Oracle*>(h);
  dispatch(*o, [&](const auto& ph) { integrate_t(*o, ph, T, U, Uold ? Uold : U, out); return 0; });
}

// Parameter derivatives of the residual at U: out = npd x n; returns npd (0
// for a physics without differentiable parameters)
int oracle_parameter_derivatives(void* h, const double* U, double time, double tstep, double lambda, double* out) {
  Oracle* o = static_cast<Oracle*>(h);
  if (o->phys != 22) return 0;
  PhysEx430T<Dual<1>> ph;
  ph.p = mk<1>(o->params.empty() ? 0.0 : o->params[0]);
  ph.p.d[0] = 1.0;
  if (out) dparams_t(*o, ph, U, time, tstep, lambda, out);
  return 1;
}

// Derivatives of the steady test-function current of species s: du (n) and,
// for a physics with differentiable parameters, dp (npd values); returns npd
int oracle_integrate_gradient(void* h, const double* T, const double* U, int s, double* du, double* dp) {
  Oracle* o = static_cast<Oracle*>(h);
  dispatch(*o, [&](const auto& ph) { integrate_grad_t(*o, ph, T, U, s, du); return 0; });
  if (o->phys != 22) return 0;
  PhysEx430T<Dual<1>> ph;
  ph.p = mk<1>(o->params.empty() ? 0.0 : o->params[0]);
  ph.p.d[0] = 1.0;
  if (dp) dp[0] = integrate_dp_t(*o, ph, T, U, s);
  return 1;
}

// the mass matrix into the entry store (read it with oracle_csr)
void oracle_mass_matrix(void* h) {
  Oracle* o = static_cast<Oracle*>(h);
  dispatch(*o, [&](const auto& ph) { mass_t(*o, ph); return 0; });
}

void oracle_init_dirichlet(void* h, double* U, double time, double lambda) {
  Oracle* o = static_cast<Oracle*>(h);
  dispatch(*o, [&](const auto& ph) { init_dirichlet_t(*o, ph, U, time, lambda); return 0; });
}

// Standalone Cartesian geometry kernels for the form-factor identity test (test/test020_formfactors.jl).
void oracle_cellfactors(int dim, const double* coord, const int* nodes, double* npar, double* epar) {
  cellfactors(dim, 0, coord, nodes, npar, epar);
}
void oracle_bfacefactors_raw(int dim, const double* coord, const int* nodes, double* npar, double* epar) {
  bfacefactors(dim, 0, coord, nodes, npar, epar);
}
void oracle_fbernoulli_pm(const double* x, double* bp, double* bm, int64_t n) {
  for (int64_t i = 0; i < n; ++i) fbernoulli_pm(x[i], bp[i], bm[i]);
}

}  // extern "C"
