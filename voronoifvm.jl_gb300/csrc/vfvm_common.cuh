// Common device/host definitions for the GB300 assembly + Newton library.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <cmath>
#include <type_traits>

#include "../../include/vfvm_gb300.h"

#define VFVM_HD __host__ __device__ __forceinline__

#define VFVM_CUDA(call)                                                                     \
  do {                                                                                      \
    cudaError_t _e = (call);                                                                \
    if (_e != cudaSuccess) {                                                                \
      fprintf(stderr, "vfvm: CUDA error %s at %s:%d: %s\n", cudaGetErrorName(_e), __FILE__, \
              __LINE__, cudaGetErrorString(_e));                                            \
      return VFVM_ERR_CUDA;                                                                 \
    }                                                                                       \
  } while (0)

namespace vfvm {

constexpr double kDirichlet = 1.0e30;  // src/vfvm_system.jl:329

// Per-thread accumulator of the Krylov dot products.  FP32 vectors (the mixed
// form) are summed in FP32 within a thread; only the per-thread partial is
// widened to FP64 for the deterministic combination across threads.  GB300
// runs FP64 at about 1/57 of its FP32 rate, so widening every element (two
// conversions and an FP64 FMA each) made these reductions FP64-bound instead
// of bandwidth-bound.  FP64 vectors accumulate in FP64.
template <typename KT>
using acc_t = typename std::conditional<std::is_same<KT, float>::value, float, double>::type;
constexpr int kMaxBlockIluColors = 32; // colour limit of the subdomain ILU0 preconditioner

// -----------------------------------------------------------------------------
// Forward-mode dual number mirroring ForwardDiff.Dual with a full chunk
// (src/vfvm_physics.jl:438): value + N partials.  The value is always FP64.
// P is the partials' type: double for the FP64 Jacobian (parity mode) or float
// for the mixed mode, where the Jacobian feeds an FP32 Krylov solve and only the
// residual (the value path) must be FP64.  GB300 runs FP64 at 1/57 of the FP32
// rate, so keeping derivative arithmetic in FP32 removes most FP64 instructions
// from the assembly.  In the mixed mode the partials are formed from `s`, the
// value carried in FP32 arithmetic of its own (computed alongside v, never
// converted from it), so no FP64 -> FP32 conversion sits on the derivative
// path.  In the FP64 mode s is v and every operation is the plain FP64 one.
// -----------------------------------------------------------------------------
template <int N, typename P = double>
struct Dual {
  double v;
  P s;
  P d[N];
};

template <typename P> constexpr bool kShadow = !std::is_same<P, double>::value;

template <int N, typename P> VFVM_HD Dual<N, P> dconst(double v) {
  Dual<N, P> r; r.v = v; r.s = P(v);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = P(0);
  return r;
}
// seed with the value in both precisions (vs: the caller's P(v), converted once)
template <int N, typename P> VFVM_HD Dual<N, P> dseed(double v, P vs, int k) {
  Dual<N, P> r; r.v = v; r.s = vs;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = (i == k) ? P(1) : P(0);
  return r;
}
template <int N, typename P> VFVM_HD Dual<N, P> dseed(double v, int k) { return dseed<N, P>(v, P(v), k); }
template <int N, typename P> VFVM_HD double val(const Dual<N, P>& a) { return a.v; }
VFVM_HD double val(double a) { return a; }

template <int N, typename P> VFVM_HD Dual<N, P> operator+(const Dual<N, P>& a, const Dual<N, P>& b) {
  Dual<N, P> r; r.v = a.v + b.v;
  if constexpr (kShadow<P>) r.s = a.s + b.s; else r.s = r.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <int N, typename P> VFVM_HD Dual<N, P> operator-(const Dual<N, P>& a, const Dual<N, P>& b) {
  Dual<N, P> r; r.v = a.v - b.v;
  if constexpr (kShadow<P>) r.s = a.s - b.s; else r.s = r.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <int N, typename P> VFVM_HD Dual<N, P> operator-(const Dual<N, P>& a) {
  Dual<N, P> r; r.v = -a.v; r.s = -a.s;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
  return r;
}
template <int N, typename P> VFVM_HD Dual<N, P> operator*(const Dual<N, P>& a, const Dual<N, P>& b) {
  Dual<N, P> r; r.v = a.v * b.v;
  if constexpr (kShadow<P>) r.s = a.s * b.s; else r.s = r.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.s + a.s * b.d[i];
  return r;
}
template <int N, typename P> VFVM_HD Dual<N, P> operator/(const Dual<N, P>& a, const Dual<N, P>& b) {
  Dual<N, P> r; r.v = a.v / b.v;
  P ib, q;
  if constexpr (kShadow<P>) { ib = P(1) / b.s; q = a.s * ib; r.s = q; }
  else { ib = 1.0 / b.v; q = r.v; r.s = r.v; }
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - q * b.d[i]) * ib;
  return r;
}
template <int N, typename P> VFVM_HD Dual<N, P> operator+(const Dual<N, P>& a, double b) {
  Dual<N, P> r = a; r.v = a.v + b;
  if constexpr (kShadow<P>) r.s = a.s + P(b); else r.s = r.v;
  return r;
}
template <int N, typename P> VFVM_HD Dual<N, P> operator+(double b, const Dual<N, P>& a) {
  Dual<N, P> r = a; r.v = b + a.v;
  if constexpr (kShadow<P>) r.s = P(b) + a.s; else r.s = r.v;
  return r;
}
template <int N, typename P> VFVM_HD Dual<N, P> operator-(const Dual<N, P>& a, double b) {
  Dual<N, P> r = a; r.v = a.v - b;
  if constexpr (kShadow<P>) r.s = a.s - P(b); else r.s = r.v;
  return r;
}
template <int N, typename P> VFVM_HD Dual<N, P> operator-(double b, const Dual<N, P>& a) {
  Dual<N, P> r; r.v = b - a.v;
  if constexpr (kShadow<P>) r.s = P(b) - a.s; else r.s = r.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
  return r;
}
template <int N, typename P> VFVM_HD Dual<N, P> operator*(const Dual<N, P>& a, double b) {
  Dual<N, P> r; r.v = a.v * b; const P bp = P(b);
  if constexpr (kShadow<P>) r.s = a.s * bp; else r.s = r.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * bp;
  return r;
}
template <int N, typename P> VFVM_HD Dual<N, P> operator*(double b, const Dual<N, P>& a) { return a * b; }
template <int N, typename P> VFVM_HD Dual<N, P> operator/(const Dual<N, P>& a, double b) {
  Dual<N, P> r; r.v = a.v / b; const P ib = P(1.0 / b);
  if constexpr (kShadow<P>) r.s = a.s * ib; else r.s = r.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * ib;
  return r;
}
template <int N, typename P> VFVM_HD Dual<N, P> operator/(double a, const Dual<N, P>& b) {
  Dual<N, P> r; r.v = a / b.v;
  P ib, q;
  if constexpr (kShadow<P>) { ib = P(1) / b.s; q = P(a) * ib; r.s = q; }
  else { ib = 1.0 / b.v; q = r.v; r.s = r.v; }
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = (-q * b.d[i]) * ib;
  return r;
}
// chain rule helper: r = f(a) with FP64 value fv and, in the partials'
// precision, value fs and derivative dfs
template <int N, typename P> VFVM_HD Dual<N, P> chain(const Dual<N, P>& a, double fv, P fs, P dfs) {
  Dual<N, P> r; r.v = fv; r.s = fs;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = dfs * a.d[i];
  return r;
}
template <int N, typename P> VFVM_HD Dual<N, P> exp(const Dual<N, P>& a) {
  const double e = ::exp(a.v);
  if constexpr (kShadow<P>) { const P es = ::expf(a.s); return chain(a, e, es, es); }
  else return chain(a, e, e, e);
}
template <int N, typename P> VFVM_HD Dual<N, P> expm1(const Dual<N, P>& a) {
  const double e = ::expm1(a.v);
  if constexpr (kShadow<P>) return chain(a, e, ::expm1f(a.s), ::expf(a.s));
  else return chain(a, e, e, ::exp(a.v));
}
template <int N, typename P> VFVM_HD Dual<N, P> log(const Dual<N, P>& a) {
  const double l = ::log(a.v);
  if constexpr (kShadow<P>) return chain(a, l, ::logf(a.s), P(1) / a.s);
  else return chain(a, l, l, 1.0 / a.v);
}
template <int N, typename P> VFVM_HD Dual<N, P> log1p(const Dual<N, P>& a) {
  const double l = ::log1p(a.v);
  if constexpr (kShadow<P>) return chain(a, l, ::log1pf(a.s), P(1) / (P(1) + a.s));
  else return chain(a, l, l, 1.0 / (1.0 + a.v));
}
template <int N, typename P> VFVM_HD Dual<N, P> pow(const Dual<N, P>& a, double p) {
  const double w = ::pow(a.v, p);
  if constexpr (kShadow<P>) { const P pp = P(p); return chain(a, w, ::powf(a.s, pp), pp * ::powf(a.s, pp - P(1))); }
  else return chain(a, w, w, p * ::pow(a.v, p - 1.0));
}
template <int N, typename P> VFVM_HD Dual<N, P> sq(const Dual<N, P>& a) { return a * a; }
template <int N, typename P> VFVM_HD Dual<N, P> cube(const Dual<N, P>& a) {
  const double c = a.v * a.v * a.v;
  if constexpr (kShadow<P>) return chain(a, c, a.s * a.s * a.s, P(3) * a.s * a.s);
  else return chain(a, c, c, 3.0 * a.v * a.v);
}
template <int N, typename P> VFVM_HD Dual<N, P> dmax(const Dual<N, P>& a, double b) { return a.v >= b ? a : dconst<N, P>(b); }

VFVM_HD double sq(double a) { return a * a; }
VFVM_HD double cube(double a) { return a * a * a; }
VFVM_HD double dmax(double a, double b) { return a > b ? a : b; }
// exp and pow for physics callbacks that run on doubles as well as on duals (storage
// is evaluated at the old values in plain doubles); a name of its own, since
// plain-double overloads of exp or pow in this namespace would collide with the
// global ones where the namespace is imported
VFVM_HD double vexp(double a) { return ::exp(a); }
template <int N, typename P> VFVM_HD Dual<N, P> vexp(const Dual<N, P>& a) { return exp(a); }
VFVM_HD double vpow(double a, double p) { return ::pow(a, p); }
template <int N, typename P> VFVM_HD Dual<N, P> vpow(const Dual<N, P>& a, double p) { return pow(a, p); }

// -----------------------------------------------------------------------------
// Bernoulli function B(x) = x/(exp(x)-1) and B(-x), with the reference's
// thresholds and Taylor-Horner branch (src/vfvm_functions.jl:2-31,78-90).
// -----------------------------------------------------------------------------
template <class T> VFVM_HD T bernoulli_horner(const T& x) {
  T y = x * (1.0 / 47900160.0);
  y = x * y;
  y = x * ((-1.0 / 1209600.0) + y);
  y = x * y;
  y = x * ((1.0 / 30240.0) + y);
  y = x * y;
  y = x * ((-1.0 / 720.0) + y);
  y = x * y;
  y = x * ((1.0 / 12.0) + y);
  y = x * ((-1.0 / 2.0) + y);
  return 1.0 + y;
}
template <class T> VFVM_HD void fbernoulli_pm(const T& x, T& bp, T& bm) {
  const double xv = val(x);
  if (xv < -50.0) { bp = -x; bm = x * 0.0; }
  else if (xv > 50.0) { bp = x * 0.0; bm = x; }
  else if (fabs(xv) < 0.25) { bp = bernoulli_horner(x); bm = x + bp; }
  else { bp = x / expm1(x); bm = x + bp; }
}

VFVM_HD double ramp(double t, double t0, double t1, double u0, double u1) {  // src/vfvm_physics.jl:516-525
  if (t < t0) return u0;
  if (t < t1) return u0 + (u1 - u0) * (t - t0) / (t1 - t0);
  return u1;
}

// -----------------------------------------------------------------------------
// Geometry item views handed to the physics callbacks (the reference's Node,
// Edge and BNode, src/vfvm_geometryitems.jl:102-578, flattened to what the
// device functors read).
// -----------------------------------------------------------------------------
struct NodeItem {
  int index, region;
  const double* x;       // coordinates of the node (dim values)
  double time, lambda;   // time and embedding parameter
  const double* data;    // per-node data (nodedata row) or nullptr
};
struct EdgeItem {
  int K, L, region;      // K = first node, L = second node
  const double* xK; const double* xL;
  double time, lambda;
  const double* dataK; const double* dataL;
  int outflownode = 0;   // boutflow: the edge's node on an outflow boundary (1 first, 2 second)
};
// boundary edge: an edge of a boundary face (the reference's BEdge,
// src/vfvm_geometryitems.jl:504-578), K = first node, L = second node
struct BEdgeItem {
  int K, L, region;      // region: the boundary region of the face
  const double* xK; const double* xL;
  double time, lambda;
};
struct BNodeItem {
  int index, region;
  const double* x;
  double time, lambda, fac;
  double Dirichlet;         // penalty (1e30, or 1e30/fac with legacy boundary data)
  double* dirichlet_value;  // written by boundary_dirichlet (Dirichlet initialisation)
};

// A physics parameter as a constant of type PT: a plain double, or a dual
// number with zero partials (parameter derivatives seed it afterwards).
template <class PT> VFVM_HD PT pconst(double v) { return v; }
template <> VFVM_HD Dual<1, double> pconst<Dual<1, double>>(double v) { return dconst<1, double>(v); }

// boundary_dirichlet!(y,u,bnode,ispec,ireg,val), src/vfvm_physics.jl:487-494
template <class T> VFVM_HD void boundary_dirichlet(T* y, const T* u, const BNodeItem& b, int ispec, int ireg, double v) {
  if (b.region == ireg) {
    y[ispec] = y[ispec] + (u[ispec] - v) * b.Dirichlet;
    if (b.dirichlet_value) b.dirichlet_value[ispec] = v;
  }
}

// the same with a dual value (the derivative with respect to a parameter that
// sets the Dirichlet value)
template <int N, typename P>
VFVM_HD void boundary_dirichlet(Dual<N, P>* y, const Dual<N, P>* u, const BNodeItem& b, int ispec, int ireg,
                                const Dual<N, P>& v) {
  if (b.region == ireg) {
    y[ispec] = y[ispec] + (u[ispec] - v) * b.Dirichlet;
    if (b.dirichlet_value) b.dirichlet_value[ispec] = v.v;
  }
}

}  // namespace vfvm
