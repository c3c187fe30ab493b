// Graph engine: device-resident damped Newton (solve_step!, src/vfvm_solver.jl:13-222) with a
// preconditioned BiCGStab linear solve (one kernel per phase; the subdomain ILU0
// request uses the global multicolour ILU0 here) in place of the reference's sparse direct
// solve (_solve_linear!, src/vfvm_linsolve.jl:6-61).
//
// Everything between two host calls runs on the device: one CUDA graph holds
//   init (Dirichlet values, norms)
//   WHILE newton_continue:
//       assemble F, J                    (vfvm_assembly.cu)
//       Krylov init (b = F, norms)
//       preconditioner setup             (block-Jacobi inverse or multicolour ILU0)
//       WHILE krylov_continue:  BiCGStab iteration (5 kernels + sweeps)
//       Newton update + solve_step! convergence logic
// The loop conditions are set from device code (cudaGraphSetConditional) by the
// last block of a deterministic two-level reduction.
#include <cstring>
#include "vfvm_solver.cuh"
#include "vfvm_physics.cuh"

namespace vfvm {

// ---------------------------------------------------------------------------
// deterministic block + grid reduction of NV doubles.  Every block writes its
// partial sums; the last block to finish (ticket) adds them in block order and
// returns true on all of its threads with the totals in out[].  MAXK selects
// max instead of sum for entries k with (maxmask >> k) & 1.
// ---------------------------------------------------------------------------
template <int NV>
__device__ __forceinline__ bool grid_reduce(double (&v)[NV], unsigned maxmask, double* partials, unsigned* ticket,
                                            double (&out)[NV]) {
  __shared__ double sh[NV][kThreads / 32];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double a = v[k];
    for (int o = 16; o > 0; o >>= 1) {
      double b = __shfl_down_sync(0xffffffffu, a, o);
      a = ((maxmask >> k) & 1) ? fmax(a, b) : a + b;
    }
    if (lane == 0) sh[k][warp] = a;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double a = sh[k][0];
      for (int w = 1; w < nw; ++w) a = ((maxmask >> k) & 1) ? fmax(a, sh[k][w]) : a + sh[k][w];
      partials[blockIdx.x * NV + k] = a;
    }
    __threadfence();
    unsigned t = atomicAdd(ticket, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  // the last block: fixed-order sum over the block partials
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double a = ((maxmask >> k) & 1) ? 0.0 : 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
      double pv = *((volatile double*)&partials[b * NV + k]);
      a = ((maxmask >> k) & 1) ? fmax(a, pv) : a + pv;
    }
    for (int o = 16; o > 0; o >>= 1) {
      double b = __shfl_down_sync(0xffffffffu, a, o);
      a = ((maxmask >> k) & 1) ? fmax(a, b) : a + b;
    }
    if (lane == 0) sh[k][warp] = a;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double a = sh[k][0];
    for (int w = 1; w < nw; ++w) a = ((maxmask >> k) & 1) ? fmax(a, sh[k][w]) : a + sh[k][w];
    out[k] = a;
  }
  if (threadIdx.x == 0) *ticket = 0u;
  return true;
}

inline int red_blocks(int64_t items) {
  int64_t b = (items + kThreads - 1) / kThreads;
  if (b < 1) b = 1;
  return (int)(b < kMaxRedBlocks ? b : kMaxRedBlocks);
}

// ---------------------------------------------------------------------------
// small dense block helpers (row-major NS x NS)
// ---------------------------------------------------------------------------
template <int NS>
__device__ __forceinline__ void block_inverse(const double* a, double* inv) {
  if constexpr (NS == 1) { inv[0] = 1.0 / a[0]; return; }
  double m[NS][2 * NS];
#pragma unroll
  for (int i = 0; i < NS; ++i)
#pragma unroll
    for (int j = 0; j < 2 * NS; ++j) m[i][j] = j < NS ? a[i * NS + j] : (j - NS == i ? 1.0 : 0.0);
#pragma unroll
  for (int c = 0; c < NS; ++c) {
    int piv = c;
    double best = fabs(m[c][c]);
#pragma unroll
    for (int r = c + 1; r < NS; ++r) if (fabs(m[r][c]) > best) { best = fabs(m[r][c]); piv = r; }
    if (piv != c) {
#pragma unroll
      for (int j = 0; j < 2 * NS; ++j) { double tmp = m[c][j]; m[c][j] = m[piv][j]; m[piv][j] = tmp; }
    }
    const double ip = 1.0 / m[c][c];
#pragma unroll
    for (int j = 0; j < 2 * NS; ++j) m[c][j] *= ip;
#pragma unroll
    for (int r = 0; r < NS; ++r) {
      if (r == c) continue;
      const double f = m[r][c];
#pragma unroll
      for (int j = 0; j < 2 * NS; ++j) m[r][j] -= f * m[c][j];
    }
  }
#pragma unroll
  for (int i = 0; i < NS; ++i)
#pragma unroll
    for (int j = 0; j < NS; ++j) inv[i * NS + j] = m[i][NS + j];
}

// ---------------------------------------------------------------------------
// Newton init: L1 norm of the (Dirichlet-initialised) start value, state reset.
// ---------------------------------------------------------------------------
__global__ void nt_init_kernel(const double* __restrict__ U, int64_t n, DevState* st, const DevControl* ctl,
                               double* partials, cudaGraphConditionalHandle ncond) {
  double v[1] = {0.0};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    v[0] += fabs(U[i]);
  double out[1];
  if (grid_reduce<1>(v, 0u, partials, &st->ticket[0], out) && threadIdx.x == 0) {
    st->rnorm = out[0];
    st->damp = ctl->is_linear ? 1.0 : ctl->damp_initial;
    st->oldnorm = 1.0;
    st->tolx = 0.0;
    st->nround = 0;
    st->niter = 1;
    st->nnewton = 0;
    st->nlin = 0;
    st->status = VFVM_OK;
    st->norm = 0.0;
    st->resnorm = 0.0;
    st->updnorm = 0.0;
    st->early = 0;
    const int go = (ctl->maxiters >= 1 && !st->abort) ? 1 : 0;
    st->finished = go ? 0 : 1;
    if (!go && !st->abort) st->status = VFVM_ERR_CONVERGENCE;
    cudaGraphSetConditional(ncond, go);
  }
}

// ---------------------------------------------------------------------------
// Krylov preparation: b = F, x = p = v = 0; max|F| over non-Dirichlet rows
// (the residual norm of the Newton loop) and the NaN check of the assembly.
// ---------------------------------------------------------------------------
template <typename KT>
__global__ void kr_prep_kernel(const double* __restrict__ F, const uint8_t* __restrict__ dirdof, int64_t n,
                               KT* __restrict__ b, KT* __restrict__ x, KT* __restrict__ p, KT* __restrict__ v,
                               DevState* st, const DevControl* ctl, double* partials, int* errflag) {
  double acc[2] = {0.0, 0.0};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double f = F[i];
    b[i] = KT(f); x[i] = KT(0); p[i] = KT(0); v[i] = KT(0);
    acc[0] += f * f;
    if (!dirdof[i]) acc[1] = fmax(acc[1], fabs(f));
  }
  double out[2];
  if (grid_reduce<2>(acc, 2u, partials, &st->ticket[1], out) && threadIdx.x == 0) {
    st->resnorm = out[1];
    if (!ctl->updatecontrol) st->norm = out[1];
    if (*errflag || isnan(out[0])) st->status = VFVM_ERR_ASSEMBLY;  // NaN assembled: AssemblyError
    // residual control: the iterate already meets the tolerance, no linear solve
    else if (!ctl->updatecontrol && !ctl->is_linear && (out[1] < ctl->abstol || out[1] < st->tolx)) st->early = 1;
  }
}

// Krylov start on the preconditioned right hand side r = M^-1 b:
// r0 = r, rho = r.r, tolerance, loop condition.
template <typename KT>
__global__ void kr_start_kernel(int64_t n, const KT* __restrict__ r, KT* __restrict__ r0, DevState* st,
                                const DevControl* ctl, double* partials, cudaGraphConditionalHandle kcond) {
  double acc[1] = {0.0};
  acc_t<KT> a0 = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const KT ri = r[i];
    r0[i] = ri;
    a0 += acc_t<KT>(ri) * acc_t<KT>(ri);
  }
  acc[0] = double(a0);
  double out[1];
  if (grid_reduce<1>(acc, 0u, partials, &st->ticket[7], out) && threadIdx.x == 0) {
    st->bnorm2 = out[0];
    st->rho = out[0];
    st->alpha = 1.0;
    st->omega = 1.0;
    st->beta = 0.0;
    st->kit = 0;
    st->kbreak = 0;
    const double tol = fmax(ctl->abstol_linear, ctl->reltol_linear * sqrt(out[0]));
    st->tol2 = tol * tol;
    st->rr = out[0];
    int go = (out[0] > st->tol2 && ctl->maxiters_linear > 0) ? 1 : 0;
    if (st->status != VFVM_OK || st->early || isnan(out[0])) go = 0;
    cudaGraphSetConditional(kcond, go);
  }
}

// z = Dinv y (block-Jacobi application)
template <int NS, typename KT>
__global__ void jacobi_apply_kernel(int N, const KT* __restrict__ dinv, const KT* __restrict__ y, KT* __restrict__ z) {
  const int K = blockIdx.x * blockDim.x + threadIdx.x;
  if (K >= N) return;
  KT yy[NS];
#pragma unroll
  for (int j = 0; j < NS; ++j) yy[j] = y[(size_t)K * NS + j];
  const KT* D = dinv + (size_t)K * NS * NS;
#pragma unroll
  for (int i = 0; i < NS; ++i) {
    KT acc = KT(0);
#pragma unroll
    for (int j = 0; j < NS; ++j) acc += D[i * NS + j] * yy[j];
    z[(size_t)K * NS + i] = acc;
  }
}

// ---------------------------------------------------------------------------
// block-Jacobi: inverse of every diagonal block
// ---------------------------------------------------------------------------
template <int NS, typename MT, typename KT>
__global__ void jacobi_setup_kernel(const MT* __restrict__ J, const int* __restrict__ diag, int N, KT* __restrict__ dinv) {
  const int K = blockIdx.x * blockDim.x + threadIdx.x;
  if (K >= N) return;
  double a[NS * NS], inv[NS * NS];
  const MT* Jd = J + (size_t)diag[K] * NS * NS;
#pragma unroll
  for (int i = 0; i < NS * NS; ++i) a[i] = double(Jd[i]);
  block_inverse<NS>(a, inv);
#pragma unroll
  for (int i = 0; i < NS * NS; ++i) dinv[(size_t)K * NS * NS + i] = KT(inv[i]);
}

// ---------------------------------------------------------------------------
// multicolour ILU(0) on the block pattern.  Rows of one colour only read rows of
// lower colours, which are complete; one launch per colour.
// ---------------------------------------------------------------------------
template <typename MT, typename KT>
__global__ void ilu_copy_kernel(const MT* __restrict__ J, KT* __restrict__ ilu, int64_t m) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
    ilu[i] = KT(J[i]);
}

__device__ __forceinline__ int find_slot(const int* __restrict__ bcol, int beg, int end, int col) {
  while (beg < end) {
    int mid = (beg + end) >> 1;
    int c = bcol[mid];
    if (c == col) return mid;
    if (c < col) beg = mid + 1; else end = mid;
  }
  return -1;
}

template <int NS, typename KT>
__global__ void ilu_factor_kernel(const int* __restrict__ cnodes, int cbeg, int cend, const int* __restrict__ color,
                                  const int* __restrict__ browptr, const int* __restrict__ bcol,
                                  const int* __restrict__ diag, const int* __restrict__ lptr,
                                  const int* __restrict__ lslots, KT* __restrict__ ilu, KT* __restrict__ dinv) {
  const int idx = cbeg + blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= cend) return;
  const int K = cnodes[idx];
  const int rb = browptr[K], re = browptr[K + 1];
  for (int q = lptr[K]; q < lptr[K + 1]; ++q) {
    const int s = lslots[q];
    const int k = bcol[s];
    const int ck = color[k];
    // L block: A_Kk <- A_Kk * inv(U_kk)
    double L[NS * NS];
    {
      double a[NS * NS], di[NS * NS];
#pragma unroll
      for (int i = 0; i < NS * NS; ++i) { a[i] = double(ilu[(size_t)s * NS * NS + i]); di[i] = double(dinv[(size_t)k * NS * NS + i]); }
#pragma unroll
      for (int i = 0; i < NS; ++i)
#pragma unroll
        for (int j = 0; j < NS; ++j) {
          double acc = 0.0;
#pragma unroll
          for (int l = 0; l < NS; ++l) acc += a[i * NS + l] * di[l * NS + j];
          L[i * NS + j] = acc;
        }
#pragma unroll
      for (int i = 0; i < NS * NS; ++i) ilu[(size_t)s * NS * NS + i] = KT(L[i]);
    }
    // A_Kj -= L * A_kj for j after k (colour(j) > colour(k)), (k,j) in the pattern
    const int kb = browptr[k], ke = browptr[k + 1];
    for (int s2 = rb; s2 < re; ++s2) {
      const int j = bcol[s2];
      if (color[j] <= ck) continue;
      const int skj = find_slot(bcol, kb, ke, j);
      if (skj < 0) continue;
      double akj[NS * NS];
#pragma unroll
      for (int i = 0; i < NS * NS; ++i) akj[i] = double(ilu[(size_t)skj * NS * NS + i]);
#pragma unroll
      for (int i = 0; i < NS; ++i)
#pragma unroll
        for (int jj = 0; jj < NS; ++jj) {
          double acc = 0.0;
#pragma unroll
          for (int l = 0; l < NS; ++l) acc += L[i * NS + l] * akj[l * NS + jj];
          ilu[(size_t)s2 * NS * NS + i * NS + jj] = KT(double(ilu[(size_t)s2 * NS * NS + i * NS + jj]) - acc);
        }
    }
  }
  double a[NS * NS], inv[NS * NS];
#pragma unroll
  for (int i = 0; i < NS * NS; ++i) a[i] = double(ilu[(size_t)diag[K] * NS * NS + i]);
  block_inverse<NS>(a, inv);
#pragma unroll
  for (int i = 0; i < NS * NS; ++i) dinv[(size_t)K * NS * NS + i] = KT(inv[i]);
}

// forward sweep of one colour: w_K = y_K - sum_{lower k} L_Kk w_k  (in place in z)
template <int NS, typename KT>
__global__ void ilu_fwd_kernel(const int* __restrict__ cnodes, int cbeg, int cend, const int* __restrict__ lptr,
                               const int* __restrict__ lslots, const int* __restrict__ bcol, const KT* __restrict__ ilu,
                               const KT* __restrict__ y, KT* __restrict__ z) {
  const int idx = cbeg + blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= cend) return;
  const int K = cnodes[idx];
  KT w[NS];
#pragma unroll
  for (int i = 0; i < NS; ++i) w[i] = y[(size_t)K * NS + i];
  for (int q = lptr[K]; q < lptr[K + 1]; ++q) {
    const int s = lslots[q];
    const int k = bcol[s];
    const KT* L = ilu + (size_t)s * NS * NS;
#pragma unroll
    for (int j = 0; j < NS; ++j) {
      const KT wk = z[(size_t)k * NS + j];
#pragma unroll
      for (int i = 0; i < NS; ++i) w[i] -= L[i * NS + j] * wk;
    }
  }
#pragma unroll
  for (int i = 0; i < NS; ++i) z[(size_t)K * NS + i] = w[i];
}

// backward sweep of one colour: z_K = inv(U_KK) (w_K - sum_{upper j} U_Kj z_j)
template <int NS, typename KT>
__global__ void ilu_bwd_kernel(const int* __restrict__ cnodes, int cbeg, int cend, const int* __restrict__ color,
                               const int* __restrict__ browptr, const int* __restrict__ bcol, const KT* __restrict__ ilu,
                               const KT* __restrict__ dinv, KT* __restrict__ z) {
  const int idx = cbeg + blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= cend) return;
  const int K = cnodes[idx];
  const int cK = color[K];
  KT w[NS];
#pragma unroll
  for (int i = 0; i < NS; ++i) w[i] = z[(size_t)K * NS + i];
  for (int s = browptr[K]; s < browptr[K + 1]; ++s) {
    const int j = bcol[s];
    if (color[j] <= cK) continue;
    const KT* Ub = ilu + (size_t)s * NS * NS;
#pragma unroll
    for (int jj = 0; jj < NS; ++jj) {
      const KT zj = z[(size_t)j * NS + jj];
#pragma unroll
      for (int i = 0; i < NS; ++i) w[i] -= Ub[i * NS + jj] * zj;
    }
  }
  const KT* D = dinv + (size_t)K * NS * NS;
#pragma unroll
  for (int i = 0; i < NS; ++i) {
    KT acc = KT(0);
#pragma unroll
    for (int j = 0; j < NS; ++j) acc += D[i * NS + j] * w[j];
    z[(size_t)K * NS + i] = acc;
  }
}

// ---------------------------------------------------------------------------
// BiCGStab, left preconditioned: solves M^-1 A x = M^-1 b.  The penalty rows of
// Dirichlet nodes (diagonal 1e30) keep an O(h) flux residual in b; after M^-1
// those rows weigh 1e-30 and no longer dominate the shadow residual or the norms.
// ---------------------------------------------------------------------------
// p = r + beta (p - omega v)
template <typename KT>
__global__ void bi_p_kernel(int64_t n, const KT* __restrict__ r, KT* __restrict__ p, const KT* __restrict__ v,
                            const DevState* st) {
  const KT beta = KT(st->beta), omega = KT(st->omega);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = r[i] + beta * (p[i] - omega * v[i]);
}

// y = A x over the block pattern; LPR lanes cooperate on one block row.
template <int NS, int LPR, typename KT>
__device__ __forceinline__ void spmv_row(int K, int N, const int* __restrict__ browptr, const int* __restrict__ bcol,
                                         const KT* __restrict__ A, const KT* __restrict__ x, KT (&yK)[NS], int sub) {
#pragma unroll
  for (int i = 0; i < NS; ++i) yK[i] = KT(0);
  if (K < N) {
    const int beg = browptr[K], end = browptr[K + 1];
    for (int s = beg + sub; s < end; s += LPR) {
      const int m = bcol[s];
      const KT* Ab = A + (size_t)s * NS * NS;
      KT xm[NS];
#pragma unroll
      for (int j = 0; j < NS; ++j) xm[j] = x[(size_t)m * NS + j];
#pragma unroll
      for (int i = 0; i < NS; ++i)
#pragma unroll
        for (int j = 0; j < NS; ++j) yK[i] += Ab[i * NS + j] * xm[j];
    }
  }
  // every lane of the warp reaches this reduction (rows past N contribute zeros)
#pragma unroll
  for (int i = 0; i < NS; ++i)
#pragma unroll
    for (int o = LPR / 2; o > 0; o >>= 1) yK[i] += __shfl_down_sync(0xffffffffu, yK[i], o, LPR);
}

// MODE 0: out = A x (no reduction)
// MODE 1: out = Dinv A x;  alpha = rho / (r0 . out)            (w = r0)
// MODE 2: out = Dinv A x;  omega = (out . s) / (out . out)      (w = s)
template <int NS, int LPR, typename KT, int MODE>
__global__ void __launch_bounds__(kThreads) spmv_kernel(int N, const int* __restrict__ browptr,
                                                        const int* __restrict__ bcol, const KT* __restrict__ A,
                                                        const KT* __restrict__ x, const KT* __restrict__ dinv,
                                                        const KT* __restrict__ w, KT* __restrict__ out, DevState* st,
                                                        double* partials) {
  const int sub = threadIdx.x % LPR;
  const int rows_per_block = kThreads / LPR;
  double acc[2] = {0.0, 0.0};
  acc_t<KT> a0 = 0, a1 = 0;
  for (int K0 = blockIdx.x * rows_per_block; K0 < N; K0 += gridDim.x * rows_per_block) {
    const int K = K0 + threadIdx.x / LPR;
    KT y[NS];
    spmv_row<NS, LPR, KT>(K, N, browptr, bcol, A, x, y, sub);
    if (K < N && sub == 0) {
      if (MODE == 0) {
#pragma unroll
        for (int i = 0; i < NS; ++i) out[(size_t)K * NS + i] = y[i];
      } else {
        const KT* D = dinv + (size_t)K * NS * NS;
#pragma unroll
        for (int i = 0; i < NS; ++i) {
          KT z = KT(0);
#pragma unroll
          for (int j = 0; j < NS; ++j) z += D[i * NS + j] * y[j];
          out[(size_t)K * NS + i] = z;
          a0 += acc_t<KT>(w[(size_t)K * NS + i]) * acc_t<KT>(z);
          a1 += acc_t<KT>(z) * acc_t<KT>(z);
        }
      }
    }
  }
  if (MODE == 0) return;
  acc[0] = double(a0);
  acc[1] = double(a1);
  double res[2];
  if (grid_reduce<2>(acc, 0u, partials, &st->ticket[2], res) && threadIdx.x == 0) {
    if (MODE == 1) {
      const double r0v = res[0];
      if (r0v == 0.0 || isnan(r0v)) { st->kbreak = 1; st->alpha = 0.0; }
      else st->alpha = st->rho / r0v;
    } else {
      st->omega = (res[1] > 0.0) ? res[0] / res[1] : 0.0;
    }
  }
}

// dot products after an ILU0 application (same outputs as MODE 1 / MODE 2)
template <typename KT, int MODE>
__global__ void dot_kernel(int64_t n, const KT* __restrict__ z, const KT* __restrict__ w, DevState* st,
                           double* partials) {
  double acc[2] = {0.0, 0.0};
  acc_t<KT> a0 = 0, a1 = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const acc_t<KT> zz = acc_t<KT>(z[i]);
    a0 += acc_t<KT>(w[i]) * zz;
    a1 += zz * zz;
  }
  acc[0] = double(a0);
  acc[1] = double(a1);
  double res[2];
  if (grid_reduce<2>(acc, 0u, partials, &st->ticket[3], res) && threadIdx.x == 0) {
    if (MODE == 1) {
      const double r0v = res[0];
      if (r0v == 0.0 || isnan(r0v)) { st->kbreak = 1; st->alpha = 0.0; }
      else st->alpha = st->rho / r0v;
    } else {
      st->omega = (res[1] > 0.0) ? res[0] / res[1] : 0.0;
    }
  }
}

// s = r - alpha v
template <typename KT>
__global__ void bi_s_kernel(int64_t n, const KT* __restrict__ r, const KT* __restrict__ v, KT* __restrict__ s,
                            const DevState* st) {
  const KT alpha = KT(st->alpha);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s[i] = r[i] - alpha * v[i];
}

// x += alpha p + omega s;  r = s - omega t;  rho_new = r0.r;  convergence test
template <typename KT>
__global__ void bi_xr_kernel(int64_t n, KT* __restrict__ x, KT* __restrict__ r, const KT* __restrict__ s,
                             const KT* __restrict__ t, const KT* __restrict__ p, const KT* __restrict__ r0,
                             DevState* st, const DevControl* ctl, double* partials, cudaGraphConditionalHandle kcond) {
  const KT alpha = KT(st->alpha), omega = KT(st->omega);
  double acc[2] = {0.0, 0.0};
  acc_t<KT> a0 = 0, a1 = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] += alpha * p[i] + omega * s[i];
    const KT rn = s[i] - omega * t[i];
    r[i] = rn;
    a0 += acc_t<KT>(r0[i]) * acc_t<KT>(rn);
    a1 += acc_t<KT>(rn) * acc_t<KT>(rn);
  }
  acc[0] = double(a0);
  acc[1] = double(a1);
  double out[2];
  if (grid_reduce<2>(acc, 0u, partials, &st->ticket[4], out) && threadIdx.x == 0) {
    const double rho_new = out[0];
    const double om = st->omega;
    st->kit += 1;
    st->nlin += 1;
    st->tot_lin += 1;
    st->rr = out[1];
    const bool brk = st->kbreak || rho_new == 0.0 || om == 0.0 || isnan(out[1]);
    st->beta = brk ? 0.0 : (rho_new / st->rho) * (st->alpha / om);
    st->rho = rho_new;
    const int go = (!brk && out[1] > st->tol2 && st->kit < ctl->maxiters_linear) ? 1 : 0;
    cudaGraphSetConditional(kcond, go);
  }
}

// ---------------------------------------------------------------------------
// Newton update and the convergence logic of solve_step! (src/vfvm_solver.jl:116-195)
// ---------------------------------------------------------------------------
template <typename KT>
__global__ void nt_update_kernel(int64_t n, double* __restrict__ U, const KT* __restrict__ x, DevState* st,
                                 const DevControl* ctl, double* partials, cudaGraphConditionalHandle ncond) {
  const double damp = st->damp;
  const bool early = st->early != 0;
  const bool skip = st->status != VFVM_OK || early;
  double acc[2] = {0.0, 0.0};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double dx = double(x[i]);
    double u = U[i];
    if (!skip) { u -= damp * dx; U[i] = u; }
    acc[0] = fmax(acc[0], fabs(dx));
    acc[1] += fabs(u);
  }
  double out[2];
  if (grid_reduce<2>(acc, 1u, partials, &st->ticket[5], out) && threadIdx.x == 0) {
    int go = 1;
    if (!skip) {
      st->nnewton += 1;
      st->tot_newton += 1;
      st->updnorm = out[0];
    }
    if (skip) {
      go = 0;
    } else if (ctl->is_linear) {
      go = 0;
    } else {
      st->damp = fmin(st->damp * ctl->damp_growth, 1.0);
      double norm = ctl->updatecontrol ? out[0] : st->norm;
      st->norm = norm;
      if (st->tolx == 0.0) st->tolx = norm * ctl->reltol;
      double dnorm = 1.0;
      const double rnorm_new = out[1];
      if (st->rnorm > 1.0e-50) dnorm = fabs((st->rnorm - rnorm_new) / st->rnorm);
      st->dnorm = dnorm;
      st->nround = (dnorm < ctl->tol_round) ? st->nround + 1 : 0;
      if (st->niter > 1 && norm / st->oldnorm > 1.0 / ctl->tol_mono) {
        st->status = VFVM_ERR_CONVERGENCE;
        go = 0;
      } else if (norm < ctl->abstol || norm < st->tolx) {
        go = 0;
      } else {
        st->oldnorm = norm;
        st->rnorm = rnorm_new;
        if (st->nround > ctl->max_round) {
          go = 0;
        } else {
          st->niter += 1;
          if (st->niter > ctl->maxiters) { st->status = VFVM_ERR_CONVERGENCE; go = 0; }
        }
      }
    }
    st->finished = 1 - go;
    cudaGraphSetConditional(ncond, go);
  }
}

// advance one implicit Euler step of fixed size: Uold = U, time += dt
__global__ void step_advance_kernel(int64_t n, const double* __restrict__ U, double* __restrict__ Uold, DevState* st) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    Uold[i] = U[i];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (st->status != VFVM_OK) st->abort = 1;
    st->time += st->dt;
    st->tstepinv = 1.0 / st->dt;
  }
}

// max |a - b| (time-step control delta), result in st->maxdiff
__global__ void maxdiff_kernel(int64_t n, const double* __restrict__ a, const double* __restrict__ b, DevState* st,
                               double* partials) {
  double v[1] = {0.0};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    v[0] = fmax(v[0], fabs(a[i] - b[i]));
  double out[1];
  if (grid_reduce<1>(v, 1u, partials, &st->ticket[6], out) && threadIdx.x == 0) st->maxdiff = out[0];
}

// ---------------------------------------------------------------------------
// Device step control (graph kind 2): the step loop of solve_transient!
// (src/vfvm_solver.jl:350-513) advanced by a one-thread controller kernel after
// every tentative step.  Same decisions in the same order as the reference:
// retry with a smaller step when Newton fails (handle_exceptions) or the change
// max|u - u_old| exceeds du_max_factor * du_opt; give up at the minimal step
// (unless the first step is forced); grow the step by dl_grow and
// du_opt / du, never past the next value of `lambdas`, and spread the last
// num_final_steps steps evenly.
// ---------------------------------------------------------------------------

// Julia's isapprox(a, b; rtol, atol)
__device__ __forceinline__ bool sc_approx(double a, double b, double rtol, double atol) {
  return a == b || (isfinite(a) && isfinite(b) && fabs(a - b) <= fmax(atol, rtol * fmax(fabs(a), fabs(b))));
}
constexpr double kSqrtEps = 1.4901161193847656e-8;

// the time / embedding values of the next tentative step from lam0 with size dl
__device__ __forceinline__ void sc_setup_try(StepCtl* sc, DevState* st) {
  sc->lam = sc->lam0 + sc->dl;
  if (sc->transient) { st->time = sc->lam; st->tstepinv = 1.0 / sc->dl; st->lambda = 0.0; }
  else { st->time = sc->time0; st->tstepinv = 0.0; st->lambda = sc->lam; }
  st->abort = 0;
}

// reserve a slot for a stored solution (the last slot is overwritten when full)
__device__ __forceinline__ void sc_store(StepCtl* sc, double t, int src) {
  int slot = -1;
  if (sc->nstored < sc->max_store) slot = sc->nstored++;
  else if (sc->max_store > 0) slot = sc->max_store - 1;
  if (slot >= 0) sc->tstore[slot] = t;
  sc->store_slot = slot;
  sc->store_src = src;
}

// first tentative step of interval i (lambdas strictly increase: checked on the host)
__device__ __forceinline__ void sc_start_interval(StepCtl* sc, DevState* st) {
  sc->dl = fmax(sc->dl, sc->dl_min);
  sc->lam = sc->lambdas[sc->i];
  sc->lam0 = sc->lam;
  sc->du = 0.0;
  sc_setup_try(sc, st);
}

__global__ void sc_begin_kernel(StepCtl* sc, DevState* st, cudaGraphConditionalHandle scond) {
  sc->copy_old = 0;
  sc->store_slot = -1;
  sc->ntries = 0;
  int go = 0;
  if (sc->i + 1 < sc->nlam) {
    sc_start_interval(sc, st);
    go = 1;
  }
  cudaGraphSetConditional(scond, go);
}

// after a tentative step (Newton done, st->maxdiff = max|u - u_old|)
__global__ void sc_finish_kernel(StepCtl* sc, DevState* st, cudaGraphConditionalHandle scond) {
  sc->copy_old = 0;
  sc->store_slot = -1;
  sc->ntries += 1;
  bool solved = true, errored = false, giveup = false;
  const int newton = st->status;
  if (newton != VFVM_OK) {
    if (!sc->handle_exceptions) { sc->status = newton; cudaGraphSetConditional(scond, 0); return; }
    solved = false;
    errored = true;
  }
  if (solved) {
    sc->du = st->maxdiff;
    if (sc->du > sc->du_max_factor * sc->du_opt) solved = false;
  }
  if (!solved) {
    if (sc_approx(sc->dl, sc->dl_min, kSqrtEps, 0.0)) {
      if (!(sc->force_first_step && sc->istep == 0) || errored) {
        sc->status = VFVM_ERR_EMBEDDING;
        if (!sc->handle_exceptions) { cudaGraphSetConditional(scond, 0); return; }
        giveup = true;
      } else {
        solved = true;  // forced first step
      }
    } else {
      sc->dl = fmax(sc->dl_min, sc->dl * sc->dl_dec);
      int go = 1;
      if (sc->ntries >= sc->max_tries) { sc->status = VFVM_ERR_EMBEDDING; go = 0; }
      else sc_setup_try(sc, st);  // retry from the same start
      cudaGraphSetConditional(scond, go);
      return;
    }
  }
  if (giveup) {  // leave the step loop; the last accepted solution is the interval's result
    if (!sc->store_all) sc_store(sc, sc->lam0, 1);
    cudaGraphSetConditional(scond, 0);
    return;
  }
  // accept the step
  sc->istep += 1;
  if (sc->store_all) sc_store(sc, sc->lam, 0);
  sc->copy_old = 1;
  const double lam = sc->lam, lend = sc->lambdas[sc->i + 1], dl = sc->dl;
  const double steps_to_go = ceil((lend - lam) / dl);
  double lam_predict = lend - lam;
  if (steps_to_go < sc->num_final_steps) lam_predict = steps_to_go > 0 ? (lend - lam) / steps_to_go : NAN;
  if (sc_approx(sc->dl_max, sc->dl_min, kSqrtEps, 0.0)) lam_predict = sc->dl_max;
  if (lam < lend) {
    // min over the candidates in order; a NaN candidate is skipped
    double cand[5] = {sc->dl_max, dl * sc->dl_grow, dl * sc->du_opt / (sc->du + 1.0e-14), lam_predict, lend - lam};
    double m = cand[0];
    for (int k = 1; k < 5; ++k) if (cand[k] < m) m = cand[k];
    sc->dl = m;
    if (sc_approx(lam + sc->dl, lend, 1.0e-15, 1.0e-15)) sc->dl = lend - lam;
    sc->lam0 = lam;
    sc->du = 0.0;
    int go = 1;
    if (sc->ntries >= sc->max_tries) { sc->status = VFVM_ERR_EMBEDDING; go = 0; }
    else sc_setup_try(sc, st);
    cudaGraphSetConditional(scond, go);
    return;
  }
  // end of interval i
  if (!sc->store_all) sc_store(sc, sc->lam0, 0);  // (u_old becomes u in the copy kernel)
  sc->i += 1;
  int go = 0;
  if (sc->i + 1 < sc->nlam && sc->ntries < sc->max_tries) {
    sc_start_interval(sc, st);
    go = 1;
  }
  cudaGraphSetConditional(scond, go);
}

// the copies the controller asked for: a stored solution, u_old = u
__global__ void sc_copy_kernel(const StepCtl* __restrict__ sc, const double* __restrict__ U) {
  const int slot = sc->store_slot, src = sc->store_src, cp = sc->copy_old;
  if (slot < 0 && !cp) return;
  const int64_t n = sc->n;
  double* __restrict__ old = sc->oldsol;
  double* __restrict__ dst = slot >= 0 ? sc->Ustore + (int64_t)slot * n : nullptr;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double u = U[i];
    if (dst) dst[i] = src == 0 ? u : old[i];
    if (cp) old[i] = u;
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
DevControl make_devcontrol(const vfvm_control& c) {
  DevControl d;
  std::memset(&d, 0, sizeof(d));
  d.abstol = c.abstol; d.reltol = c.reltol; d.tol_round = c.tol_round; d.tol_mono = c.tol_mono;
  d.damp_initial = c.damp_initial; d.damp_growth = c.damp_growth;
  d.reltol_linear = c.reltol_linear; d.abstol_linear = c.abstol_linear;
  d.maxiters = c.maxiters; d.max_round = c.max_round; d.is_linear = c.is_linear;
  d.updatecontrol = c.updatecontrol; d.maxiters_linear = c.maxiters_linear;
  d.krylov = c.krylov; d.gmres_restart = c.gmres_restart;
  d.batch_tail = c.batch_krylov_tail > 0 ? c.batch_krylov_tail : 0;
  return d;
}

void destroy_workspace(Workspace* w) {
  if (!w) return;
  for (auto& g : w->graphs) cudaGraphExecDestroy(g.second);
  for (auto& g : w->graph_defs) cudaGraphDestroy(g.second);
  if (w->st) cudaFree(w->st);
  if (w->st_host) cudaFreeHost(w->st_host);
  if (w->ctl) cudaFree(w->ctl);
  if (w->sc) cudaFree(w->sc);
  if (w->ev0) cudaEventDestroy(w->ev0);
  if (w->ev1) cudaEventDestroy(w->ev1);
  delete w;
}

template <typename KT>
static cudaError_t alloc_kvecs(KVecs<KT>& k, const vfvm_ctx* c) {
  cudaError_t e;
  const size_t n = (size_t)c->N * c->ns, nblk = (size_t)c->nnzb, b2 = (size_t)c->ns * c->ns;
  DBuf<KT>* v[] = {&k.b, &k.x, &k.r, &k.r0, &k.p, &k.ph, &k.v, &k.s, &k.sh, &k.t};
  for (auto* b : v) {
    if (b->n == n) continue;
    if ((e = b->alloc(n)) != cudaSuccess) return e;
    if ((e = cudaMemset(b->p, 0, n * sizeof(KT))) != cudaSuccess) return e;
  }
  if (k.ilu.n != nblk * b2 && (e = k.ilu.alloc(nblk * b2)) != cudaSuccess) return e;
  const size_t ne = (size_t)c->ell_w * c->N * b2, nl = (size_t)std::max(c->lo_w, 1) * c->N * b2,
               nu = (size_t)std::max(c->up_w, 1) * c->N * b2;
  if (k.ell_val.n != ne && (e = k.ell_val.alloc(ne)) != cudaSuccess) return e;
  if (k.lo_val.n != nl && (e = k.lo_val.alloc(nl)) != cudaSuccess) return e;
  if (k.up_val.n != nu && (e = k.up_val.alloc(nu)) != cudaSuccess) return e;
  return cudaSuccess;
}

int ensure_workspace(vfvm_ctx* c, int precision) {
  if (!c->ws) {
    Workspace* w = new Workspace;
    c->ws = w;
    VFVM_CUDA(cudaMalloc(&w->st, sizeof(DevState)));
    VFVM_CUDA(cudaMemset(w->st, 0, sizeof(DevState)));
    VFVM_CUDA(cudaMallocHost(&w->st_host, sizeof(DevState)));
    VFVM_CUDA(cudaMalloc(&w->ctl, sizeof(DevControl)));
    VFVM_CUDA(w->partials.alloc((size_t)kMaxRedBlocks * 4));
    VFVM_CUDA(w->Uinit.alloc((size_t)c->N * c->ns));
    VFVM_CUDA(cudaEventCreate(&w->ev0));
    VFVM_CUDA(cudaEventCreate(&w->ev1));
    VFVM_CUDA(cudaFuncSetAttribute(coarse_invert_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)coarse_smem_bytes(kCoarseMax)));
    // node colours for the ILU0 ordering
    std::vector<int> col(c->N, 0);
    for (int q = 0; q < c->ncolors; ++q) {
      std::vector<int> tmp(c->h_color_ptr[q + 1] - c->h_color_ptr[q]);
      VFVM_CUDA(cudaMemcpy(tmp.data(), c->color_nodes.p + c->h_color_ptr[q], tmp.size() * sizeof(int), cudaMemcpyDeviceToHost));
      for (int k : tmp) col[k] = q;
    }
    VFVM_CUDA(w->node_color.upload(col));
  }
  Workspace* w = c->ws;
  const size_t n = (size_t)c->N * c->ns;
  if (precision == VFVM_PRECISION_FP64) {
    VFVM_CUDA(alloc_kvecs(w->k64, c));
    if (w->k64.dinv.n != (size_t)c->N * c->ns * c->ns) VFVM_CUDA(w->k64.dinv.alloc((size_t)c->N * c->ns * c->ns));
  } else {
    VFVM_CUDA(alloc_kvecs(w->k32, c));
    if (w->k32.dinv.n != (size_t)c->N * c->ns * c->ns) VFVM_CUDA(w->k32.dinv.alloc((size_t)c->N * c->ns * c->ns));
    if (c->Jf.n != (size_t)c->nnzb * c->ns * c->ns) VFVM_CUDA(c->Jf.alloc((size_t)c->nnzb * c->ns * c->ns));
  }
  return VFVM_OK;
}

// lanes per block row for the SpMV: the smallest power of two >= the mean row length
static int choose_lpr(const vfvm_ctx* c) {
  const double avg = double(c->nnzb) / double(c->N);
  if (avg <= 4.0) return 4;
  if (avg <= 8.0) return 8;
  if (avg <= 16.0) return 16;
  return 32;
}

template <int NS, typename KT>
static void record_ilu_apply(vfvm_ctx* c, KVecs<KT>& k, const KT* y, KT* z, cudaStream_t s) {
  Workspace* w = c->ws;
  for (int q = 0; q < c->ncolors; ++q) {
    const int cb = c->h_color_ptr[q], ce = c->h_color_ptr[q + 1];
    const int b = (ce - cb + 127) / 128;
    if (b > 0)
      ilu_fwd_kernel<NS, KT><<<b, 128, 0, s>>>(c->color_nodes.p, cb, ce, c->lower_ptr.p, c->lower_slots.p, c->bcol.p,
                                              k.ilu.p, y, z);
  }
  for (int q = c->ncolors - 1; q >= 0; --q) {
    const int cb = c->h_color_ptr[q], ce = c->h_color_ptr[q + 1];
    const int b = (ce - cb + 127) / 128;
    if (b > 0)
      ilu_bwd_kernel<NS, KT><<<b, 128, 0, s>>>(c->color_nodes.p, cb, ce, w->node_color.p, c->browptr.p, c->bcol.p,
                                               k.ilu.p, k.dinv.p, z);
  }
}

// z += P A_c^-1 P^T y (coarse-grid correction stage)
template <int NS, typename KT>
static void record_coarse_add(vfvm_ctx* c, const KT* y, KT* z, cudaStream_t s) {
  const CoarseData cd = c->coarse_data();
  if (!cd.nc) return;
  const int64_t n = (int64_t)c->N * NS;
  coarse_restrict_kernel<NS, KT><<<(cd.nagg * 32 + 255) / 256, 256, 0, s>>>(cd, y);
  coarse_matvec_kernel<<<(cd.nc * 32 + 255) / 256, 256, 0, s>>>(cd);
  coarse_prolong_kernel<NS, KT><<<red_blocks(n), kThreads, 0, s>>>(cd, z, n);
}

// z = M^-1 y
template <int NS, typename KT>
static void record_precon_apply(vfvm_ctx* c, KVecs<KT>& k, int precon, const KT* y, KT* z, cudaStream_t s) {
  if (precon == VFVM_PRECON_JACOBI)
    jacobi_apply_kernel<NS, KT><<<(c->N + 127) / 128, 128, 0, s>>>(c->N, k.dinv.p, y, z);
  else
    record_ilu_apply<NS, KT>(c, k, y, z, s);
  record_coarse_add<NS, KT>(c, y, z, s);
}

template <int NS, int LPR, typename KT>
static void record_krylov_iteration(vfvm_ctx* c, KVecs<KT>& k, const KT* A, int precon, cudaGraphConditionalHandle kcond,
                                    cudaStream_t s) {
  Workspace* w = c->ws;
  const int N = c->N;
  const int64_t n = (int64_t)N * NS;
  const int rpb = kThreads / LPR;
  int sblocks = (N + rpb - 1) / rpb;
  if (sblocks > kMaxRedBlocks) sblocks = kMaxRedBlocks;
  // block Jacobi without a coarse stage: SpMV, Jacobi and dot product fused
  const bool jac = precon == VFVM_PRECON_JACOBI && c->coarse_data().nc == 0;
  const int eb = red_blocks(n);
  bi_p_kernel<KT><<<eb, kThreads, 0, s>>>(n, k.r.p, k.p.p, k.v.p, w->st);
  // v = M^-1 A p,  alpha = rho / (r0 . v)
  if (jac) {
    spmv_kernel<NS, LPR, KT, 1><<<sblocks, kThreads, 0, s>>>(N, c->browptr.p, c->bcol.p, A, k.p.p, k.dinv.p, k.r0.p,
                                                             k.v.p, w->st, w->partials.p);
  } else {
    spmv_kernel<NS, LPR, KT, 0><<<sblocks, kThreads, 0, s>>>(N, c->browptr.p, c->bcol.p, A, k.p.p, nullptr, nullptr,
                                                             k.b.p, w->st, w->partials.p);
    record_precon_apply<NS, KT>(c, k, precon, k.b.p, k.v.p, s);
    dot_kernel<KT, 1><<<eb, kThreads, 0, s>>>(n, k.v.p, k.r0.p, w->st, w->partials.p);
  }
  bi_s_kernel<KT><<<eb, kThreads, 0, s>>>(n, k.r.p, k.v.p, k.s.p, w->st);
  // t = M^-1 A s,  omega = (t . s) / (t . t)
  if (jac) {
    spmv_kernel<NS, LPR, KT, 2><<<sblocks, kThreads, 0, s>>>(N, c->browptr.p, c->bcol.p, A, k.s.p, k.dinv.p, k.s.p,
                                                             k.t.p, w->st, w->partials.p);
  } else {
    spmv_kernel<NS, LPR, KT, 0><<<sblocks, kThreads, 0, s>>>(N, c->browptr.p, c->bcol.p, A, k.s.p, nullptr, nullptr,
                                                             k.b.p, w->st, w->partials.p);
    record_precon_apply<NS, KT>(c, k, precon, k.b.p, k.t.p, s);
    dot_kernel<KT, 2><<<eb, kThreads, 0, s>>>(n, k.t.p, k.s.p, w->st, w->partials.p);
  }
  bi_xr_kernel<KT><<<eb, kThreads, 0, s>>>(n, k.x.p, k.r.p, k.s.p, k.t.p, k.p.p, k.r0.p, w->st, w->ctl, w->partials.p,
                                           kcond);
}

template <int NS, typename KT, typename MT>
static void record_precon_setup(vfvm_ctx* c, KVecs<KT>& k, const MT* J, int precon, cudaStream_t s) {
  Workspace* w = c->ws;
  const int N = c->N;
  if (precon == VFVM_PRECON_JACOBI) {
    jacobi_setup_kernel<NS, MT, KT><<<(N + 127) / 128, 128, 0, s>>>(J, c->diag.p, N, k.dinv.p);
  } else {
    const int64_t m = c->nnzb * NS * NS;
    ilu_copy_kernel<MT, KT><<<red_blocks(m), kThreads, 0, s>>>(J, k.ilu.p, m);
    for (int q = 0; q < c->ncolors; ++q) {
      const int cb = c->h_color_ptr[q], ce = c->h_color_ptr[q + 1];
      const int b = (ce - cb + 127) / 128;
      if (b > 0)
        ilu_factor_kernel<NS, KT><<<b, 128, 0, s>>>(c->color_nodes.p, cb, ce, w->node_color.p, c->browptr.p, c->bcol.p,
                                                    c->diag.p, c->lower_ptr.p, c->lower_slots.p, k.ilu.p, k.dinv.p);
    }
  }
  const CoarseData cd = c->coarse_data();
  if (cd.nc) {  // Galerkin coarse matrix and its inverse
    cudaMemsetAsync(cd.A, 0, (size_t)cd.nc * cd.nc * sizeof(float), s);
    coarse_galerkin_kernel<NS, MT><<<(cd.npairs * 32 + 255) / 256, 256, 0, s>>>(cd, c->bcol.p, J);
    coarse_invert_kernel<<<1, 1024, coarse_smem_bytes(cd.nc), s>>>(cd.A, cd.nc);
  }
}

// Build the Newton graph: [init] + WHILE(newton){ assemble; kr_init; precon; WHILE(krylov){iter}; update }.
// appends a conditional WHILE node after the leaves of g (nodes without
// dependents); returns the node and its body graph
static cudaError_t add_while_node(cudaGraph_t g, cudaGraphConditionalHandle h, cudaGraphNode_t* node,
                                  cudaGraph_t* body) {
  size_t nn = 0;
  cudaError_t e = cudaGraphGetNodes(g, nullptr, &nn);
  if (e != cudaSuccess) return e;
  std::vector<cudaGraphNode_t> nodes(nn), leaves;
  if ((e = cudaGraphGetNodes(g, nodes.data(), &nn)) != cudaSuccess) return e;
  for (auto nd : nodes) {
    size_t nd_out = 0;
    if ((e = cudaGraphNodeGetDependentNodes(nd, nullptr, nullptr, &nd_out)) != cudaSuccess) return e;
    if (nd_out == 0) leaves.push_back(nd);
  }
  cudaGraphNodeParams wp = {};
  wp.type = cudaGraphNodeTypeConditional;
  wp.conditional.handle = h;
  wp.conditional.type = cudaGraphCondTypeWhile;
  wp.conditional.size = 1;
  if ((e = cudaGraphAddNode(node, g, leaves.data(), nullptr, leaves.size(), &wp)) != cudaSuccess) return e;
  *body = wp.conditional.phGraph_out[0];
  return cudaSuccess;
}

template <int NS, typename KT>
static int record_newton_body(vfvm_ctx* c, int precision, int precon, cudaGraph_t body,
                              cudaGraphConditionalHandle ncond, cudaGraphConditionalHandle kcond);

// kind 0: full solve (copies Uinit -> U, Uinit -> Uold first); kind 1: fixed-step
// implicit Euler step (advance Uold = U, time += dt, then solve); kind 2: the
// whole step loop of solve_transient! with device step control: WHILE (step
// controller) { U = Uold = u_old; Newton WHILE; max|U - u_old|; controller;
// copies }.
template <int NS, typename KT>
static int build_graph_t(vfvm_ctx* c, int precision, int precon, int kind, cudaGraph_t* out) {
  Workspace* w = c->ws;
  const int N = c->N;
  const int64_t n = (int64_t)N * NS;
  cudaGraph_t g;
  VFVM_CUDA(cudaGraphCreate(&g, 0));
  cudaGraphConditionalHandle ncond, kcond, scond;
  VFVM_CUDA(cudaGraphConditionalHandleCreate(&ncond, g, 0, 0));
  VFVM_CUDA(cudaGraphConditionalHandleCreate(&kcond, g, 0, 0));
  cudaStream_t s = c->stream;
  cudaGraph_t gcap;
  cudaGraph_t host = g;  // the graph that holds the Newton WHILE node
  if (kind == 2) {
    VFVM_CUDA(cudaGraphConditionalHandleCreate(&scond, g, 0, 0));
    VFVM_CUDA(cudaStreamBeginCaptureToGraph(s, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    sc_begin_kernel<<<1, 1, 0, s>>>(w->sc, w->st, scond);
    VFVM_CUDA(cudaStreamEndCapture(s, &gcap));
    cudaGraphNode_t snode;
    VFVM_CUDA(add_while_node(g, scond, &snode, &host));
  }

  // --- prologue of a Newton solve
  VFVM_CUDA(cudaStreamBeginCaptureToGraph(s, host, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  if (kind == 0 || kind == 2) {
    cudaMemcpyAsync(c->U.p, w->Uinit.p, n * sizeof(double), cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(c->Uold.p, w->Uinit.p, n * sizeof(double), cudaMemcpyDeviceToDevice, s);
  } else {
    step_advance_kernel<<<red_blocks(n), kThreads, 0, s>>>(n, c->U.p, c->Uold.p, w->st);
  }
  cudaMemsetAsync(c->errflag.p, 0, sizeof(int), s);
  launch_init_dirichlet(c, c->U.p, &w->st->time, s);
  nt_init_kernel<<<red_blocks(n), kThreads, 0, s>>>(c->U.p, n, w->st, w->ctl, w->partials.p, ncond);
  VFVM_CUDA(cudaStreamEndCapture(s, &gcap));
  cudaGraphNode_t wnode;
  cudaGraph_t body;
  VFVM_CUDA(add_while_node(host, ncond, &wnode, &body));
  if (int rc = record_newton_body<NS, KT>(c, precision, precon, body, ncond, kcond)) return rc;
  if (kind == 2) {  // step control after the Newton loop
    VFVM_CUDA(cudaStreamBeginCaptureToGraph(s, host, &wnode, nullptr, 1, cudaStreamCaptureModeThreadLocal));
    maxdiff_kernel<<<red_blocks(n), kThreads, 0, s>>>(n, c->U.p, w->Uinit.p, w->st, w->partials.p);
    sc_finish_kernel<<<1, 1, 0, s>>>(w->sc, w->st, scond);
    sc_copy_kernel<<<red_blocks(n), kThreads, 0, s>>>(w->sc, c->U.p);
    VFVM_CUDA(cudaStreamEndCapture(s, &gcap));
  }
  *out = g;
  return VFVM_OK;
}

// The Newton loop body: assembly, Krylov preparation, preconditioner setup,
// WHILE (BiCGStab iteration), Newton update and the solve_step! logic.
template <int NS, typename KT>
static int record_newton_body(vfvm_ctx* c, int precision, int precon, cudaGraph_t body,
                              cudaGraphConditionalHandle ncond, cudaGraphConditionalHandle kcond) {
  Workspace* w = c->ws;
  KVecs<KT>& k = *reinterpret_cast<KVecs<KT>*>(precision == VFVM_PRECISION_FP64 ? (void*)&w->k64 : (void*)&w->k32);
  const int64_t n = (int64_t)c->N * NS;
  cudaStream_t s = c->stream;

  // --- Newton body
  VFVM_CUDA(cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  if (precision == VFVM_PRECISION_FP64) launch_assemble(c, c->U.p, c->Uold.p, &w->st->time, c->F.p, c->J.p, nullptr, s);
  else launch_assemble(c, c->U.p, c->Uold.p, &w->st->time, c->F.p, nullptr, c->Jf.p, s);
  kr_prep_kernel<KT><<<red_blocks(n), kThreads, 0, s>>>(c->F.p, c->dirichlet_dof.p, n, k.b.p, k.x.p, k.p.p, k.v.p,
                                                         w->st, w->ctl, w->partials.p, c->errflag.p);
  const KT* A = precision == VFVM_PRECISION_FP64 ? (const KT*)c->J.p : (const KT*)c->Jf.p;
  record_precon_setup<NS, KT, KT>(c, k, A, precon, s);
  record_precon_apply<NS, KT>(c, k, precon, k.b.p, k.r.p, s);  // r = M^-1 b
  kr_start_kernel<KT><<<red_blocks(n), kThreads, 0, s>>>(n, k.r.p, k.r0.p, w->st, w->ctl, w->partials.p, kcond);
  cudaGraph_t bcap;
  VFVM_CUDA(cudaStreamEndCapture(s, &bcap));
  size_t nb_nodes = 0;
  VFVM_CUDA(cudaGraphGetNodes(body, nullptr, &nb_nodes));
  std::vector<cudaGraphNode_t> bnodes(nb_nodes);
  VFVM_CUDA(cudaGraphGetNodes(body, bnodes.data(), &nb_nodes));
  std::vector<cudaGraphNode_t> bleaves;
  for (auto nd : bnodes) {
    size_t nd_out = 0;
    VFVM_CUDA(cudaGraphNodeGetDependentNodes(nd, nullptr, nullptr, &nd_out));
    if (nd_out == 0) bleaves.push_back(nd);
  }
  cudaGraphNodeParams kp = {};
  kp.type = cudaGraphNodeTypeConditional;
  kp.conditional.handle = kcond;
  kp.conditional.type = cudaGraphCondTypeWhile;
  kp.conditional.size = 1;
  cudaGraphNode_t knode;
  VFVM_CUDA(cudaGraphAddNode(&knode, body, bleaves.data(), nullptr, bleaves.size(), &kp));
  cudaGraph_t kbody = kp.conditional.phGraph_out[0];

  // --- Krylov body
  VFVM_CUDA(cudaStreamBeginCaptureToGraph(s, kbody, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  const int lpr = choose_lpr(c);
  if (lpr == 4) record_krylov_iteration<NS, 4, KT>(c, k, A, precon, kcond, s);
  else if (lpr == 8) record_krylov_iteration<NS, 8, KT>(c, k, A, precon, kcond, s);
  else if (lpr == 16) record_krylov_iteration<NS, 16, KT>(c, k, A, precon, kcond, s);
  else record_krylov_iteration<NS, 32, KT>(c, k, A, precon, kcond, s);
  cudaGraph_t kcap;
  VFVM_CUDA(cudaStreamEndCapture(s, &kcap));

  // --- Newton update after the Krylov loop
  VFVM_CUDA(cudaStreamBeginCaptureToGraph(s, body, &knode, nullptr, 1, cudaStreamCaptureModeThreadLocal));
  nt_update_kernel<KT><<<red_blocks(n), kThreads, 0, s>>>(n, c->U.p, k.x.p, w->st, w->ctl, w->partials.p, ncond);
  VFVM_CUDA(cudaStreamEndCapture(s, &bcap));
  return VFVM_OK;
}


int get_graph(vfvm_ctx* c, int precision, int precon, int kind, cudaGraphExec_t* out) {
  Workspace* w = c->ws;
  GraphKey key{precision, precon, kind, c->coarse ? c->coarse->target : 0};
  auto it = w->graphs.find(key);
  if (it != w->graphs.end()) { *out = it->second; return VFVM_OK; }
  cudaGraph_t g = nullptr;
  int rc = VFVM_ERR_INPUT;
  const bool f64 = precision == VFVM_PRECISION_FP64;
  switch (c->ns) {
    case 1: rc = f64 ? build_graph_t<1, double>(c, precision, precon, kind, &g) : build_graph_t<1, float>(c, precision, precon, kind, &g); break;
    case 2: rc = f64 ? build_graph_t<2, double>(c, precision, precon, kind, &g) : build_graph_t<2, float>(c, precision, precon, kind, &g); break;
    case 3: rc = f64 ? build_graph_t<3, double>(c, precision, precon, kind, &g) : build_graph_t<3, float>(c, precision, precon, kind, &g); break;
  }
  if (rc != VFVM_OK) return rc;
  VFVM_CUDA(cudaGetLastError());
  cudaGraphExec_t exec;
  VFVM_CUDA(cudaGraphInstantiate(&exec, g, 0));
  w->graph_defs[key] = g;
  w->graphs[key] = exec;
  *out = exec;
  return VFVM_OK;
}

int launch_maxdiff(vfvm_ctx* c, const double* a, const double* b) {
  const int64_t n = (int64_t)c->N * c->ns;
  maxdiff_kernel<<<red_blocks(n), kThreads, 0, c->stream>>>(n, a, b, c->ws->st, c->ws->partials.p);
  VFVM_CUDA(cudaGetLastError());
  return VFVM_OK;
}

}  // namespace vfvm
