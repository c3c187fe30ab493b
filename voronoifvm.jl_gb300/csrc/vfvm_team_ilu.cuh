// Team-generic multicolour ILU(0) on the block pattern and the left-ILU0
// preconditioned BiCGStab built on it.
//
// Nodes are greedily coloured (no two neighbours share a colour); the
// elimination order is (colour, node index).  Rows of one colour only read rows
// of lower colours, so the factorisation and both triangular sweeps run one
// colour at a time with a team barrier in between.
#pragma once
#include "vfvm_krylov.cuh"

namespace vfvm {

constexpr int kMaxColors = kMaxBlockIluColors;  // subdomain ILU0 keeps per-colour ranges in shared memory

template <typename KT>
struct IluData {
  int ncolors;
  const int* color_ptr;    // ncolors+1 (device)
  const int* color_nodes;  // nodes sorted by (colour, index)
  const int* node_color;   // colour per node
  const int* lower_ptr;    // per node: lower-colour slots in elimination order
  const int* lower_slots;
  KT* ilu;                 // nnzb * NS * NS factor values
  KT* y;                   // temporary vector (N * NS)
  // ELL copies of the factor's couplings by colour position (entry w of
  // position p at w*N + p; node -1 = padding): lower (elimination) and upper
  int lw, uw;
  const int* lo_node;
  const int* lo_slot;
  const int* up_node;
  const int* up_slot;
  KT* lo_val;
  KT* up_val;
};

// ---------------------------------------------------------------------------
// ELL kernels of the Krylov solve.  One thread per row: the row's index and
// value loads are independent of each other (fixed width, column-major), so a
// thread has all of them in flight at once; the vector gathers follow.
// ---------------------------------------------------------------------------

// ell_val <- A (rows [r0, r1), thread tid of nt)
template <int NS, typename KT>
__device__ __forceinline__ void pack_ell_rows(const KrylovData<NS, KT>& d, int r0, int r1, int tid, int nt) {
  constexpr int B = NS * NS;
  for (int w = 0; w < d.ew; ++w)
    for (int K = r0 + tid; K < r1; K += nt) {
      const int64_t e = (int64_t)w * d.N + K;
      const int s = d.ell_slot[e];
#pragma unroll
      for (int i = 0; i < B; ++i) d.ell_val[e * B + i] = s >= 0 ? __ldcg(&d.A[(int64_t)s * B + i]) : KT(0);
    }
}

// out = A x on rows [r0, r1); two rows per thread and pass
template <int NS, typename KT>
__device__ __forceinline__ void spmv_ell_rows(const KrylovData<NS, KT>& d, const KT* __restrict__ x,
                                              KT* __restrict__ out, int r0, int r1, int tid, int nt) {
  constexpr int B = NS * NS;
  constexpr int R = 2;
  const int N = d.N;
  const int* __restrict__ col = d.ell_col;
  const KT* __restrict__ val = d.ell_val;
  for (int K0 = r0 + tid; K0 < r1; K0 += R * nt) {
    KT y[R][NS];
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
      for (int i = 0; i < NS; ++i) y[r][i] = KT(0);
#pragma unroll 4
    for (int w = 0; w < d.ew; ++w) {
      int m[R];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int K = K0 + r * nt;
        m[r] = K < r1 ? col[(int64_t)w * N + K] : -1;
      }
#pragma unroll
      for (int r = 0; r < R; ++r) {
        if (m[r] < 0) continue;
        const KT* Ab = val + ((int64_t)w * N + K0 + r * nt) * B;
#pragma unroll
        for (int j = 0; j < NS; ++j) {
          const KT xm = x[(size_t)m[r] * NS + j];
#pragma unroll
          for (int i = 0; i < NS; ++i) y[r][i] += Ab[i * NS + j] * xm;
        }
      }
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int K = K0 + r * nt;
      if (K < r1) {
#pragma unroll
        for (int i = 0; i < NS; ++i) out[(size_t)K * NS + i] = y[r][i];
      }
    }
  }
}

// lo_val/up_val <- the factor's couplings for colour positions [p0, p1);
// couplings to nodes outside [K0, K1) become 0 (subdomain ILU0)
template <int NS, typename KT>
__device__ __forceinline__ void pack_ilu_positions(const IluData<KT>& il, int N, int p0, int p1, int tid, int nt,
                                                   int K0, int K1) {
  constexpr int B = NS * NS;
  for (int w = 0; w < il.lw; ++w)
    for (int p = p0 + tid; p < p1; p += nt) {
      const int64_t e = (int64_t)w * N + p;
      const int sl = il.lo_slot[e], k = il.lo_node[e];
      const bool keep = sl >= 0 && k >= K0 && k < K1;
#pragma unroll
      for (int i = 0; i < B; ++i) il.lo_val[e * B + i] = keep ? __ldcg(&il.ilu[(int64_t)sl * B + i]) : KT(0);
    }
  for (int w = 0; w < il.uw; ++w)
    for (int p = p0 + tid; p < p1; p += nt) {
      const int64_t e = (int64_t)w * N + p;
      const int sl = il.up_slot[e], k = il.up_node[e];
      const bool keep = sl >= 0 && k >= K0 && k < K1;
#pragma unroll
      for (int i = 0; i < B; ++i) il.up_val[e * B + i] = keep ? __ldcg(&il.ilu[(int64_t)sl * B + i]) : KT(0);
    }
}

// forward sweep of one colour: z_K = y_K - sum L_Kk z_k over positions [p0, p1);
// two positions per thread and pass
template <int NS, typename KT>
__device__ __forceinline__ void ilu_fwd_positions(const IluData<KT>& il, int N, const KT* __restrict__ y,
                                                  KT* __restrict__ z, int p0, int p1, int tid, int nt) {
  constexpr int B = NS * NS;
  constexpr int R = 2;
  const int* __restrict__ lnode = il.lo_node;
  const KT* __restrict__ lval = il.lo_val;
  for (int pb = p0 + tid; pb < p1; pb += R * nt) {
    int K[R];
    KT w[R][NS];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int p = pb + r * nt;
      K[r] = p < p1 ? il.color_nodes[p] : -1;
    }
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
      for (int i = 0; i < NS; ++i) w[r][i] = K[r] >= 0 ? y[(size_t)K[r] * NS + i] : KT(0);
#pragma unroll 4
    for (int l = 0; l < il.lw; ++l) {
      int k[R];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int p = pb + r * nt;
        k[r] = p < p1 ? lnode[(int64_t)l * N + p] : -1;
      }
#pragma unroll
      for (int r = 0; r < R; ++r) {
        if (k[r] < 0) continue;
        const KT* Lb = lval + ((int64_t)l * N + pb + r * nt) * B;
#pragma unroll
        for (int j = 0; j < NS; ++j) {
          const KT zk = z[(size_t)k[r] * NS + j];
#pragma unroll
          for (int i = 0; i < NS; ++i) w[r][i] -= Lb[i * NS + j] * zk;
        }
      }
    }
#pragma unroll
    for (int r = 0; r < R; ++r)
      if (K[r] >= 0) {
#pragma unroll
        for (int i = 0; i < NS; ++i) z[(size_t)K[r] * NS + i] = w[r][i];
      }
  }
}

// backward sweep of one colour: z_K = D_K^-1 (z_K - sum U_Kj z_j); two positions per pass
template <int NS, typename KT>
__device__ __forceinline__ void ilu_bwd_positions(const IluData<KT>& il, const KT* __restrict__ dinv, int N,
                                                  KT* __restrict__ z, int p0, int p1, int tid, int nt) {
  constexpr int B = NS * NS;
  constexpr int R = 2;
  const int* __restrict__ unode = il.up_node;
  const KT* __restrict__ uval = il.up_val;
  for (int pb = p0 + tid; pb < p1; pb += R * nt) {
    int K[R];
    KT w[R][NS];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int p = pb + r * nt;
      K[r] = p < p1 ? il.color_nodes[p] : -1;
    }
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
      for (int i = 0; i < NS; ++i) w[r][i] = K[r] >= 0 ? z[(size_t)K[r] * NS + i] : KT(0);
#pragma unroll 4
    for (int l = 0; l < il.uw; ++l) {
      int j[R];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int p = pb + r * nt;
        j[r] = p < p1 ? unode[(int64_t)l * N + p] : -1;
      }
#pragma unroll
      for (int r = 0; r < R; ++r) {
        if (j[r] < 0) continue;
        const KT* Ub = uval + ((int64_t)l * N + pb + r * nt) * B;
#pragma unroll
        for (int jj = 0; jj < NS; ++jj) {
          const KT zj = z[(size_t)j[r] * NS + jj];
#pragma unroll
          for (int i = 0; i < NS; ++i) w[r][i] -= Ub[i * NS + jj] * zj;
        }
      }
    }
#pragma unroll
    for (int r = 0; r < R; ++r)
      if (K[r] >= 0) {
        const KT* D = dinv + (size_t)K[r] * B;
#pragma unroll
        for (int i = 0; i < NS; ++i) {
          KT acc = KT(0);
#pragma unroll
          for (int jj = 0; jj < NS; ++jj) acc += D[i * NS + jj] * w[r][jj];
          z[(size_t)K[r] * NS + i] = acc;
        }
      }
  }
}

__device__ __forceinline__ int slot_of(const int* __restrict__ col, int beg, int end, int c) {
  while (beg < end) {
    const int mid = (beg + end) >> 1;
    const int cm = col[mid];
    if (cm == c) return mid;
    if (cm < c) beg = mid + 1; else end = mid;
  }
  return -1;
}

template <int NS, typename KT>
__device__ __forceinline__ void ilu_factor_row(int K, const KrylovData<NS, KT>& d, const IluData<KT>& il) {
  const int rb = d.rowptr[K], re = d.rowptr[K + 1];
  for (int q = il.lower_ptr[K]; q < il.lower_ptr[K + 1]; ++q) {
    const int s = il.lower_slots[q];
    const int k = d.col[s];
    const int ck = il.node_color[k];
    double L[NS * NS];
    {
      double a[NS * NS], di[NS * NS];
#pragma unroll
      for (int i = 0; i < NS * NS; ++i) { a[i] = double(il.ilu[(size_t)s * NS * NS + i]); di[i] = double(d.dinv[(size_t)k * NS * NS + i]); }
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
      for (int i = 0; i < NS * NS; ++i) il.ilu[(size_t)s * NS * NS + i] = KT(L[i]);
    }
    const int kb = d.rowptr[k], ke = d.rowptr[k + 1];
    for (int s2 = rb; s2 < re; ++s2) {
      const int j = d.col[s2];
      if (il.node_color[j] <= ck) continue;
      const int skj = slot_of(d.col, kb, ke, j);
      if (skj < 0) continue;
#pragma unroll
      for (int i = 0; i < NS; ++i)
#pragma unroll
        for (int jj = 0; jj < NS; ++jj) {
          double acc = 0.0;
#pragma unroll
          for (int l = 0; l < NS; ++l) acc += L[i * NS + l] * double(il.ilu[(size_t)skj * NS * NS + l * NS + jj]);
          KT& dst = il.ilu[(size_t)s2 * NS * NS + i * NS + jj];
          dst = KT(double(dst) - acc);
        }
    }
  }
  double a[NS * NS], inv[NS * NS];
#pragma unroll
  for (int i = 0; i < NS * NS; ++i) a[i] = double(il.ilu[(size_t)d.diag[K] * NS * NS + i]);
  small_inverse<NS>(a, inv);
#pragma unroll
  for (int i = 0; i < NS * NS; ++i) d.dinv[(size_t)K * NS * NS + i] = KT(inv[i]);
}

// ILU(0) factorisation of d.A into il.ilu (+ inverted diagonal blocks in d.dinv)
template <class Team, int NS, typename KT>
__device__ bool team_ilu_factor(Team& team, const KrylovData<NS, KT>& d, const IluData<KT>& il, int64_t nvals) {
  for (int64_t q = team.rank(); q < nvals; q += team.size()) il.ilu[q] = d.A[q];
  if (!team.sync()) return false;
  for (int c = 0; c < il.ncolors; ++c) {
    for (int idx = il.color_ptr[c] + team.rank(); idx < il.color_ptr[c + 1]; idx += team.size())
      ilu_factor_row<NS, KT>(il.color_nodes[idx], d, il);
    if (!team.sync()) return false;
  }
  return true;
}

// ---------------------------------------------------------------------------
// BiCGStab vector updates, four elements per thread per pass (q, q+st, q+2st,
// q+3st: each load instruction stays coalesced across the threads, and a
// thread issues all loads of a pass before its first store).  Element q is
// always handled by the same thread (q = start mod st), the ownership that
// lets the coarse prolongation skip a barrier.
// ---------------------------------------------------------------------------
constexpr int kVecU = 4;

// p = r + beta (p - omega v)
template <typename KT>
__device__ __forceinline__ void vec_p_update(KT* __restrict__ p, const KT* __restrict__ r, const KT* __restrict__ v,
                                             KT beta, KT omega, int64_t q0, int64_t q1, int64_t st) {
  for (int64_t q = q0; q < q1; q += kVecU * st) {
    KT rr[kVecU], pp[kVecU], vv[kVecU];
#pragma unroll
    for (int u = 0; u < kVecU; ++u) {
      const int64_t e = q + u * st;
      if (e < q1) { rr[u] = r[e]; pp[u] = p[e]; vv[u] = v[e]; }
    }
#pragma unroll
    for (int u = 0; u < kVecU; ++u) {
      const int64_t e = q + u * st;
      if (e < q1) p[e] = rr[u] + beta * (pp[u] - omega * vv[u]);
    }
  }
}

// s = r - alpha v
template <typename KT>
__device__ __forceinline__ void vec_s_update(KT* __restrict__ s, const KT* __restrict__ r, const KT* __restrict__ v,
                                             KT alpha, int64_t q0, int64_t q1, int64_t st) {
  for (int64_t q = q0; q < q1; q += kVecU * st) {
    KT rr[kVecU], vv[kVecU];
#pragma unroll
    for (int u = 0; u < kVecU; ++u) {
      const int64_t e = q + u * st;
      if (e < q1) { rr[u] = r[e]; vv[u] = v[e]; }
    }
#pragma unroll
    for (int u = 0; u < kVecU; ++u) {
      const int64_t e = q + u * st;
      if (e < q1) s[e] = rr[u] - alpha * vv[u];
    }
  }
}

// acc[0] += w.z, acc[1] += z.z
template <typename KT>
__device__ __forceinline__ void vec_dots(const KT* __restrict__ w, const KT* __restrict__ z, int64_t q0, int64_t q1,
                                         int64_t st, double (&acc)[2]) {
  acc_t<KT> a0 = 0, a1 = 0;
  for (int64_t q = q0; q < q1; q += kVecU * st) {
    KT ww[kVecU], zz[kVecU];
#pragma unroll
    for (int u = 0; u < kVecU; ++u) {
      const int64_t e = q + u * st;
      ww[u] = e < q1 ? w[e] : KT(0);
      zz[u] = e < q1 ? z[e] : KT(0);
    }
#pragma unroll
    for (int u = 0; u < kVecU; ++u) {
      a0 += acc_t<KT>(ww[u]) * acc_t<KT>(zz[u]);
      a1 += acc_t<KT>(zz[u]) * acc_t<KT>(zz[u]);
    }
  }
  acc[0] += double(a0);
  acc[1] += double(a1);
}

// x += alpha p + omega s;  r = s - omega t;  acc += (r0.r, r.r)
template <typename KT>
__device__ __forceinline__ void vec_xr_update(KT* __restrict__ x, KT* __restrict__ r, const KT* __restrict__ p,
                                              const KT* __restrict__ s, const KT* __restrict__ t,
                                              const KT* __restrict__ r0, KT alpha, KT omega, int64_t q0, int64_t q1,
                                              int64_t st, double (&acc)[2]) {
  acc_t<KT> a0 = 0, a1 = 0;
  for (int64_t q = q0; q < q1; q += kVecU * st) {
    KT xx[kVecU], pp[kVecU], ss[kVecU], tt[kVecU], r0r[kVecU];
#pragma unroll
    for (int u = 0; u < kVecU; ++u) {
      const int64_t e = q + u * st;
      if (e < q1) { xx[u] = x[e]; pp[u] = p[e]; ss[u] = s[e]; tt[u] = t[e]; r0r[u] = r0[e]; }
    }
#pragma unroll
    for (int u = 0; u < kVecU; ++u) {
      const int64_t e = q + u * st;
      if (e < q1) {
        x[e] = xx[u] + alpha * pp[u] + omega * ss[u];
        const KT rn = ss[u] - omega * tt[u];
        r[e] = rn;
        a0 += acc_t<KT>(r0r[u]) * acc_t<KT>(rn);
        a1 += acc_t<KT>(rn) * acc_t<KT>(rn);
      }
    }
  }
  acc[0] += double(a0);
  acc[1] += double(a1);
}

// z = (LU)^-1 y with the ELL couplings; ends with a team barrier
template <class Team, int NS, typename KT>
__device__ bool team_ilu_apply_ell(Team& team, const KrylovData<NS, KT>& d, const IluData<KT>& il,
                                   const KT* __restrict__ y, KT* __restrict__ z) {
  for (int c = 0; c < il.ncolors; ++c) {
    ilu_fwd_positions<NS, KT>(il, d.N, y, z, il.color_ptr[c], il.color_ptr[c + 1], team.rank(), team.size());
    if (!team.sync()) return false;
  }
  for (int c = il.ncolors - 1; c >= 0; --c) {
    ilu_bwd_positions<NS, KT>(il, d.dinv, d.N, z, il.color_ptr[c], il.color_ptr[c + 1], team.rank(), team.size());
    if (!team.sync()) return false;
  }
  return true;
}

// Left multicolour-ILU0 BiCGStab (ELL SpMV and sweeps, optional coarse stage):
// solves A x = b from x = 0; `iters` is set on every thread.
template <class Team, int NS, int LPR, typename KT>
__device__ bool team_bicgstab_ilu(Team& team, const KrylovData<NS, KT>& d, const IluData<KT>& il, const KrylovCtl& c,
                                  int64_t nvals, int& iters) {
  const int64_t n = (int64_t)d.N * NS;
  iters = 0;
  if (!team_ilu_factor<Team, NS, KT>(team, d, il, nvals)) return false;
  pack_ell_rows<NS, KT>(d, 0, d.N, team.rank(), team.size());
  pack_ilu_positions<NS, KT>(il, d.N, 0, d.N, team.rank(), team.size(), 0, d.N);
  if (d.cd.nc && !team_coarse_setup<Team, NS, KT>(team, d.cd, d.col, d.A)) return false;  // (ends with a barrier)
  if (!d.cd.nc && !team.sync()) return false;
  if (!team_ilu_apply_ell<Team, NS, KT>(team, d, il, d.b, d.r)) return false;  // r = M^-1 b
  if (d.cd.nc && !team_coarse_add<Team, NS, KT>(team, d.cd, d.b, d.r, n)) return false;
  double acc1[1] = {0.0};
  acc_t<KT> a1 = 0;
  for (int64_t q = team.rank(); q < n; q += team.size()) {
    const KT rq = d.r[q];
    d.r0[q] = rq; d.x[q] = KT(0); d.p[q] = KT(0); d.v[q] = KT(0);
    a1 += acc_t<KT>(rq) * acc_t<KT>(rq);
  }
  acc1[0] = double(a1);
  double red1[1];
  if (!team.template reduce<1>(acc1, 0u, red1)) return false;
  double rho = red1[0];
  const double tol = fmax(c.abstol, c.reltol * sqrt(red1[0]));
  const double tol2 = tol * tol;
  double rr = red1[0], alpha = 1.0, omega = 1.0, beta = 0.0;
  if (!(rr > tol2) || c.maxiters <= 0 || isnan(rr)) return true;
  int it = 0, brk = 0;
  const int64_t q0 = team.rank(), qs = team.size();
  while (true) {
    vec_p_update<KT>(d.p, d.r, d.v, KT(beta), KT(omega), q0, n, qs);
    if (!team.sync()) return false;
    spmv_ell_rows<NS, KT>(d, d.p, il.y, 0, d.N, team.rank(), team.size());
    if (!team.sync()) return false;
    if (!team_ilu_apply_ell<Team, NS, KT>(team, d, il, il.y, d.v)) return false;
    if (d.cd.nc && !team_coarse_add<Team, NS, KT>(team, d.cd, il.y, d.v, n)) return false;
    double acc[2] = {0.0, 0.0}, red[2];
    vec_dots<KT>(d.r0, d.v, q0, n, qs, acc);
    if (!team.template reduce<2>(acc, 0u, red)) return false;
    if (red[0] == 0.0 || isnan(red[0])) { brk = 1; alpha = 0.0; }
    else alpha = rho / red[0];
    vec_s_update<KT>(d.s, d.r, d.v, KT(alpha), q0, n, qs);
    if (!team.sync()) return false;
    spmv_ell_rows<NS, KT>(d, d.s, il.y, 0, d.N, team.rank(), team.size());
    if (!team.sync()) return false;
    if (!team_ilu_apply_ell<Team, NS, KT>(team, d, il, il.y, d.t)) return false;
    if (d.cd.nc && !team_coarse_add<Team, NS, KT>(team, d.cd, il.y, d.t, n)) return false;
    acc[0] = acc[1] = 0.0;
    vec_dots<KT>(d.s, d.t, q0, n, qs, acc);
    if (!team.template reduce<2>(acc, 0u, red)) return false;
    omega = red[1] > 0.0 ? red[0] / red[1] : 0.0;
    acc[0] = acc[1] = 0.0;
    vec_xr_update<KT>(d.x, d.r, d.p, d.s, d.t, d.r0, KT(alpha), KT(omega), q0, n, qs, acc);
    if (!team.template reduce<2>(acc, 0u, red)) return false;
    ++it;
    rr = red[1];
    brk = brk || red[0] == 0.0 || omega == 0.0 || isnan(rr);
    if (brk || !(rr > tol2) || it >= c.maxiters) break;
    beta = (red[0] / rho) * (alpha / omega);
    rho = red[0];
  }
  iters = it;
  return true;
}

}  // namespace vfvm

namespace vfvm {

// ---------------------------------------------------------------------------
// Subdomain (block) ILU(0): every CTA of the team owns the contiguous node
// range [K0, K1) and factors / applies ILU(0) on the couplings inside it only
// (multicolour order, __syncthreads between colours).  The preconditioner then
// needs no team-wide barrier; a BiCGStab iteration costs 5 team barriers.  For
// a one-CTA team the subdomain is the whole system (exact ILU(0)).
// ---------------------------------------------------------------------------
struct Subdomain {
  int K0, K1;
  int cb[kMaxColors + 1];  // per colour: [cb[c], ce[c]) range in color_nodes inside [K0, K1)
  int ce[kMaxColors + 1];
};

__device__ __forceinline__ int lower_bound_int(const int* __restrict__ a, int lo, int hi, int v) {
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (a[mid] < v) lo = mid + 1; else hi = mid;
  }
  return lo;
}

template <int NS, typename KT>
__device__ __forceinline__ void make_subdomain(Subdomain& sd, int N, int cta, int ncta, const IluData<KT>& il) {
  sd.K0 = (int)((int64_t)N * cta / ncta);
  sd.K1 = (int)((int64_t)N * (cta + 1) / ncta);
  for (int c = 0; c < il.ncolors && c < kMaxColors; ++c) {
    const int b = il.color_ptr[c], e = il.color_ptr[c + 1];
    sd.cb[c] = lower_bound_int(il.color_nodes, b, e, sd.K0);
    sd.ce[c] = lower_bound_int(il.color_nodes, b, e, sd.K1);
  }
}

template <int NS, typename KT>
__device__ __forceinline__ void bilu_factor_row(int K, const Subdomain& sd, const KrylovData<NS, KT>& d,
                                                const IluData<KT>& il) {
  const int rb = d.rowptr[K], re = d.rowptr[K + 1];
  for (int q = il.lower_ptr[K]; q < il.lower_ptr[K + 1]; ++q) {
    const int s = il.lower_slots[q];
    const int k = d.col[s];
    if (k < sd.K0 || k >= sd.K1) continue;  // coupling leaves the subdomain: dropped
    const int ck = il.node_color[k];
    double L[NS * NS];
    {
      double a[NS * NS], di[NS * NS];
#pragma unroll
      for (int i = 0; i < NS * NS; ++i) { a[i] = double(il.ilu[(size_t)s * NS * NS + i]); di[i] = double(d.dinv[(size_t)k * NS * NS + i]); }
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
      for (int i = 0; i < NS * NS; ++i) il.ilu[(size_t)s * NS * NS + i] = KT(L[i]);
    }
    const int kb = d.rowptr[k], ke = d.rowptr[k + 1];
    for (int s2 = rb; s2 < re; ++s2) {
      const int j = d.col[s2];
      if (j < sd.K0 || j >= sd.K1 || il.node_color[j] <= ck) continue;
      const int skj = slot_of(d.col, kb, ke, j);
      if (skj < 0) continue;
#pragma unroll
      for (int i = 0; i < NS; ++i)
#pragma unroll
        for (int jj = 0; jj < NS; ++jj) {
          double acc = 0.0;
#pragma unroll
          for (int l = 0; l < NS; ++l) acc += L[i * NS + l] * double(il.ilu[(size_t)skj * NS * NS + l * NS + jj]);
          KT& dst = il.ilu[(size_t)s2 * NS * NS + i * NS + jj];
          dst = KT(double(dst) - acc);
        }
    }
  }
  double a[NS * NS], inv[NS * NS];
#pragma unroll
  for (int i = 0; i < NS * NS; ++i) a[i] = double(il.ilu[(size_t)d.diag[K] * NS * NS + i]);
  small_inverse<NS>(a, inv);
#pragma unroll
  for (int i = 0; i < NS * NS; ++i) d.dinv[(size_t)K * NS * NS + i] = KT(inv[i]);
}

// CTA-local factorisation of the subdomain (copies the subdomain's block rows first)
template <int NS, typename KT>
__device__ void bilu_factor(const Subdomain& sd, const KrylovData<NS, KT>& d, const IluData<KT>& il) {
  const int64_t v0 = (int64_t)d.rowptr[sd.K0] * NS * NS, v1 = (int64_t)d.rowptr[sd.K1] * NS * NS;
  for (int64_t q = v0 + threadIdx.x; q < v1; q += blockDim.x) il.ilu[q] = d.A[q];
  __syncthreads();
  for (int c = 0; c < il.ncolors; ++c) {
    for (int idx = sd.cb[c] + threadIdx.x; idx < sd.ce[c]; idx += blockDim.x) bilu_factor_row<NS, KT>(il.color_nodes[idx], sd, d, il);
    __syncthreads();
  }
}

// CTA-local z = (LU)^-1 y on the subdomain's positions with the ELL couplings
// (couplings that leave the subdomain were packed as 0); ends with __syncthreads
template <int NS, typename KT>
__device__ void bilu_apply_ell(const Subdomain& sd, const KrylovData<NS, KT>& d, const IluData<KT>& il,
                               const KT* __restrict__ y, KT* __restrict__ z) {
  for (int c = 0; c < il.ncolors; ++c) {
    ilu_fwd_positions<NS, KT>(il, d.N, y, z, sd.cb[c], sd.ce[c], threadIdx.x, blockDim.x);
    __syncthreads();
  }
  for (int c = il.ncolors - 1; c >= 0; --c) {
    ilu_bwd_positions<NS, KT>(il, d.dinv, d.N, z, sd.cb[c], sd.ce[c], threadIdx.x, blockDim.x);
    __syncthreads();
  }
}

template <class Team>
__device__ __forceinline__ int team_cta(const Team& t);
template <>
__device__ __forceinline__ int team_cta<GroupTeam>(const GroupTeam& t) { return t.bid; }
template <>
__device__ __forceinline__ int team_cta<CtaTeam>(const CtaTeam&) { return 0; }
template <class Team>
__device__ __forceinline__ int team_ncta(const Team& t);
template <>
__device__ __forceinline__ int team_ncta<GroupTeam>(const GroupTeam& t) { return t.nblk; }
template <>
__device__ __forceinline__ int team_ncta<CtaTeam>(const CtaTeam&) { return 1; }

// Left subdomain-ILU0 BiCGStab: solves A x = b (x starts at 0); all vector work
// on the CTA's own subdomain rows; `iters` is set on every thread.
template <class Team, int NS, int LPR, typename KT>
__device__ bool team_bicgstab_bilu(Team& team, const KrylovData<NS, KT>& d, const IluData<KT>& il, const KrylovCtl& c,
                                   int& iters) {
  iters = 0;
  __shared__ Subdomain sd;
  if (threadIdx.x == 0) make_subdomain<NS, KT>(sd, d.N, team_cta(team), team_ncta(team), il);
  __syncthreads();
  const int64_t q0 = (int64_t)sd.K0 * NS, q1 = (int64_t)sd.K1 * NS;
  bilu_factor<NS, KT>(sd, d, il);
  pack_ell_rows<NS, KT>(d, sd.K0, sd.K1, threadIdx.x, blockDim.x);
  for (int c = 0; c < il.ncolors && c < kMaxColors; ++c)
    pack_ilu_positions<NS, KT>(il, d.N, sd.cb[c], sd.ce[c], threadIdx.x, blockDim.x, sd.K0, sd.K1);
  __syncthreads();
  if (d.cd.nc && !team_coarse_setup<Team, NS, KT>(team, d.cd, d.col, d.A)) return false;
  bilu_apply_ell<NS, KT>(sd, d, il, d.b, d.r);  // r = M^-1 b (subdomain-local)
  if (d.cd.nc && !team_coarse_add_range<Team, NS, KT>(team, d.cd, d.b, d.r, q0, q1)) return false;
  double acc1[1] = {0.0};
  acc_t<KT> a1 = 0;
  for (int64_t q = q0 + threadIdx.x; q < q1; q += blockDim.x) {
    const KT rq = d.r[q];
    d.r0[q] = rq; d.x[q] = KT(0); d.p[q] = KT(0); d.v[q] = KT(0);
    a1 += acc_t<KT>(rq) * acc_t<KT>(rq);
  }
  acc1[0] = double(a1);
  double red1[1];
  if (!team.template reduce<1>(acc1, 0u, red1)) return false;
  double rho = red1[0];
  const double tol = fmax(c.abstol, c.reltol * sqrt(red1[0]));
  const double tol2 = tol * tol;
  double rr = red1[0], alpha = 1.0, omega = 1.0, beta = 0.0;
  if (!(rr > tol2) || c.maxiters <= 0 || isnan(rr)) return true;
  int it = 0, brk = 0;
  while (true) {
    vec_p_update<KT>(d.p, d.r, d.v, KT(beta), KT(omega), q0 + threadIdx.x, q1, blockDim.x);
    if (!team.sync()) return false;  // SpMV reads neighbouring subdomains' p
    spmv_ell_rows<NS, KT>(d, d.p, il.y, sd.K0, sd.K1, threadIdx.x, blockDim.x);
    __syncthreads();
    bilu_apply_ell<NS, KT>(sd, d, il, il.y, d.v);
    if (d.cd.nc && !team_coarse_add_range<Team, NS, KT>(team, d.cd, il.y, d.v, q0, q1)) return false;
    double acc[2] = {0.0, 0.0}, red[2];
    vec_dots<KT>(d.r0, d.v, q0 + threadIdx.x, q1, blockDim.x, acc);
    acc[1] = 0.0;
    if (!team.template reduce<2>(acc, 0u, red)) return false;
    if (red[0] == 0.0 || isnan(red[0])) { brk = 1; alpha = 0.0; }
    else alpha = rho / red[0];
    vec_s_update<KT>(d.s, d.r, d.v, KT(alpha), q0 + threadIdx.x, q1, blockDim.x);
    if (!team.sync()) return false;  // SpMV reads neighbouring subdomains' s
    spmv_ell_rows<NS, KT>(d, d.s, il.y, sd.K0, sd.K1, threadIdx.x, blockDim.x);
    __syncthreads();
    bilu_apply_ell<NS, KT>(sd, d, il, il.y, d.t);
    if (d.cd.nc && !team_coarse_add_range<Team, NS, KT>(team, d.cd, il.y, d.t, q0, q1)) return false;
    acc[0] = acc[1] = 0.0;
    vec_dots<KT>(d.s, d.t, q0 + threadIdx.x, q1, blockDim.x, acc);
    if (!team.template reduce<2>(acc, 0u, red)) return false;
    omega = red[1] > 0.0 ? red[0] / red[1] : 0.0;
    acc[0] = acc[1] = 0.0;
    vec_xr_update<KT>(d.x, d.r, d.p, d.s, d.t, d.r0, KT(alpha), KT(omega), q0 + threadIdx.x, q1, blockDim.x, acc);
    if (!team.template reduce<2>(acc, 0u, red)) return false;
    ++it;
    rr = red[1];
    brk = brk || red[0] == 0.0 || omega == 0.0 || isnan(rr);
    if (brk || !(rr > tol2) || it >= c.maxiters) break;
    beta = (red[0] / rho) * (alpha / omega);
    rho = red[0];
  }
  iters = it;
  return true;
}

}  // namespace vfvm
