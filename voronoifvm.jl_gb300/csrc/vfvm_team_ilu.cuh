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
};

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

// z = (LU)^-1 y; ends with a team barrier
template <class Team, int NS, typename KT>
__device__ bool team_ilu_apply(Team& team, const KrylovData<NS, KT>& d, const IluData<KT>& il, const KT* __restrict__ y,
                               KT* __restrict__ z) {
  for (int c = 0; c < il.ncolors; ++c) {
    for (int idx = il.color_ptr[c] + team.rank(); idx < il.color_ptr[c + 1]; idx += team.size()) {
      const int K = il.color_nodes[idx];
      KT w[NS];
#pragma unroll
      for (int i = 0; i < NS; ++i) w[i] = y[(size_t)K * NS + i];
      for (int q = il.lower_ptr[K]; q < il.lower_ptr[K + 1]; ++q) {
        const int s = il.lower_slots[q];
        const int k = d.col[s];
        const KT* Lb = il.ilu + (size_t)s * NS * NS;
#pragma unroll
        for (int j = 0; j < NS; ++j) {
          const KT wk = z[(size_t)k * NS + j];
#pragma unroll
          for (int i = 0; i < NS; ++i) w[i] -= Lb[i * NS + j] * wk;
        }
      }
#pragma unroll
      for (int i = 0; i < NS; ++i) z[(size_t)K * NS + i] = w[i];
    }
    if (!team.sync()) return false;
  }
  for (int c = il.ncolors - 1; c >= 0; --c) {
    for (int idx = il.color_ptr[c] + team.rank(); idx < il.color_ptr[c + 1]; idx += team.size()) {
      const int K = il.color_nodes[idx];
      KT w[NS];
#pragma unroll
      for (int i = 0; i < NS; ++i) w[i] = z[(size_t)K * NS + i];
      for (int s = d.rowptr[K]; s < d.rowptr[K + 1]; ++s) {
        const int j = d.col[s];
        if (il.node_color[j] <= c) continue;
        const KT* Ub = il.ilu + (size_t)s * NS * NS;
#pragma unroll
        for (int jj = 0; jj < NS; ++jj) {
          const KT zj = z[(size_t)j * NS + jj];
#pragma unroll
          for (int i = 0; i < NS; ++i) w[i] -= Ub[i * NS + jj] * zj;
        }
      }
      const KT* D = d.dinv + (size_t)K * NS * NS;
#pragma unroll
      for (int i = 0; i < NS; ++i) {
        KT acc = KT(0);
#pragma unroll
        for (int j = 0; j < NS; ++j) acc += D[i * NS + j] * w[j];
        z[(size_t)K * NS + i] = acc;
      }
    }
    if (!team.sync()) return false;
  }
  return true;
}

// out = A x (plain), LPR lanes per block row
template <class Team, int NS, int LPR, typename KT>
__device__ __forceinline__ void team_spmv(Team& team, const KrylovData<NS, KT>& d, const KT* __restrict__ xin,
                                          KT* __restrict__ out) {
  const int sub = team.rank() % LPR;
  const int group = team.rank() / LPR;
  const int ngroups = team.size() / LPR;
  const int warp_first_group = (team.rank() & ~31) / LPR;
  for (int base = warp_first_group; base < d.N; base += ngroups) {
    const int K = base + (group - warp_first_group);
    KT y[NS];
#pragma unroll
    for (int i = 0; i < NS; ++i) y[i] = KT(0);
    if (K < d.N) {
      const int beg = d.rowptr[K], end = d.rowptr[K + 1];
      for (int s = beg + sub; s < end; s += LPR) {
        const int m = d.col[s];
        const KT* Ab = d.A + (size_t)s * NS * NS;
#pragma unroll
        for (int j = 0; j < NS; ++j) {
          const KT xm = xin[(size_t)m * NS + j];
#pragma unroll
          for (int i = 0; i < NS; ++i) y[i] += Ab[i * NS + j] * xm;
        }
      }
    }
#pragma unroll
    for (int i = 0; i < NS; ++i)
#pragma unroll
      for (int o = LPR / 2; o > 0; o >>= 1) y[i] += __shfl_down_sync(0xffffffffu, y[i], o, LPR);
    if (K < d.N && sub == 0) {
#pragma unroll
      for (int i = 0; i < NS; ++i) out[(size_t)K * NS + i] = y[i];
    }
  }
}

// dot products w.z and z.z over the team's dofs
template <class Team, typename KT>
__device__ __forceinline__ void team_dots(Team& team, int64_t n, const KT* __restrict__ w, const KT* __restrict__ z,
                                          double (&acc)[2]) {
  for (int64_t q = team.rank(); q < n; q += team.size()) {
    const double zz = double(z[q]);
    acc[0] += double(w[q]) * zz;
    acc[1] += zz * zz;
  }
}

// Left-ILU0-preconditioned BiCGStab: solves A x = b (x starts at 0).  `iters`
// receives the iteration count on every thread.  Returns false if a barrier expired.
template <class Team, int NS, int LPR, typename KT>
__device__ bool team_bicgstab_ilu(Team& team, const KrylovData<NS, KT>& d, const IluData<KT>& il, const KrylovCtl& c,
                                  int64_t nvals, int& iters) {
  const int64_t n = (int64_t)d.N * NS;
  iters = 0;
  if (!team_ilu_factor<Team, NS, KT>(team, d, il, nvals)) return false;
  if (d.cd.nc && !team_coarse_setup<Team, NS, KT>(team, d.cd, d.col, d.A)) return false;
  if (!team_ilu_apply<Team, NS, KT>(team, d, il, d.b, d.r)) return false;  // r = M^-1 b
  if (d.cd.nc && !team_coarse_add<Team, NS, KT>(team, d.cd, d.b, d.r, n)) return false;
  double acc1[1] = {0.0};
  for (int64_t q = team.rank(); q < n; q += team.size()) {
    const KT rq = d.r[q];
    d.r0[q] = rq; d.x[q] = KT(0); d.p[q] = KT(0); d.v[q] = KT(0);
    acc1[0] += double(rq) * double(rq);
  }
  double red1[1];
  if (!team.template reduce<1>(acc1, 0u, red1)) return false;
  double rho = red1[0];
  const double tol = fmax(c.abstol, c.reltol * sqrt(red1[0]));
  const double tol2 = tol * tol;
  double rr = red1[0], alpha = 1.0, omega = 1.0, beta = 0.0;
  if (!(rr > tol2) || c.maxiters <= 0 || isnan(rr)) return true;
  int it = 0, brk = 0;
  while (true) {
    for (int64_t q = team.rank(); q < n; q += team.size()) d.p[q] = d.r[q] + KT(beta) * (d.p[q] - KT(omega) * d.v[q]);
    if (!team.sync()) return false;
    team_spmv<Team, NS, LPR, KT>(team, d, d.p, il.y);
    if (!team.sync()) return false;
    if (!team_ilu_apply<Team, NS, KT>(team, d, il, il.y, d.v)) return false;
    if (d.cd.nc && !team_coarse_add<Team, NS, KT>(team, d.cd, il.y, d.v, n)) return false;
    double acc[2] = {0.0, 0.0}, red[2];
    team_dots<Team, KT>(team, n, d.r0, d.v, acc);
    if (!team.template reduce<2>(acc, 0u, red)) return false;
    if (red[0] == 0.0 || isnan(red[0])) { brk = 1; alpha = 0.0; }
    else alpha = rho / red[0];
    for (int64_t q = team.rank(); q < n; q += team.size()) d.s[q] = d.r[q] - KT(alpha) * d.v[q];
    if (!team.sync()) return false;
    team_spmv<Team, NS, LPR, KT>(team, d, d.s, il.y);
    if (!team.sync()) return false;
    if (!team_ilu_apply<Team, NS, KT>(team, d, il, il.y, d.t)) return false;
    if (d.cd.nc && !team_coarse_add<Team, NS, KT>(team, d.cd, il.y, d.t, n)) return false;
    acc[0] = acc[1] = 0.0;
    team_dots<Team, KT>(team, n, d.s, d.t, acc);
    if (!team.template reduce<2>(acc, 0u, red)) return false;
    omega = red[1] > 0.0 ? red[0] / red[1] : 0.0;
    acc[0] = acc[1] = 0.0;
    for (int64_t q = team.rank(); q < n; q += team.size()) {
      d.x[q] += KT(alpha) * d.p[q] + KT(omega) * d.s[q];
      const KT rn = d.s[q] - KT(omega) * d.t[q];
      d.r[q] = rn;
      acc[0] += double(d.r0[q]) * double(rn);
      acc[1] += double(rn) * double(rn);
    }
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

// CTA-local z = (LU)^-1 y on the subdomain's rows; ends with __syncthreads
template <int NS, typename KT>
__device__ void bilu_apply(const Subdomain& sd, const KrylovData<NS, KT>& d, const IluData<KT>& il,
                           const KT* __restrict__ y, KT* __restrict__ z) {
  for (int c = 0; c < il.ncolors; ++c) {
    for (int idx = sd.cb[c] + threadIdx.x; idx < sd.ce[c]; idx += blockDim.x) {
      const int K = il.color_nodes[idx];
      KT w[NS];
#pragma unroll
      for (int i = 0; i < NS; ++i) w[i] = y[(size_t)K * NS + i];
      for (int q = il.lower_ptr[K]; q < il.lower_ptr[K + 1]; ++q) {
        const int s = il.lower_slots[q];
        const int k = d.col[s];
        if (k < sd.K0 || k >= sd.K1) continue;
        const KT* Lb = il.ilu + (size_t)s * NS * NS;
#pragma unroll
        for (int j = 0; j < NS; ++j) {
          const KT wk = z[(size_t)k * NS + j];
#pragma unroll
          for (int i = 0; i < NS; ++i) w[i] -= Lb[i * NS + j] * wk;
        }
      }
#pragma unroll
      for (int i = 0; i < NS; ++i) z[(size_t)K * NS + i] = w[i];
    }
    __syncthreads();
  }
  for (int c = il.ncolors - 1; c >= 0; --c) {
    for (int idx = sd.cb[c] + threadIdx.x; idx < sd.ce[c]; idx += blockDim.x) {
      const int K = il.color_nodes[idx];
      KT w[NS];
#pragma unroll
      for (int i = 0; i < NS; ++i) w[i] = z[(size_t)K * NS + i];
      for (int s = d.rowptr[K]; s < d.rowptr[K + 1]; ++s) {
        const int j = d.col[s];
        if (j < sd.K0 || j >= sd.K1 || il.node_color[j] <= c) continue;
        const KT* Ub = il.ilu + (size_t)s * NS * NS;
#pragma unroll
        for (int jj = 0; jj < NS; ++jj) {
          const KT zj = z[(size_t)j * NS + jj];
#pragma unroll
          for (int i = 0; i < NS; ++i) w[i] -= Ub[i * NS + jj] * zj;
        }
      }
      const KT* D = d.dinv + (size_t)K * NS * NS;
#pragma unroll
      for (int i = 0; i < NS; ++i) {
        KT acc = KT(0);
#pragma unroll
        for (int j = 0; j < NS; ++j) acc += D[i * NS + j] * w[j];
        z[(size_t)K * NS + i] = acc;
      }
    }
    __syncthreads();
  }
}

// y = A x on the subdomain's rows, LPR lanes per block row, CTA threads only
template <int NS, int LPR, typename KT>
__device__ __forceinline__ void cta_spmv(const Subdomain& sd, const KrylovData<NS, KT>& d, const KT* __restrict__ xin,
                                         KT* __restrict__ out) {
  const int sub = threadIdx.x % LPR;
  const int group = threadIdx.x / LPR;
  const int ngroups = blockDim.x / LPR;
  const int warp_first_group = (threadIdx.x & ~31) / LPR;
  for (int base = sd.K0 + warp_first_group; base < sd.K1; base += ngroups) {
    const int K = base + (group - warp_first_group);
    KT y[NS];
#pragma unroll
    for (int i = 0; i < NS; ++i) y[i] = KT(0);
    if (K < sd.K1) {
      const int beg = d.rowptr[K], end = d.rowptr[K + 1];
      for (int s = beg + sub; s < end; s += LPR) {
        const int m = d.col[s];
        const KT* Ab = d.A + (size_t)s * NS * NS;
#pragma unroll
        for (int j = 0; j < NS; ++j) {
          const KT xm = xin[(size_t)m * NS + j];
#pragma unroll
          for (int i = 0; i < NS; ++i) y[i] += Ab[i * NS + j] * xm;
        }
      }
    }
#pragma unroll
    for (int i = 0; i < NS; ++i)
#pragma unroll
      for (int o = LPR / 2; o > 0; o >>= 1) y[i] += __shfl_down_sync(0xffffffffu, y[i], o, LPR);
    if (K < sd.K1 && sub == 0) {
#pragma unroll
      for (int i = 0; i < NS; ++i) out[(size_t)K * NS + i] = y[i];
    }
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
  if (d.cd.nc && !team_coarse_setup<Team, NS, KT>(team, d.cd, d.col, d.A)) return false;
  bilu_apply<NS, KT>(sd, d, il, d.b, d.r);  // r = M^-1 b (subdomain-local)
  if (d.cd.nc && !team_coarse_add_range<Team, NS, KT>(team, d.cd, d.b, d.r, q0, q1)) return false;
  double acc1[1] = {0.0};
  for (int64_t q = q0 + threadIdx.x; q < q1; q += blockDim.x) {
    const KT rq = d.r[q];
    d.r0[q] = rq; d.x[q] = KT(0); d.p[q] = KT(0); d.v[q] = KT(0);
    acc1[0] += double(rq) * double(rq);
  }
  double red1[1];
  if (!team.template reduce<1>(acc1, 0u, red1)) return false;
  double rho = red1[0];
  const double tol = fmax(c.abstol, c.reltol * sqrt(red1[0]));
  const double tol2 = tol * tol;
  double rr = red1[0], alpha = 1.0, omega = 1.0, beta = 0.0;
  if (!(rr > tol2) || c.maxiters <= 0 || isnan(rr)) return true;
  int it = 0, brk = 0;
  while (true) {
    for (int64_t q = q0 + threadIdx.x; q < q1; q += blockDim.x) d.p[q] = d.r[q] + KT(beta) * (d.p[q] - KT(omega) * d.v[q]);
    if (!team.sync()) return false;  // SpMV reads neighbouring subdomains' p
    cta_spmv<NS, LPR, KT>(sd, d, d.p, il.y);
    __syncthreads();
    bilu_apply<NS, KT>(sd, d, il, il.y, d.v);
    if (d.cd.nc && !team_coarse_add_range<Team, NS, KT>(team, d.cd, il.y, d.v, q0, q1)) return false;
    double acc[2] = {0.0, 0.0}, red[2];
    for (int64_t q = q0 + threadIdx.x; q < q1; q += blockDim.x) acc[0] += double(d.r0[q]) * double(d.v[q]);
    if (!team.template reduce<2>(acc, 0u, red)) return false;
    if (red[0] == 0.0 || isnan(red[0])) { brk = 1; alpha = 0.0; }
    else alpha = rho / red[0];
    for (int64_t q = q0 + threadIdx.x; q < q1; q += blockDim.x) d.s[q] = d.r[q] - KT(alpha) * d.v[q];
    if (!team.sync()) return false;  // SpMV reads neighbouring subdomains' s
    cta_spmv<NS, LPR, KT>(sd, d, d.s, il.y);
    __syncthreads();
    bilu_apply<NS, KT>(sd, d, il, il.y, d.t);
    if (d.cd.nc && !team_coarse_add_range<Team, NS, KT>(team, d.cd, il.y, d.t, q0, q1)) return false;
    acc[0] = acc[1] = 0.0;
    for (int64_t q = q0 + threadIdx.x; q < q1; q += blockDim.x) {
      const double tt = double(d.t[q]);
      acc[0] += tt * double(d.s[q]);
      acc[1] += tt * tt;
    }
    if (!team.template reduce<2>(acc, 0u, red)) return false;
    omega = red[1] > 0.0 ? red[0] / red[1] : 0.0;
    acc[0] = acc[1] = 0.0;
    for (int64_t q = q0 + threadIdx.x; q < q1; q += blockDim.x) {
      d.x[q] += KT(alpha) * d.p[q] + KT(omega) * d.s[q];
      const KT rn = d.s[q] - KT(omega) * d.t[q];
      d.r[q] = rn;
      acc[0] += double(d.r0[q]) * double(rn);
      acc[1] += double(rn) * double(rn);
    }
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
