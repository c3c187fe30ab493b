// Team-generic, left-preconditioned BiCGStab with block-Jacobi (inverse of the
// NS x NS diagonal blocks) on a block-CSR matrix.  Runs inside one persistent
// launch: a whole grid (GridTeam) or one CTA (CtaTeam).
#pragma once
#include "vfvm_coarse.cuh"
#include "vfvm_team.cuh"

namespace vfvm {

template <int NS, typename KT>
struct KrylovData {
  int N;                    // block rows
  const int* rowptr;        // N+1
  const int* col;           // block columns
  const KT* A;              // nnzb * NS * NS, row-major blocks
  const int* diag;          // slot of the diagonal block per row
  KT* dinv;                 // N * NS * NS
  const KT* b;              // N * NS
  KT* x;                    // N * NS (output; initial guess 0)
  KT *r, *r0, *p, *v, *s, *t;
  CoarseData cd;            // coarse-grid correction stage (cd.nc == 0: none)
  // ELL copy of the matrix (entry w of row K at w*N + K; column -1 = padding)
  int ew;
  const int* ell_col;
  const int* ell_slot;      // block slot of each ELL entry
  KT* ell_val;              // packed from A after each assembly
  KT* gv;                   // GMRES Krylov basis: (restart + 1) vectors of N * NS (null: BiCGStab only)
};

struct KrylovCtl {
  double reltol, abstol;
  int maxiters;
};

struct KrylovOut {
  int iters, status, breakdown, pad;
  double res0, res;
};

template <int NS>
__device__ __forceinline__ void small_inverse(const double* a, double* inv) {
  if constexpr (NS == 1) {
    inv[0] = 1.0 / a[0];
  } else {
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
      for (int r = c + 1; r < NS; ++r)
        if (fabs(m[r][c]) > best) { best = fabs(m[r][c]); piv = r; }
      if (piv != c) {
#pragma unroll
        for (int j = 0; j < 2 * NS; ++j) { const double tmp = m[c][j]; m[c][j] = m[piv][j]; m[piv][j] = tmp; }
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
}

// out_K = Dinv_K (A x)_K for the rows of this team; returns the thread's
// contributions sum_K w_K . out_K (acc[0]) and out_K . out_K (acc[1]).
// LPR lanes cooperate on one block row; all lanes of a warp run the same trip count.
template <class Team, int NS, int LPR, typename KT>
__device__ __forceinline__ void team_spmv_jac(Team& team, const KrylovData<NS, KT>& d, const KT* __restrict__ xin,
                                              KT* __restrict__ out, const KT* __restrict__ w, double (&acc)[2]) {
  const int sub = team.rank() % LPR;
  const int group = team.rank() / LPR;
  const int ngroups = team.size() / LPR;
  const int warp_first_group = (team.rank() & ~31) / LPR;
  acc_t<KT> a0 = 0, a1 = 0;
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
      const KT* D = d.dinv + (size_t)K * NS * NS;
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
  acc[0] += double(a0);
  acc[1] += double(a1);
}

// Solves A x = b (x starts at 0).  Returns false if a team barrier expired.
template <class Team, int NS, int LPR, typename KT>
__device__ bool team_bicgstab_jacobi(Team& team, const KrylovData<NS, KT>& d, const KrylovCtl& c, KrylovOut* out,
                                     int* iters_all = nullptr) {
  const int64_t n = (int64_t)d.N * NS;
  if (iters_all) *iters_all = 0;
  // block-Jacobi setup, x = 0, r = Dinv b, r0 = r
  double acc1[1] = {0.0};
  for (int K = team.rank(); K < d.N; K += team.size()) {
    double a[NS * NS], inv[NS * NS];
    const KT* Ad = d.A + (size_t)d.diag[K] * NS * NS;
#pragma unroll
    for (int i = 0; i < NS * NS; ++i) a[i] = double(Ad[i]);
    small_inverse<NS>(a, inv);
#pragma unroll
    for (int i = 0; i < NS * NS; ++i) d.dinv[(size_t)K * NS * NS + i] = KT(inv[i]);
#pragma unroll
    for (int i = 0; i < NS; ++i) {
      double z = 0.0;
#pragma unroll
      for (int j = 0; j < NS; ++j) z += inv[i * NS + j] * double(d.b[(size_t)K * NS + j]);
      const size_t q = (size_t)K * NS + i;
      d.x[q] = KT(0); d.p[q] = KT(0); d.v[q] = KT(0);
      d.r[q] = KT(z); d.r0[q] = KT(z);
      acc1[0] += double(KT(z)) * double(KT(z));
    }
  }
  double red1[1];
  if (!team.template reduce<1>(acc1, 0u, red1)) return false;
  double rho = red1[0];
  const double tol = fmax(c.abstol, c.reltol * sqrt(red1[0]));
  const double tol2 = tol * tol;
  int it = 0, brk = 0;
  double rr = red1[0], alpha = 1.0, omega = 1.0, beta = 0.0;
  if (!(rr > tol2) || c.maxiters <= 0 || isnan(rr)) {
    if (team.rank() == 0 && out) { out->iters = 0; out->res0 = sqrt(red1[0]); out->res = sqrt(rr); out->breakdown = 0; }
    return true;
  }
  while (true) {
    // p = r + beta (p - omega v)
    for (int64_t q = team.rank(); q < n; q += team.size())
      d.p[q] = d.r[q] + KT(beta) * (d.p[q] - KT(omega) * d.v[q]);
    if (!team.sync()) return false;
    // v = Dinv A p ; alpha = rho / (r0 . v)
    double acc[2] = {0.0, 0.0};
    team_spmv_jac<Team, NS, LPR, KT>(team, d, d.p, d.v, d.r0, acc);
    double red[2];
    if (!team.template reduce<2>(acc, 0u, red)) return false;
    if (red[0] == 0.0 || isnan(red[0])) { brk = 1; alpha = 0.0; }
    else alpha = rho / red[0];
    // s = r - alpha v
    for (int64_t q = team.rank(); q < n; q += team.size()) d.s[q] = d.r[q] - KT(alpha) * d.v[q];
    if (!team.sync()) return false;
    // t = Dinv A s ; omega = (t.s)/(t.t)
    acc[0] = acc[1] = 0.0;
    team_spmv_jac<Team, NS, LPR, KT>(team, d, d.s, d.t, d.s, acc);
    if (!team.template reduce<2>(acc, 0u, red)) return false;
    omega = red[1] > 0.0 ? red[0] / red[1] : 0.0;
    // x += alpha p + omega s ; r = s - omega t
    acc_t<KT> a0 = 0, a1 = 0;
    for (int64_t q = team.rank(); q < n; q += team.size()) {
      d.x[q] += KT(alpha) * d.p[q] + KT(omega) * d.s[q];
      const KT rn = d.s[q] - KT(omega) * d.t[q];
      d.r[q] = rn;
      a0 += acc_t<KT>(d.r0[q]) * acc_t<KT>(rn);
      a1 += acc_t<KT>(rn) * acc_t<KT>(rn);
    }
    acc[0] = double(a0);
    acc[1] = double(a1);
    if (!team.template reduce<2>(acc, 0u, red)) return false;
    ++it;
    rr = red[1];
    brk = brk || red[0] == 0.0 || omega == 0.0 || isnan(rr);
    if (brk || !(rr > tol2) || it >= c.maxiters) break;
    beta = (red[0] / rho) * (alpha / omega);
    rho = red[0];
  }
  if (team.rank() == 0 && out) { out->iters = it; out->res0 = sqrt(red1[0]); out->res = sqrt(rr); out->breakdown = brk; }
  if (iters_all) *iters_all = it;
  return true;
}

}  // namespace vfvm
