// Coarse-grid correction: the second stage of the preconditioner.
//
//   M^-1 r = M_1^-1 r + P A_c^-1 P^T r
//
// M_1 is the one-level preconditioner (ILU0 or block Jacobi); P is piecewise
// constant on aggregates of nodes (boxes of a coarse tensor grid over the
// grid's bounding box), per species, restricted to the dofs without a
// Dirichlet penalty; A_c = P^T A P is the Galerkin coarse matrix, assembled on
// the device after every Jacobian assembly and inverted densely in FP32 by
// Gauss-Jordan elimination with partial pivoting inside one CTA's shared
// memory.  The one-level ILU0 needs O(grid width) Krylov iterations; the
// coarse stage removes the smooth error components that cause this.
#pragma once
#include "vfvm_common.cuh"

namespace vfvm {

constexpr int kCoarseMax = 208;  // coarse unknowns: the dense FP32 matrix (173 KB) fits one CTA's shared memory

inline size_t coarse_smem_bytes(int nc) { return ((size_t)nc * nc + 2 * (size_t)nc + 64) * sizeof(float); }

// Device view of a coarse space.  Vectors written inside a persistent launch by
// other CTAs (A, rc, zc, the restricted input) are read with __ldcg (L2).
struct CoarseData {
  int nagg = 0, nc = 0;          // aggregates, coarse unknowns (nagg * NS); nc == 0: no coarse stage
  int npairs = 0;
  const uint8_t* dirdof = nullptr;    // N * NS: 1 where a Dirichlet penalty acts (excluded from P)
  const int* agg_of_node = nullptr;   // N
  const int* agg_ptr = nullptr;       // nagg + 1
  const int* agg_nodes = nullptr;     // nodes grouped by aggregate
  const int* pair_ptr = nullptr;      // npairs + 1
  const int* pair_ij = nullptr;       // npairs: I * nagg + J
  const int* pair_slot = nullptr;     // nnzb: block slots grouped by aggregate pair
  const int* pair_row = nullptr;      // nnzb: block row of each listed slot
  float* A = nullptr;                 // nc * nc: Galerkin matrix, overwritten by its inverse
  float* rc = nullptr;                // nc: restricted vector
  float* zc = nullptr;                // nc: coarse solution
};

// One warp per aggregate pair: A_c[(I,a),(J,b)] = sum of the (a,b) entries of the
// listed blocks whose row dof (node, a) and column dof (col, b) are free.
// Warp `w` of `nw` in the team/grid; deterministic (fixed order + shuffle tree).
template <int NS, typename MT>
__device__ __forceinline__ void coarse_galerkin_warps(const CoarseData& cd, const int* __restrict__ col,
                                                      const MT* __restrict__ J, int w, int nw) {
  const uint8_t* __restrict__ dirdof = cd.dirdof;
  const int lane = threadIdx.x & 31;
  for (int p = w; p < cd.npairs; p += nw) {
    const int I = cd.pair_ij[p] / cd.nagg, Jg = cd.pair_ij[p] % cd.nagg;
    const int b = cd.pair_ptr[p], e = cd.pair_ptr[p + 1];
    float acc[NS * NS];
#pragma unroll
    for (int k = 0; k < NS * NS; ++k) acc[k] = 0.f;
    for (int q = b + lane; q < e; q += 32) {
      const int s = cd.pair_slot[q], r = cd.pair_row[q], c = col[s];
#pragma unroll
      for (int a = 0; a < NS; ++a)
#pragma unroll
        for (int bb = 0; bb < NS; ++bb)
          if (!dirdof[(int64_t)r * NS + a] && !dirdof[(int64_t)c * NS + bb])
            acc[a * NS + bb] += float(__ldcg(&J[(int64_t)s * NS * NS + a * NS + bb]));
    }
#pragma unroll
    for (int k = 0; k < NS * NS; ++k)
      for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_down_sync(0xffffffffu, acc[k], o);
    if (lane == 0) {
#pragma unroll
      for (int a = 0; a < NS; ++a)
#pragma unroll
        for (int bb = 0; bb < NS; ++bb) cd.A[(size_t)(I * NS + a) * cd.nc + Jg * NS + bb] = acc[a * NS + bb];
    }
  }
}

// In-place inverse of the nc x nc matrix in shared memory `a` by Gauss-Jordan
// elimination with partial pivoting, by one CTA.  Coarse unknowns without any
// free fine dof have an all-zero row and column: they get a unit pivot and a
// zero inverse entry (they drop out).  A pivot below 1e-7 of the largest
// diagonal entry (a singular direction, e.g. the constants of a pure Neumann
// problem) is skipped in the same way.  scratch: 2 * nc + 64 floats.
__device__ __forceinline__ void coarse_invert_smem(float* a, int nc, float* scratch) {
  float* colk = scratch;          // nc: column k before elimination
  int* perm = reinterpret_cast<int*>(scratch + nc);  // nc: row swapped into position k
  float* red = scratch + 2 * nc;  // 64: pivot search / flags
  const int tid = threadIdx.x, nt = blockDim.x;
  // scale for the singular-pivot test and empty coarse unknowns
  if (tid < 32) {
    float m = 0.f;
    for (int i = tid; i < nc; i += 32) m = fmaxf(m, fabsf(a[i * nc + i]));
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (tid == 0) red[40] = m;
  }
  __syncthreads();
  const float tiny = 1e-7f * red[40];
  for (int i = tid; i < nc; i += nt)
    if (a[i * nc + i] == 0.f) {
      bool empty = true;
      for (int j = 0; j < nc; ++j) empty = empty && a[i * nc + j] == 0.f && a[j * nc + i] == 0.f;
      if (empty) a[i * nc + i] = 1.f;
    }
  __syncthreads();
  for (int k = 0; k < nc; ++k) {
    // pivot: largest |a[i][k]|, i >= k (warp 0; ties -> smallest i)
    if (tid < 32) {
      float best = -1.f;
      int bi = k;
      for (int i = k + tid; i < nc; i += 32) {
        const float v = fabsf(a[i * nc + k]);
        if (v > best) { best = v; bi = i; }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const float ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      if (tid == 0) { perm[k] = bi; red[0] = best; }
    }
    __syncthreads();
    const int p = perm[k];
    const bool skip = !(red[0] > tiny);
    if (p != k)
      for (int j = tid; j < nc; j += nt) {
        const float t = a[k * nc + j];
        a[k * nc + j] = a[p * nc + j];
        a[p * nc + j] = t;
      }
    __syncthreads();
    if (skip) {  // singular direction: zero row and column k of the inverse
      for (int j = tid; j < nc; j += nt) { a[k * nc + j] = 0.f; a[j * nc + k] = 0.f; }
      __syncthreads();
      continue;
    }
    for (int i = tid; i < nc; i += nt) colk[i] = a[i * nc + k];
    __syncthreads();
    const float pinv = 1.f / colk[k];
    for (int j = tid; j < nc; j += nt) a[k * nc + j] = (j == k ? 1.f : a[k * nc + j]) * pinv;
    __syncthreads();
    {
      const int lane = tid & 31, nwp = nt >> 5;
      for (int i = tid >> 5; i < nc; i += nwp) {
        if (i == k) continue;
        const float f = colk[i];
        float* ai = a + (size_t)i * nc;
        for (int j = lane; j < nc; j += 32) ai[j] = (j == k ? 0.f : ai[j]) - f * a[k * nc + j];
      }
    }
    __syncthreads();
  }
  // undo the row swaps as column swaps, last first
  for (int k = nc - 1; k >= 0; --k) {
    const int p = perm[k];
    if (p != k)
      for (int i = tid; i < nc; i += nt) {
        const float t = a[i * nc + k];
        a[i * nc + k] = a[i * nc + p];
        a[i * nc + p] = t;
      }
    __syncthreads();
  }
}

// Restriction by warps: rc[I*NS+a] = sum of y over the free dofs (node, a), node in I.
template <int NS, typename KT>
__device__ __forceinline__ void coarse_restrict_warps(const CoarseData& cd, const KT* __restrict__ y, int w, int nw) {
  const uint8_t* __restrict__ dirdof = cd.dirdof;
  const int lane = threadIdx.x & 31;
  for (int I = w; I < cd.nagg; I += nw) {
    float acc[NS];
#pragma unroll
    for (int a = 0; a < NS; ++a) acc[a] = 0.f;
    // four of the lane's nodes per pass, their loads issued before the sums
    // (the lane's summation order is unchanged)
    const int q1 = cd.agg_ptr[I + 1];
    for (int q = cd.agg_ptr[I] + lane; q < q1; q += 4 * 32) {
      int64_t K[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) K[u] = q + 32 * u < q1 ? (int64_t)cd.agg_nodes[q + 32 * u] : -1;
      float yv[4][NS];
      uint8_t dv[4][NS];
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int a = 0; a < NS; ++a) {
          dv[u][a] = K[u] >= 0 ? dirdof[K[u] * NS + a] : (uint8_t)1;
          yv[u][a] = K[u] >= 0 ? float(__ldcg(&y[K[u] * NS + a])) : 0.f;
        }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int a = 0; a < NS; ++a)
          if (!dv[u][a]) acc[a] += yv[u][a];
    }
#pragma unroll
    for (int a = 0; a < NS; ++a)
      for (int o = 16; o > 0; o >>= 1) acc[a] += __shfl_down_sync(0xffffffffu, acc[a], o);
    if (lane == 0) {
#pragma unroll
      for (int a = 0; a < NS; ++a) cd.rc[I * NS + a] = acc[a];
    }
  }
}

// Coarse solve by warps: zc = A_c^-1 rc (A holds the inverse), one warp per row.
__device__ __forceinline__ void coarse_matvec_warps(const CoarseData& cd, int w, int nw) {
  const int lane = threadIdx.x & 31;
  for (int i = w; i < cd.nc; i += nw) {
    float acc = 0.f;
    for (int j = lane; j < cd.nc; j += 32) acc += __ldcg(&cd.A[(size_t)i * cd.nc + j]) * __ldcg(&cd.rc[j]);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) cd.zc[i] = acc;
  }
}

// z[q] += zc[agg(node(q)) * NS + species(q)] on the free dofs.
template <int NS, typename KT>
__device__ __forceinline__ void coarse_prolong_add(const CoarseData& cd, KT* __restrict__ z, int64_t q) {
  if (cd.dirdof[q]) return;
  const int64_t K = q / NS;
  const int a = (int)(q - K * NS);
  z[q] += KT(__ldcg(&cd.zc[cd.agg_of_node[K] * NS + a]));
}

// ---- standalone kernels (graph engine) ----

template <int NS, typename MT>
__global__ void coarse_galerkin_kernel(CoarseData cd, const int* __restrict__ col, const MT* __restrict__ J) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  coarse_galerkin_warps<NS, MT>(cd, col, J, w, nw);
}

static __global__ void coarse_invert_kernel(float* A, int nc) {
  extern __shared__ float csm[];
  for (int e = threadIdx.x; e < nc * nc; e += blockDim.x) csm[e] = A[e];
  __syncthreads();
  coarse_invert_smem(csm, nc, csm + (size_t)nc * nc);
  for (int e = threadIdx.x; e < nc * nc; e += blockDim.x) A[e] = csm[e];
}

template <int NS, typename KT>
__global__ void coarse_restrict_kernel(CoarseData cd, const KT* __restrict__ y) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  coarse_restrict_warps<NS, KT>(cd, y, w, nw);
}

static __global__ void coarse_matvec_kernel(CoarseData cd) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  coarse_matvec_warps(cd, w, nw);
}

template <int NS, typename KT>
__global__ void coarse_prolong_kernel(CoarseData cd, KT* __restrict__ z, int64_t n) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
    coarse_prolong_add<NS, KT>(cd, z, q);
}

// ---- team versions (persistent and batched engines) ----

// Galerkin assembly by all warps of the team, inversion by the team's first CTA
// in its dynamic shared memory `smem` (coarse_smem_bytes(nc)).
template <class Team, int NS, typename MT>
__device__ bool team_coarse_setup(Team& team, const CoarseData& cd, const int* col, const MT* J) {
  extern __shared__ float vfvm_coarse_smem[];
  const bool first_cta = team.rank() < (int)blockDim.x;
  float* smem = vfvm_coarse_smem;
  for (int64_t e = team.rank(); e < (int64_t)cd.nc * cd.nc; e += team.size()) cd.A[e] = 0.f;
  if (!team.sync()) return false;
  coarse_galerkin_warps<NS, MT>(cd, col, J, team.rank() >> 5, team.size() >> 5);
  if (!team.sync()) return false;
  if (first_cta) {
    for (int e = threadIdx.x; e < cd.nc * cd.nc; e += blockDim.x) smem[e] = __ldcg(&cd.A[e]);
    __syncthreads();
    coarse_invert_smem(smem, cd.nc, smem + (size_t)cd.nc * cd.nc);
    for (int e = threadIdx.x; e < cd.nc * cd.nc; e += blockDim.x) cd.A[e] = smem[e];
  }
  return team.sync();
}

// out += P A_c^-1 P^T in.  The prolongation writes out[q] for q = rank + k*size,
// the ownership of the team's vector loops, so no barrier follows it.
template <class Team, int NS, typename KT>
__device__ bool team_coarse_add(Team& team, const CoarseData& cd, const KT* in, KT* out, int64_t n) {
  coarse_restrict_warps<NS, KT>(cd, in, team.rank() >> 5, team.size() >> 5);
  if (!team.sync()) return false;
  coarse_matvec_warps(cd, team.rank() >> 5, team.size() >> 5);
  if (!team.sync()) return false;
  for (int64_t q = team.rank(); q < n; q += team.size()) coarse_prolong_add<NS, KT>(cd, out, q);
  return true;
}

// Subdomain variant: `in` was written CTA-locally, so a team barrier comes
// first; the prolongation covers this CTA's dof range [q0, q1).
template <class Team, int NS, typename KT>
__device__ bool team_coarse_add_range(Team& team, const CoarseData& cd, const KT* in, KT* out, int64_t q0,
                                      int64_t q1) {
  if (!team.sync()) return false;
  coarse_restrict_warps<NS, KT>(cd, in, team.rank() >> 5, team.size() >> 5);
  if (!team.sync()) return false;
  coarse_matvec_warps(cd, team.rank() >> 5, team.size() >> 5);
  if (!team.sync()) return false;
  for (int64_t q = q0 + threadIdx.x; q < q1; q += blockDim.x) coarse_prolong_add<NS, KT>(cd, out, q);
  __syncthreads();
  return true;
}

}  // namespace vfvm
