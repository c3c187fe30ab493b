// Team-generic building blocks for persistent solvers.
//
// A "team" is either the whole grid of a cooperative launch (GridTeam: all CTAs
// co-resident, synchronised by a bounded software grid barrier) or one CTA
// (CtaTeam: __syncthreads).  Solver phases are written once against the team
// interface:
//   team.rank(), team.size()         thread index / count inside the team
//   team.sync()                      barrier (returns false if a bounded wait expired)
//   team.reduce<NV>(v, maxmask, out) deterministic all-reduce of NV doubles
// Reductions are deterministic: block partials are combined in block order by
// every block (grid team) or in warp order (CTA team).
#pragma once
#include "vfvm_common.cuh"

namespace vfvm {

constexpr int kTeamMaxWarps = 32;

// block-level reduction of NV doubles; result valid in all threads
template <int NV>
__device__ __forceinline__ void block_allreduce(double (&v)[NV], unsigned maxmask, double (*sh)[kTeamMaxWarps]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double a = v[k];
    for (int o = 16; o > 0; o >>= 1) {
      const double b = __shfl_down_sync(0xffffffffu, a, o);
      a = ((maxmask >> k) & 1) ? fmax(a, b) : a + b;
    }
    if (lane == 0) sh[k][warp] = a;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double a = sh[k][0];
    for (int w = 1; w < nw; ++w) a = ((maxmask >> k) & 1) ? fmax(a, sh[k][w]) : a + sh[k][w];
    v[k] = a;
  }
  __syncthreads();
}

// Barrier/reduction scratch of a team (device memory, zero-initialised):
//   bar[0] arrival counter, bar[1] generation, bar[2] error flag
//   partials: 2 * nblocks * 8 doubles (double-buffered)
struct GridSync {
  unsigned* bar;
  double* partials;
};

constexpr long long kBarrierSpinLimit = 1ll << 24;  // ~0.5-1 s of polling, then VFVM_ERR_TIMEOUT

// A team of `nblk` co-resident CTAs (a whole cooperative grid, or a group of
// CTAs inside one); `bid` is this CTA's index in the team.
struct GroupTeam {
  GridSync gs;
  int nblk, bid;
  unsigned parity;  // alternates the partials buffer between consecutive reductions
  __device__ __forceinline__ int rank() const { return bid * blockDim.x + threadIdx.x; }
  __device__ __forceinline__ int size() const { return nblk * blockDim.x; }

  // Bounded generation barrier over the team's CTAs.  Returns false (on every
  // thread of every CTA that observes it) once any CTA's wait expired.
  __device__ __forceinline__ bool sync() {
    __shared__ int ok_sh;
    __syncthreads();
    if (threadIdx.x == 0) {
      volatile unsigned* vbar = gs.bar;
      const unsigned gen = vbar[1];
      __threadfence();
      const unsigned arrived = atomicAdd(&gs.bar[0], 1u);
      int ok = 1;
      if (arrived == (unsigned)nblk - 1u) {
        gs.bar[0] = 0u;
        __threadfence();
        atomicAdd(&gs.bar[1], 1u);
      } else {
        long long spins = 0;
        while (vbar[1] == gen) {
          if (vbar[2] != 0u || ++spins > kBarrierSpinLimit) { ok = 0; break; }
          if (spins > 64) __nanosleep(32);
        }
        if (!ok) atomicExch(&gs.bar[2], 1u);
      }
      __threadfence();
      ok_sh = ok && (vbar[2] == 0u);
    }
    __syncthreads();
    return ok_sh != 0;
  }

  template <int NV>
  __device__ __forceinline__ bool reduce(double (&v)[NV], unsigned maxmask, double (&out)[NV]) {
    __shared__ double sh[NV][kTeamMaxWarps];
    block_allreduce<NV>(v, maxmask, sh);
    double* buf = gs.partials + (size_t)parity * nblk * 8;
    parity ^= 1u;
    if (threadIdx.x == 0) {
#pragma unroll
      for (int k = 0; k < NV; ++k) buf[bid * 8 + k] = v[k];
    }
    if (!sync()) return false;
    // every CTA sums the partials in CTA order (deterministic, identical everywhere);
    // L2 loads (ld.global.cg) see the other CTAs' fenced writes and can all be in flight
    __shared__ double tot[NV];
    if (threadIdx.x < 32) {
#pragma unroll
      for (int k = 0; k < NV; ++k) {
        double a = 0.0;
        constexpr int kChunk = 8;
        for (int b0 = threadIdx.x; b0 < nblk; b0 += 32 * kChunk) {
          double pv[kChunk];
#pragma unroll
          for (int j = 0; j < kChunk; ++j) {
            const int b = b0 + 32 * j;
            pv[j] = b < nblk ? __ldcg(&buf[b * 8 + k]) : 0.0;
          }
#pragma unroll
          for (int j = 0; j < kChunk; ++j) a = ((maxmask >> k) & 1) ? fmax(a, pv[j]) : a + pv[j];
        }
        for (int o = 16; o > 0; o >>= 1) {
          const double bb = __shfl_down_sync(0xffffffffu, a, o);
          a = ((maxmask >> k) & 1) ? fmax(a, bb) : a + bb;
        }
        if (threadIdx.x == 0) tot[k] = a;
      }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; ++k) out[k] = tot[k];
    __syncthreads();
    return true;
  }
};

// The whole cooperative grid as one team.
__device__ __forceinline__ GroupTeam grid_team(const GridSync& gs) { return GroupTeam{gs, (int)gridDim.x, (int)blockIdx.x, 0u}; }
using GridTeam = GroupTeam;

struct CtaTeam {
  __device__ __forceinline__ int rank() const { return threadIdx.x; }
  __device__ __forceinline__ int size() const { return blockDim.x; }
  __device__ __forceinline__ bool sync() { __syncthreads(); return true; }
  template <int NV>
  __device__ __forceinline__ bool reduce(double (&v)[NV], unsigned maxmask, double (&out)[NV]) {
    __shared__ double sh[NV][kTeamMaxWarps];
    block_allreduce<NV>(v, maxmask, sh);
#pragma unroll
    for (int k = 0; k < NV; ++k) out[k] = v[k];
    return true;
  }
};

}  // namespace vfvm
