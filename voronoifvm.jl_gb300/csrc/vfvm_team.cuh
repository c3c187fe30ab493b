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

// Barrier/reduction scratch of a grid team (device memory, zero-initialised):
//   bar[0] arrival counter, bar[1] generation, bar[2] error flag, bar[3] reduction parity
//   partials: 2 * nblocks * 8 doubles (double-buffered)
struct GridSync {
  unsigned* bar;
  double* partials;
};

constexpr long long kBarrierSpinLimit = 1ll << 24;  // ~0.5-1 s of polling, then VFVM_ERR_TIMEOUT

struct GridTeam {
  GridSync gs;
  unsigned parity;  // alternates the partials buffer between consecutive reductions
  __device__ __forceinline__ int rank() const { return blockIdx.x * blockDim.x + threadIdx.x; }
  __device__ __forceinline__ int size() const { return gridDim.x * blockDim.x; }
  __device__ __forceinline__ int nblocks() const { return gridDim.x; }

  // Bounded sense-free generation barrier.  Returns false (on every thread of
  // every block that observes it) once any block's wait expired.
  __device__ __forceinline__ bool sync() {
    __shared__ int ok_sh;
    __syncthreads();
    if (threadIdx.x == 0) {
      volatile unsigned* vbar = gs.bar;
      const unsigned gen = vbar[1];
      __threadfence();
      const unsigned arrived = atomicAdd(&gs.bar[0], 1u);
      int ok = 1;
      if (arrived == gridDim.x - 1) {
        gs.bar[0] = 0u;
        __threadfence();
        atomicAdd(&gs.bar[1], 1u);
      } else {
        long long spins = 0;
        while (vbar[1] == gen) {
          if (vbar[2] != 0u || ++spins > kBarrierSpinLimit) { ok = 0; break; }
          __nanosleep(64);
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
    double* buf = gs.partials + (size_t)parity * gridDim.x * 8;
    parity ^= 1u;
    if (threadIdx.x == 0) {
#pragma unroll
      for (int k = 0; k < NV; ++k) buf[blockIdx.x * 8 + k] = v[k];
    }
    if (!sync()) return false;
    // every block sums the partials in block order (deterministic, identical on all blocks)
    __shared__ double tot[NV];
    if (threadIdx.x < 32) {
#pragma unroll
      for (int k = 0; k < NV; ++k) {
        double a = 0.0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += 32) {
          const double pv = *((volatile double*)&buf[b * 8 + k]);
          a = ((maxmask >> k) & 1) ? fmax(a, pv) : a + pv;
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
