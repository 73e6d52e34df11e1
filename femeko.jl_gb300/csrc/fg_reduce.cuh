// Deterministic grid reductions shared by the solvers: compensated FP32 (hi, lo)
// sums and the two-level "last block finishes" pattern.
#pragma once

#include <stdint.h>

struct ff {
  float hi, lo;
};

__device__ __forceinline__ ff ff_add(ff a, ff b) {
  float s = a.hi + b.hi;
  float bb = s - a.hi;
  float e = (a.hi - (s - bb)) + (b.hi - bb);
  return ff{s, e + a.lo + b.lo};
}

// Block partials -> one total, in two parallel levels so that no single block reads
// every partial.  Block b writes its partial and arrives on counter[1 + b % 64]; the
// last block of each of those groups sums the group's partials (one per thread) and
// arrives on counter[0]; the last group finisher sums the group totals.  Each sum is a
// fixed-shape tree over a fixed index order, so results do not depend on scheduling.
// Group totals sit right after the block partials (gridDim.x * N doubles).  Returns
// true in thread 0 of the finishing block, with the totals in tot.
constexpr int FG_ARRIVE_GROUPS = 64;
// The arrival counter of single-level "last block finishes" reductions (above the
// counters the two-level reduction uses, 0..FG_ARRIVE_GROUPS).
constexpr int FG_LAST1_COUNTER = 100;

// Arrival: an atomic add with release (the partials written before it are visible to
// whoever acquires the counter later) and acquire semantics at GPU scope; lighter
// than a full fence followed by a relaxed add.
__device__ __forceinline__ unsigned atom_add_acq_rel(unsigned *p, unsigned v) {
  unsigned old;
  asm volatile("atom.acq_rel.gpu.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}

// Compensated FP32 block sum kept as (hi, lo) pairs in thread 0.
template <int N>
__device__ __forceinline__ void block_sum_ff_pair(ff (&v)[N], ff (*sh)[32]) {
#pragma unroll
  for (int j = 0; j < N; ++j)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      ff other{__shfl_down_sync(0xffffffffu, v[j].hi, o), __shfl_down_sync(0xffffffffu, v[j].lo, o)};
      v[j] = ff_add(v[j], other);
    }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0)
#pragma unroll
    for (int j = 0; j < N; ++j) sh[j][w] = v[j];
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int j = 0; j < N; ++j) {
      v[j] = (l < nw) ? sh[j][l] : ff{0.f, 0.f};
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        ff other{__shfl_down_sync(0xffffffffu, v[j].hi, o), __shfl_down_sync(0xffffffffu, v[j].lo, o)};
        v[j] = ff_add(v[j], other);
      }
    }
  }
}

// grid_finish for the FP32 iterations' compensated dot products: the same two
// levels and fixed order, with the partials kept as (hi, lo) float pairs and summed
// on the FP32 pipe; only the totals become doubles.  GB300 runs FP64 at 1/64 of the
// FP32 rate: two levels of double block sums on the finishing path cost ~3 us per
// launch at 96^3.  v: the block's sums in thread 0.
// Grids of at most FG_LAST1_MAX_BLOCKS blocks finish in one level instead: every
// block arrives on one counter and the last one adds all partials (index order,
// strided over its threads), which at a few hundred blocks ends sooner than two
// chained levels of arrivals; larger grids keep the two levels.  The counter array
// holds at least FG_LAST1_COUNTER + 1 entries.
constexpr unsigned FG_LAST1_MAX_BLOCKS = 1024;
template <int N>
__device__ __forceinline__ bool grid_finish_ff(const ff (&v)[N], float2 *partials, unsigned *counter,
                                               double (&tot)[N]) {
  __shared__ int s_role;
  __shared__ ff shg[N][32], shf[N][32];
  const unsigned G = gridDim.x;
  if (G <= FG_LAST1_MAX_BLOCKS) {
    if (threadIdx.x == 0) {
#pragma unroll
      for (int j = 0; j < N; ++j) partials[(size_t)blockIdx.x * N + j] = make_float2(v[j].hi, v[j].lo);
      s_role = (atom_add_acq_rel(counter + FG_LAST1_COUNTER, 1u) == G - 1) ? 1 : 0;
    }
    __syncthreads();
    if (s_role == 0) return false;
    __threadfence();
    ff acc[N];
#pragma unroll
    for (int j = 0; j < N; ++j) acc[j] = ff{0.f, 0.f};
    for (unsigned k = threadIdx.x; k < G; k += blockDim.x) {
      float2 q[N];
#pragma unroll
      for (int j = 0; j < N; ++j) q[j] = __ldcg(partials + (size_t)k * N + j);
#pragma unroll
      for (int j = 0; j < N; ++j) acc[j] = ff_add(acc[j], ff{q[j].x, q[j].y});
    }
    block_sum_ff_pair<N>(acc, shf);
    if (threadIdx.x == 0) counter[FG_LAST1_COUNTER] = 0u;
#pragma unroll
    for (int j = 0; j < N; ++j) tot[j] = (double)acc[j].hi + (double)acc[j].lo;
    return threadIdx.x == 0;
  }
  const unsigned grp = blockIdx.x % FG_ARRIVE_GROUPS;
  const unsigned ngroups = G < FG_ARRIVE_GROUPS ? G : FG_ARRIVE_GROUPS;
  const unsigned gsize = (G - grp + FG_ARRIVE_GROUPS - 1) / FG_ARRIVE_GROUPS;
  float2 *gpart = partials + (size_t)G * N;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int j = 0; j < N; ++j) partials[(size_t)blockIdx.x * N + j] = make_float2(v[j].hi, v[j].lo);
    s_role = (atom_add_acq_rel(counter + 1 + grp, 1u) == gsize - 1) ? 1 : 0;
  }
  __syncthreads();
  if (s_role == 0) return false;
  __threadfence();
  ff acc[N];
#pragma unroll
  for (int j = 0; j < N; ++j) acc[j] = ff{0.f, 0.f};
  for (unsigned k = threadIdx.x; k < gsize; k += blockDim.x)
#pragma unroll
    for (int j = 0; j < N; ++j) {
      const float2 q = __ldcg(partials + (size_t)(grp + k * FG_ARRIVE_GROUPS) * N + j);
      acc[j] = ff_add(acc[j], ff{q.x, q.y});
    }
  block_sum_ff_pair<N>(acc, shg);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int j = 0; j < N; ++j) gpart[(size_t)grp * N + j] = make_float2(acc[j].hi, acc[j].lo);
    counter[1 + grp] = 0u;  // every member of the group has arrived
    s_role = (atom_add_acq_rel(counter, 1u) == ngroups - 1) ? 2 : 0;
  }
  __syncthreads();
  if (s_role != 2) return false;
  __threadfence();
#pragma unroll
  for (int j = 0; j < N; ++j) acc[j] = ff{0.f, 0.f};
  for (unsigned g = threadIdx.x; g < ngroups; g += blockDim.x)
#pragma unroll
    for (int j = 0; j < N; ++j) {
      const float2 q = __ldcg(gpart + (size_t)g * N + j);
      acc[j] = ff_add(acc[j], ff{q.x, q.y});
    }
  block_sum_ff_pair<N>(acc, shf);
  if (threadIdx.x == 0) counter[0] = 0u;
#pragma unroll
  for (int j = 0; j < N; ++j) tot[j] = (double)acc[j].hi + (double)acc[j].lo;
  return threadIdx.x == 0;
}

