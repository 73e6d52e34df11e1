// SpMV and Jacobi-preconditioned CG on the SELL-32x4 operator.
//
// The reference solves with IterativeSolvers.cg (Magnetostatics/2DmagneticField.jl:139,
// Micromagnetics/LL.jl:185, Femeko_jl_C++/Magnetostatics/run.jl:141) or Eigen's
// diagonal-preconditioned ConjugateGradient (magnetostatics.cpp:26-38).
//
// Layout: one thread per row; a row's slots come in groups of 4, so each group is one
// 128-bit load of values (float4, or two double2) and one load of column indices
// (int4, or short4 holding column - row when the matrix bandwidth fits 16 bits).
// A warp's group loads are contiguous (512 B of FP32 values).
//
// The CG recurrences are those of Chronopoulos & Gear (1989): with u = D^-1 r,
// w = A u, s = A p, one reduction per iteration (gamma = r.u, delta = w.u and r.r)
// gives beta = gamma_new / gamma and alpha = gamma_new / (delta - beta gamma_new / alpha);
// then s = w + beta s, p = u + beta p, x += alpha p, r -= alpha s, u = D^-1 r, w = A u.
//
// Mixed precision (FP32 operator and vectors): ONE kernel per iteration.  Each row
// gathers its neighbours' (r, w, s, D^-1) -- one 16-byte load per entry, double
// buffered -- and recomputes their new u = D^-1 (r - alpha (w + beta s)) on the fly,
// so the vector updates and the SpMV share one pass over memory.  Dot products use
// compensated (TwoSum) FP32 sums per thread and per block and FP64 across blocks.
//
// FP64 operator and vectors: two kernels per iteration (the pointwise updates, then
// w = A u with the dot products).  On GB300 an FP64 FMA costs ~64 FP32 FMAs, so
// recomputing u at every gathered entry would triple the SpMV's FP64 work.
//
// Scalars never leave the device; the host reads the "done" flag once per block of
// iterations, each block replayed as a CUDA graph.  An FP64 residual b - A x (FP64
// operator) drives iterative refinement around the FP32 solves; in the Newton solver
// the Newton loop itself is that refinement.
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "fg_async.cuh"
#include "fg_common.cuh"
#include "fg_reduce.cuh"
// ------------------------------------------------------------------ reductions
// Sum N doubles over the block; thread 0 gets the result.
template <int N>
__device__ __forceinline__ void block_sum(double (&v)[N], double (*sh)[32]) {
#pragma unroll
  for (int j = 0; j < N; ++j)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[j] += __shfl_down_sync(0xffffffffu, v[j], o);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0)
#pragma unroll
    for (int j = 0; j < N; ++j) sh[j][w] = v[j];
  __syncthreads();
  if (w == 0) {
    int nw = blockDim.x >> 5;
#pragma unroll
    for (int j = 0; j < N; ++j) {
      v[j] = (l < nw) ? sh[j][l] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v[j] += __shfl_down_sync(0xffffffffu, v[j], o);
    }
  }
}

// Per-thread accumulators: a plain FP64 sum for FP64 vectors, a compensated
// (TwoSum) FP32 pair for FP32 vectors.
template <typename S>
struct Acc;
template <>
struct Acc<double> {
  double v = 0.0;
  __device__ __forceinline__ void add(double x) { v += x; }
};
template <>
struct Acc<float> {
  ff v{0.f, 0.f};
  __device__ __forceinline__ void add(float x) { v = ff_add(v, ff{x, 0.f}); }
};

// The grid reduction of fg_reduce.cuh with FP64 partials (one level up to
// FG_LAST1_MAX_BLOCKS blocks, two above): true in thread 0 of the finishing block,
// with the totals in tot.
template <int N>
__device__ __forceinline__ bool grid_finish(const double (&v)[N], double *partials, unsigned *counter,
                                            double (&tot)[N]) {
  __shared__ int s_role;
  __shared__ double shg[N][32], shf[N][32];
  const unsigned G = gridDim.x;
  if (G <= FG_LAST1_MAX_BLOCKS) {
    if (threadIdx.x == 0) {
#pragma unroll
      for (int j = 0; j < N; ++j) partials[(size_t)blockIdx.x * N + j] = v[j];
      s_role = (atom_add_acq_rel(counter + FG_LAST1_COUNTER, 1u) == G - 1) ? 1 : 0;
    }
    __syncthreads();
    if (s_role == 0) return false;
    __threadfence();
    double acc[N];
#pragma unroll
    for (int j = 0; j < N; ++j) acc[j] = 0.0;
    for (unsigned k = threadIdx.x; k < G; k += blockDim.x)
#pragma unroll
      for (int j = 0; j < N; ++j) acc[j] += __ldcg(partials + (size_t)k * N + j);
    block_sum<N>(acc, shf);
    if (threadIdx.x == 0) counter[FG_LAST1_COUNTER] = 0u;
#pragma unroll
    for (int j = 0; j < N; ++j) tot[j] = acc[j];
    return threadIdx.x == 0;
  }
  const unsigned grp = blockIdx.x % FG_ARRIVE_GROUPS;
  const unsigned ngroups = G < FG_ARRIVE_GROUPS ? G : FG_ARRIVE_GROUPS;
  const unsigned gsize = (G - grp + FG_ARRIVE_GROUPS - 1) / FG_ARRIVE_GROUPS;
  double *gpart = partials + (size_t)G * N;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int j = 0; j < N; ++j) partials[(size_t)blockIdx.x * N + j] = v[j];
    s_role = (atom_add_acq_rel(counter + 1 + grp, 1u) == gsize - 1) ? 1 : 0;
  }
  __syncthreads();
  if (s_role == 0) return false;
  __threadfence();
  double acc[N];
#pragma unroll
  for (int j = 0; j < N; ++j) acc[j] = 0.0;
  for (unsigned k = threadIdx.x; k < gsize; k += blockDim.x)
#pragma unroll
    for (int j = 0; j < N; ++j) acc[j] += __ldcg(partials + (size_t)(grp + k * FG_ARRIVE_GROUPS) * N + j);
  block_sum<N>(acc, shg);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int j = 0; j < N; ++j) gpart[(size_t)grp * N + j] = acc[j];
    counter[1 + grp] = 0u;  // every member of the group has arrived
    s_role = (atom_add_acq_rel(counter, 1u) == ngroups - 1) ? 2 : 0;
  }
  __syncthreads();
  if (s_role != 2) return false;
  __threadfence();
#pragma unroll
  for (int j = 0; j < N; ++j) acc[j] = 0.0;
  for (unsigned g = threadIdx.x; g < ngroups; g += blockDim.x)
#pragma unroll
    for (int j = 0; j < N; ++j) acc[j] += __ldcg(gpart + (size_t)g * N + j);
  block_sum<N>(acc, shf);
  if (threadIdx.x == 0) counter[0] = 0u;
#pragma unroll
  for (int j = 0; j < N; ++j) tot[j] = acc[j];
  return threadIdx.x == 0;
}

// The three dot products of an FP32 CG iteration (per-thread compensated sums):
// block sums, then grid_finish_ff.  True in thread 0 of the finishing block.
__device__ __forceinline__ bool finish_dots32(const Acc<float> (&dots)[3], double *partials, unsigned *counter,
                                              double (&tot)[3]) {
  __shared__ ff shb[3][32];
  ff v[3] = {dots[0].v, dots[1].v, dots[2].v};
  block_sum_ff_pair<3>(v, shb);
  return grid_finish_ff<3>(v, reinterpret_cast<float2 *>(partials), counter, tot);
}

// ------------------------------------------------------------------ index helpers
// Column loads: absolute int32 columns (int4 per group) or 16-bit offsets from the
// row (short4 per group).
struct ColAbs {
  typedef int T;
  typedef int4 T4;
  static __device__ __forceinline__ int col(T c, int64_t) { return c; }
};
struct ColRel {
  typedef int16_t T;
  typedef short4 T4;
  static __device__ __forceinline__ int col(T c, int64_t row) { return (int)row + (int)c; }
};

__device__ __forceinline__ int4 ld_cols(const int4 *p) { return __ldg(p); }
__device__ __forceinline__ short4 ld_cols(const short4 *p) { return __ldg(p); }


// Scalar slots of the Chronopoulos-Gear recurrences (device doubles in scal[]):
// S_RZ gamma = r.u, S_ALPHA, S_BETA, S_RR r.r, S_TOL2 stop threshold on r.r.

// Last-block tail shared by the FP32 and FP64 iterations: from (gamma_new, delta,
// r.r) the next alpha and beta, the iteration count and the stopping test.  The first
// call after an initialisation (iteration count < 0) sets beta = 0, alpha =
// gamma/delta and turns the relative threshold absolute (times r0.r0).  cgcg_next is
// the arithmetic on explicit inputs (the previous gamma and alpha, the threshold, the
// previous count); cgcg_scalars applies it to the run's scalar slots.
struct CgNext {
  double gam, rr, alpha, beta, tol2;
  int it;
  int done;    // -1: unchanged, else the new done flag
  int status;  // -1: unchanged, else the new status
};
__device__ __forceinline__ CgNext cgcg_next(const double (&tot)[3], double gold, double aold, double tol2,
                                            int it_prev, int maxit) {
  const double gam = tot[0], del = tot[1], rr = tot[2];
  CgNext o;
  o.it = it_prev + 1;
  o.beta = 0.0;
  o.done = -1;
  o.status = -1;
  o.tol2 = tol2;
  if (o.it == 0) {
    o.alpha = (del != 0.0) ? gam / del : 0.0;
    o.tol2 = tol2 * rr;
    o.done = (rr == 0.0 || rr <= o.tol2) ? 1 : 0;
  } else {
    o.beta = (gold != 0.0) ? gam / gold : 0.0;
    const double den = del - o.beta * gam / aold;
    o.alpha = (den != 0.0) ? gam / den : 0.0;
    if (!isfinite(rr)) { o.status = 2; o.done = 1; }
    else if (rr <= tol2) { o.status = 0; o.done = 1; }
    else if (o.it >= maxit) { o.status = 1; o.done = 1; }
  }
  o.gam = gam;
  o.rr = rr;
  return o;
}

__device__ __forceinline__ void cgcg_store(const CgNext &o, double *scal, int *ictl) {
  scal[S_TOL2] = o.tol2;
  if (o.status >= 0) ictl[I_STATUS] = o.status;
  if (o.done >= 0) ictl[I_DONE] = o.done;
  scal[S_RZ] = o.gam;
  scal[S_RR] = o.rr;
  scal[S_ALPHA] = o.alpha;
  scal[S_BETA] = o.beta;
  ictl[I_ITERS] = o.it;
}

__device__ __forceinline__ void cgcg_scalars(const double (&tot)[3], double *scal, int *ictl) {
  cgcg_store(cgcg_next(tot, scal[S_RZ], scal[S_ALPHA], scal[S_TOL2], ictl[I_ITERS], ictl[I_MAXIT]), scal, ictl);
}

// The previous scalars cgcg_next needs, loaded by a finishing thread before it sums
// the partials (the loads then overlap those of the partials instead of following
// the block sum).  Nothing in the running launch writes them before its finish.
struct CgPrev {
  double gold, aold, tol2;
  int it, maxit;
};
__device__ __forceinline__ CgPrev cgcg_prev(const double *scal, const int *ictl) {
  return CgPrev{__ldcg(scal + S_RZ), __ldcg(scal + S_ALPHA), __ldcg(scal + S_TOL2), __ldcg(ictl + I_ITERS),
                __ldcg(ictl + I_MAXIT)};
}
__device__ __forceinline__ void cgcg_scalars(const double (&tot)[3], const CgPrev &pv, double *scal, int *ictl) {
  cgcg_store(cgcg_next(tot, pv.gold, pv.aold, pv.tol2, pv.it, pv.maxit), scal, ictl);
}

// ------------------------------------------------------------------ FP32 CG (fused)
// State per row in a float4 pair buffer: (r, w, s, dinv).  `first` computes
// w0 = A u0 from (r0, -, -, dinv) with alpha = beta = 0 (then s stays 0); later
// iterations apply the full recurrences.  HOIST: issue all loads of a row before the
// FMAs (rows of up to 16 slots).  BS: threads per block (autotuned).
template <class CI, bool HOIST, int BS>
__global__ void __launch_bounds__(BS) k_cg32_iter(int64_t n, const int *__restrict__ sl_ptr,
                                                  const int *__restrict__ sl_len,
                                                  const typename CI::T *__restrict__ col,
                                                  const float *__restrict__ val, const float4 *__restrict__ st_in,
                                                  float4 *__restrict__ st_out, float *__restrict__ p,
                                                  float *__restrict__ x, double *scal, int *ictl, double *partials,
                                                  unsigned *counter) {
  if (ictl[I_DONE]) return;
  const bool first = ictl[I_ITERS] < 0;
  const float alpha = first ? 0.f : (float)scal[S_ALPHA];
  const float beta = first ? 0.f : (float)scal[S_BETA];
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  Acc<float> dots[3];
  if (i < n) {
    const int s = (int)(i >> 5), lane = (int)(i & 31);
    const int64_t base = (int64_t)sl_ptr[s] + lane * FG_GROUP;
    const int G = sl_len[s];
    const float4 *v4 = reinterpret_cast<const float4 *>(val + base);
    const typename CI::T4 *c4 = reinterpret_cast<const typename CI::T4 *>(col + base);
    // u_new of a neighbour from its (r, w, s, dinv)
    auto unew = [&](const float4 a) { return a.w * fmaf(-alpha, fmaf(beta, a.z, a.y), a.x); };
    float acc = 0.f;
    if (HOIST && G <= 4) {
      float4 vv[4];
      typename CI::T4 cc[4];
#pragma unroll
      for (int g = 0; g < 4; ++g)
        if (g < G) {
          vv[g] = __ldg(v4 + (int64_t)g * FG_SLICE);
          cc[g] = ld_cols(c4 + (int64_t)g * FG_SLICE);
        }
#pragma unroll
      for (int g = 0; g < 4; ++g)
        if (g < G) {
          acc = fmaf(vv[g].x, unew(__ldg(st_in + CI::col(cc[g].x, i))), acc);
          acc = fmaf(vv[g].y, unew(__ldg(st_in + CI::col(cc[g].y, i))), acc);
          acc = fmaf(vv[g].z, unew(__ldg(st_in + CI::col(cc[g].z, i))), acc);
          acc = fmaf(vv[g].w, unew(__ldg(st_in + CI::col(cc[g].w, i))), acc);
        }
    } else {
#pragma unroll 4
      for (int g = 0; g < G; ++g) {
        const float4 vv = __ldg(v4 + (int64_t)g * FG_SLICE);
        const typename CI::T4 cc = ld_cols(c4 + (int64_t)g * FG_SLICE);
        const float4 a = __ldg(st_in + CI::col(cc.x, i));
        const float4 b = __ldg(st_in + CI::col(cc.y, i));
        const float4 c = __ldg(st_in + CI::col(cc.z, i));
        const float4 d = __ldg(st_in + CI::col(cc.w, i));
        acc = fmaf(vv.x, unew(a), acc);
        acc = fmaf(vv.y, unew(b), acc);
        acc = fmaf(vv.z, unew(c), acc);
        acc = fmaf(vv.w, unew(d), acc);
      }
    }
    // own row: s, p, x, r, u updates (same arithmetic as unew for the neighbours)
    const float4 o = __ldg(st_in + i);
    const float snew = fmaf(beta, o.z, o.y);
    const float rnew = fmaf(-alpha, snew, o.x);
    const float unw = o.w * rnew;
    if (!first) {
      const float pnew = fmaf(beta, p[i], o.w * o.x);
      p[i] = pnew;
      x[i] = fmaf(alpha, pnew, x[i]);
    }
    st_out[i] = make_float4(rnew, acc, snew, o.w);
    dots[0].add(rnew * unw);
    dots[1].add(acc * unw);
    dots[2].add(rnew * rnew);
  }
  double tot[3];
  if (finish_dots32(dots, partials, counter, tot)) cgcg_scalars(tot, scal, ictl);
}

// The same iteration with halo staging: the CTA first turns each distinct neighbour
// state of its R rows into the new u once, into shared memory (coalesced loads of a
// sorted column list), then every row reads its neighbours' u from shared memory
// through 16-bit local indices.  R = rows per CTA (the halo block size).
template <int R>
__global__ void __launch_bounds__(R) k_cg32_iter_halo(int64_t n, const int *__restrict__ sl_ptr,
                                                      const int *__restrict__ sl_len,
                                                      const uint16_t *__restrict__ lcol,
                                                      const float *__restrict__ val, const int *__restrict__ halo_col,
                                                      const int *__restrict__ halo_len, int hcap,
                                                      const float4 *__restrict__ st_in, float4 *__restrict__ st_out,
                                                      float *__restrict__ p, float *__restrict__ x, double *scal,
                                                      int *ictl, double *partials, unsigned *counter) {
  extern __shared__ float us[];
  if (ictl[I_DONE]) return;
  const bool first = ictl[I_ITERS] < 0;
  const float alpha = first ? 0.f : (float)scal[S_ALPHA];
  const float beta = first ? 0.f : (float)scal[S_BETA];
  {
    const int hl = halo_len[blockIdx.x];
    const int *hc = halo_col + (int64_t)blockIdx.x * hcap;
    for (int h = threadIdx.x; h < hl; h += R) {
      const float4 a = __ldg(st_in + __ldg(hc + h));
      us[h] = a.w * fmaf(-alpha, fmaf(beta, a.z, a.y), a.x);
    }
  }
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * R + threadIdx.x;
  Acc<float> dots[3];
  if (i < n) {
    const int s = (int)(i >> 5), lane = (int)(i & 31);
    const int64_t base = (int64_t)sl_ptr[s] + lane * FG_GROUP;
    const int G = sl_len[s];
    const float4 *v4 = reinterpret_cast<const float4 *>(val + base);
    const ushort4 *c4 = reinterpret_cast<const ushort4 *>(lcol + base);
    float acc = 0.f;
#pragma unroll 4
    for (int g = 0; g < G; ++g) {
      const float4 vv = __ldg(v4 + (int64_t)g * FG_SLICE);
      const ushort4 cc = __ldg(c4 + (int64_t)g * FG_SLICE);
      acc = fmaf(vv.x, us[cc.x], acc);
      acc = fmaf(vv.y, us[cc.y], acc);
      acc = fmaf(vv.z, us[cc.z], acc);
      acc = fmaf(vv.w, us[cc.w], acc);
    }
    const float4 o = __ldg(st_in + i);
    const float snew = fmaf(beta, o.z, o.y);
    const float rnew = fmaf(-alpha, snew, o.x);
    const float unw = o.w * rnew;
    if (!first) {
      const float pnew = fmaf(beta, p[i], o.w * o.x);
      p[i] = pnew;
      x[i] = fmaf(alpha, pnew, x[i]);
    }
    st_out[i] = make_float4(rnew, acc, snew, o.w);
    dots[0].add(rnew * unw);
    dots[1].add(acc * unw);
    dots[2].add(rnew * rnew);
  }
  double tot[3];
  if (finish_dots32(dots, partials, counter, tot)) cgcg_scalars(tot, scal, ictl);
}

// The halo iteration as a persistent, software-pipelined kernel.  Each CTA walks the
// row blocks (tiles) b = blockIdx.x, blockIdx.x + gridDim.x, ... with two shared-memory
// stages: while tile k is computed, tile k+1's neighbour states are in flight
// (16-byte cp.async gathers) and tile k+2's halo list, matrix values and local
// column indices are in flight as bulk copies (cp.async.bulk completing on an
// mbarrier).  So the loads of the next tiles overlap the current one instead of
// waiting on each dependent gather.  Dots accumulate over the CTA's tiles and are
// reduced once at the end.
struct PipeArgs {
  int64_t n;
  int ntiles, nslices, hcap;
  int HM, TM;  // halo entries and matrix entries per stage (capacities)
  const int *sl_ptr, *sl_len, *halo_col, *halo_len;
  const uint16_t *lcol;
  const float *val;
};

__host__ __device__ __forceinline__ size_t pipe_align(size_t b) { return (b + 127) & ~(size_t)127; }
// stage layout: halo columns (int), halo states (float4), halo u (float), values, columns
__host__ __device__ __forceinline__ size_t pipe_stage_bytes(int HM, int TM) {
  return pipe_align((size_t)HM * 4) + pipe_align((size_t)HM * 16) + pipe_align((size_t)HM * 4) +
         pipe_align((size_t)TM * 4) + pipe_align((size_t)TM * 2);
}

template <int R>
__global__ void __launch_bounds__(R) k_cg32_iter_pipe(PipeArgs a, const float4 *__restrict__ st_in,
                                                      float4 *__restrict__ st_out, float *__restrict__ p,
                                                      float *__restrict__ x, double *scal, int *ictl,
                                                      double *partials, unsigned *counter) {
  extern __shared__ __align__(128) unsigned char sm_pipe[];
  __shared__ __align__(8) uint64_t bar[2];
  if (ictl[I_DONE]) return;
  const bool first = ictl[I_ITERS] < 0;
  const float alpha = first ? 0.f : (float)scal[S_ALPHA];
  const float beta = first ? 0.f : (float)scal[S_BETA];
  const int tid = threadIdx.x;
  const size_t o_hst = pipe_align((size_t)a.HM * 4), o_u = o_hst + pipe_align((size_t)a.HM * 16);
  const size_t o_val = o_u + pipe_align((size_t)a.HM * 4), o_col = o_val + pipe_align((size_t)a.TM * 4);
  const size_t stage = pipe_stage_bytes(a.HM, a.TM);
  auto hidx = [&](int s) { return reinterpret_cast<int *>(sm_pipe + s * stage); };
  auto hst = [&](int s) { return reinterpret_cast<float4 *>(sm_pipe + s * stage + o_hst); };
  auto uh = [&](int s) { return reinterpret_cast<float *>(sm_pipe + s * stage + o_u); };
  auto vals = [&](int s) { return reinterpret_cast<const float *>(sm_pipe + s * stage + o_val); };
  auto cols = [&](int s) { return reinterpret_cast<const uint16_t *>(sm_pipe + s * stage + o_col); };
  constexpr int SPT = R / FG_SLICE;  // slices per tile
  const int K = (a.ntiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x;
  auto tile_of = [&](int k) { return (int)blockIdx.x + k * (int)gridDim.x; };

  // thread 0: bulk copies of a tile's halo list, values and local columns into stage s
  auto issue_bulk = [&](int tile, int s) {
    const int s0 = tile * SPT, s1 = min(s0 + SPT, a.nslices);
    const int e0 = a.sl_ptr[s0], e1 = a.sl_ptr[s1];
    const uint32_t hb = (uint32_t)((a.halo_len[tile] * 4 + 15) & ~15);
    const uint32_t vb = (uint32_t)(e1 - e0) * 4u, cb = (uint32_t)(e1 - e0) * 2u;
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(&bar[s], hb + vb + cb);
    bulk_g2s(hidx(s), a.halo_col + (int64_t)tile * a.hcap, hb, &bar[s]);
    bulk_g2s(sm_pipe + s * stage + o_val, a.val + e0, vb, &bar[s]);
    bulk_g2s(sm_pipe + s * stage + o_col, a.lcol + e0, cb, &bar[s]);
  };
  // all threads: 16-byte gathers of the tile's neighbour states into stage s
  auto issue_gather = [&](int tile, int s) {
    const int hl = a.halo_len[tile];
    const int *hi = hidx(s);
    float4 *dst = hst(s);
    for (int h = tid; h < hl; h += R) cp_async16(dst + h, st_in + hi[h]);
    cp_async_commit();
  };

  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_proxy_async_smem();
  }
  __syncthreads();
  uint32_t phases = 0u;  // bit s: parity of stage s's next barrier phase
  bool ok = true;
  if (tid == 0) {
    issue_bulk(tile_of(0), 0);
    if (K > 1) issue_bulk(tile_of(1), 1);
  }
  ok = mbar_wait(&bar[0], 0u);
  phases ^= 1u;
  if (__syncthreads_or(!ok)) ok = false;
  if (ok) issue_gather(tile_of(0), 0);

  Acc<float> dots[3];
  for (int k = 0; k < K && ok; ++k) {
    const int s = k & 1, tile = tile_of(k);
    const int64_t i = (int64_t)tile * R + tid;
    // own row: issued before the waits so that they overlap them
    float4 o = make_float4(0.f, 0.f, 0.f, 0.f);
    float pi = 0.f, xi = 0.f;
    int G = 0, base = 0;
    const bool row = i < a.n;
    if (row) {
      o = __ldg(st_in + i);
      if (!first) { pi = p[i]; xi = x[i]; }
      const int sl = (int)(i >> 5);
      G = a.sl_len[sl];
      base = a.sl_ptr[sl] - a.sl_ptr[tile * SPT] + (int)(i & 31) * FG_GROUP;
    }
    const int hl = a.halo_len[tile];
    cp_async_wait_all();
    __syncthreads();
    {
      const float4 *hs = hst(s);
      float *u = uh(s);
      for (int h = tid; h < hl; h += R) {
        const float4 q = hs[h];
        u[h] = q.w * fmaf(-alpha, fmaf(beta, q.z, q.y), q.x);
      }
    }
    if (k + 1 < K) {
      const int s1 = s ^ 1;
      const bool got = mbar_wait(&bar[s1], (phases >> s1) & 1u);
      phases ^= 1u << s1;
      if (__syncthreads_or(!got)) { ok = false; break; }
      issue_gather(tile_of(k + 1), s1);
    }
    __syncthreads();
    if (row) {
      const float *v = vals(s);
      const uint16_t *c = cols(s);
      const float *u = uh(s);
      float acc = 0.f;
#pragma unroll 4
      for (int g = 0; g < G; ++g) {
        const float4 vv = *reinterpret_cast<const float4 *>(v + base + g * FG_SLICE * FG_GROUP);
        const ushort4 cc = *reinterpret_cast<const ushort4 *>(c + base + g * FG_SLICE * FG_GROUP);
        acc = fmaf(vv.x, u[cc.x], acc);
        acc = fmaf(vv.y, u[cc.y], acc);
        acc = fmaf(vv.z, u[cc.z], acc);
        acc = fmaf(vv.w, u[cc.w], acc);
      }
      const float snew = fmaf(beta, o.z, o.y);
      const float rnew = fmaf(-alpha, snew, o.x);
      const float unw = o.w * rnew;
      if (!first) {
        const float pnew = fmaf(beta, pi, o.w * o.x);
        p[i] = pnew;
        x[i] = fmaf(alpha, pnew, xi);
      }
      st_out[i] = make_float4(rnew, acc, snew, o.w);
      dots[0].add(rnew * unw);
      dots[1].add(acc * unw);
      dots[2].add(rnew * rnew);
    }
    __syncthreads();
    if (k + 2 < K && tid == 0) issue_bulk(tile_of(k + 2), s);
  }
  if (!ok) {
    // a bulk copy did not arrive: report, drain what is in flight (bounded), stop the CG
    cp_async_wait_all();
    mbar_wait(&bar[0], phases & 1u, 1 << 20);
    mbar_wait(&bar[1], (phases >> 1) & 1u, 1 << 20);
    if (tid == 0) {
      atomicExch(ictl + I_FAULT, 1);
      atomicExch(ictl + I_DONE, 1);
    }
  }
  double tot[3];
  if (finish_dots32(dots, partials, counter, tot) && ok) cgcg_scalars(tot, scal, ictl);
}

// Programmatic dependent launch: a kernel launched with programmatic stream
// serialisation may start while the previous kernel in the stream finishes;
// griddep_wait() returns once that kernel has completed and its writes are visible,
// griddep_release() lets the next kernel start launching.  Both are no-ops for a
// kernel launched without the attribute.
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void griddep_release() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// FP32 Chronopoulos-Gear iteration split in two passes, as the FP64 one: a streaming
// vector update (s = w + beta s, p = u + beta p, x += alpha p, r -= alpha s,
// u = D^-1 r; four rows per thread) and w = A u with the three dot products.  The
// SpMV then gathers 4-byte entries of u instead of 16-byte neighbour states.  The u
// of the previous iteration is formed again as D^-1 r (the same single rounding that
// wrote it, here and in k_cg32s_init) instead of being read: 24 B read and 20 B
// written per row.
__global__ void __launch_bounds__(256) k_cg32s_vec(int64_t n4, float4 *__restrict__ r, const float4 *__restrict__ w,
                                                   float4 *__restrict__ s, float4 *__restrict__ p,
                                                   float4 *__restrict__ u, float4 *__restrict__ x,
                                                   const float4 *__restrict__ dinv, const double *scal,
                                                   const int *ictl) {
  griddep_wait();
  griddep_release();
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n4) return;
  // the flag, the scalars and the vectors are loaded together
  const int done = ictl[I_DONE];
  const double alpha_d = scal[S_ALPHA], beta_d = scal[S_BETA];
  const float4 ww = w[j], dd = dinv[j];
  float4 ss = s[j], pp = p[j], xx = x[j], rr = r[j];
  if (done) return;
  const float4 uu = make_float4(dd.x * rr.x, dd.y * rr.y, dd.z * rr.z, dd.w * rr.w);
  const float alpha = (float)alpha_d, beta = (float)beta_d;
  ss.x = fmaf(beta, ss.x, ww.x); ss.y = fmaf(beta, ss.y, ww.y); ss.z = fmaf(beta, ss.z, ww.z); ss.w = fmaf(beta, ss.w, ww.w);
  pp.x = fmaf(beta, pp.x, uu.x); pp.y = fmaf(beta, pp.y, uu.y); pp.z = fmaf(beta, pp.z, uu.z); pp.w = fmaf(beta, pp.w, uu.w);
  xx.x = fmaf(alpha, pp.x, xx.x); xx.y = fmaf(alpha, pp.y, xx.y); xx.z = fmaf(alpha, pp.z, xx.z); xx.w = fmaf(alpha, pp.w, xx.w);
  rr.x = fmaf(-alpha, ss.x, rr.x); rr.y = fmaf(-alpha, ss.y, rr.y); rr.z = fmaf(-alpha, ss.z, rr.z); rr.w = fmaf(-alpha, ss.w, rr.w);
  s[j] = ss;
  p[j] = pp;
  x[j] = xx;
  r[j] = rr;
  u[j] = make_float4(dd.x * rr.x, dd.y * rr.y, dd.z * rr.z, dd.w * rr.w);
}

// PERSIST: a grid of at most the resident blocks walks the 256-row blocks with a
// grid stride, so each block reduces and arrives once for several row blocks.  At
// any moment all blocks work on neighbouring rows and gather the same stretch of u
// (contiguous row ranges per block, which spread the gathers over the whole vector,
// measured 41 us per iteration against 36 us at 96^3).
template <class CI, bool PERSIST>
__global__ void __launch_bounds__(256) k_cg32s_spmv(int64_t n, const int *__restrict__ sl_ptr,
                                                    const int *__restrict__ sl_len,
                                                    const typename CI::T *__restrict__ col,
                                                    const float *__restrict__ val, const float *__restrict__ u,
                                                    const float *__restrict__ r, const float *__restrict__ rw,
                                                    float *__restrict__ w, double *scal, int *ictl,
                                                    double *partials, unsigned *counter) {
  griddep_wait();
  griddep_release();
  // the done flag is loaded together with the first row's metadata: its latency
  // overlaps theirs instead of preceding them
  const int done = ictl[I_DONE];
  Acc<float> dots[3];
  const int64_t nrb = (n + 255) / 256;
  bool first_block = true;
  for (int64_t rb = blockIdx.x; rb < (PERSIST ? nrb : (int64_t)blockIdx.x + 1); rb += gridDim.x) {
  const int64_t i = rb * 256 + threadIdx.x;
  int G = 0;
  int64_t base = 0;
  if (i < n) {
    const int s = (int)(i >> 5), lane = (int)(i & 31);
    base = (int64_t)sl_ptr[s] + lane * FG_GROUP;
    G = sl_len[s];
  }
  if (first_block) {
    if (done) return;
    first_block = false;
  }
  if (i < n) {
    const float4 *v4 = reinterpret_cast<const float4 *>(val + base);
    const typename CI::T4 *c4 = reinterpret_cast<const typename CI::T4 *>(col + base);
    float acc = 0.f;
#pragma unroll 4
    for (int g = 0; g < G; ++g) {
      const float4 vv = __ldg(v4 + (int64_t)g * FG_SLICE);
      const typename CI::T4 cc = ld_cols(c4 + (int64_t)g * FG_SLICE);
      acc = fmaf(vv.x, __ldg(u + CI::col(cc.x, i)), acc);
      acc = fmaf(vv.y, __ldg(u + CI::col(cc.y, i)), acc);
      acc = fmaf(vv.z, __ldg(u + CI::col(cc.z, i)), acc);
      acc = fmaf(vv.w, __ldg(u + CI::col(cc.w, i)), acc);
    }
    w[i] = acc;
    const float ui = u[i], ri = r[i];
    dots[0].add(ri * ui);
    dots[1].add(acc * ui);
    // rw (the scaled system): r.r of the unscaled residual, sum of D_ii r'_i^2
    dots[2].add(rw ? ri * ri * __ldg(rw + i) : ri * ri);
  }
  }
  double tot[3];
  if (finish_dots32(dots, partials, counter, tot)) cgcg_scalars(tot, scal, ictl);
}

// The split SpMV with halo staging of u (4 bytes per distinct neighbour).
template <int R>
__global__ void __launch_bounds__(R) k_cg32s_spmv_halo(int64_t n, const int *__restrict__ sl_ptr,
                                                       const int *__restrict__ sl_len,
                                                       const uint16_t *__restrict__ lcol,
                                                       const float *__restrict__ val, const int *__restrict__ halo_col,
                                                       const int *__restrict__ halo_len, int hcap,
                                                       const float *__restrict__ u, const float *__restrict__ r,
                                                       float *__restrict__ w, double *scal, int *ictl,
                                                       double *partials, unsigned *counter) {
  extern __shared__ float uhs[];
  griddep_wait();
  griddep_release();
  if (ictl[I_DONE]) return;
  {
    const int hl = halo_len[blockIdx.x];
    const int *hc = halo_col + (int64_t)blockIdx.x * hcap;
    for (int h = threadIdx.x; h < hl; h += R) uhs[h] = __ldg(u + __ldg(hc + h));
  }
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * R + threadIdx.x;
  Acc<float> dots[3];
  if (i < n) {
    const int s = (int)(i >> 5), lane = (int)(i & 31);
    const int64_t base = (int64_t)sl_ptr[s] + lane * FG_GROUP;
    const int G = sl_len[s];
    const float4 *v4 = reinterpret_cast<const float4 *>(val + base);
    const ushort4 *c4 = reinterpret_cast<const ushort4 *>(lcol + base);
    float acc = 0.f;
#pragma unroll 4
    for (int g = 0; g < G; ++g) {
      const float4 vv = __ldg(v4 + (int64_t)g * FG_SLICE);
      const ushort4 cc = __ldg(c4 + (int64_t)g * FG_SLICE);
      acc = fmaf(vv.x, uhs[cc.x], acc);
      acc = fmaf(vv.y, uhs[cc.y], acc);
      acc = fmaf(vv.z, uhs[cc.z], acc);
      acc = fmaf(vv.w, uhs[cc.w], acc);
    }
    w[i] = acc;
    const float ui = u[i], ri = r[i];
    dots[0].add(ri * ui);
    dots[1].add(acc * ui);
    dots[2].add(ri * ri);
  }
  double tot[3];
  if (finish_dots32(dots, partials, counter, tot)) cgcg_scalars(tot, scal, ictl);
}

// Thread-level part of the sum of nparts per-block (hi, lo) partials of three dot
// products by a 256-thread block: thread t adds partials t, t + 256, t + 512, ... in
// that order, with the loads of U consecutive ones issued before any add (a block
// that waits on L2 once instead of U times).
template <int U>
__device__ __forceinline__ void sum_partials_ff3(const float2 *__restrict__ partials, int nparts, ff (&acc)[3]) {
  for (int base = threadIdx.x; base < nparts; base += 256 * U) {
    float2 q[U][3];
#pragma unroll
    for (int i = 0; i < U; ++i) {
      const int k = base + 256 * i;
#pragma unroll
      for (int j = 0; j < 3; ++j) q[i][j] = (k < nparts) ? __ldcg(partials + (size_t)k * 3 + j) : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int i = 0; i < U; ++i)
      if (base + 256 * i < nparts)
#pragma unroll
        for (int j = 0; j < 3; ++j) acc[j] = ff_add(acc[j], ff{q[i][j].x, q[i][j].y});
  }
}

// The split SpMV with the matrix entries staged by the bulk-copy engine: a persistent
// grid whose blocks walk their 256-row blocks; while a block computes one, the values
// and column offsets of its next one (two contiguous ranges of the SELL layout) are
// in flight into the other shared-memory stage (cp.async.bulk completing on an
// mbarrier).  Threads read their row's entries from shared memory and gather u from
// global memory.  cap: the most padded entries of one 256-row block.  A stage that
// does not arrive within the bounded wait stops the CG with I_FAULT set.  SPLIT: each
// block leaves its compensated partials (float pairs) and returns; with LAST1 the
// last block to arrive (one counter) then adds all of them, in the order and with the
// arithmetic of k_cg32_dots_finish, and sets the scalars: one level of arrivals and no
// separate finishing launch.
template <class CI, bool SPLIT = false, bool LAST1 = false>
__global__ void __launch_bounds__(256) k_cg32s_spmv_bulk(int64_t n, int nslices, int cap,
                                                         const int *__restrict__ sl_ptr,
                                                         const int *__restrict__ sl_len,
                                                         const typename CI::T *__restrict__ col,
                                                         const float *__restrict__ val, const float *__restrict__ u,
                                                         const float *__restrict__ r, float *__restrict__ w,
                                                         double *scal, int *ictl, double *partials,
                                                         unsigned *counter) {
  using T = typename CI::T;
  using T4 = typename CI::T4;
  extern __shared__ __align__(128) unsigned char sm_bulk[];
  __shared__ __align__(8) uint64_t bar[2];
  if (ictl[I_DONE]) return;
  const int tid = threadIdx.x;
  const size_t o_col = pipe_align((size_t)cap * 4);
  const size_t stage = o_col + pipe_align((size_t)cap * sizeof(T));
  const int64_t nrb = (n + 255) / 256;
  const int K = (int)((nrb - (int64_t)blockIdx.x + gridDim.x - 1) / gridDim.x);
  auto rowblock = [&](int k) { return (int64_t)blockIdx.x + (int64_t)k * gridDim.x; };
  // thread 0: the values and columns of the k-th row block of this CTA into stage st
  auto issue = [&](int k, int st) {
    const int s0 = (int)(rowblock(k) * (256 / FG_SLICE)), s1 = min(s0 + 256 / FG_SLICE, nslices);
    const int e0 = sl_ptr[s0], e1 = sl_ptr[s1];
    const uint32_t vb = (uint32_t)(e1 - e0) * 4u, cb = (uint32_t)(e1 - e0) * (uint32_t)sizeof(T);
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(&bar[st], vb + cb);
    bulk_g2s(sm_bulk + st * stage, val + e0, vb, &bar[st]);
    bulk_g2s(sm_bulk + st * stage + o_col, col + e0, cb, &bar[st]);
  };
  uint32_t inflight = 0u;  // bit st: a copy into stage st not yet waited for
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_proxy_async_smem();
  }
  __syncthreads();
  if (tid == 0) {
    issue(0, 0);
    if (K > 1) issue(1, 1);
  }
  inflight = (K > 1) ? 3u : 1u;
  uint32_t phase = 0u;  // bit st: parity of stage st's next phase
  bool ok = true;
  Acc<float> dots[3];
  for (int k = 0; k < K; ++k) {
    const int st = k & 1;
    const int64_t rb = rowblock(k);
    const int64_t i = rb * 256 + tid;
    const bool row = i < n;
    int G = 0, base = 0;
    float ui = 0.f, ri = 0.f;
    if (row) {
      // own row's metadata and vector entries, issued before the wait
      const int s = (int)(i >> 5);
      G = sl_len[s];
      base = sl_ptr[s] - sl_ptr[rb * (256 / FG_SLICE)] + (tid & 31) * FG_GROUP;
      ui = u[i];
      ri = r[i];
    }
    const bool got = mbar_wait(&bar[st], (phase >> st) & 1u);
    if (got) {
      phase ^= 1u << st;
      inflight &= ~(1u << st);
    }
    if (__syncthreads_or(!got)) { ok = false; break; }
    if (row) {
      const float *v = reinterpret_cast<const float *>(sm_bulk + st * stage);
      const T *c = reinterpret_cast<const T *>(sm_bulk + st * stage + o_col);
      float acc = 0.f;
#pragma unroll 4
      for (int g = 0; g < G; ++g) {
        const float4 vv = *reinterpret_cast<const float4 *>(v + base + g * FG_SLICE * FG_GROUP);
        const T4 cc = *reinterpret_cast<const T4 *>(c + base + g * FG_SLICE * FG_GROUP);
        acc = fmaf(vv.x, __ldg(u + CI::col(cc.x, i)), acc);
        acc = fmaf(vv.y, __ldg(u + CI::col(cc.y, i)), acc);
        acc = fmaf(vv.z, __ldg(u + CI::col(cc.z, i)), acc);
        acc = fmaf(vv.w, __ldg(u + CI::col(cc.w, i)), acc);
      }
      w[i] = acc;
      dots[0].add(ri * ui);
      dots[1].add(acc * ui);
      dots[2].add(ri * ri);
    }
    // every thread is done with stage st: refill it with the row block after next
    __syncthreads();
    if (k + 2 < K) {
      if (tid == 0) issue(k + 2, st);
      inflight |= 1u << st;
    }
  }
  if (!ok) {
    // a stage did not arrive: wait (bounded) for the copies in flight, stop the CG
    if (tid == 0) {
      for (int st = 0; st < 2; ++st)
        if (inflight & (1u << st)) mbar_wait(&bar[st], (phase >> st) & 1u, 1 << 20);
      atomicExch(ictl + I_FAULT, 1);
      atomicExch(ictl + I_DONE, 1);
    }
    __syncthreads();
  }
  if (SPLIT) {
    // the block's compensated sums only; k_cg32_dots_finish adds them up
    __shared__ ff shs[3][32];
    ff v[3] = {dots[0].v, dots[1].v, dots[2].v};
    block_sum_ff_pair<3>(v, shs);
    if (tid == 0) {
      float2 *fp = reinterpret_cast<float2 *>(partials);
      for (int j = 0; j < 3; ++j) fp[(size_t)blockIdx.x * 3 + j] = make_float2(v[j].hi, v[j].lo);
    }
    if (!LAST1) return;
    __shared__ int s_last;
    if (tid == 0) {
      // release: the partials above are visible to the block that arrives last
      s_last = (atom_add_acq_rel(counter + FG_LAST1_COUNTER, 1u) == gridDim.x - 1) ? 1 : 0;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    CgPrev pv{};
    if (tid == 0) pv = cgcg_prev(scal, ictl);
    ff acc[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    sum_partials_ff3<4>(reinterpret_cast<const float2 *>(partials), (int)gridDim.x, acc);
    block_sum_ff_pair<3>(acc, shs);
    if (tid == 0) {
      counter[FG_LAST1_COUNTER] = 0u;
      double tot[3];
      for (int j = 0; j < 3; ++j) tot[j] = (double)acc[j].hi + (double)acc[j].lo;
      cgcg_scalars(tot, pv, scal, ictl);
    }
    return;
  }
  double tot[3];
  if (finish_dots32(dots, partials, counter, tot) && ok) cgcg_scalars(tot, scal, ictl);
}

// The dot products of the split-reduction SpMV (k_cg32s_spmv_bulk<CI, true>): one
// block sums the nparts per-block partials in index order and sets the iteration's
// scalars.  A kernel of its own instead of the last-arriving block of the SpMV: no
// block of the SpMV waits on arrival counters, and the sum starts once every block
// has finished, in one block, without the two-level arrival chain.
__global__ void __launch_bounds__(256) k_cg32_dots_finish(const float2 *__restrict__ partials, int nparts,
                                                          double *scal, int *ictl) {
  if (ictl[I_DONE]) return;
  CgPrev pv{};
  if (threadIdx.x == 0) pv = cgcg_prev(scal, ictl);
  ff acc[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
  sum_partials_ff3<4>(partials, nparts, acc);
  __shared__ ff shr[3][32];
  block_sum_ff_pair<3>(acc, shr);
  if (threadIdx.x == 0) {
    double tot[3];
    for (int j = 0; j < 3; ++j) tot[j] = (double)acc[j].hi + (double)acc[j].lo;
    cgcg_scalars(tot, pv, scal, ictl);
  }
}

// ------------------------------------------------------------------ FP32 CG, one launch
// The split FP32 iteration (vector pass, then w = A u with its dot products) run by
// ONE persistent cooperative launch for many iterations: the grid barrier between
// the two phases and the one closing an iteration replace two kernel boundaries, the
// last block to reach the closing barrier finishes the dot products (fixed order)
// and sets the scalars before it releases the others, and each block's first two
// row blocks of matrix entries are already in flight (bulk copies) while the vector
// pass and the barriers run.  Every block handles the same 256-row blocks in both
// phases, so a block reads back only its own vector writes; the gathers of u, written
// by other blocks in this launch, bypass L1 (ld.global.cg).  Every wait is bounded:
// a barrier or a copy that does not complete stops the CG with I_FAULT set.
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u32(unsigned *p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Waits (bounded) until the barrier generation differs from g; false on timeout.
__device__ __forceinline__ bool coop_wait_gen(const unsigned *gen, unsigned g) {
  for (int it = 0; it < (1 << 24); ++it) {
    if (ld_acquire_u32(gen) != g) return true;
    __nanosleep(32);
  }
  return false;
}

template <class CI>
__global__ void __launch_bounds__(256) k_cg32_coop(int64_t n, int nslices, int cap, const int *__restrict__ sl_ptr,
                                                   const int *__restrict__ sl_len,
                                                   const typename CI::T *__restrict__ col,
                                                   const float *__restrict__ val, float *__restrict__ r,
                                                   float *__restrict__ w, float *__restrict__ s,
                                                   float *__restrict__ p, float *__restrict__ u,
                                                   float *__restrict__ x, const float *__restrict__ dinv,
                                                   double *scal, int *ictl, float2 *partials, unsigned *bar,
                                                   int iters) {
  using T = typename CI::T;
  using T4 = typename CI::T4;
  extern __shared__ __align__(128) unsigned char sm_bulk[];
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ int s_last, s_ok;
  const int tid = threadIdx.x;
  const unsigned G = gridDim.x;
  unsigned *count = bar, *gen = bar + 1;
  const size_t o_col = pipe_align((size_t)cap * 4);
  const size_t stage = o_col + pipe_align((size_t)cap * sizeof(T));
  const int64_t nrb = (n + 255) / 256;
  const int K = (int)((nrb - (int64_t)blockIdx.x + G - 1) / G);
  auto rowblock = [&](int k) { return (int64_t)blockIdx.x + (int64_t)k * G; };
  // matrix items are consumed in the order (iteration, row block); item q uses stage
  // q & 1 and holds row block q mod K
  const int64_t nitems = (int64_t)iters * K;
  auto issue = [&](int64_t q) {
    const int st = (int)(q & 1);
    const int s0 = (int)(rowblock((int)(q % K)) * (256 / FG_SLICE)), s1 = min(s0 + 256 / FG_SLICE, nslices);
    const int e0 = sl_ptr[s0], e1 = sl_ptr[s1];
    const uint32_t vb = (uint32_t)(e1 - e0) * 4u, cb = (uint32_t)(e1 - e0) * (uint32_t)sizeof(T);
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(&mbar[st], vb + cb);
    bulk_g2s(sm_bulk + st * stage, val + e0, vb, &mbar[st]);
    bulk_g2s(sm_bulk + st * stage + o_col, col + e0, cb, &mbar[st]);
  };
  if (tid == 0) {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    fence_proxy_async_smem();
  }
  __syncthreads();
  uint32_t inflight = 0u, phase = 0u;
  // the first two items are in flight from the start, during the first vector pass
  for (int64_t q = 0; q < 2 && q < nitems; ++q) {
    if (tid == 0) issue(q);
    inflight |= 1u << (q & 1);
  }
  int64_t qc = 0;  // items consumed
  unsigned g_seen = ld_acquire_u32(gen);
  bool ok = true;
  // a barrier of every block (false when a wait ran out); with reduce_last, the last
  // block to arrive adds the blocks' dot-product partials and sets the scalars first
  auto barrier = [&](bool reduce_last) -> bool {
    __syncthreads();
    if (tid == 0) s_last = (atom_add_acq_rel(count, 1u) == G - 1) ? 1 : 0;
    __syncthreads();
    const bool last = s_last != 0;
    if (last) {
      if (reduce_last) {
        ff acc[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
        for (unsigned k = tid; k < G; k += 256)
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            const float2 v2 = __ldcg(partials + (size_t)k * 3 + j);
            acc[j] = ff_add(acc[j], ff{v2.x, v2.y});
          }
        __shared__ ff shr[3][32];
        block_sum_ff_pair<3>(acc, shr);
        if (tid == 0) {
          double tot[3];
          for (int j = 0; j < 3; ++j) tot[j] = (double)acc[j].hi + (double)acc[j].lo;
          cgcg_scalars(tot, scal, ictl);
        }
      }
      if (tid == 0) {
        *count = 0u;
        st_release_u32(gen, g_seen + 1u);
        s_ok = 1;
      }
    } else if (tid == 0) {
      s_ok = coop_wait_gen(gen, g_seen) ? 1 : 0;
    }
    __syncthreads();
    ++g_seen;
    return s_ok != 0;
  };
  for (int itn = 0; itn < iters && ok; ++itn) {
    if (__ldcg(ictl + I_DONE)) break;
    // ---- vector pass on this block's rows
    const float alpha = (float)__ldcg(scal + S_ALPHA), beta = (float)__ldcg(scal + S_BETA);
    for (int k = 0; k < K; ++k) {
      const int64_t i = rowblock(k) * 256 + tid;
      if (i < n) {
        const float ww = w[i], dd = dinv[i];
        float ss = s[i], pp = p[i], xx = x[i], rr = r[i];
        const float uu = u[i];
        ss = fmaf(beta, ss, ww);
        pp = fmaf(beta, pp, uu);
        xx = fmaf(alpha, pp, xx);
        rr = fmaf(-alpha, ss, rr);
        s[i] = ss;
        p[i] = pp;
        x[i] = xx;
        r[i] = rr;
        u[i] = dd * rr;
      }
    }
    if (!barrier(false)) { ok = false; break; }
    // ---- w = A u and the dot products on this block's rows
    Acc<float> dots[3];
    for (int k = 0; k < K; ++k, ++qc) {
      const int st = (int)(qc & 1);
      const int64_t rb = rowblock(k);
      const int64_t i = rb * 256 + tid;
      const bool row = i < n;
      int Gs = 0, base = 0;
      float ui = 0.f, ri = 0.f;
      if (row) {
        const int sl = (int)(i >> 5);
        Gs = sl_len[sl];
        base = sl_ptr[sl] - sl_ptr[rb * (256 / FG_SLICE)] + (tid & 31) * FG_GROUP;
        ui = u[i];
        ri = r[i];
      }
      const bool got = mbar_wait(&mbar[st], (phase >> st) & 1u);
      if (got) {
        phase ^= 1u << st;
        inflight &= ~(1u << st);
      }
      if (__syncthreads_or(!got)) { ok = false; break; }
      if (row) {
        const float *v = reinterpret_cast<const float *>(sm_bulk + st * stage);
        const T *c = reinterpret_cast<const T *>(sm_bulk + st * stage + o_col);
        float acc = 0.f;
#pragma unroll 4
        for (int gg = 0; gg < Gs; ++gg) {
          const float4 vv = *reinterpret_cast<const float4 *>(v + base + gg * FG_SLICE * FG_GROUP);
          const T4 cc = *reinterpret_cast<const T4 *>(c + base + gg * FG_SLICE * FG_GROUP);
          acc = fmaf(vv.x, __ldcg(u + CI::col(cc.x, i)), acc);
          acc = fmaf(vv.y, __ldcg(u + CI::col(cc.y, i)), acc);
          acc = fmaf(vv.z, __ldcg(u + CI::col(cc.z, i)), acc);
          acc = fmaf(vv.w, __ldcg(u + CI::col(cc.w, i)), acc);
        }
        w[i] = acc;
        dots[0].add(ri * ui);
        dots[1].add(acc * ui);
        dots[2].add(ri * ri);
      }
      // every thread is done with the stage: refill it with item qc + 2 (the row
      // block after next, or one of the next iteration's first two: the matrix does
      // not change)
      __syncthreads();
      if (qc + 2 < nitems) {
        if (tid == 0) issue(qc + 2);
        inflight |= 1u << st;
      }
    }
    if (!ok) break;
    {
      __shared__ ff shb[3][32];
      ff v3[3] = {dots[0].v, dots[1].v, dots[2].v};
      block_sum_ff_pair<3>(v3, shb);
      if (tid == 0)
        for (int j = 0; j < 3; ++j) partials[(size_t)blockIdx.x * 3 + j] = make_float2(v3[j].hi, v3[j].lo);
    }
    if (!barrier(true)) { ok = false; break; }
  }
  // drain the copies still in flight (the prefetch for an iteration that did not run)
  if (tid == 0) {
    for (int st = 0; st < 2; ++st)
      if (inflight & (1u << st))
        if (mbar_wait(&mbar[st], (phase >> st) & 1u, 1 << 20)) inflight &= ~(1u << st);
    if (!ok || inflight) {
      atomicExch(ictl + I_FAULT, 1);
      atomicExch(ictl + I_DONE, 1);
    }
  }
  __syncthreads();
}

// ------------------------------------------------------------------ FP32 pipelined CG
// Pipelined Jacobi-PCG (Ghysels and Vanroose, "Hiding global synchronization latency
// in the preconditioned Conjugate Gradient algorithm", Parallel Computing 40, 2014):
// the dot products of iteration i are formed by the vector pass of iteration i - 1,
// and their grid-wide sum is finished by one extra block of the SpMV of iteration i
// while the other blocks compute n = A m, so no block waits for a reduction tail.
// With M = D^-1 the preconditioned vectors u = D r and q = D s need no storage:
//   gamma = r.Dr, delta = w.Dr, |r|^2          (partials of the previous vector pass)
//   n = A m                                    (SpMV; its extra block finishes the dots:
//   beta = gamma / gamma_old, alpha = gamma / (delta - beta gamma / alpha_old))
//   z = n + beta z, s = w + beta s, p = Dr + beta p,
//   x += alpha p, r -= alpha s, w -= alpha z, m = D w     (vector pass)
// in exact arithmetic w = A D r, s = A p, z = A D s.  Start: r = r0, m = D r, w = A m
// (plain SpMV), then one vector pass with alpha = beta = 0 gives m = D w and the
// first dots.  Stopping test on the recursive |r|^2, as the other variants.

// r = scale * rin (FP32), m = D r, x = s = p = z = n = 0; scalars and control words.
__global__ void k_pcg32_init(int64_t n, int64_t np, const double *__restrict__ rin, double scale,
                             const float *__restrict__ dinv, float *__restrict__ r, float *__restrict__ m,
                             float *__restrict__ x, float *__restrict__ s, float *__restrict__ p,
                             float *__restrict__ z, float *__restrict__ nv, double tol2_rel, int maxit, double *scal,
                             int *ictl) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < np; i += stride) {
    const float ri = (i < n) ? (float)(scale * rin[i]) : 0.f;
    r[i] = ri;
    m[i] = dinv[i] * ri;
    x[i] = 0.f;
    s[i] = 0.f;
    p[i] = 0.f;
    z[i] = 0.f;
    nv[i] = 0.f;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    scal[S_TOL2] = tol2_rel;
    scal[S_ALPHA] = 0.0;
    scal[S_BETA] = 0.0;
    scal[S_RZ] = 0.0;
    ictl[I_ITERS] = 0;
    ictl[I_MAXIT] = maxit;
    ictl[I_STATUS] = 0;
    ictl[I_FAULT] = 0;
    ictl[I_DONE] = 0;
    ictl[I_BODIES] = 0;
    ictl[I_PIPE_FIRST] = 1;
  }
}

// Scalars of one pipelined iteration from gamma, delta and |r|^2 (one thread).
__device__ __forceinline__ void pcg_scalars(const double (&tot)[3], double *scal, int *ictl) {
  const double gam = tot[0], del = tot[1], rr = tot[2];
  const int it = ictl[I_ITERS];
  if (ictl[I_PIPE_FIRST]) {
    scal[S_TOL2] = scal[S_TOL2] * rr;  // relative threshold -> absolute, from r0.r0
    ictl[I_PIPE_FIRST] = 0;
  }
  scal[S_RR] = rr;
  int st = -1;
  if (!isfinite(rr) || !isfinite(gam) || !isfinite(del)) st = 2;
  else if (rr == 0.0 || rr <= scal[S_TOL2]) st = 0;
  else if (it >= ictl[I_MAXIT]) st = 1;
  if (st >= 0) {
    ictl[I_STATUS] = st;
    ictl[I_DONE] = 1;
    return;
  }
  double alpha, beta = 0.0;
  if (it == 0) {
    alpha = (del != 0.0) ? gam / del : 0.0;
  } else {
    const double gold = scal[S_RZ], aold = scal[S_ALPHA];
    beta = (gold != 0.0) ? gam / gold : 0.0;
    const double den = del - beta * gam / aold;
    alpha = (den != 0.0) ? gam / den : 0.0;
  }
  scal[S_RZ] = gam;
  scal[S_ALPHA] = alpha;
  scal[S_BETA] = beta;
  ictl[I_ITERS] = it + 1;
}

// Vector pass of the pipelined iteration, four rows per thread; each block leaves its
// compensated partial sums of gamma, delta and |r|^2 in partials[block][3].
__global__ void __launch_bounds__(256) k_pcg32_vec(int64_t n4, float4 *__restrict__ x, float4 *__restrict__ r,
                                                   float4 *__restrict__ w, float4 *__restrict__ s,
                                                   float4 *__restrict__ p, float4 *__restrict__ z,
                                                   const float4 *__restrict__ nv, float4 *__restrict__ m,
                                                   const float4 *__restrict__ dinv, const double *scal,
                                                   const int *ictl, float2 *__restrict__ partials) {
  if (ictl[I_DONE]) return;
  const float alpha = (float)scal[S_ALPHA], beta = (float)scal[S_BETA];
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  ff acc[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
  if (j < n4) {
    const float4 nn = nv[j], dd = dinv[j];
    float4 zz = z[j], ww = w[j], ss = s[j], rr = r[j], pp = p[j], xx = x[j];
    float4 mm;
#define FG_PCG_LANE(c)                                \
  {                                                   \
    zz.c = fmaf(beta, zz.c, nn.c);                    \
    ss.c = fmaf(beta, ss.c, ww.c);                    \
    pp.c = fmaf(beta, pp.c, dd.c * rr.c);             \
    xx.c = fmaf(alpha, pp.c, xx.c);                   \
    rr.c = fmaf(-alpha, ss.c, rr.c);                  \
    ww.c = fmaf(-alpha, zz.c, ww.c);                  \
    mm.c = dd.c * ww.c;                               \
    const float uc = dd.c * rr.c;                     \
    acc[0] = ff_add(acc[0], ff{rr.c * uc, 0.f});      \
    acc[1] = ff_add(acc[1], ff{ww.c * uc, 0.f});      \
    acc[2] = ff_add(acc[2], ff{rr.c * rr.c, 0.f});    \
  }
    FG_PCG_LANE(x) FG_PCG_LANE(y) FG_PCG_LANE(z) FG_PCG_LANE(w)
#undef FG_PCG_LANE
    z[j] = zz;
    s[j] = ss;
    p[j] = pp;
    x[j] = xx;
    r[j] = rr;
    w[j] = ww;
    m[j] = mm;
  }
  __shared__ ff shb[3][32];
  block_sum_ff_pair<3>(acc, shb);
  if (threadIdx.x == 0)
    for (int k = 0; k < 3; ++k) partials[(size_t)blockIdx.x * 3 + k] = make_float2(acc[k].hi, acc[k].lo);
}

// out = A in with the matrix entries staged by bulk copies (as k_cg32s_spmv_bulk, no
// dot products).  With nparts > 0, block 0 does no SpMV work: it sums the nparts
// partials of the last vector pass in index order and sets the iteration's scalars,
// while blocks 1.. walk the 256-row blocks.
template <class CI>
__global__ void __launch_bounds__(256) k_pcg32_spmv_bulk(int64_t n, int nslices, int cap,
                                                         const int *__restrict__ sl_ptr,
                                                         const int *__restrict__ sl_len,
                                                         const typename CI::T *__restrict__ col,
                                                         const float *__restrict__ val, const float *__restrict__ in,
                                                         float *__restrict__ out, double *scal, int *ictl,
                                                         const float2 *__restrict__ partials, int nparts) {
  using T = typename CI::T;
  using T4 = typename CI::T4;
  extern __shared__ __align__(128) unsigned char sm_bulk[];
  __shared__ __align__(8) uint64_t bar[2];
  if (ictl[I_DONE]) return;
  const int tid = threadIdx.x;
  if (nparts > 0 && blockIdx.x == 0) {
    ff acc[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    for (int k = tid; k < nparts; k += 256)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const float2 q = __ldcg(partials + (size_t)k * 3 + j);
        acc[j] = ff_add(acc[j], ff{q.x, q.y});
      }
    __shared__ ff shr[3][32];
    block_sum_ff_pair<3>(acc, shr);
    if (tid == 0) {
      double tot[3];
      for (int j = 0; j < 3; ++j) tot[j] = (double)acc[j].hi + (double)acc[j].lo;
      pcg_scalars(tot, scal, ictl);
    }
    return;
  }
  const int off = nparts > 0 ? 1 : 0;
  const int nb = (int)gridDim.x - off, b = (int)blockIdx.x - off;
  const size_t o_col = pipe_align((size_t)cap * 4);
  const size_t stage = o_col + pipe_align((size_t)cap * sizeof(T));
  const int64_t nrb = (n + 255) / 256;
  const int K = (int)((nrb - (int64_t)b + nb - 1) / nb);
  auto rowblock = [&](int k) { return (int64_t)b + (int64_t)k * nb; };
  auto issue = [&](int k, int st) {
    const int s0 = (int)(rowblock(k) * (256 / FG_SLICE)), s1 = min(s0 + 256 / FG_SLICE, nslices);
    const int e0 = sl_ptr[s0], e1 = sl_ptr[s1];
    const uint32_t vb = (uint32_t)(e1 - e0) * 4u, cb = (uint32_t)(e1 - e0) * (uint32_t)sizeof(T);
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(&bar[st], vb + cb);
    bulk_g2s(sm_bulk + st * stage, val + e0, vb, &bar[st]);
    bulk_g2s(sm_bulk + st * stage + o_col, col + e0, cb, &bar[st]);
  };
  uint32_t inflight = 0u;
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_proxy_async_smem();
  }
  __syncthreads();
  if (tid == 0) {
    if (K > 0) issue(0, 0);
    if (K > 1) issue(1, 1);
  }
  inflight = (K > 1) ? 3u : (K > 0 ? 1u : 0u);
  uint32_t phase = 0u;
  bool ok = true;
  for (int k = 0; k < K; ++k) {
    const int st = k & 1;
    const int64_t rb = rowblock(k);
    const int64_t i = rb * 256 + tid;
    const bool row = i < n;
    int G = 0, base = 0;
    if (row) {
      const int sl = (int)(i >> 5);
      G = sl_len[sl];
      base = sl_ptr[sl] - sl_ptr[rb * (256 / FG_SLICE)] + (tid & 31) * FG_GROUP;
    }
    const bool got = mbar_wait(&bar[st], (phase >> st) & 1u);
    if (got) {
      phase ^= 1u << st;
      inflight &= ~(1u << st);
    }
    if (__syncthreads_or(!got)) { ok = false; break; }
    if (row) {
      const float *v = reinterpret_cast<const float *>(sm_bulk + st * stage);
      const T *c = reinterpret_cast<const T *>(sm_bulk + st * stage + o_col);
      float acc = 0.f;
#pragma unroll 4
      for (int g = 0; g < G; ++g) {
        const float4 vv = *reinterpret_cast<const float4 *>(v + base + g * FG_SLICE * FG_GROUP);
        const T4 cc = *reinterpret_cast<const T4 *>(c + base + g * FG_SLICE * FG_GROUP);
        acc = fmaf(vv.x, __ldg(in + CI::col(cc.x, i)), acc);
        acc = fmaf(vv.y, __ldg(in + CI::col(cc.y, i)), acc);
        acc = fmaf(vv.z, __ldg(in + CI::col(cc.z, i)), acc);
        acc = fmaf(vv.w, __ldg(in + CI::col(cc.w, i)), acc);
      }
      out[i] = acc;
    }
    __syncthreads();
    if (k + 2 < K) {
      if (tid == 0) issue(k + 2, st);
      inflight |= 1u << st;
    }
  }
  if (!ok && tid == 0) {
    // a stage did not arrive: wait (bounded) for the copies in flight, stop the CG
    for (int st = 0; st < 2; ++st)
      if (inflight & (1u << st)) mbar_wait(&bar[st], (phase >> st) & 1u, 1 << 20);
    atomicExch(ictl + I_FAULT, 1);
    atomicExch(ictl + I_DONE, 1);
  }
}

// Jacobi-PCG as plain CG on the symmetrically scaled system (the scaled split
// variant): A' = S A S with S = D^-1/2 (sdiag = sqrt of the Jacobi inverse, 0 on
// Dirichlet rows), b' = S b, x = S y.  The iterates are those of Jacobi-PCG; the
// preconditioned residual u = r' needs no vector of its own, and the stopping test
// measures the unscaled residual |r| = |S^-1 r'| (r.r = sum D_ii r'_i^2), as
// Jacobi-PCG does.
__global__ void k_sdiag32(int64_t np, const float *__restrict__ dinv, float *__restrict__ sdiag,
                          float *__restrict__ diag) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const float d = dinv[i];
  sdiag[i] = sqrtf(d);
  diag[i] = (d > 0.f) ? 1.f / d : 0.f;  // D_ii, the weight of r'_i^2 in the unscaled r.r
}

template <class CI>
__global__ void k_scale_op32(int64_t n, const int *__restrict__ sl_ptr, const int *__restrict__ sl_len,
                             const typename CI::T *__restrict__ col, const float *__restrict__ val,
                             const float *__restrict__ sdiag, float *__restrict__ vals) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int s = (int)(i >> 5), lane = (int)(i & 31);
  const float si = sdiag[i];
  const int L = FG_GROUP * sl_len[s];
  for (int q = 0; q < L; ++q) {
    const int64_t e = sell_pos(sl_ptr[s], lane, q);
    vals[e] = val[e] * si * sdiag[CI::col(col[e], i)];
  }
}

// r' = S (scale rin), s = p = y = 0.
__global__ void k_cg32ss_init(int64_t n, int64_t np, const double *__restrict__ rin, double scale,
                              const float *__restrict__ sdiag, float *__restrict__ r, float *__restrict__ s,
                              float *__restrict__ p, float *__restrict__ y, double tol2_rel, int maxit, double *scal,
                              int *ictl) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < np; i += stride) {
    r[i] = (i < n) ? (float)(scale * rin[i]) * sdiag[i] : 0.f;
    s[i] = 0.f;
    p[i] = 0.f;
    y[i] = 0.f;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    scal[S_TOL2] = tol2_rel;
    scal[S_ALPHA] = 0.0;
    scal[S_BETA] = 0.0;
    ictl[I_ITERS] = -1;
    ictl[I_MAXIT] = maxit;
    ictl[I_STATUS] = 0;
    ictl[I_FAULT] = 0;
    ictl[I_DONE] = 0;
    ictl[I_BODIES] = 0;
  }
}

// s = w + beta s, p = r + beta p, y += alpha p, r -= alpha s (four rows per thread).
__global__ void __launch_bounds__(256) k_cg32ss_vec(int64_t n4, float4 *__restrict__ r, const float4 *__restrict__ w,
                                                    float4 *__restrict__ s, float4 *__restrict__ p,
                                                    float4 *__restrict__ y, const double *scal, const int *ictl) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n4) return;
  const int done = ictl[I_DONE];
  const double alpha_d = scal[S_ALPHA], beta_d = scal[S_BETA];
  const float4 ww = w[j];
  float4 ss = s[j], pp = p[j], yy = y[j], rr = r[j];
  if (done) return;
  const float alpha = (float)alpha_d, beta = (float)beta_d;
  ss.x = fmaf(beta, ss.x, ww.x); ss.y = fmaf(beta, ss.y, ww.y); ss.z = fmaf(beta, ss.z, ww.z); ss.w = fmaf(beta, ss.w, ww.w);
  pp.x = fmaf(beta, pp.x, rr.x); pp.y = fmaf(beta, pp.y, rr.y); pp.z = fmaf(beta, pp.z, rr.z); pp.w = fmaf(beta, pp.w, rr.w);
  yy.x = fmaf(alpha, pp.x, yy.x); yy.y = fmaf(alpha, pp.y, yy.y); yy.z = fmaf(alpha, pp.z, yy.z); yy.w = fmaf(alpha, pp.w, yy.w);
  rr.x = fmaf(-alpha, ss.x, rr.x); rr.y = fmaf(-alpha, ss.y, rr.y); rr.z = fmaf(-alpha, ss.z, rr.z); rr.w = fmaf(-alpha, ss.w, rr.w);
  s[j] = ss;
  p[j] = pp;
  y[j] = yy;
  r[j] = rr;
}

// x += scale * S y (the solution of the unscaled system).
__global__ void k_axpy_scaled_to64(int64_t n, double scale, const float *__restrict__ sdiag,
                                   const float *__restrict__ y, double *__restrict__ x) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] += scale * (double)(sdiag[i] * y[i]);
}

// r = scale * rin, u = D^-1 r, s = p = x = 0 for the split FP32 iteration.
__global__ void k_cg32s_init(int64_t n, int64_t np, const double *__restrict__ rin, double scale,
                             const float *__restrict__ dinv, float *__restrict__ r, float *__restrict__ u,
                             float *__restrict__ s, float *__restrict__ p, float *__restrict__ x, double tol2_rel,
                             int maxit, double *scal, int *ictl) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < np; i += stride) {
    const float ri = (i < n) ? (float)(scale * rin[i]) : 0.f;
    r[i] = ri;
    u[i] = dinv[i] * ri;
    s[i] = 0.f;
    p[i] = 0.f;
    x[i] = 0.f;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    scal[S_TOL2] = tol2_rel;
    scal[S_ALPHA] = 0.0;
    scal[S_BETA] = 0.0;
    ictl[I_ITERS] = -1;
    ictl[I_MAXIT] = maxit;
    ictl[I_STATUS] = 0;
    ictl[I_FAULT] = 0;
    ictl[I_DONE] = 0;
    ictl[I_BODIES] = 0;
  }
}

// r0 = scale * rin, state (r0, 0, 0, dinv) in both buffers, p = x = 0.  The threshold
// tol2_rel becomes absolute (times r0.r0) in the first iteration.
__global__ void k_cg32_init(int64_t n, int64_t np, const double *__restrict__ rin, double scale,
                            const float *__restrict__ dinv, float4 *__restrict__ st0, float4 *__restrict__ st1,
                            float *__restrict__ p, float *__restrict__ x, double tol2_rel, int maxit, double *scal,
                            int *ictl) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < np; i += stride) {
    const float ri = (i < n) ? (float)(scale * rin[i]) : 0.f;
    const float4 v = make_float4(ri, 0.f, 0.f, dinv[i]);
    st0[i] = v;
    st1[i] = v;
    p[i] = 0.f;
    x[i] = 0.f;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    scal[S_TOL2] = tol2_rel;
    scal[S_ALPHA] = 0.0;
    scal[S_BETA] = 0.0;
    ictl[I_ITERS] = -1;
    ictl[I_MAXIT] = maxit;
    ictl[I_STATUS] = 0;
    ictl[I_FAULT] = 0;
    ictl[I_DONE] = 0;
    ictl[I_BODIES] = 0;
  }
}

// ------------------------------------------------------------------ FP64 CG
// Pointwise part: s = w + beta s, p = u + beta p, x += alpha p, r -= alpha s, u = D^-1 r
// (two rows per thread, double2).
__global__ void __launch_bounds__(256) k_cg64_vec(int64_t n2, double2 *__restrict__ r, const double2 *__restrict__ w,
                                                  double2 *__restrict__ s, double2 *__restrict__ p,
                                                  double2 *__restrict__ u, double2 *__restrict__ x,
                                                  const double2 *__restrict__ dinv, const double *scal,
                                                  const int *ictl) {
  if (ictl[I_DONE]) return;
  const double alpha = scal[S_ALPHA], beta = scal[S_BETA];
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n2) return;
  const double2 ww = w[j], dd = dinv[j], uu = u[j];
  double2 ss = s[j], pp = p[j], xx = x[j], rr = r[j];
  ss.x = fma(beta, ss.x, ww.x); ss.y = fma(beta, ss.y, ww.y);
  pp.x = fma(beta, pp.x, uu.x); pp.y = fma(beta, pp.y, uu.y);
  xx.x = fma(alpha, pp.x, xx.x); xx.y = fma(alpha, pp.y, xx.y);
  rr.x = fma(-alpha, ss.x, rr.x); rr.y = fma(-alpha, ss.y, rr.y);
  s[j] = ss;
  p[j] = pp;
  x[j] = xx;
  r[j] = rr;
  u[j] = make_double2(dd.x * rr.x, dd.y * rr.y);
}

// w = A u with gamma = r.u, delta = w.u and r.r reduced; the last block sets the
// next alpha, beta and the stopping test.
// PERSIST: a grid of a few blocks per SM walks the 256-row blocks (one reduction per
// block for all of its rows, as in k_cg32s_spmv).
template <class CI, bool PERSIST>
__global__ void __launch_bounds__(256) k_cg64_spmv(int64_t n, const int *__restrict__ sl_ptr,
                                                   const int *__restrict__ sl_len,
                                                   const typename CI::T *__restrict__ col,
                                                   const double *__restrict__ val, const double *__restrict__ u,
                                                   const double *__restrict__ r, double *__restrict__ w,
                                                   double *scal, int *ictl, double *partials, unsigned *counter) {
  if (ictl[I_DONE]) return;
  double d3[3] = {0.0, 0.0, 0.0};
  const int64_t nrb = (n + 255) / 256;
  for (int64_t rb = blockIdx.x; rb < (PERSIST ? nrb : (int64_t)blockIdx.x + 1); rb += gridDim.x) {
  const int64_t i = rb * 256 + threadIdx.x;
  if (i < n) {
    const int s = (int)(i >> 5), lane = (int)(i & 31);
    const int64_t base = (int64_t)sl_ptr[s] + lane * FG_GROUP;
    const int G = sl_len[s];
    const double2 *v2 = reinterpret_cast<const double2 *>(val + base);
    const typename CI::T4 *c4 = reinterpret_cast<const typename CI::T4 *>(col + base);
    double acc = 0.0;
#pragma unroll 4
    for (int g = 0; g < G; ++g) {
      const double2 va = __ldg(v2 + (int64_t)g * 2 * FG_SLICE);
      const double2 vb = __ldg(v2 + (int64_t)g * 2 * FG_SLICE + 1);
      const typename CI::T4 cc = ld_cols(c4 + (int64_t)g * FG_SLICE);
      acc = fma(va.x, __ldg(u + CI::col(cc.x, i)), acc);
      acc = fma(va.y, __ldg(u + CI::col(cc.y, i)), acc);
      acc = fma(vb.x, __ldg(u + CI::col(cc.z, i)), acc);
      acc = fma(vb.y, __ldg(u + CI::col(cc.w, i)), acc);
    }
    w[i] = acc;
    const double ui = u[i], ri = r[i];
    d3[0] = fma(ri, ui, d3[0]);
    d3[1] = fma(acc, ui, d3[1]);
    d3[2] = fma(ri, ri, d3[2]);
  }
  }
  __shared__ double shd[3][32];
  block_sum<3>(d3, shd);
  double tot[3];
  if (grid_finish<3>(d3, partials, counter, tot)) cgcg_scalars(tot, scal, ictl);
}

// FP64 w = A u with halo staging of u (see k_cg32_iter_halo) and the dot products.
template <int R>
__global__ void __launch_bounds__(R) k_cg64_spmv_halo(int64_t n, const int *__restrict__ sl_ptr,
                                                      const int *__restrict__ sl_len,
                                                      const uint16_t *__restrict__ lcol,
                                                      const double *__restrict__ val, const int *__restrict__ halo_col,
                                                      const int *__restrict__ halo_len, int hcap,
                                                      const double *__restrict__ u, const double *__restrict__ r,
                                                      double *__restrict__ w, double *scal, int *ictl,
                                                      double *partials, unsigned *counter) {
  extern __shared__ double ud[];
  if (ictl[I_DONE]) return;
  {
    constexpr int HB = 8;  // a batch of indices, then their values: HB independent gathers in flight
    const int hl = halo_len[blockIdx.x];
    const int *hc = halo_col + (int64_t)blockIdx.x * hcap;
    for (int h0 = threadIdx.x; h0 < hl; h0 += HB * R) {
      int idx[HB];
#pragma unroll
      for (int k = 0; k < HB; ++k) idx[k] = (h0 + k * R < hl) ? __ldg(hc + h0 + k * R) : -1;
      double v[HB];
#pragma unroll
      for (int k = 0; k < HB; ++k) v[k] = (idx[k] >= 0) ? __ldg(u + idx[k]) : 0.0;
#pragma unroll
      for (int k = 0; k < HB; ++k)
        if (idx[k] >= 0) ud[h0 + k * R] = v[k];
    }
  }
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * R + threadIdx.x;
  double d3[3] = {0.0, 0.0, 0.0};
  if (i < n) {
    const int s = (int)(i >> 5), lane = (int)(i & 31);
    const int64_t base = (int64_t)sl_ptr[s] + lane * FG_GROUP;
    const int G = sl_len[s];
    const double2 *v2 = reinterpret_cast<const double2 *>(val + base);
    const ushort4 *c4 = reinterpret_cast<const ushort4 *>(lcol + base);
    double acc = 0.0;
#pragma unroll 4
    for (int g = 0; g < G; ++g) {
      const double2 va = __ldg(v2 + (int64_t)g * 2 * FG_SLICE);
      const double2 vb = __ldg(v2 + (int64_t)g * 2 * FG_SLICE + 1);
      const ushort4 cc = __ldg(c4 + (int64_t)g * FG_SLICE);
      acc = fma(va.x, ud[cc.x], acc);
      acc = fma(va.y, ud[cc.y], acc);
      acc = fma(vb.x, ud[cc.z], acc);
      acc = fma(vb.y, ud[cc.w], acc);
    }
    w[i] = acc;
    const double ui = u[i], ri = r[i];
    d3[0] = ri * ui;
    d3[1] = acc * ui;
    d3[2] = ri * ri;
  }
  __shared__ double shd[3][32];
  block_sum<3>(d3, shd);
  double tot[3];
  if (grid_finish<3>(d3, partials, counter, tot)) cgcg_scalars(tot, scal, ictl);
}

// r = scale * rin, u = D^-1 r, s = p = x = 0 (w comes from the first SpMV).
__global__ void k_cg64_init(int64_t n, int64_t np, const double *__restrict__ rin, double scale,
                            const double *__restrict__ dinv, double *__restrict__ r, double *__restrict__ u,
                            double *__restrict__ s, double *__restrict__ p, double *__restrict__ x, double tol2_rel,
                            int maxit, double *scal, int *ictl) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < np; i += stride) {
    const double ri = (i < n) ? scale * rin[i] : 0.0;
    r[i] = ri;
    u[i] = dinv[i] * ri;
    s[i] = 0.0;
    p[i] = 0.0;
    x[i] = 0.0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    scal[S_TOL2] = tol2_rel;
    scal[S_ALPHA] = 0.0;
    scal[S_BETA] = 0.0;
    ictl[I_ITERS] = -1;
    ictl[I_MAXIT] = maxit;
    ictl[I_STATUS] = 0;
    ictl[I_FAULT] = 0;
    ictl[I_DONE] = 0;
    ictl[I_BODIES] = 0;
  }
}

// ------------------------------------------------------------------ FP64 helpers
// y = A x (FP64 operator); with b != null, r = b - A x.  Rows with fixed[i] are set
// to 0.  Reduces r.r into scal[slot] when slot >= 0.
template <class CI>
__global__ void __launch_bounds__(256) k_spmv64(int64_t n, const int *__restrict__ sl_ptr,
                                                const int *__restrict__ sl_len, const typename CI::T *__restrict__ col,
                                                const double *__restrict__ val, const double *__restrict__ x,
                                                const double *__restrict__ b, double *__restrict__ y,
                                                const uint8_t *__restrict__ fixed, int slot, double *scal,
                                                double *partials, unsigned *counter) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double rr = 0.0;
  if (i < n) {
    const int s = (int)(i >> 5), lane = (int)(i & 31);
    const int64_t base = (int64_t)sl_ptr[s] + lane * FG_GROUP;
    const int G = sl_len[s];
    double acc = 0.0;
    for (int g = 0; g < G; ++g) {
      const typename CI::T4 cc = ld_cols(reinterpret_cast<const typename CI::T4 *>(col + base) + (int64_t)g * FG_SLICE);
      const double *vg = val + base + (int64_t)g * FG_GROUP * FG_SLICE;
      acc = fma(vg[0], x[CI::col(cc.x, i)], acc);
      acc = fma(vg[1], x[CI::col(cc.y, i)], acc);
      acc = fma(vg[2], x[CI::col(cc.z, i)], acc);
      acc = fma(vg[3], x[CI::col(cc.w, i)], acc);
    }
    double v = b ? b[i] - acc : acc;
    if (fixed && fixed[i]) v = 0.0;
    y[i] = v;
    rr = v * v;
  }
  if (slot < 0) return;
  __shared__ double shd[1][32];
  double part[1] = {rr};
  block_sum<1>(part, shd);
  double tot[1];
  if (grid_finish<1>(part, partials, counter, tot)) scal[slot] = tot[0];
}

__global__ void __launch_bounds__(256) k_dot64(int64_t n, const double *__restrict__ x, const double *__restrict__ y,
                                               const uint8_t *__restrict__ fixed, int slot, double *scal,
                                               double *partials, unsigned *counter) {
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (!fixed || !fixed[i]) acc += x[i] * (y ? y[i] : 1.0);
  __shared__ double shd[1][32];
  double part[1] = {acc};
  block_sum<1>(part, shd);
  double tot[1];
  if (grid_finish<1>(part, partials, counter, tot)) scal[slot] = tot[0];
}

// (y.y, y.z, z.z) over the rows with mask 0: the coefficients of |y + a z|^2 on those
// rows as a quadratic in a; and (u.u, u.du, du.du) over all rows, those of
// |u + a du|^2 (fixed-order grid reduction).
__global__ void __launch_bounds__(256) k_lin_quad(int64_t n, const double *__restrict__ y, const double *__restrict__ z,
                                                  const uint8_t *__restrict__ mask, const double *__restrict__ u,
                                                  const double *__restrict__ du, double *out, double *partials,
                                                  unsigned *counter) {
  double v[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  auto add = [&](double a, double b, bool in, double p, double q) {
    if (in) {
      v[0] = fma(a, a, v[0]);
      v[1] = fma(a, b, v[1]);
      v[2] = fma(b, b, v[2]);
    }
    v[3] = fma(p, p, v[3]);
    v[4] = fma(p, q, v[4]);
    v[5] = fma(q, q, v[5]);
  };
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  // four rows' loads in flight before their sums, which keep the row order of a plain
  // grid-stride loop
  for (; i + 3 * stride < n; i += 4 * stride) {
    double a[4], b[4], p[4], q[4];
    bool in[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int64_t j = i + r * stride;
      a[r] = y[j];
      b[r] = z[j];
      p[r] = u[j];
      q[r] = du[j];
      in[r] = !mask || !mask[j];
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) add(a[r], b[r], in[r], p[r], q[r]);
  }
  for (; i < n; i += stride) add(y[i], z[i], !mask || !mask[i], u[i], du[i]);
  __shared__ double shd[6][32];
  block_sum<6>(v, shd);
  double tot[6];
  if (grid_finish<6>(v, partials, counter, tot))
    for (int j = 0; j < 6; ++j) out[j] = tot[j];
}

// F <- -F with the sum of squares of the result (one pass instead of a negation and
// a separate dot product)
__global__ void __launch_bounds__(256) k_negate_norm64(int64_t n, double *__restrict__ F, int slot, double *scal,
                                                       double *partials, unsigned *counter) {
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double f = -F[i];
    F[i] = f;
    acc += f * f;
  }
  __shared__ double shd[1][32];
  double part[1] = {acc};
  block_sum<1>(part, shd);
  double tot[1];
  if (grid_finish<1>(part, partials, counter, tot)) scal[slot] = tot[0];
}

// x += scale * d
template <typename S>
__global__ void k_axpy_to64(int64_t n, double scale, const S *__restrict__ d, double *__restrict__ x) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] += scale * (double)d[i];
}

__global__ void k_fill64(int64_t n, double v, double *__restrict__ x) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] = v;
}

// ------------------------------------------------------------------ host helpers
static unsigned red_grid(int64_t n) {
  unsigned g = grid_for(n, 256);
  return g > (unsigned)FG_RED_BLOCKS ? (unsigned)FG_RED_BLOCKS : g;
}
static unsigned row_grid(const fg_mesh *m) { return grid_for(m->nv, 256); }

// Grid of the FP64 vector reductions: resident blocks walking the vector with a grid
// stride (4 per SM), so that each block reduces once for several thousand entries and
// the arrival chain at the end is short.
static unsigned dot_grid(const fg_mesh *m, int64_t n) {
  return std::min<unsigned>(red_grid(n), 4u * (unsigned)std::max(m->sm_count, 1));
}

void fg_dot_enqueue(fg_mesh *m, const double *x, const double *y, int64_t n, bool mask_fixed, int slot) {
  k_dot64<<<dot_grid(m, n), 256, 0, m->stream>>>(n, x, y, (mask_fixed && m->has_fixed) ? m->fixed : nullptr, slot,
                                                 m->scal, m->red.partials, m->red.counter);
  FG_CUDA_TRY(cudaGetLastError());
  FG_LAUNCHED(1);
}

void fg_lin_quad_enqueue(fg_mesh *m, const double *d_y, const double *d_z, const uint8_t *mask, const double *d_u,
                         const double *d_du, double *d_out) {
  k_lin_quad<<<dot_grid(m, m->nv), 256, 0, m->stream>>>(m->nv, d_y, d_z, mask, d_u, d_du, d_out, m->red.partials,
                                                         m->red.counter);
  FG_CUDA_TRY(cudaGetLastError());
  FG_LAUNCHED(1);
}

void fg_negate_norm2_enqueue(fg_mesh *m, double *F) {
  k_negate_norm64<<<dot_grid(m, m->nv), 256, 0, m->stream>>>(m->nv, F, FG_SLOT_FNORM2, m->scal, m->red.partials,
                                                              m->red.counter);
  FG_CUDA_TRY(cudaGetLastError());
  FG_LAUNCHED(1);
}

double fg_slot_sqrt(fg_mesh *m, int slot) {
  FG_CUDA_TRY(cudaMemcpyAsync(m->hbuf, m->scal + slot, sizeof(double), cudaMemcpyDeviceToHost, m->stream));
  fg_sync(m);
  return std::sqrt(m->hbuf[0]);
}

double fg_dot_dev(fg_mesh *m, const double *x, const double *y, int64_t n, bool mask_fixed) {
  const int slot = 8;
  fg_dot_enqueue(m, x, y, n, mask_fixed, slot);
  FG_CUDA_TRY(cudaMemcpyAsync(m->hbuf, m->scal + slot, sizeof(double), cudaMemcpyDeviceToHost, m->stream));
  fg_sync(m);
  return m->hbuf[0];
}

double fg_norm2_dev(fg_mesh *m, const double *x, int64_t n, bool mask_fixed) {
  return std::sqrt(fg_dot_dev(m, x, x, n, mask_fixed));
}

static void spmv64_launch(fg_mesh *m, const double *x, const double *b, double *y, const uint8_t *fx, int slot) {
  FG_REQUIRE(m->val64 != nullptr, FG_BAD_ARG, "no FP64 operator assembled");
  if (m->use_dcol)
    k_spmv64<ColRel><<<row_grid(m), 256, 0, m->stream>>>(m->nv, m->sl_ptr, m->sl_len, m->sl_dcol, m->val64, x, b, y,
                                                         fx, slot, m->scal, m->red.partials, m->red.counter);
  else
    k_spmv64<ColAbs><<<row_grid(m), 256, 0, m->stream>>>(m->nv, m->sl_ptr, m->sl_len, m->sl_col, m->val64, x, b, y,
                                                         fx, slot, m->scal, m->red.partials, m->red.counter);
  FG_CUDA_TRY(cudaGetLastError());
  FG_LAUNCHED(1);
}

void fg_spmv64_dev(fg_mesh *m, const double *x, double *y) { spmv64_launch(m, x, nullptr, y, nullptr, -1); }

void fg_spmv64_vals(fg_mesh *m, const double *vals, const double *x, double *y) {
  const uint8_t *fx = m->has_fixed ? m->fixed : nullptr;
  if (m->use_dcol)
    k_spmv64<ColRel><<<row_grid(m), 256, 0, m->stream>>>(m->nv, m->sl_ptr, m->sl_len, m->sl_dcol, vals, x, nullptr, y,
                                                         fx, -1, m->scal, m->red.partials, m->red.counter);
  else
    k_spmv64<ColAbs><<<row_grid(m), 256, 0, m->stream>>>(m->nv, m->sl_ptr, m->sl_len, m->sl_col, vals, x, nullptr, y,
                                                         fx, -1, m->scal, m->red.partials, m->red.counter);
  FG_CUDA_TRY(cudaGetLastError());
  FG_LAUNCHED(1);
}

// CG vectors, padded to whole slices and zeroed once (pads stay zero).
// FP32: v32[0] x, v32[1] p, v32[2] / v32[3] the two (r, w, s, dinv) state buffers of
// the fused iteration; the split iteration uses v32[4] r, [5] w, [6] s, [7] u.
// FP64: v64[0] x, v64[1] r, v64[2] u, v64[3] s, v64[4] p, v64[12] w.
static void ensure_cg32(fg_mesh *m) {
  for (int j = 0; j < 8; ++j)
    if (!m->v32[j]) {
      size_t len = (size_t)m->nvp * ((j == 2 || j == 3) ? 4 : 1);
      m->v32[j] = dev_alloc<float>(m, len);
      FG_CUDA_TRY(cudaMemsetAsync(m->v32[j], 0, sizeof(float) * len, m->stream));
    }
  for (int j = 0; j < 3; ++j)
    if (!m->pv32[j]) {
      m->pv32[j] = dev_alloc<float>(m, (size_t)m->nvp);
      FG_CUDA_TRY(cudaMemsetAsync(m->pv32[j], 0, sizeof(float) * (size_t)m->nvp, m->stream));
    }
}
static void ensure_cg64(fg_mesh *m) {
  const int idx[6] = {0, 1, 2, 3, 4, 12};
  for (int j : idx)
    if (!m->v64[j]) {
      m->v64[j] = dev_alloc<double>(m, (size_t)m->nvp);
      FG_CUDA_TRY(cudaMemsetAsync(m->v64[j], 0, sizeof(double) * (size_t)m->nvp, m->stream));
    }
}

// FP32 iteration variants (block size x load scheduling) for the autotuner.
// 0-3 fused iteration with direct gathers, 4 fused with halo staging, 5 fused and
// pipelined, 6 split (vector pass + SpMV) with direct gathers, 7 split with halo
// staging, 8 split with direct gathers in a persistent grid, 9 the same launched with
// programmatic dependent launch, 10 the same with the matrix values held in L2,
// 11-15 persistent grids of 4, 3, 5, 6 and 7 blocks per SM, 16 CG on the
// symmetrically Jacobi-scaled system with the SpMV of variant 14, 17-19 split with
// the matrix entries staged by bulk copies (4, 3, 2 blocks per SM), 20 and 21 variants
// 16 and 17 with the matrix values held in L2, 22 and 23 variants 17 and 18 with the
// dot products finished by a one-block kernel after the SpMV, 24 and 25 the
// pipelined CG (its dot products finished by one block of the bulk-staged SpMV; 4
// and 3 blocks per SM).  The pipelined variants are timed by the autotuner but
// never chosen by it: in FP32 their recurrences lose accuracy faster than CG's, so
// inner solves asked for 1e-6 stall (Newton's tight Eisenstat-Walker steps), and on
// singular systems they diverge; they run only when forced.  26: the split iteration
// of 22 run by one persistent cooperative launch for many iterations (grid barriers
// in place of kernel boundaries, the matrix prefetched across them).  27 and 28:
// variants 22 and 23 with the partials added by the last SpMV block to arrive instead
// of a one-block kernel (one launch fewer per iteration, the same iterates).
constexpr int FG_N_SPMV32 = 29;
// Split FP32 variants on the scaled system, with the values in the L2 window, and
// with the matrix entries staged by bulk copies.
static inline bool v_scaled(int v) { return v == 16 || v == 20; }
static inline bool v_window(int v) { return v == 10 || v == 20 || v == 21; }
static inline bool v_bulk(int v) { return (v >= 17 && v <= 19) || (v >= 21 && v <= 23) || v == 27 || v == 28; }
static inline bool v_splitred(int v) { return v == 22 || v == 23; }
static inline bool v_last1(int v) { return v == 27 || v == 28; }
static inline bool split32(int v) { return v >= 6; }
static inline bool v_pipe(int v) { return v == 24 || v == 25; }
static inline bool v_coop(int v) { return v == 26; }
constexpr int FG_N_SPMV64 = 4;   // 0 direct gathers, 1 halo staging, 2/3 persistent with 4/8 blocks per SM

template <class CI>
static void iter32_variant(fg_mesh *m, int v, const typename CI::T *col, const float4 *in, float4 *out) {
  auto go = [&](auto kern, int bs) {
    kern<<<grid_for(m->nv, bs), bs, 0, m->stream>>>(m->nv, m->sl_ptr, m->sl_len, col, m->val32, in, out, m->v32[1],
                                                     m->v32[0], m->scal, m->ictl, m->red.partials, m->red.counter);
  };
  switch (v) {
    case 1: go(k_cg32_iter<CI, true, 256>, 256); break;
    case 2: go(k_cg32_iter<CI, false, 128>, 128); break;
    case 3: go(k_cg32_iter<CI, false, 512>, 512); break;
    default: go(k_cg32_iter<CI, false, 256>, 256); break;
  }
}

// Launch of a halo kernel instantiated for the handle's rows per CTA.
template <template <int> class K, class... Args>
static void halo_launch(fg_mesh *m, size_t elem_bytes, Args... args) {
  const size_t smem = (size_t)std::max(m->hmax, 1) * elem_bytes;
  auto go = [&](auto kern, int R) {
    if (smem > 48 * 1024)
      FG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<m->nhblocks, R, smem, m->stream>>>(args...);
  };
  switch (m->hrows) {
    case 512: go(K<512>::fn, 512); break;
    case 256: go(K<256>::fn, 256); break;
    case 128: go(K<128>::fn, 128); break;
    case 64: go(K<64>::fn, 64); break;
    default: go(K<32>::fn, 32); break;
  }
}
template <int R>
struct Iter32Halo {
  static constexpr auto fn = k_cg32_iter_halo<R>;
};
template <int R>
struct Spmv64Halo {
  static constexpr auto fn = k_cg64_spmv_halo<R>;
};

template <int R>
struct Iter32Pipe {
  static constexpr auto fn = k_cg32_iter_pipe<R>;
};

// Persistent pipelined iteration: two stages of shared memory per CTA, as many CTAs
// as fit on the GPU at once (never more than there are row blocks).  Sized on first
// use; pipe_grid = -1 when one CTA's stages do not fit in shared memory.
static bool pipe_available(fg_mesh *m) {
  if (!fg_ensure_halo(m)) return false;
  if (m->pipe_grid != 0) return m->pipe_grid > 0;
  const int HM = (m->hmax + 3) & ~3;
  const size_t smem = 2 * pipe_stage_bytes(HM, m->tmax);
  int dev_max = 0;
  FG_CUDA_TRY(cudaDeviceGetAttribute(&dev_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, m->device));
  if (smem + 4096 > (size_t)dev_max) { m->pipe_grid = -1; return false; }
  int per_sm = 0;
  auto size = [&](auto kern, int R) {
    FG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    FG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, R, smem));
  };
  switch (m->hrows) {
    case 512: size(Iter32Pipe<512>::fn, 512); break;
    case 256: size(Iter32Pipe<256>::fn, 256); break;
    case 128: size(Iter32Pipe<128>::fn, 128); break;
    case 64: size(Iter32Pipe<64>::fn, 64); break;
    default: size(Iter32Pipe<32>::fn, 32); break;
  }
  if (per_sm < 1) { m->pipe_grid = -1; return false; }
  m->pipe_grid = std::min(m->nhblocks, per_sm * std::max(m->sm_count, 1));
  return true;
}

static void pipe_launch32(fg_mesh *m, const float4 *in, float4 *out) {
  PipeArgs a;
  a.n = m->nv;
  a.ntiles = m->nhblocks;
  a.nslices = m->nslices;
  a.hcap = m->hcap;
  a.HM = (m->hmax + 3) & ~3;
  a.TM = m->tmax;
  a.sl_ptr = m->sl_ptr;
  a.sl_len = m->sl_len;
  a.halo_col = m->halo_col;
  a.halo_len = m->halo_len;
  a.lcol = m->sl_lcol;
  a.val = m->val32;
  const size_t smem = 2 * pipe_stage_bytes(a.HM, a.TM);
  auto go = [&](auto kern, int R) {
    FG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<m->pipe_grid, R, smem, m->stream>>>(a, in, out, m->v32[1], m->v32[0], m->scal, m->ictl, m->red.partials,
                                                m->red.counter);
  };
  switch (m->hrows) {
    case 512: go(Iter32Pipe<512>::fn, 512); break;
    case 256: go(Iter32Pipe<256>::fn, 256); break;
    case 128: go(Iter32Pipe<128>::fn, 128); break;
    case 64: go(Iter32Pipe<64>::fn, 64); break;
    default: go(Iter32Pipe<32>::fn, 32); break;
  }
}

template <int R>
struct Spmv32sHalo {
  static constexpr auto fn = k_cg32s_spmv_halo<R>;
};

// w = A u and the dots of the split FP32 iteration
// Launch with programmatic stream serialisation (the kernel waits for its
// predecessor with griddep_wait, so its launch overlaps the predecessor's tail).
template <typename... KArgs, typename... Args>
static void pdl_launch(bool pdl, void (*kern)(KArgs...), unsigned grid, unsigned block, size_t smem,
                       cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  FG_CUDA_TRY(cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...));
}

// L2 residency of the FP32 matrix values (variants 10 and 20): an access-policy
// window on the SpMV launches marks the values persisting in a set-aside part of L2,
// so that the iterations of an inner solve read them from L2 instead of HBM.  The
// set-aside is a limit of this process's context.  It exists only while a solve with
// such a variant runs: every other solve (FP64, or FP32 without the window) first
// returns the whole L2 to normal use (l2_for_solve), and the last handle destroyed
// releases it for good.
namespace {
std::mutex g_l2_lock;
size_t g_l2_setaside[64] = {0};
int g_l2_users[64] = {0};
}  // namespace

// Whether the device offers persisting L2 lines and access-policy windows.
static bool l2_supported(fg_mesh *m) {
  if (m->device < 0 || m->device >= 64) return false;
  int max_persist = 0, max_win = 0;
  if (cudaDeviceGetAttribute(&max_persist, cudaDevAttrMaxPersistingL2CacheSize, m->device) != cudaSuccess ||
      cudaDeviceGetAttribute(&max_win, cudaDevAttrMaxAccessPolicyWindowSize, m->device) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return max_persist > 0 && max_win > 0;
}

// Sizes the window over the FP32 values and makes sure the set-aside is in place.
static bool prepare_l2(fg_mesh *m) {
  if (m->l2_win_bytes < 0 || !m->val32) return false;
  if (!l2_supported(m)) {
    m->l2_win_bytes = -1;
    return false;
  }
  int max_persist = 0, max_win = 0;
  cudaDeviceGetAttribute(&max_persist, cudaDevAttrMaxPersistingL2CacheSize, m->device);
  cudaDeviceGetAttribute(&max_win, cudaDevAttrMaxAccessPolicyWindowSize, m->device);
  // the values only: a set-aside for values and columns (81 MB of the 135 MB L2 at
  // 96^3) left too little L2 for everything else and was slower
  const size_t want = sizeof(float) * (size_t)m->nsell;
  std::lock_guard<std::mutex> g(g_l2_lock);
  const size_t setaside = std::min(want, (size_t)max_persist);
  if (setaside > g_l2_setaside[m->device]) {
    FG_CUDA_TRY(cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, setaside));
    g_l2_setaside[m->device] = setaside;
  }
  if (m->l2_win_bytes == 0) ++g_l2_users[m->device];
  m->l2_win_bytes = (int64_t)std::min(want, (size_t)max_win);
  m->l2_hit_ratio = (float)std::min(1.0, (double)g_l2_setaside[m->device] / (double)m->l2_win_bytes);
  return true;
}

// Before a solve: the set-aside for a window variant, none for any other.
static void l2_for_solve(fg_mesh *m, bool window) {
  if (window) {
    prepare_l2(m);
    return;
  }
  std::lock_guard<std::mutex> g(g_l2_lock);
  if (m->device < 0 || m->device >= 64 || g_l2_setaside[m->device] == 0) return;
  cudaCtxResetPersistingL2Cache();
  cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, 0);
  cudaGetLastError();
  g_l2_setaside[m->device] = 0;
}

// Returns every line the process's context holds as persisting to normal, so that
// a timing does not profit from lines an earlier variant's L2 window left behind.
static void reset_persisting_l2(fg_mesh *m) {
  std::lock_guard<std::mutex> g(g_l2_lock);
  if (m->device < 0 || m->device >= 64 || g_l2_setaside[m->device] == 0) return;
  cudaCtxResetPersistingL2Cache();
  cudaGetLastError();
}

void fg_release_l2(fg_mesh *m) {
  if (m->l2_win_bytes <= 0) return;
  std::lock_guard<std::mutex> g(g_l2_lock);
  if (--g_l2_users[m->device] == 0 && g_l2_setaside[m->device] > 0) {
    cudaCtxResetPersistingL2Cache();
    cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, 0);
    g_l2_setaside[m->device] = 0;
  }
  cudaGetLastError();
  m->l2_win_bytes = 0;
}

// A launch whose accesses to the window [win, win + l2_win_bytes) persist in L2.
template <typename... KArgs, typename... Args>
static void l2_launch(fg_mesh *m, const float *win, void (*kern)(KArgs...), unsigned grid, unsigned block,
                      size_t smem, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = m->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeAccessPolicyWindow;
  attr[0].val.accessPolicyWindow.base_ptr = (void *)win;
  attr[0].val.accessPolicyWindow.num_bytes = (size_t)m->l2_win_bytes;
  attr[0].val.accessPolicyWindow.hitRatio = m->l2_hit_ratio;
  attr[0].val.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
  attr[0].val.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  FG_CUDA_TRY(cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...));
}

// The scaled operator of variant 16, rebuilt when the operator changed.
static void ensure_scaled(fg_mesh *m) {
  if (!m->val32s) m->val32s = dev_alloc<float>(m, (size_t)m->nsell);
  if (!m->sdiag32) {
    m->sdiag32 = dev_alloc<float>(m, (size_t)m->nvp);
    m->diag32 = dev_alloc<float>(m, (size_t)m->nvp);
    FG_CUDA_TRY(cudaMemsetAsync(m->sdiag32, 0, sizeof(float) * (size_t)m->nvp, m->stream));
    FG_CUDA_TRY(cudaMemsetAsync(m->diag32, 0, sizeof(float) * (size_t)m->nvp, m->stream));
  }
  if (m->val32s_version == m->op_version) return;
  k_sdiag32<<<grid_for(m->nvp, 256), 256, 0, m->stream>>>(m->nvp, m->dinv32, m->sdiag32, m->diag32);
  if (m->use_dcol)
    k_scale_op32<ColRel><<<grid_for(m->nv, 256), 256, 0, m->stream>>>(m->nv, m->sl_ptr, m->sl_len, m->sl_dcol,
                                                                      m->val32, m->sdiag32, m->val32s);
  else
    k_scale_op32<ColAbs><<<grid_for(m->nv, 256), 256, 0, m->stream>>>(m->nv, m->sl_ptr, m->sl_len, m->sl_col,
                                                                      m->val32, m->sdiag32, m->val32s);
  FG_CUDA_TRY(cudaGetLastError());
  FG_LAUNCHED(2);
  m->val32s_version = m->op_version;
}

// Shared memory of the bulk-staged SpMV: two stages of the largest 256-row block.
static size_t bulk_smem(const fg_mesh *m) {
  const size_t cb = m->use_dcol ? sizeof(int16_t) : sizeof(int);
  return 2 * (pipe_align((size_t)m->tmax256 * 4) + pipe_align((size_t)m->tmax256 * cb));
}

// Blocks per SM of the bulk-staged variants 17, 18, 19 (4, 3, 2 wanted), or 0 where
// two stages do not fit; sized once per handle.  The kernels may take up to the
// device's opt-in shared memory (set once per process).
static int bulk_per_sm(fg_mesh *m, int v) {
  // 17-19, (20: not bulk), 21: 17 with the L2 window, 22 and 23: 17 and 18 with the
  // split reduction, (24-26 sized elsewhere), 27 and 28: 22 and 23 finished by the
  // last block
  static const int kWant[12] = {4, 3, 2, 4, 4, 4, 3, 4, 3, 4, 4, 3};
  if (m->bulk_fit < 0) {
    static std::once_flag attr_once;
    static int dyn_max = 0;  // opt-in shared memory less the kernels' static shared memory
    std::call_once(attr_once, [&]() {
      int dev_max = 0;
      cudaFuncAttributes fa[2];
      if (cudaDeviceGetAttribute(&dev_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, m->device) != cudaSuccess ||
          cudaFuncGetAttributes(&fa[0], k_cg32s_spmv_bulk<ColRel>) != cudaSuccess ||
          cudaFuncGetAttributes(&fa[1], k_cg32s_spmv_bulk<ColAbs>) != cudaSuccess) {
        cudaGetLastError();
        return;
      }
      const int d = dev_max - (int)std::max(fa[0].sharedSizeBytes, fa[1].sharedSizeBytes);
      if (cudaFuncSetAttribute(k_cg32s_spmv_bulk<ColRel>, cudaFuncAttributeMaxDynamicSharedMemorySize, d) !=
              cudaSuccess ||
          cudaFuncSetAttribute(k_cg32s_spmv_bulk<ColAbs>, cudaFuncAttributeMaxDynamicSharedMemorySize, d) !=
              cudaSuccess ||
          cudaFuncSetAttribute(k_cg32s_spmv_bulk<ColRel, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, d) !=
              cudaSuccess ||
          cudaFuncSetAttribute(k_cg32s_spmv_bulk<ColAbs, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, d) !=
              cudaSuccess ||
          cudaFuncSetAttribute(k_cg32s_spmv_bulk<ColRel, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               d) != cudaSuccess ||
          cudaFuncSetAttribute(k_cg32s_spmv_bulk<ColAbs, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               d) != cudaSuccess) {
        cudaGetLastError();
        return;
      }
      dyn_max = d;
    });
    const size_t smem = bulk_smem(m);
    int per_sm = 0;
    if (m->tmax256 > 0 && smem <= (size_t)dyn_max) {
      if (m->use_dcol)
        FG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg32s_spmv_bulk<ColRel>, 256, smem));
      else
        FG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg32s_spmv_bulk<ColAbs>, 256, smem));
    }
    m->bulk_fit = per_sm;
  }
  return std::min(m->bulk_fit, kWant[v - 17]);
}

static void bulk_launch32(fg_mesh *m, int v) {
  const int per_sm = bulk_per_sm(m, v);
  FG_REQUIRE(per_sm > 0, FG_UNSUPPORTED, "bulk-staged SpMV: row blocks too large for shared memory");
  const unsigned g = std::min<unsigned>(grid_for(m->nv, 256), (unsigned)per_sm * (unsigned)std::max(m->sm_count, 1));
  const size_t smem = bulk_smem(m);
  if (v_window(v) && m->l2_win_bytes > 0) {
    // the bulk copies of the values read them from the L2 window
    if (m->use_dcol)
      l2_launch(m, m->val32, k_cg32s_spmv_bulk<ColRel>, g, 256, smem, m->nv, m->nslices, m->tmax256, m->sl_ptr,
                m->sl_len, m->sl_dcol, m->val32, m->v32[7], m->v32[4], m->v32[5], m->scal, m->ictl,
                m->red.partials, m->red.counter);
    else
      l2_launch(m, m->val32, k_cg32s_spmv_bulk<ColAbs>, g, 256, smem, m->nv, m->nslices, m->tmax256, m->sl_ptr,
                m->sl_len, m->sl_col, m->val32, m->v32[7], m->v32[4], m->v32[5], m->scal, m->ictl,
                m->red.partials, m->red.counter);
  } else if (v_last1(v)) {
    // per-block partials; the last block to arrive adds them and sets the scalars
    if (m->use_dcol)
      k_cg32s_spmv_bulk<ColRel, true, true><<<g, 256, smem, m->stream>>>(
          m->nv, m->nslices, m->tmax256, m->sl_ptr, m->sl_len, m->sl_dcol, m->val32, m->v32[7], m->v32[4],
          m->v32[5], m->scal, m->ictl, m->red.partials, m->red.counter);
    else
      k_cg32s_spmv_bulk<ColAbs, true, true><<<g, 256, smem, m->stream>>>(
          m->nv, m->nslices, m->tmax256, m->sl_ptr, m->sl_len, m->sl_col, m->val32, m->v32[7], m->v32[4],
          m->v32[5], m->scal, m->ictl, m->red.partials, m->red.counter);
  } else if (v_splitred(v)) {
    // per-block partials, then one block adds them and sets the scalars
    if (m->use_dcol)
      k_cg32s_spmv_bulk<ColRel, true><<<g, 256, smem, m->stream>>>(
          m->nv, m->nslices, m->tmax256, m->sl_ptr, m->sl_len, m->sl_dcol, m->val32, m->v32[7], m->v32[4],
          m->v32[5], m->scal, m->ictl, m->red.partials, m->red.counter);
    else
      k_cg32s_spmv_bulk<ColAbs, true><<<g, 256, smem, m->stream>>>(
          m->nv, m->nslices, m->tmax256, m->sl_ptr, m->sl_len, m->sl_col, m->val32, m->v32[7], m->v32[4],
          m->v32[5], m->scal, m->ictl, m->red.partials, m->red.counter);
    k_cg32_dots_finish<<<1, 256, 0, m->stream>>>(reinterpret_cast<const float2 *>(m->red.partials), (int)g, m->scal,
                                                 m->ictl);
  } else if (m->use_dcol)
    k_cg32s_spmv_bulk<ColRel><<<g, 256, smem, m->stream>>>(m->nv, m->nslices, m->tmax256, m->sl_ptr, m->sl_len,
                                                           m->sl_dcol, m->val32, m->v32[7], m->v32[4], m->v32[5],
                                                           m->scal, m->ictl, m->red.partials, m->red.counter);
  else
    k_cg32s_spmv_bulk<ColAbs><<<g, 256, smem, m->stream>>>(m->nv, m->nslices, m->tmax256, m->sl_ptr, m->sl_len,
                                                           m->sl_col, m->val32, m->v32[7], m->v32[4], m->v32[5],
                                                           m->scal, m->ictl, m->red.partials, m->red.counter);
}

// Blocks per SM of the pipelined variants 24 and 25 (4, 3 wanted), or 0 where two
// stages of a 256-row block do not fit; sized once per handle.
static int pipe_per_sm(fg_mesh *m, int v) {
  if (m->pipe_fit < 0) {
    static std::once_flag attr_once;
    static int dyn_max = 0;
    std::call_once(attr_once, [&]() {
      int dev_max = 0;
      cudaFuncAttributes fa[2];
      if (cudaDeviceGetAttribute(&dev_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, m->device) != cudaSuccess ||
          cudaFuncGetAttributes(&fa[0], k_pcg32_spmv_bulk<ColRel>) != cudaSuccess ||
          cudaFuncGetAttributes(&fa[1], k_pcg32_spmv_bulk<ColAbs>) != cudaSuccess) {
        cudaGetLastError();
        return;
      }
      const int d = dev_max - (int)std::max(fa[0].sharedSizeBytes, fa[1].sharedSizeBytes);
      if (cudaFuncSetAttribute(k_pcg32_spmv_bulk<ColRel>, cudaFuncAttributeMaxDynamicSharedMemorySize, d) !=
              cudaSuccess ||
          cudaFuncSetAttribute(k_pcg32_spmv_bulk<ColAbs>, cudaFuncAttributeMaxDynamicSharedMemorySize, d) !=
              cudaSuccess) {
        cudaGetLastError();
        return;
      }
      dyn_max = d;
    });
    const size_t smem = bulk_smem(m);
    int per_sm = 0;
    if (m->tmax256 > 0 && smem <= (size_t)dyn_max) {
      if (m->use_dcol)
        FG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg32_spmv_bulk<ColRel>, 256, smem));
      else
        FG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg32_spmv_bulk<ColAbs>, 256, smem));
    }
    m->pipe_fit = per_sm;
  }
  return std::min(m->pipe_fit, v == 24 ? 4 : 3);
}

// Blocks of the pipelined variants' vector pass (four rows per thread), also the
// number of dot-product partials the next SpMV's first block sums.
static unsigned pipe_vec_grid(const fg_mesh *m) { return grid_for(m->nvp / 4, 256); }

// out = A in for the pipelined variants; with `reduce` the first block finishes the
// dot products of the last vector pass instead of taking rows.  The grid never
// exceeds the resident blocks, so that reducing block runs from the start.
static void pipe_spmv32(fg_mesh *m, int v, bool reduce, const float *in, float *out) {
  const int per_sm = pipe_per_sm(m, v);
  FG_REQUIRE(per_sm > 0, FG_UNSUPPORTED, "pipelined CG: row blocks too large for shared memory");
  const unsigned resident = (unsigned)per_sm * (unsigned)std::max(m->sm_count, 1);
  const unsigned rows = grid_for(m->nv, 256);
  const unsigned g = reduce ? std::min(rows + 1, resident) : std::min(rows, resident);
  const size_t smem = bulk_smem(m);
  const int nparts = reduce ? (int)pipe_vec_grid(m) : 0;
  const float2 *parts = reinterpret_cast<const float2 *>(m->red.partials);
  if (m->use_dcol)
    k_pcg32_spmv_bulk<ColRel><<<g, 256, smem, m->stream>>>(m->nv, m->nslices, m->tmax256, m->sl_ptr, m->sl_len,
                                                           m->sl_dcol, m->val32, in, out, m->scal, m->ictl, parts,
                                                           nparts);
  else
    k_pcg32_spmv_bulk<ColAbs><<<g, 256, smem, m->stream>>>(m->nv, m->nslices, m->tmax256, m->sl_ptr, m->sl_len,
                                                           m->sl_col, m->val32, in, out, m->scal, m->ictl, parts,
                                                           nparts);
}

static void pipe_vec32(fg_mesh *m) {
  k_pcg32_vec<<<pipe_vec_grid(m), 256, 0, m->stream>>>(
      m->nvp / 4, reinterpret_cast<float4 *>(m->v32[0]), reinterpret_cast<float4 *>(m->v32[4]),
      reinterpret_cast<float4 *>(m->v32[5]), reinterpret_cast<float4 *>(m->v32[6]),
      reinterpret_cast<float4 *>(m->v32[1]), reinterpret_cast<float4 *>(m->pv32[0]),
      reinterpret_cast<const float4 *>(m->pv32[1]), reinterpret_cast<float4 *>(m->pv32[2]),
      reinterpret_cast<const float4 *>(m->dinv32), (const double *)m->scal, (const int *)m->ictl,
      reinterpret_cast<float2 *>(m->red.partials));
}

// One of the two kernels of the split-reduction variants alone (for timing): the
// SpMV that leaves per-block partials, or (finish) the one-block sum of them.
static void launch_split_parts(fg_mesh *m, int v, bool finish) {
  const int per_sm = bulk_per_sm(m, v);
  FG_REQUIRE(per_sm > 0, FG_UNSUPPORTED, "bulk-staged SpMV: row blocks too large for shared memory");
  const unsigned g = std::min<unsigned>(grid_for(m->nv, 256), (unsigned)per_sm * (unsigned)std::max(m->sm_count, 1));
  if (finish) {
    k_cg32_dots_finish<<<1, 256, 0, m->stream>>>(reinterpret_cast<const float2 *>(m->red.partials), (int)g, m->scal,
                                                 m->ictl);
    return;
  }
  const size_t smem = bulk_smem(m);
  if (m->use_dcol)
    k_cg32s_spmv_bulk<ColRel, true><<<g, 256, smem, m->stream>>>(
        m->nv, m->nslices, m->tmax256, m->sl_ptr, m->sl_len, m->sl_dcol, m->val32, m->v32[7], m->v32[4], m->v32[5],
        m->scal, m->ictl, m->red.partials, m->red.counter);
  else
    k_cg32s_spmv_bulk<ColAbs, true><<<g, 256, smem, m->stream>>>(
        m->nv, m->nslices, m->tmax256, m->sl_ptr, m->sl_len, m->sl_col, m->val32, m->v32[7], m->v32[4], m->v32[5],
        m->scal, m->ictl, m->red.partials, m->red.counter);
}

static void launch_spmv32s(fg_mesh *m, int v) {
  if (v_coop(v)) {
    // outside the persistent launch (the first SpMV of a solve, kernel timings): the
    // split-reduction SpMV and its one-block finish
    bulk_launch32(m, 22);
    return;
  }
  if (v_pipe(v)) {
    pipe_spmv32(m, v, true, m->pv32[2], m->pv32[1]);
    return;
  }
  const bool pdl = (v == 9);
  if (v == 20 && m->l2_win_bytes > 0) {
    // the scaled system (16) with its values in the L2 window
    const unsigned g = std::min<unsigned>(grid_for(m->nv, 256), 6u * (unsigned)std::max(m->sm_count, 1));
    if (m->use_dcol)
      l2_launch(m, m->val32s, k_cg32s_spmv<ColRel, true>, g, 256, 0, m->nv, m->sl_ptr, m->sl_len, m->sl_dcol,
                m->val32s, m->v32[4], m->v32[4], m->diag32, m->v32[5], m->scal, m->ictl, m->red.partials,
                m->red.counter);
    else
      l2_launch(m, m->val32s, k_cg32s_spmv<ColAbs, true>, g, 256, 0, m->nv, m->sl_ptr, m->sl_len, m->sl_col,
                m->val32s, m->v32[4], m->v32[4], m->diag32, m->v32[5], m->scal, m->ictl, m->red.partials,
                m->red.counter);
    return;
  }
  if (v_scaled(v)) {
    // w = A' r' with the dots r'.r', w.r' and r.r = sum D_ii r'_i^2 (u = r' on the scaled
    // system; the stopping test is on the unscaled residual, as in Jacobi-PCG)
    const unsigned g = std::min<unsigned>(grid_for(m->nv, 256), 6u * (unsigned)std::max(m->sm_count, 1));
    if (m->use_dcol)
      k_cg32s_spmv<ColRel, true><<<g, 256, 0, m->stream>>>(m->nv, m->sl_ptr, m->sl_len, m->sl_dcol, m->val32s,
                                                           m->v32[4], m->v32[4], m->diag32, m->v32[5], m->scal,
                                                           m->ictl, m->red.partials, m->red.counter);
    else
      k_cg32s_spmv<ColAbs, true><<<g, 256, 0, m->stream>>>(m->nv, m->sl_ptr, m->sl_len, m->sl_col, m->val32s,
                                                           m->v32[4], m->v32[4], m->diag32, m->v32[5], m->scal,
                                                           m->ictl, m->red.partials, m->red.counter);
    return;
  }
  if (v == 10 && m->l2_win_bytes > 0) {
    // the persistent grid of 14 (6 blocks per SM) with the values in the L2 window
    const unsigned g = std::min<unsigned>(grid_for(m->nv, 256), 6u * (unsigned)std::max(m->sm_count, 1));
    if (m->use_dcol)
      l2_launch(m, m->val32, k_cg32s_spmv<ColRel, true>, g, 256, 0, m->nv, m->sl_ptr, m->sl_len, m->sl_dcol, m->val32,
                m->v32[7], m->v32[4], (const float *)nullptr, m->v32[5], m->scal, m->ictl, m->red.partials,
                m->red.counter);
    else
      l2_launch(m, m->val32, k_cg32s_spmv<ColAbs, true>, g, 256, 0, m->nv, m->sl_ptr, m->sl_len, m->sl_col, m->val32,
                m->v32[7], m->v32[4], (const float *)nullptr, m->v32[5], m->scal, m->ictl, m->red.partials,
                m->red.counter);
    return;
  }
  if (v_bulk(v)) {
    bulk_launch32(m, v);
  } else if (v >= 8) {
    // persistent: 8 (variants 8-10), 4 (11), 3 (12), 5 (13), 6 (14) or 7 (15)
    // resident 256-thread blocks per SM; fewer blocks walk more row blocks each and
    // reduce once for all of them
    static const unsigned kPerSm[16] = {0, 0, 0, 0, 0, 0, 0, 0, 8, 8, 8, 4, 3, 5, 6, 7};
    const unsigned per_sm = kPerSm[v];
    const unsigned g = std::min<unsigned>(grid_for(m->nv, 256), per_sm * (unsigned)std::max(m->sm_count, 1));
    if (m->use_dcol)
      pdl_launch(pdl, k_cg32s_spmv<ColRel, true>, g, 256, 0, m->stream, m->nv, m->sl_ptr, m->sl_len, m->sl_dcol,
                 m->val32, m->v32[7], m->v32[4], (const float *)nullptr, m->v32[5], m->scal, m->ictl,
                 m->red.partials, m->red.counter);
    else
      pdl_launch(pdl, k_cg32s_spmv<ColAbs, true>, g, 256, 0, m->stream, m->nv, m->sl_ptr, m->sl_len, m->sl_col,
                 m->val32, m->v32[7], m->v32[4], (const float *)nullptr, m->v32[5], m->scal, m->ictl,
                 m->red.partials, m->red.counter);
  } else if (v == 7 && m->halo_col)
    halo_launch<Spmv32sHalo>(m, sizeof(float), m->nv, (const int *)m->sl_ptr, (const int *)m->sl_len,
                             (const uint16_t *)m->sl_lcol, (const float *)m->val32, (const int *)m->halo_col,
                             (const int *)m->halo_len, m->hcap, (const float *)m->v32[7], (const float *)m->v32[4],
                             m->v32[5], m->scal, m->ictl, m->red.partials, m->red.counter);
  else if (m->use_dcol)
    pdl_launch(false, k_cg32s_spmv<ColRel, false>, grid_for(m->nv, 256), 256, 0, m->stream, m->nv, m->sl_ptr,
               m->sl_len, m->sl_dcol, m->val32, m->v32[7], m->v32[4], (const float *)nullptr, m->v32[5], m->scal,
               m->ictl, m->red.partials, m->red.counter);
  else
    pdl_launch(false, k_cg32s_spmv<ColAbs, false>, grid_for(m->nv, 256), 256, 0, m->stream, m->nv, m->sl_ptr,
               m->sl_len, m->sl_col, m->val32, m->v32[7], m->v32[4], (const float *)nullptr, m->v32[5], m->scal,
               m->ictl, m->red.partials, m->red.counter);
}

static void launch_vec32s(fg_mesh *m, int v) {
  if (v_pipe(v)) {
    pipe_vec32(m);
    return;
  }
  if (v_scaled(v)) {
    k_cg32ss_vec<<<grid_for(m->nvp / 4, 256), 256, 0, m->stream>>>(
        m->nvp / 4, reinterpret_cast<float4 *>(m->v32[4]), reinterpret_cast<const float4 *>(m->v32[5]),
        reinterpret_cast<float4 *>(m->v32[6]), reinterpret_cast<float4 *>(m->v32[1]),
        reinterpret_cast<float4 *>(m->v32[0]), m->scal, m->ictl);
    return;
  }
  const bool pdl = (v == 9);
  pdl_launch(pdl, k_cg32s_vec, grid_for(m->nvp / 4, 256), 256, 0, m->stream, m->nvp / 4,
             reinterpret_cast<float4 *>(m->v32[4]), reinterpret_cast<const float4 *>(m->v32[5]),
             reinterpret_cast<float4 *>(m->v32[6]), reinterpret_cast<float4 *>(m->v32[1]),
             reinterpret_cast<float4 *>(m->v32[7]), reinterpret_cast<float4 *>(m->v32[0]),
             reinterpret_cast<const float4 *>(m->dinv32), (const double *)m->scal, (const int *)m->ictl);
}

static void launch_iter32(fg_mesh *m, int v, bool from_first_buffer) {
  if (v_pipe(v)) {
    // the SpMV (its first block finishing the last vector pass's dots), then the
    // vector pass with those scalars
    launch_spmv32s(m, v);
    launch_vec32s(m, v);
    return;
  }
  if (split32(v)) {
    launch_vec32s(m, v);
    launch_spmv32s(m, v);
    return;
  }
  const float4 *in = reinterpret_cast<const float4 *>(from_first_buffer ? m->v32[2] : m->v32[3]);
  float4 *out = reinterpret_cast<float4 *>(from_first_buffer ? m->v32[3] : m->v32[2]);
  if (v == 5 && pipe_available(m))
    pipe_launch32(m, in, out);
  else if (v >= 4)
    halo_launch<Iter32Halo>(m, sizeof(float), m->nv, (const int *)m->sl_ptr, (const int *)m->sl_len,
                            (const uint16_t *)m->sl_lcol, (const float *)m->val32, (const int *)m->halo_col,
                            (const int *)m->halo_len, m->hcap, in, out, m->v32[1], m->v32[0], m->scal, m->ictl,
                            m->red.partials, m->red.counter);
  else if (m->use_dcol) iter32_variant<ColRel>(m, v, m->sl_dcol, in, out);
  else iter32_variant<ColAbs>(m, v, m->sl_col, in, out);
}

static void launch_spmv64cg(fg_mesh *m) {
  if (m->spmv_variant64 == 2 || m->spmv_variant64 == 3) {
    const unsigned per_sm = (m->spmv_variant64 == 2) ? 4u : 8u;
    const unsigned g = std::min<unsigned>(grid_for(m->nv, 256), per_sm * (unsigned)std::max(m->sm_count, 1));
    if (m->use_dcol)
      k_cg64_spmv<ColRel, true><<<g, 256, 0, m->stream>>>(m->nv, m->sl_ptr, m->sl_len, m->sl_dcol, m->val64,
                                                           m->v64[2], m->v64[1], m->v64[12], m->scal, m->ictl,
                                                           m->red.partials, m->red.counter);
    else
      k_cg64_spmv<ColAbs, true><<<g, 256, 0, m->stream>>>(m->nv, m->sl_ptr, m->sl_len, m->sl_col, m->val64,
                                                           m->v64[2], m->v64[1], m->v64[12], m->scal, m->ictl,
                                                           m->red.partials, m->red.counter);
  } else if (m->spmv_variant64 == 1)
    halo_launch<Spmv64Halo>(m, sizeof(double), m->nv, (const int *)m->sl_ptr, (const int *)m->sl_len,
                            (const uint16_t *)m->sl_lcol, (const double *)m->val64, (const int *)m->halo_col,
                            (const int *)m->halo_len, m->hcap, (const double *)m->v64[2], (const double *)m->v64[1],
                            m->v64[12], m->scal, m->ictl, m->red.partials, m->red.counter);
  else if (m->use_dcol)
    k_cg64_spmv<ColRel, false><<<row_grid(m), 256, 0, m->stream>>>(m->nv, m->sl_ptr, m->sl_len, m->sl_dcol, m->val64,
                                                            m->v64[2], m->v64[1], m->v64[12], m->scal, m->ictl,
                                                            m->red.partials, m->red.counter);
  else
    k_cg64_spmv<ColAbs, false><<<row_grid(m), 256, 0, m->stream>>>(m->nv, m->sl_ptr, m->sl_len, m->sl_col, m->val64,
                                                            m->v64[2], m->v64[1], m->v64[12], m->scal, m->ictl,
                                                            m->red.partials, m->red.counter);
}

static void launch_vec64(fg_mesh *m) {
  k_cg64_vec<<<grid_for(m->nvp / 2, 256), 256, 0, m->stream>>>(
      m->nvp / 2, reinterpret_cast<double2 *>(m->v64[1]), reinterpret_cast<const double2 *>(m->v64[12]),
      reinterpret_cast<double2 *>(m->v64[3]), reinterpret_cast<double2 *>(m->v64[4]),
      reinterpret_cast<double2 *>(m->v64[2]), reinterpret_cast<double2 *>(m->v64[0]),
      reinterpret_cast<const double2 *>(m->dinv64), m->scal, m->ictl);
}

// Initialisation and the first pass (w0 = A u0 and the first alpha): FP32 state
// buffer 0 -> 1, so the iteration blocks start reading buffer 1.
static void start_cg(fg_mesh *m, bool mixed, const double *r64, double scale, double tol2_rel, int maxit) {
  const unsigned g = red_grid(m->nvp);
  l2_for_solve(m, mixed && v_window(m->spmv_variant32));
  if (mixed && v_scaled(m->spmv_variant32)) {
    ensure_scaled(m);
    k_cg32ss_init<<<g, 256, 0, m->stream>>>(m->nv, m->nvp, r64, scale, m->sdiag32, m->v32[4], m->v32[6], m->v32[1],
                                            m->v32[0], tol2_rel, maxit, m->scal, m->ictl);
    launch_spmv32s(m, m->spmv_variant32);
  } else if (mixed && v_pipe(m->spmv_variant32)) {
    // r, m = D r; w = A m; one vector pass with alpha = beta = 0 gives m = D w and the
    // partials of the first dot products
    k_pcg32_init<<<g, 256, 0, m->stream>>>(m->nv, m->nvp, r64, scale, m->dinv32, m->v32[4], m->pv32[2], m->v32[0],
                                           m->v32[6], m->v32[1], m->pv32[0], m->pv32[1], tol2_rel, maxit, m->scal,
                                           m->ictl);
    pipe_spmv32(m, m->spmv_variant32, false, m->pv32[2], m->v32[5]);
    pipe_vec32(m);
    FG_LAUNCHED(1);
  } else if (mixed && split32(m->spmv_variant32)) {
    k_cg32s_init<<<g, 256, 0, m->stream>>>(m->nv, m->nvp, r64, scale, m->dinv32, m->v32[4], m->v32[7], m->v32[6],
                                           m->v32[1], m->v32[0], tol2_rel, maxit, m->scal, m->ictl);
    launch_spmv32s(m, m->spmv_variant32);
  } else if (mixed) {
    k_cg32_init<<<g, 256, 0, m->stream>>>(m->nv, m->nvp, r64, scale, m->dinv32,
                                          reinterpret_cast<float4 *>(m->v32[2]), reinterpret_cast<float4 *>(m->v32[3]),
                                          m->v32[1], m->v32[0], tol2_rel, maxit, m->scal, m->ictl);
    launch_iter32(m, m->spmv_variant32, true);
  } else {
    k_cg64_init<<<g, 256, 0, m->stream>>>(m->nv, m->nvp, r64, scale, m->dinv64, m->v64[1], m->v64[2], m->v64[3],
                                          m->v64[4], m->v64[0], tol2_rel, maxit, m->scal, m->ictl);
    launch_spmv64cg(m);
  }
  FG_CUDA_TRY(cudaGetLastError());
  FG_LAUNCHED(2);
}

// Closes each body of the whole-solve loop graph: the WHILE node runs the body again
// while the CG is not done, and never more than max_it / body + 2 times (a bound that
// holds even if no iteration of a body counted).
__global__ void k_cg_continue(cudaGraphConditionalHandle h, int *ictl, int body) {
  if (threadIdx.x != 0) return;
  const int b = ictl[I_BODIES] + 1;
  ictl[I_BODIES] = b;
  const bool more = ictl[I_DONE] == 0 && b < ictl[I_MAXIT] / body + 2;
  cudaGraphSetConditional(h, more ? 1u : 0u);
}

// Captures `enqueue` (one body of iterations) into a graph: a plain block of
// iterations, or a WHILE conditional node around the body and k_cg_continue, so that
// one launch runs the solve to its end without host round trips.  Returns false,
// with the stream out of capture and the error cleared, when the loop graph cannot
// be built (the caller then replays plain blocks).
template <class F>
static bool capture_iterations(fg_mesh *m, GraphCache &gc, int body, bool loop, F &&enqueue) {
  cudaGraph_t graph = nullptr, target = nullptr;
  cudaGraphConditionalHandle h = 0;
  if (loop) {
    if (cudaGraphCreate(&graph, 0) != cudaSuccess ||
        cudaGraphConditionalHandleCreate(&h, graph, 1u, cudaGraphCondAssignDefault) != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      cudaGetLastError();
      return false;
    }
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    if (cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &np) != cudaSuccess) {
      cudaGraphDestroy(graph);
      cudaGetLastError();
      return false;
    }
    target = np.conditional.phGraph_out[0];
    FG_CUDA_TRY(cudaStreamBeginCaptureToGraph(m->stream, target, nullptr, nullptr, 0,
                                              cudaStreamCaptureModeThreadLocal));
  } else {
    FG_CUDA_TRY(cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal));
  }
  bool ok = true;
  try {
    enqueue();
    if (loop) k_cg_continue<<<1, 32, 0, m->stream>>>(h, m->ictl, body);
    ok = cudaGetLastError() == cudaSuccess;
  } catch (const FgError &) {
    ok = false;
  }
  cudaGraph_t captured = nullptr;
  ok = (cudaStreamEndCapture(m->stream, &captured) == cudaSuccess) && ok;
  if (!loop) graph = captured;
  if (ok) ok = cudaGraphInstantiate(&gc.exec, graph, 0) == cudaSuccess;
  if (graph) cudaGraphDestroy(graph);
  if (!ok) {
    gc.exec = nullptr;
    cudaGetLastError();
    FG_REQUIRE(loop, FG_CUDA, "CG graph capture failed");
  }
  return ok;
}

// Runs CG iterations until the device sets "done".  Returns the iteration count.
// use_graph 1: one launch of a WHILE-node graph (bodies of check_every iterations)
// runs the whole solve; where that graph cannot be built (launch attributes the
// conditional body does not take), and with use_graph 2, blocks of check_every
// iterations are replayed with a host check of the done flag between them.
// loop_ms (may be null): device time from the first launch to the end of the last
// one, host checks included (the autotuner's measure of a variant).
// Blocks per SM of the cooperative variant (4 wanted; 0 where two stages do not fit
// or the device has no cooperative launch); sized once per handle.
static int coop_per_sm(fg_mesh *m) {
  if (m->coop_fit < 0) {
    int coop = 0;
    if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, m->device) != cudaSuccess) {
      cudaGetLastError();
      coop = 0;
    }
    int per_sm = 0;
    const size_t smem = bulk_smem(m);
    int dev_max = 0;
    FG_CUDA_TRY(cudaDeviceGetAttribute(&dev_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, m->device));
    if (coop && m->tmax256 > 0 && smem + 1024 <= (size_t)dev_max) {
      auto size = [&](auto kern) {
        FG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        FG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, smem));
      };
      if (m->use_dcol) size(k_cg32_coop<ColRel>);
      else size(k_cg32_coop<ColAbs>);
    }
    m->coop_fit = per_sm;
  }
  return std::min(m->coop_fit, 4);
}

// Launches the persistent cooperative CG for at most `iters` iterations (it stops
// earlier at convergence, the cap or a fault).  Every block is resident (cooperative
// launch), so its grid barriers cannot wait on a block that never runs.
static void coop_launch32(fg_mesh *m, int iters) {
  const int per_sm = coop_per_sm(m);
  FG_REQUIRE(per_sm > 0, FG_UNSUPPORTED, "cooperative CG: not available on this operator or device");
  const unsigned g = std::min<unsigned>(grid_for(m->nv, 256), (unsigned)per_sm * (unsigned)std::max(m->sm_count, 1));
  if (!m->coop_bar) m->coop_bar = dev_alloc<unsigned>(m, 2);
  FG_CUDA_TRY(cudaMemsetAsync(m->coop_bar, 0, 2 * sizeof(unsigned), m->stream));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(g);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = bulk_smem(m);
  cfg.stream = m->stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  float2 *parts = reinterpret_cast<float2 *>(m->red.partials);
  if (m->use_dcol)
    FG_CUDA_TRY(cudaLaunchKernelEx(&cfg, k_cg32_coop<ColRel>, (int64_t)m->nv, m->nslices, m->tmax256,
                                   (const int *)m->sl_ptr, (const int *)m->sl_len, (const int16_t *)m->sl_dcol,
                                   (const float *)m->val32, m->v32[4], m->v32[5], m->v32[6], m->v32[1], m->v32[7],
                                   m->v32[0], (const float *)m->dinv32, m->scal, m->ictl, parts, m->coop_bar, iters));
  else
    FG_CUDA_TRY(cudaLaunchKernelEx(&cfg, k_cg32_coop<ColAbs>, (int64_t)m->nv, m->nslices, m->tmax256,
                                   (const int *)m->sl_ptr, (const int *)m->sl_len, (const int *)m->sl_col,
                                   (const float *)m->val32, m->v32[4], m->v32[5], m->v32[6], m->v32[1], m->v32[7],
                                   m->v32[0], (const float *)m->dinv32, m->scal, m->ictl, parts, m->coop_bar, iters));
  FG_LAUNCHED(1);
}

// The solve loop of the cooperative variant: launches of up to 1024 iterations with a
// host check of the done flag between them (no graph).
static int run_cg_coop(fg_mesh *m, int *status, float *loop_ms) {
  if (loop_ms) FG_CUDA_TRY(cudaEventRecord(m->ev0, m->stream));
  for (;;) {
    coop_launch32(m, 1024);
    if (loop_ms) FG_CUDA_TRY(cudaEventRecord(m->ev1, m->stream));
    FG_CUDA_TRY(cudaMemcpyAsync(m->hint, m->ictl, sizeof(int) * (I_BODIES + 1), cudaMemcpyDeviceToHost,
                                m->stream));
    fg_sync(m);
    FG_REQUIRE(m->hint[I_FAULT] == 0, FG_CUDA,
               "CG kernel: an asynchronous shared-memory copy or a grid barrier did not complete");
    if (m->hint[I_DONE]) break;
  }
  if (status) *status = m->hint[I_STATUS];
  if (loop_ms) FG_CUDA_TRY(cudaEventElapsedTime(loop_ms, m->ev0, m->ev1));
  return std::max(m->hint[I_ITERS], 0);
}

static int run_cg(fg_mesh *m, bool mixed, const fg_solve_opts &o, int *status, float *loop_ms = nullptr) {
  if (mixed && v_coop(m->spmv_variant32)) return run_cg_coop(m, status, loop_ms);
  int block = o.check_every > 0 ? o.check_every : 32;
  if (block & 1) ++block;
  const int per_iter = (mixed && !split32(m->spmv_variant32)) ? 1 : (mixed && v_splitred(m->spmv_variant32)) ? 3 : 2;
  GraphCache &gc = m->graph[mixed ? 1 : 0];
  const bool use_graph = o.use_graph != 0;
  // programmatic-launch edges keep the host-checked blocks
  const bool want_loop = o.use_graph == 1 && !(mixed && m->spmv_variant32 == 9);
  const int body = block;
  const void *key[5] = {mixed ? (const void *)m->val32 : (const void *)m->val64,
                        mixed ? (const void *)(intptr_t)(m->spmv_variant32 + 1) : (const void *)m->v64[0],
                        (const void *)(intptr_t)body, (const void *)(intptr_t)m->use_dcol,
                        (const void *)(intptr_t)(mixed ? 0 : m->spmv_variant64 + 1)};
  auto enqueue_block = [&](int n) {
    for (int it = 0; it < n; ++it) {
      if (mixed) launch_iter32(m, m->spmv_variant32, (it & 1) != 0);
      else { launch_vec64(m); launch_spmv64cg(m); }
    }
  };
  bool loop = false;
  if (use_graph) {
    bool match = gc.exec && gc.iters == body && gc.loop == want_loop;
    for (int j = 0; j < 5 && match; ++j) match = (gc.key[j] == key[j]);
    if (!match) {
      if (gc.exec) { cudaGraphExecDestroy(gc.exec); gc.exec = nullptr; }
      gc.loop = want_loop && capture_iterations(m, gc, body, true, [&]() { enqueue_block(body); });
      if (!gc.loop) capture_iterations(m, gc, block, false, [&]() { enqueue_block(block); });
      gc.iters = gc.loop ? body : block;
      for (int j = 0; j < 5; ++j) gc.key[j] = key[j];
      if (!gc.loop) gc.key[2] = (const void *)(intptr_t)-1;  // a plain block: rebuilt for a new request
    }
    loop = gc.loop;
  }
  // the whole solve in one launch (bodies of an even number of iterations keep the
  // fused variants' state buffers in step); launches are counted from the bodies run
  if (loop_ms) FG_CUDA_TRY(cudaEventRecord(m->ev0, m->stream));
  if (loop) FG_CUDA_TRY(cudaGraphLaunch(gc.exec, m->stream));
  int bodies = 0;
  for (;;) {
    if (loop_ms) FG_CUDA_TRY(cudaEventRecord(m->ev1, m->stream));
    FG_CUDA_TRY(cudaMemcpyAsync(m->hint, m->ictl, sizeof(int) * (I_BODIES + 1), cudaMemcpyDeviceToHost,
                                m->stream));
    fg_sync(m);
    if (loop) {
      FG_LAUNCHED((long long)(m->hint[I_BODIES] - bodies) * (per_iter * body + 1));
      bodies = m->hint[I_BODIES];
    }
    FG_REQUIRE(m->hint[I_FAULT] == 0, FG_CUDA, "CG kernel: an asynchronous shared-memory copy did not complete");
    if (m->hint[I_DONE]) break;
    if (use_graph) {
      FG_CUDA_TRY(cudaGraphLaunch(gc.exec, m->stream));
    } else {
      enqueue_block(block);
      FG_CUDA_TRY(cudaGetLastError());
    }
    if (!loop) FG_LAUNCHED((long long)per_iter * block);
  }
  if (status) *status = m->hint[I_STATUS];
  if (loop_ms) FG_CUDA_TRY(cudaEventElapsedTime(loop_ms, m->ev0, m->ev1));
  return std::max(m->hint[I_ITERS], 0);
}

// Microseconds per iteration of the handle's current variant run the way the solver
// runs it (start_cg, then run_cg with default options: the whole-solve graph where it
// can be built), over `reps` iterations after an untimed run that builds the graph.
static double loop_us_per_iteration(fg_mesh *m, bool mixed, int reps) {
  fg_solve_opts o;
  fg_solve_opts_default(&o);
  if (!m->v64[5]) m->v64[5] = dev_alloc<double>(m, (size_t)m->nvp);
  k_fill64<<<red_grid(m->nv), 256, 0, m->stream>>>(m->nv, 1.0, m->v64[5]);
  FG_LAUNCHED(1);
  if (mixed) ensure_cg32(m);
  else ensure_cg64(m);
  float ms = 0.f;
  int its = 0;
  for (int pass = 0; pass < 2; ++pass) {
    start_cg(m, mixed, m->v64[5], 1.0, 0.0, reps);
    its = run_cg(m, mixed, o, nullptr, pass == 1 ? &ms : nullptr);
  }
  return 1e3 * (double)ms / std::max(its, 1);
}

fg_status fg_autotune_spmv32(fg_mesh *m, int reps, int *chosen, double *us_per_variant);
fg_status fg_autotune_spmv64(fg_mesh *m, int reps, int *chosen, double *us_per_variant);

// Process-wide memory of the autotuner's choices, keyed by the device and the shape
// of the operator (rows, padded entries, longest row, column format; the halo rows
// per block follow from the longest row): a new handle for a mesh of the same
// structure (the one-shot entry points create one per call) reuses the choice
// instead of timing the variants again.
namespace {
std::mutex g_tune_lock;
std::map<std::tuple<int, int64_t, int64_t, int, int, bool>, int> g_tune;
std::tuple<int, int64_t, int64_t, int, int, bool> tune_key(const fg_mesh *m, bool mixed) {
  return std::make_tuple(m->device, m->nv, m->nsell, m->maxrow4, (int)m->use_dcol, mixed);
}
}  // namespace

static bool tune_cache_get(fg_mesh *m, bool mixed) {
  std::lock_guard<std::mutex> g(g_tune_lock);
  auto it = g_tune.find(tune_key(m, mixed));
  if (it == g_tune.end()) return false;
  if (mixed) { m->spmv_variant32 = it->second; m->tuned32 = true; }
  else { m->spmv_variant64 = it->second; m->tuned64 = true; }
  return true;
}

static void tune_cache_put(fg_mesh *m, bool mixed) {
  std::lock_guard<std::mutex> g(g_tune_lock);
  g_tune[tune_key(m, mixed)] = mixed ? m->spmv_variant32 : m->spmv_variant64;
}

// Whether FP32 variant v can run on this handle (the L2 window: whether the device
// has persisting L2; the set-aside itself is made when a solve starts).
static bool variant32_available(fg_mesh *m, int v) {
  if (v < 0 || v >= FG_N_SPMV32) return false;
  if ((v == 4 || v == 7) && !fg_ensure_halo(m)) return false;
  if (v == 5 && !pipe_available(m)) return false;
  if (v_bulk(v) && bulk_per_sm(m, v) == 0) return false;
  if (v_pipe(v) && pipe_per_sm(m, v) == 0) return false;
  if (v_coop(v) && (coop_per_sm(m) == 0 || bulk_per_sm(m, 22) == 0)) return false;
  if (v_window(v) && !l2_supported(m)) return false;
  return true;
}

// Inner solve of A d = scale * r64 from d = 0 to relative residual `inner`, then
// x += d / scale.  Returns iterations; *ist = 0 converged, 1 cap, 2 non-finite.
static int inner_solve(fg_mesh *m, bool mixed, const double *r64, double rn, double inner, int maxit,
                       const fg_solve_opts &o, double *d_x, int *ist) {
  int its;
  if (mixed) {
    ensure_cg32(m);
    if (o.spmv > 0 && o.spmv <= FG_N_SPMV32) {
      // a forced variant that this operator cannot run (no halo lists, stages too
      // large for shared memory) falls back to the plain gather kernel
      const int v = o.spmv - 1;
      m->spmv_variant32 = variant32_available(m, v) ? v : 0;
    } else if (!m->tuned32 && !tune_cache_get(m, true)) {
      fg_autotune_spmv32(m, 20, nullptr, nullptr);
      tune_cache_put(m, true);
    } else if (!variant32_available(m, m->spmv_variant32)) {
      // a variant remembered from another handle of this operator shape that this
      // handle cannot run as it is (its halo lists or pipeline grid not built, the
      // stages too large): time the variants on this handle instead
      fg_autotune_spmv32(m, 20, nullptr, nullptr);
    }
    if (v_window(m->spmv_variant32) && !prepare_l2(m)) {
      // no persisting L2 after all: the same variant without the window
      const int v = m->spmv_variant32;
      m->spmv_variant32 = (v == 10) ? 14 : (v == 20) ? 16 : 17;
    }
    start_cg(m, true, r64, 1.0 / rn, inner * inner, maxit);
    its = run_cg(m, true, o, ist);
    if (v_scaled(m->spmv_variant32))
      k_axpy_scaled_to64<<<grid_for(m->nv, 256), 256, 0, m->stream>>>(m->nv, rn, m->sdiag32, m->v32[0], d_x);
    else
      k_axpy_to64<float><<<red_grid(m->nv), 256, 0, m->stream>>>(m->nv, rn, m->v32[0], d_x);
  } else {
    ensure_cg64(m);
    if (!m->tuned64 && !tune_cache_get(m, false)) {
      fg_autotune_spmv64(m, 20, nullptr, nullptr);
      tune_cache_put(m, false);
    } else if (m->spmv_variant64 == 1 && !fg_ensure_halo(m)) {
      m->spmv_variant64 = 0;  // the halo-staged SpMV needs this handle's halo lists
    }
    start_cg(m, false, r64, 1.0 / rn, inner * inner, maxit);
    its = run_cg(m, false, o, ist);
    k_axpy_to64<double><<<red_grid(m->nv), 256, 0, m->stream>>>(m->nv, rn, m->v64[0], d_x);
  }
  FG_CUDA_TRY(cudaGetLastError());
  FG_LAUNCHED(1);
  return its;
}

int fg_pcg_solve(fg_mesh *m, const double *d_b, double *d_x, const fg_solve_opts &o, fg_solve_stats *st,
                 bool newton_inner, double b_norm) {
  const bool mixed = o.precision == FG_MIXED;
  FG_REQUIRE(mixed ? m->val32 != nullptr : m->val64 != nullptr, FG_BAD_ARG, "operator not assembled");
  if (!m->v64[6]) m->v64[6] = dev_alloc<double>(m, (size_t)m->nvp);
  double *r64 = m->v64[6];
  const uint8_t *fx = m->has_fixed ? m->fixed : nullptr;
  FG_CUDA_TRY(cudaEventRecord(m->ev0, m->stream));
  int total = 0, refinements = 0, status = 0;
  double rn0 = -1.0, rn = 0.0;
  const int max_ref = newton_inner ? 1 : 50;
  for (int ref = 0; ref < max_ref; ++ref) {
    if (newton_inner) {
      // x = 0, residual = b
      FG_CUDA_TRY(cudaMemcpyAsync(r64, d_b, sizeof(double) * (size_t)m->nv, cudaMemcpyDeviceToDevice, m->stream));
      rn = (b_norm >= 0.0) ? b_norm : fg_norm2_dev(m, r64, m->nv, true);
    } else {
      FG_REQUIRE(m->val64 != nullptr, FG_BAD_ARG, "refinement needs the FP64 operator");
      spmv64_launch(m, d_x, d_b, r64, fx, 9);
      FG_CUDA_TRY(cudaMemcpyAsync(m->hbuf, m->scal + 9, sizeof(double), cudaMemcpyDeviceToHost, m->stream));
      fg_sync(m);
      rn = std::sqrt(m->hbuf[0]);
    }
    if (rn0 < 0) rn0 = rn;
    if (!std::isfinite(rn)) { status = 2; break; }
    double target = o.rtol * rn0;
    if (rn <= target || rn == 0.0) break;
    if (total >= o.maxiter) { status = 1; break; }
    double rel = target / rn;  // inner relative target that would finish the job
    double inner = mixed ? std::max(rel, o.inner_rtol) : rel;
    if (newton_inner) inner = o.inner_rtol;
    int ist = 0;
    total += inner_solve(m, mixed, r64, rn, inner, o.maxiter - total, o, d_x, &ist);
    ++refinements;
    if (ist == 2) { status = 2; break; }
    if (newton_inner) { status = ist; break; }
  }
  // a Newton step continues on the stream: its solve is not timed (no wait here)
  const bool timed = !newton_inner;
  if (timed) {
    FG_CUDA_TRY(cudaEventRecord(m->ev1, m->stream));
    fg_sync(m);
  }
  if (st) {
    float ms = 0.f;
    if (timed) cudaEventElapsedTime(&ms, m->ev0, m->ev1);
    st->iterations = total;
    st->refinements = refinements;
    st->converged = (status == 0);
    st->relres = (rn0 > 0) ? rn / rn0 : 0.0;
    st->ms = ms;
  }
  if (status == 2) throw FgError{FG_NAN, "CG produced a non-finite residual"};
  return status;
}

// ------------------------------------------------------------------ C ABI
extern "C" void fg_solve_opts_default(fg_solve_opts *o) {
  if (!o) return;
  o->precision = FG_FP64;
  o->rtol = 1e-10;
  o->maxiter = 1000000;
  o->inner_rtol = 1e-5;
  o->check_every = 32;
  o->use_graph = 1;
  o->spmv = FG_SPMV_AUTO;
  o->reserved_ = 0;
}

// A standalone operator from a symmetric CSC matrix: a handle with the pattern and
// values in SELL-32x4 layout but no mesh.
static fg_mesh *matrix_handle(int64_t n, const int64_t *colptr, const int64_t *rowval, const double *nzval, int base,
                              bool want32) {
  FG_REQUIRE(n > 0 && n < ((int64_t)1 << 30), FG_BAD_ARG, "matrix size out of range");
  FG_REQUIRE(base == 0 || base == 1, FG_BAD_ARG, "index_base must be 0 or 1");
  int64_t nnz = colptr[n] - base;
  FG_REQUIRE(nnz >= 0 && nnz < ((int64_t)1 << 31), FG_BAD_ARG, "nnz out of range");
  fg_mesh *m = new fg_mesh();
  try {
    FG_CUDA_TRY(cudaGetDevice(&m->device));
    FG_CUDA_TRY(cudaDeviceGetAttribute(&m->sm_count, cudaDevAttrMultiProcessorCount, m->device));
    fg_pool_init(m->device);
    FG_CUDA_TRY(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
    FG_CUDA_TRY(cudaEventCreate(&m->ev0));
    FG_CUDA_TRY(cudaEventCreate(&m->ev1));
    m->nv = n;
    m->nnz = nnz;
    m->nslices = (int)((n + FG_SLICE - 1) / FG_SLICE);
    m->nvp = (int64_t)m->nslices * FG_SLICE;
    std::vector<int> sl_len(m->nslices), sl_ptr(m->nslices + 1);
    int64_t acc = 0;
    for (int s = 0; s < m->nslices; ++s) {
      int64_t mx = 1;
      for (int64_t r = (int64_t)s * FG_SLICE; r < std::min<int64_t>(n, (int64_t)(s + 1) * FG_SLICE); ++r)
        mx = std::max<int64_t>(mx, colptr[r + 1] - colptr[r]);
      int groups = (int)((mx + FG_GROUP - 1) / FG_GROUP);
      sl_len[s] = groups;
      sl_ptr[s] = (int)acc;
      acc += (int64_t)groups * FG_GROUP * FG_SLICE;
      FG_REQUIRE(acc < ((int64_t)1 << 31), FG_BAD_ARG, "padded matrix too large");
    }
    sl_ptr[m->nslices] = (int)acc;
    m->nsell = acc;
    // largest 256-row block in padded entries (the bulk-staged SpMV stages one)
    for (int s0 = 0; s0 < m->nslices; s0 += 256 / FG_SLICE)
      m->tmax256 = std::max(m->tmax256, sl_ptr[std::min(s0 + 256 / FG_SLICE, m->nslices)] - sl_ptr[s0]);
    std::vector<int> col(acc);
    std::vector<int16_t> dcol(acc, 0);
    std::vector<double> val(acc, 0.0);
    std::vector<double> dinv(m->nvp, 0.0);
    bool wide = false;
    for (int64_t r = 0; r < n; ++r) {
      int s = (int)(r / FG_SLICE), lane = (int)(r % FG_SLICE);
      int64_t b = colptr[r] - base, e = colptr[r + 1] - base;
      int k = 0;
      double diag = 0.0;
      for (int64_t qq = b; qq < e; ++qq, ++k) {
        int64_t c = rowval[qq] - base;
        FG_REQUIRE(c >= 0 && c < n, FG_BAD_ARG, "row index out of range");
        int64_t pos = sell_pos(sl_ptr[s], lane, k);
        col[pos] = (int)c;
        val[pos] = nzval[qq];
        int64_t d = c - r;
        if (d < -32768 || d > 32767) wide = true; else dcol[pos] = (int16_t)d;
        if (c == r) diag += nzval[qq];
      }
      for (; k < FG_GROUP * sl_len[s]; ++k) col[sell_pos(sl_ptr[s], lane, k)] = (int)r;
      dinv[r] = diag != 0.0 ? 1.0 / diag : 0.0;
    }
    m->use_dcol = !wide;
    m->sl_ptr = dev_alloc<int>(m, (size_t)m->nslices + 1);
    m->sl_len = dev_alloc<int>(m, (size_t)m->nslices);
    m->sl_col = dev_alloc<int>(m, (size_t)acc);
    m->sl_dcol = dev_alloc<int16_t>(m, (size_t)acc);
    m->val64 = dev_alloc<double>(m, (size_t)acc);
    m->dinv64 = dev_alloc<double>(m, (size_t)m->nvp);
    FG_CUDA_TRY(cudaMemcpyAsync(m->sl_ptr, sl_ptr.data(), sizeof(int) * (m->nslices + 1), cudaMemcpyHostToDevice, m->stream));
    FG_CUDA_TRY(cudaMemcpyAsync(m->sl_len, sl_len.data(), sizeof(int) * m->nslices, cudaMemcpyHostToDevice, m->stream));
    FG_CUDA_TRY(cudaMemcpyAsync(m->sl_col, col.data(), sizeof(int) * acc, cudaMemcpyHostToDevice, m->stream));
    FG_CUDA_TRY(cudaMemcpyAsync(m->sl_dcol, dcol.data(), sizeof(int16_t) * acc, cudaMemcpyHostToDevice, m->stream));
    FG_CUDA_TRY(cudaMemcpyAsync(m->val64, val.data(), sizeof(double) * acc, cudaMemcpyHostToDevice, m->stream));
    FG_CUDA_TRY(cudaMemcpyAsync(m->dinv64, dinv.data(), sizeof(double) * m->nvp, cudaMemcpyHostToDevice, m->stream));
    if (want32) {
      std::vector<float> v32(val.begin(), val.end()), d32(dinv.begin(), dinv.end());
      m->val32 = dev_alloc<float>(m, (size_t)acc);
      m->dinv32 = dev_alloc<float>(m, (size_t)m->nvp);
      FG_CUDA_TRY(cudaMemcpyAsync(m->val32, v32.data(), sizeof(float) * acc, cudaMemcpyHostToDevice, m->stream));
      FG_CUDA_TRY(cudaMemcpyAsync(m->dinv32, d32.data(), sizeof(float) * m->nvp, cudaMemcpyHostToDevice, m->stream));
    }
    m->red.partials = dev_alloc<double>(m, ((size_t)grid_for(n, FG_SLICE) + FG_RED_BLOCKS) * 4);
    m->red.counter = dev_alloc<unsigned int>(m, 128);
    FG_CUDA_TRY(cudaMemsetAsync(m->red.counter, 0, 128 * sizeof(unsigned int), m->stream));
    m->scal = dev_alloc<double>(m, S_NSCAL);
    m->ictl = dev_alloc<int>(m, I_NINT);
    m->flags = dev_alloc<int>(m, 4);
    FG_CUDA_TRY(cudaMemsetAsync(m->flags, 0, 4 * sizeof(int), m->stream));
    m->hbuf = static_cast<double *>(fg_pinned_block_get());
    m->hint = reinterpret_cast<int *>(m->hbuf + 64);
    int64_t mr = 1;
    for (int64_t r = 0; r < n; ++r) mr = std::max<int64_t>(mr, colptr[r + 1] - colptr[r]);
    m->maxrow = (int)mr;
    m->maxrow4 = (int)((mr + FG_GROUP - 1) / FG_GROUP * FG_GROUP);
    fg_sync(m);
  } catch (...) {
    fg_mesh_destroy(m);
    throw;
  }
  return m;
}

extern "C" fg_status fg_cg_csc(int64_t n, const int64_t *colptr, const int64_t *rowval, const double *nzval,
                               int32_t index_base, const double *b, double *x, const fg_solve_opts *o,
                               fg_solve_stats *s) {
  fg_mesh *m = nullptr;
  fg_status st = fg_guard([&]() -> fg_status {
    FG_REQUIRE(colptr && rowval && nzval && b && x, FG_BAD_ARG, "fg_cg_csc: null pointer");
    fg_solve_opts opts;
    fg_solve_opts_default(&opts);
    if (o) opts = *o;
    m = matrix_handle(n, colptr, rowval, nzval, index_base, opts.precision == FG_MIXED);
    double *db = dev_alloc<double>(m, (size_t)n), *dx = dev_alloc<double>(m, (size_t)n);
    FG_CUDA_TRY(cudaMemcpyAsync(db, b, sizeof(double) * n, cudaMemcpyHostToDevice, m->stream));
    FG_CUDA_TRY(cudaMemcpyAsync(dx, x, sizeof(double) * n, cudaMemcpyHostToDevice, m->stream));
    int status = fg_pcg_solve(m, db, dx, opts, s, false);
    FG_CUDA_TRY(cudaMemcpyAsync(x, dx, sizeof(double) * n, cudaMemcpyDeviceToHost, m->stream));
    fg_sync(m);
    return status == 0 ? FG_OK : FG_NOT_CONVERGED;
  });
  if (m) fg_mesh_destroy(m);
  return st;
}

extern "C" fg_status fg_spmv_csc(int64_t n, const int64_t *colptr, const int64_t *rowval, const double *nzval,
                                 int32_t index_base, const double *x, double *y) {
  fg_mesh *m = nullptr;
  fg_status st = fg_guard([&]() -> fg_status {
    FG_REQUIRE(colptr && rowval && nzval && x && y, FG_BAD_ARG, "fg_spmv_csc: null pointer");
    m = matrix_handle(n, colptr, rowval, nzval, index_base, false);
    double *dx = dev_alloc<double>(m, (size_t)n), *dy = dev_alloc<double>(m, (size_t)n);
    FG_CUDA_TRY(cudaMemcpyAsync(dx, x, sizeof(double) * n, cudaMemcpyHostToDevice, m->stream));
    fg_spmv64_dev(m, dx, dy);
    FG_CUDA_TRY(cudaMemcpyAsync(y, dy, sizeof(double) * n, cudaMemcpyDeviceToHost, m->stream));
    fg_sync(m);
    return FG_OK;
  });
  if (m) fg_mesh_destroy(m);
  return st;
}


// ------------------------------------------------------------------ timing and tuning
// A CG state for timing: residual of ones, zero tolerance, no iteration cap, then the
// first pass.  Uses v64[5] as its scratch right-hand side (the refinement residual in
// v64[6] stays untouched).
static void timing_state(fg_mesh *m, bool mixed) {
  if (!m->v64[5]) m->v64[5] = dev_alloc<double>(m, (size_t)m->nvp);
  k_fill64<<<red_grid(m->nv), 256, 0, m->stream>>>(m->nv, 1.0, m->v64[5]);
  if (mixed) ensure_cg32(m);
  else ensure_cg64(m);
  start_cg(m, mixed, m->v64[5], 1.0, 0.0, 1 << 30);
  FG_LAUNCHED(1);
}

// Average duration of one CG kernel launch on the handle's current operator (events
// on the handle's stream): which = 0 the FP32 fused iteration or the FP64 SpMV with
// its dot products, 1 the FP64 pointwise update.  Leaves the CG vectors in an
// unspecified state.
fg_status fg_bench_cg_kernel(fg_mesh *m, int which, int precision, int reps, double *ms_per_launch) {
  const bool mixed = precision == FG_MIXED;
  FG_REQUIRE(mixed ? m->val32 != nullptr : m->val64 != nullptr, FG_BAD_ARG, "operator not assembled");
  if (which == 6) {
    // whole iterations the way the solver runs them (its graph loop), reps of them
    *ms_per_launch = 1e-3 * loop_us_per_iteration(m, mixed, std::max(reps, 2));
    return FG_OK;
  }
  timing_state(m, mixed);
  const int v = m->spmv_variant32;
  auto body = [&](int n) {
    for (int r = 0; r < n; ++r) {
      if (mixed && (!split32(v) || which == 3)) launch_iter32(m, v, (r & 1) != 0);
      else if (mixed && (which == 0 || which == 9) && v_splitred(v)) launch_split_parts(m, v, which == 9);
      else if (mixed && which == 0) launch_spmv32s(m, v);
      else if (mixed) launch_vec32s(m, v);
      else if (which == 0) launch_spmv64cg(m);
      else if (which == 1) launch_vec64(m);
      else { launch_vec64(m); launch_spmv64cg(m); }
    }
    FG_LAUNCHED(n);
  };
  body(2);
  FG_CUDA_TRY(cudaEventRecord(m->ev0, m->stream));
  body(reps & ~1);
  FG_CUDA_TRY(cudaEventRecord(m->ev1, m->stream));
  FG_CUDA_TRY(cudaGetLastError());
  fg_sync(m);
  float ms = 0.f;
  FG_CUDA_TRY(cudaEventElapsedTime(&ms, m->ev0, m->ev1));
  *ms_per_launch = ms / (reps & ~1);
  return FG_OK;
}

// Autotuner: times every FP32 CG iteration variant on the handle's current operator,
// each run as the solver runs it (CUDA events around its graph loop), and keeps the
// fastest for the handle.  Runs at the first mixed-precision solve of an operator
// shape (or on request).  The variants that hold their values in a persisting-L2
// window set L2 aside for the whole context (every other kernel of the process
// loses it): one is kept only when it beats the fastest variant without a window
// by more than kWindowMargin.  The pipelined variants are never kept, and neither are
// those on the Jacobi-scaled system (16, 20): the same iterates as Jacobi-PCG in exact
// arithmetic, but in FP32 a 96^3 Newton solve took 1,427 CG iterations with them
// against 1,329, which a per-iteration timing does not see.
// Near-ties (within kTieMargin of the fastest) go to the bulk-staged split variants
// with the split reduction (22, 23, 27, 28): entries staged through shared memory, the
// SpMV nearest the copy bandwidth when timed alone, so that the choice between
// variants a few tenths of a microsecond apart does not follow timing noise.
constexpr double kWindowMargin = 0.05;
constexpr double kTieMargin = 0.015;
fg_status fg_autotune_spmv32(fg_mesh *m, int reps, int *chosen, double *us_per_variant) {
  FG_REQUIRE(m->val32 != nullptr, FG_BAD_ARG, "autotune: no FP32 operator assembled");
  reps = std::max(64, (reps + 31) / 32 * 32);  // whole bodies of the solver's graph loop
  int best = 0, best_win = -1, best_pref = -1;
  double best_us = 1e30, best_win_us = 1e30, best_pref_us = 1e30;
  for (int v = 0; v < FG_N_SPMV32; ++v) {
    if (!variant32_available(m, v) || (v_window(v) && !prepare_l2(m))) {  // not available here
      if (us_per_variant) us_per_variant[v] = 0.0;
      continue;
    }
    m->spmv_variant32 = v;
    // timed as the solver runs them, from an L2 without persisting lines
    reset_persisting_l2(m);
    const double us = loop_us_per_iteration(m, true, reps);
    if (us_per_variant) us_per_variant[v] = us;
    if (v_pipe(v) || v_scaled(v)) continue;
    if (v_window(v)) {
      if (us < best_win_us) { best_win_us = us; best_win = v; }
    } else if (us < best_us) {
      best_us = us;
      best = v;
    }
    if ((v_splitred(v) || v_last1(v)) && us < best_pref_us) { best_pref_us = us; best_pref = v; }
  }
  double chosen_us = best_us;
  if (best_win >= 0 && best_win_us < (1.0 - kWindowMargin) * best_us) { best = best_win; chosen_us = best_win_us; }
  if (best_pref >= 0 && best_pref_us <= (1.0 + kTieMargin) * chosen_us) best = best_pref;
  m->spmv_variant32 = best;
  m->tuned32 = true;
  if (chosen) *chosen = best;
  return FG_OK;
}

// The same for the FP64 iteration (SpMV with direct gathers, halo staging, or a
// persistent grid of 4 or 8 blocks per SM), timed per whole iteration.
fg_status fg_autotune_spmv64(fg_mesh *m, int reps, int *chosen, double *us_per_variant) {
  FG_REQUIRE(m->val64 != nullptr, FG_BAD_ARG, "autotune: no FP64 operator assembled");
  reps = std::max(64, (reps + 31) / 32 * 32);
  int best = 0;
  double best_us = 1e30;
  for (int v = 0; v < FG_N_SPMV64; ++v) {
    if (v == 1 && !fg_ensure_halo(m)) {
      if (us_per_variant) us_per_variant[v] = 0.0;
      continue;
    }
    m->spmv_variant64 = v;
    // timed as the solver runs them
    const double us = loop_us_per_iteration(m, false, reps);
    if (us_per_variant) us_per_variant[v] = us;
    if (us < best_us && !v_pipe(v)) { best_us = us; best = v; }
  }
  m->spmv_variant64 = best;
  m->tuned64 = true;
  if (m->graph[0].exec) { cudaGraphExecDestroy(m->graph[0].exec); m->graph[0].exec = nullptr; }
  if (chosen) *chosen = best;
  return FG_OK;
}

extern "C" fg_status fg_set_cg_variant(fg_mesh *m, int32_t precision, int32_t variant) {
  return fg_guard([&]() -> fg_status {
    FG_REQUIRE(m != nullptr, FG_BAD_ARG, "fg_set_cg_variant: null handle");
    if (precision == FG_MIXED) {
      FG_REQUIRE(variant >= 0 && variant <= FG_N_SPMV32, FG_BAD_ARG, "fg_set_cg_variant: no such variant");
      if (variant == 0) { m->tuned32 = false; return FG_OK; }
      const int v = variant - 1;
      FG_REQUIRE(variant32_available(m, v), FG_UNSUPPORTED,
                 "fg_set_cg_variant: variant not available for this operator");
      m->spmv_variant32 = v;
      m->tuned32 = true;
    } else {
      FG_REQUIRE(variant >= 0 && variant <= FG_N_SPMV64, FG_BAD_ARG, "fg_set_cg_variant: no such variant");
      if (variant == 0) { m->tuned64 = false; return FG_OK; }
      FG_REQUIRE(variant != 2 || fg_ensure_halo(m), FG_UNSUPPORTED, "fg_set_cg_variant: variant not available");
      m->spmv_variant64 = variant - 1;
      m->tuned64 = true;
    }
    return FG_OK;
  });
}

extern "C" fg_status fg_get_cg_variant(const fg_mesh *m, int32_t precision, int32_t *variant) {
  return fg_guard([&]() -> fg_status {
    FG_REQUIRE(m != nullptr && variant != nullptr, FG_BAD_ARG, "fg_get_cg_variant: null argument");
    const bool mixed = precision == FG_MIXED;
    const bool tuned = mixed ? m->tuned32 : m->tuned64;
    *variant = tuned ? 1 + (mixed ? m->spmv_variant32 : m->spmv_variant64) : 0;
    return FG_OK;
  });
}

extern "C" fg_status fg_autotune(fg_mesh *m, int32_t precision, int32_t *variant, double *us_per_variant,
                                 int32_t n_slots) {
  return fg_guard([&]() -> fg_status {
    FG_REQUIRE(m != nullptr, FG_BAD_ARG, "fg_autotune: null handle");
    double us[32] = {0};
    int chosen = 0, nv = 0;
    fg_status st;
    if (precision == FG_MIXED) {
      st = fg_autotune_spmv32(m, 50, &chosen, us);
      nv = FG_N_SPMV32;
    } else {
      st = fg_autotune_spmv64(m, 50, &chosen, us);
      nv = FG_N_SPMV64;
    }
    tune_cache_put(m, precision == FG_MIXED);
    if (variant) *variant = chosen;
    if (us_per_variant)
      for (int v = 0; v < nv && v < n_slots; ++v) us_per_variant[v] = us[v];
    return st;
  });
}

// ------------------------------------------------------------------ BiCGStab (FP64)
// Jacobi right-preconditioned BiCGStab (van der Vorst 1992) for the nonsymmetric
// backward-Euler transport operator.  One iteration is five kernels, each reading
// the scalars the previous one finished on the device:
//   p = r + beta (p - omega v), ph = D p          k_bcg_p
//   v = A ph, alpha = rho / (rh . v)              k_bcg_spmv<0>
//   s = r - alpha v, sh = D s                     k_bcg_s
//   t = A sh, omega = (t . s) / (t . t)           k_bcg_spmv<1>
//   x += alpha ph + omega sh, r = s - omega t,
//   rho' = rh . r, beta = (rho'/rho)(alpha/omega) k_bcg_update
// Every kernel returns at once when the control word says the solve is done, so a
// captured body of several iterations can run past convergence at no cost.
enum { Q_RHO = 0, Q_ALPHA, Q_OMEGA, Q_BETA, Q_RR, Q_TOL2, Q_BB };
enum { BCG_X = 0, BCG_R, BCG_RH, BCG_P, BCG_PH, BCG_V, BCG_S, BCG_SH, BCG_T, BCG_B, BCG_NVEC };
constexpr int FG_BCG_BODY = 8;  // iterations per captured graph body

__global__ void __launch_bounds__(256) k_bcg_start(int64_t n, const double *__restrict__ b,
                                                   const double *__restrict__ r, double *__restrict__ rh,
                                                   double *__restrict__ p, double *__restrict__ v, double tol, int maxit,
                                                   double *scal, int *ictl, double *partials, unsigned *counter) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double d[2] = {0.0, 0.0};
  if (i < n) {
    const double ri = r[i], bi = b[i];
    rh[i] = ri;
    p[i] = 0.0;
    v[i] = 0.0;
    d[0] = ri * ri;
    d[1] = bi * bi;
  }
  __shared__ double sh[2][32];
  block_sum<2>(d, sh);
  double tot[2];
  if (grid_finish<2>(d, partials, counter, tot)) {
    const double tol2 = tol * tol * tot[1];
    scal[Q_RHO] = tot[0];
    scal[Q_ALPHA] = 1.0;
    scal[Q_OMEGA] = 1.0;
    scal[Q_BETA] = 0.0;
    scal[Q_RR] = tot[0];
    scal[Q_BB] = tot[1];
    scal[Q_TOL2] = tol2;
    ictl[I_ITERS] = 0;
    ictl[I_MAXIT] = maxit;
    ictl[I_STATUS] = isfinite(tot[0]) ? 0 : 2;
    ictl[I_DONE] = (tot[0] <= tol2 || !isfinite(tot[0])) ? 1 : 0;
  }
}

__global__ void __launch_bounds__(256) k_bcg_p(int64_t n, const double *__restrict__ r, const double *__restrict__ v,
                                               double *__restrict__ p, double *__restrict__ ph,
                                               const double *__restrict__ dinv, const double *scal, const int *ictl) {
  if (ictl[I_DONE]) return;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double beta = scal[Q_BETA], omega = scal[Q_OMEGA];
  const double pi = r[i] + beta * (p[i] - omega * v[i]);
  p[i] = pi;
  ph[i] = dinv[i] * pi;
}

// MODE 0: y = v = A ph, alpha = rho / (rh . v).  MODE 1: y = t = A sh, omega = (t.s)/(t.t).
template <class CI, int MODE>
__global__ void __launch_bounds__(256) k_bcg_spmv(int64_t n, const int *__restrict__ sl_ptr,
                                                  const int *__restrict__ sl_len, const typename CI::T *__restrict__ col,
                                                  const double *__restrict__ val, const double *__restrict__ x,
                                                  double *__restrict__ y, const double *__restrict__ w,
                                                  double *scal, int *ictl, double *partials, unsigned *counter) {
  if (ictl[I_DONE]) return;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double d[2] = {0.0, 0.0};
  if (i < n) {
    const int s = (int)(i >> 5), lane = (int)(i & 31);
    const int64_t base = (int64_t)sl_ptr[s] + lane * FG_GROUP;
    const int G = sl_len[s];
    double acc = 0.0;
    for (int g = 0; g < G; ++g) {
      const typename CI::T4 cc = ld_cols(reinterpret_cast<const typename CI::T4 *>(col + base) + (int64_t)g * FG_SLICE);
      const double *vg = val + base + (int64_t)g * FG_GROUP * FG_SLICE;
      acc = fma(vg[0], x[CI::col(cc.x, i)], acc);
      acc = fma(vg[1], x[CI::col(cc.y, i)], acc);
      acc = fma(vg[2], x[CI::col(cc.z, i)], acc);
      acc = fma(vg[3], x[CI::col(cc.w, i)], acc);
    }
    y[i] = acc;
    d[0] = w[i] * acc;          // rh . v  or  s . t
    d[1] = MODE ? acc * acc : 0.0;
  }
  __shared__ double sh[2][32];
  block_sum<2>(d, sh);
  double tot[2];
  if (grid_finish<2>(d, partials, counter, tot)) {
    if (MODE == 0) {
      if (tot[0] == 0.0 || !isfinite(tot[0])) {
        ictl[I_STATUS] = 2;
        ictl[I_DONE] = 1;
      } else {
        scal[Q_ALPHA] = scal[Q_RHO] / tot[0];
      }
    } else {
      scal[Q_OMEGA] = tot[1] > 0.0 ? tot[0] / tot[1] : 0.0;
    }
  }
}

__global__ void __launch_bounds__(256) k_bcg_s(int64_t n, const double *__restrict__ r, const double *__restrict__ v,
                                               double *__restrict__ s, double *__restrict__ sh,
                                               const double *__restrict__ dinv, const double *scal, const int *ictl) {
  if (ictl[I_DONE]) return;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double si = r[i] - scal[Q_ALPHA] * v[i];
  s[i] = si;
  sh[i] = dinv[i] * si;
}

__global__ void __launch_bounds__(256) k_bcg_update(int64_t n, double *__restrict__ x, double *__restrict__ r,
                                                    const double *__restrict__ ph, const double *__restrict__ sh,
                                                    const double *__restrict__ s, const double *__restrict__ t,
                                                    const double *__restrict__ rh, double *scal, int *ictl,
                                                    double *partials, unsigned *counter) {
  if (ictl[I_DONE]) return;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double d[2] = {0.0, 0.0};
  if (i < n) {
    const double alpha = scal[Q_ALPHA], omega = scal[Q_OMEGA];
    x[i] += alpha * ph[i] + omega * sh[i];
    const double ri = s[i] - omega * t[i];
    r[i] = ri;
    d[0] = rh[i] * ri;
    d[1] = ri * ri;
  }
  __shared__ double shd[2][32];
  block_sum<2>(d, shd);
  double tot[2];
  if (grid_finish<2>(d, partials, counter, tot)) {
    const int it = ++ictl[I_ITERS];
    const double omega = scal[Q_OMEGA];
    scal[Q_RR] = tot[1];
    if (tot[1] <= scal[Q_TOL2]) {
      ictl[I_STATUS] = 0;
      ictl[I_DONE] = 1;
    } else if (!isfinite(tot[1]) || tot[0] == 0.0 || omega == 0.0) {
      ictl[I_STATUS] = 2;
      ictl[I_DONE] = 1;
    } else if (it >= ictl[I_MAXIT]) {
      ictl[I_STATUS] = 1;
      ictl[I_DONE] = 1;
    } else {
      scal[Q_BETA] = (tot[0] / scal[Q_RHO]) * (scal[Q_ALPHA] / omega);
      scal[Q_RHO] = tot[0];
    }
  }
}

void fg_spmv64_plain(fg_mesh *m, const double *vals, const double *x, double *y) {
  if (m->use_dcol)
    k_spmv64<ColRel><<<row_grid(m), 256, 0, m->stream>>>(m->nv, m->sl_ptr, m->sl_len, m->sl_dcol, vals, x, nullptr, y,
                                                         nullptr, -1, m->scal, m->red.partials, m->red.counter);
  else
    k_spmv64<ColAbs><<<row_grid(m), 256, 0, m->stream>>>(m->nv, m->sl_ptr, m->sl_len, m->sl_col, vals, x, nullptr, y,
                                                         nullptr, -1, m->scal, m->red.partials, m->red.counter);
  FG_CUDA_TRY(cudaGetLastError());
  FG_LAUNCHED(1);
}

template <class CI>
static void bcg_enqueue_body(fg_mesh *m, const typename CI::T *col) {
  double **v = m->bcg;
  const unsigned g = row_grid(m);
  const int64_t n = m->nv;
  for (int k = 0; k < FG_BCG_BODY; ++k) {
    k_bcg_p<<<g, 256, 0, m->stream>>>(n, v[BCG_R], v[BCG_V], v[BCG_P], v[BCG_PH], m->dinv64, m->scal, m->ictl);
    k_bcg_spmv<CI, 0><<<g, 256, 0, m->stream>>>(n, m->sl_ptr, m->sl_len, col, m->val64, v[BCG_PH], v[BCG_V],
                                                v[BCG_RH], m->scal, m->ictl, m->red.partials, m->red.counter);
    k_bcg_s<<<g, 256, 0, m->stream>>>(n, v[BCG_R], v[BCG_V], v[BCG_S], v[BCG_SH], m->dinv64, m->scal, m->ictl);
    k_bcg_spmv<CI, 1><<<g, 256, 0, m->stream>>>(n, m->sl_ptr, m->sl_len, col, m->val64, v[BCG_SH], v[BCG_T],
                                                v[BCG_S], m->scal, m->ictl, m->red.partials, m->red.counter);
    k_bcg_update<<<g, 256, 0, m->stream>>>(n, v[BCG_X], v[BCG_R], v[BCG_PH], v[BCG_SH], v[BCG_S], v[BCG_T],
                                           v[BCG_RH], m->scal, m->ictl, m->red.partials, m->red.counter);
  }
}

static void bcg_body(fg_mesh *m) {
  if (m->use_dcol) bcg_enqueue_body<ColRel>(m, m->sl_dcol);
  else bcg_enqueue_body<ColAbs>(m, m->sl_col);
}

int fg_bicgstab_solve(fg_mesh *m, const double *d_b, double *d_x, const fg_solve_opts &o, fg_solve_stats *st) {
  FG_REQUIRE(m->val64 && m->dinv64, FG_BAD_ARG, "BiCGStab: no FP64 operator assembled");
  for (int j = 0; j < BCG_NVEC; ++j)
    if (!m->bcg[j]) {
      m->bcg[j] = dev_alloc<double>(m, (size_t)m->nvp);
      FG_CUDA_TRY(cudaMemsetAsync(m->bcg[j], 0, sizeof(double) * (size_t)m->nvp, m->stream));
    }
  double **v = m->bcg;
  const int64_t n = m->nv;
  if (d_x != v[BCG_X])
    FG_CUDA_TRY(cudaMemcpyAsync(v[BCG_X], d_x, sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, m->stream));
  if (d_b != v[BCG_B])
    FG_CUDA_TRY(cudaMemcpyAsync(v[BCG_B], d_b, sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, m->stream));
  // r = b - A x
  if (m->use_dcol)
    k_spmv64<ColRel><<<row_grid(m), 256, 0, m->stream>>>(n, m->sl_ptr, m->sl_len, m->sl_dcol, m->val64, v[BCG_X],
                                                         v[BCG_B], v[BCG_R], nullptr, -1, m->scal, m->red.partials,
                                                         m->red.counter);
  else
    k_spmv64<ColAbs><<<row_grid(m), 256, 0, m->stream>>>(n, m->sl_ptr, m->sl_len, m->sl_col, m->val64, v[BCG_X],
                                                         v[BCG_B], v[BCG_R], nullptr, -1, m->scal, m->red.partials,
                                                         m->red.counter);
  const int maxit = o.maxiter > 0 ? o.maxiter : (int)std::min<int64_t>(2 * n + 10, 1 << 30);
  k_bcg_start<<<row_grid(m), 256, 0, m->stream>>>(n, v[BCG_B], v[BCG_R], v[BCG_RH], v[BCG_P], v[BCG_V], o.rtol, maxit,
                                                  m->scal, m->ictl, m->red.partials, m->red.counter);
  FG_CUDA_TRY(cudaGetLastError());
  FG_LAUNCHED(2);
  if (!m->bcg_exec || m->bcg_dcol != m->use_dcol) {
    if (m->bcg_exec) cudaGraphExecDestroy(m->bcg_exec);
    m->bcg_exec = nullptr;
    cudaGraph_t graph = nullptr;
    FG_CUDA_TRY(cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal));
    bcg_body(m);
    FG_CUDA_TRY(cudaStreamEndCapture(m->stream, &graph));
    const cudaError_t e = cudaGraphInstantiate(&m->bcg_exec, graph, 0);
    cudaGraphDestroy(graph);
    FG_CUDA_TRY(e);
    m->bcg_dcol = m->use_dcol;
  }
  int *h = m->hint;
  const int64_t max_bodies = maxit / FG_BCG_BODY + 2;
  for (int64_t b = 0; b < max_bodies; ++b) {
    FG_CUDA_TRY(cudaGraphLaunch(m->bcg_exec, m->stream));
    FG_LAUNCHED(5 * FG_BCG_BODY);
    FG_CUDA_TRY(cudaMemcpyAsync(h, m->ictl, sizeof(int) * 4, cudaMemcpyDeviceToHost, m->stream));
    fg_sync(m);
    if (h[I_DONE]) break;
  }
  FG_CUDA_TRY(cudaMemcpyAsync(m->hbuf, m->scal, sizeof(double) * 8, cudaMemcpyDeviceToHost, m->stream));
  FG_CUDA_TRY(cudaMemcpyAsync(h, m->ictl, sizeof(int) * 4, cudaMemcpyDeviceToHost, m->stream));
  if (d_x != v[BCG_X])
    FG_CUDA_TRY(cudaMemcpyAsync(d_x, v[BCG_X], sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, m->stream));
  fg_sync(m);
  const int status = h[I_DONE] ? h[I_STATUS] : 1;
  if (st) {
    st->iterations = h[I_ITERS];
    st->refinements = 0;
    st->converged = status == 0;
    st->pad_ = 0;
    const double bb = m->hbuf[Q_BB];
    st->relres = bb > 0.0 ? std::sqrt(m->hbuf[Q_RR] / bb) : std::sqrt(m->hbuf[Q_RR]);
    st->ms = 0.f;
  }
  return status;
}

// r = b - A x with the given SELL values (no Dirichlet masking); returns ||r||.
double fg_residual_norm(fg_mesh *m, const double *vals, const double *x, const double *b, double *r) {
  constexpr int slot = 9;
  if (m->use_dcol)
    k_spmv64<ColRel><<<row_grid(m), 256, 0, m->stream>>>(m->nv, m->sl_ptr, m->sl_len, m->sl_dcol, vals, x, b, r,
                                                         nullptr, slot, m->scal, m->red.partials, m->red.counter);
  else
    k_spmv64<ColAbs><<<row_grid(m), 256, 0, m->stream>>>(m->nv, m->sl_ptr, m->sl_len, m->sl_col, vals, x, b, r,
                                                         nullptr, slot, m->scal, m->red.partials, m->red.counter);
  FG_CUDA_TRY(cudaGetLastError());
  FG_LAUNCHED(1);
  FG_CUDA_TRY(cudaMemcpyAsync(m->hbuf, m->scal + slot, sizeof(double), cudaMemcpyDeviceToHost, m->stream));
  fg_sync(m);
  return std::sqrt(m->hbuf[0]);
}
