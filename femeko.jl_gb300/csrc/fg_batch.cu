// Many independent linear magnetostatic problems (meshes of uneven size) solved in
// ONE graph launch: each problem gets a thread-block cluster that runs its whole
// Jacobi-PCG (Magnetostatics/magneticField.jl:89-132 per mesh, the solve
// IterativeSolvers.cg does there) without returning to the host.  The cluster's CTAs
// split the problem's rows; dot products are reduced through distributed shared
// memory (every CTA reads the CTAs' partials in rank order, so all of them get the
// same value), and the cluster barrier separates the phases.
// Load balance: a problem's work grows with its rows (and its iteration count with
// them), so the cluster size follows the rows: 16, 8, 4 or 2 CTAs, the largest problem
// getting 16 where the device places 16-CTA clusters.  One launch per cluster size,
// the launches on parallel branches of one captured graph, largest problems first in
// each.
#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <numeric>
#include <type_traits>
#include <vector>

#include "fg_common.cuh"

namespace cgrp = cooperative_groups;

// Threads per CTA.  The FP64 kernel runs two CTAs per SM (64 registers a thread; its
// FP64 pipe is the limit, and two CTAs per SM pack the batch into fewer waves); the
// mixed kernel one CTA per SM with 128 registers a thread, which keeps more of a row's
// loads in flight (17 against 22 us per iteration on a 69k-row problem; two rows per
// thread in flight and 16-bit column offsets were measured slower or no faster).
constexpr int FG_BATCH_THREADS = 512;
constexpr int FG_BATCH_WARPS = FG_BATCH_THREADS / 32;
// FP64 refinement steps of a mixed-precision problem at most (as the single-mesh solver)
constexpr int FG_BATCH_MAX_REF = 50;

struct BatchProb {
  int64_t n;
  int nslices;
  const int *sl_ptr, *sl_len, *sl_col;
  const double *val, *dinv;
  const float *val32, *dinv32;  // FP32 operator (mixed precision; null in FP64)
  const uint8_t *fixed;         // may be null
  double *x, *r, *z, *p, *q;    // FP64 vectors (mixed: x and the FP64 residual r only)
  float4 *sa32, *sb32;  // mixed: the two buffers of the inner rows' state (r, w, s, D^-1)
  float *p32, *d32;     // mixed: inner search direction and correction
  double tol2_rel;
  double inner_rtol;  // mixed: relative target of each inner FP32 solve at least
  int maxit;
  int *iters;       // out: iterations (mixed: inner FP32 iterations in total)
  double *relres;   // out: ||r|| / ||r0||
  int *status;      // out: 0 converged, 1 cap, 2 non-finite / breakdown
  int *refs;        // out: FP64 refinement steps (mixed), 0 in FP64
};

// One CTA's shared state for the cluster reductions: the per-thread (FP64) or per-warp
// (FP32) partials, the CTA's published sums (read by the other CTAs of the cluster; two
// slots used alternately) and the scalars thread 0 broadcasts to the CTA.
template <int NV>
struct BatchShared {
  double part[NV][FG_BATCH_THREADS];
  double slot[2][NV];
  double bc[4];
};

// Cluster barrier with release (arrive) and acquire (wait) semantics at cluster scope:
// the global and shared writes of every thread before it are visible to every thread of
// the cluster after it (the default semantics of barrier.cluster, spelled out).
__device__ __forceinline__ void cluster_sync_acqrel() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Cluster-wide sums of NV values held by every thread.  Inside the CTA, FP32 values are
// added by warp shuffles and the 16 warp sums by warp 0 in FP64; FP64 values are stored
// per thread and warp 0 adds them (lane l: threads l, l + 32, ... in order, then a
// shuffle tree), so the FP64 additions run on one warp instead of all 512 threads (FP64
// issues at 1/64 of the FP32 rate).  The CTA's sums go to its slot; after the cluster
// barrier warp 0 of every CTA reads the CL slots (lane k: rank k) and adds them by the
// same shuffle tree, so all CTAs of the cluster get the same bits and take the same
// branches.  Result: tot[] in every lane of warp 0 (undefined in the other warps).
// `which` alternates between calls: a CTA rewrites a slot only after the next cluster
// barrier, when every reader of the slot's previous value is done.
template <int CL, int NV, int NS, typename T>
__device__ __forceinline__ void cluster_sums(cgrp::cluster_group &cl, BatchShared<NS> &sh, const T (&v)[NV],
                                             int which, double (&tot)[NV]) {
  static_assert(NV <= NS, "more values than shared slots");
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if constexpr (std::is_same<T, float>::value) {
    float a[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) a[k] = v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
      for (int k = 0; k < NV; ++k) a[k] += __shfl_down_sync(0xffffffffu, a[k], o);
    if (l == 0)
#pragma unroll
      for (int k = 0; k < NV; ++k) sh.part[k][w] = (double)a[k];
  } else {
#pragma unroll
    for (int k = 0; k < NV; ++k) sh.part[k][threadIdx.x] = v[k];
  }
  __syncthreads();
  if (w == 0) {
    double s[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      if constexpr (std::is_same<T, float>::value) {
        s[k] = l < FG_BATCH_WARPS ? sh.part[k][l] : 0.0;
      } else {
        s[k] = 0.0;
#pragma unroll 4
        for (int j = l; j < FG_BATCH_THREADS; j += 32) s[k] += sh.part[k][j];
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
      for (int k = 0; k < NV; ++k) s[k] += __shfl_down_sync(0xffffffffu, s[k], o);
    if (l == 0)
#pragma unroll
      for (int k = 0; k < NV; ++k) sh.slot[which][k] = s[k];
  }
  cluster_sync_acqrel();
  if (w == 0) {
    double t[NV];
    const double *remote = l < CL ? cl.map_shared_rank(&sh.slot[which][0], l) : nullptr;
#pragma unroll
    for (int k = 0; k < NV; ++k) t[k] = l < CL ? remote[k] : 0.0;
#pragma unroll
    for (int o = CL / 2; o > 0; o >>= 1)
#pragma unroll
      for (int k = 0; k < NV; ++k) t[k] += __shfl_down_sync(0xffffffffu, t[k], o);
#pragma unroll
    for (int k = 0; k < NV; ++k) tot[k] = __shfl_sync(0xffffffffu, t[k], 0);
  }
}

// FP32 form for the inner iterations of the mixed-precision solve: warp shuffles, warp
// 0 adds the 16 warp sums into the CTA's slot, and after the cluster barrier EVERY warp
// reads the CL slots and adds them by the same shuffle tree, so all threads of the
// cluster hold the same bits without a broadcast through shared memory (one CTA
// barrier and one cluster barrier per call).
template <int NV>
struct BatchShared32 {
  float wsum[NV][FG_BATCH_WARPS];
  float slot[2][NV];
};
template <int CL, int NV, int NS>
__device__ __forceinline__ void cluster_sums_f32(cgrp::cluster_group &cl, BatchShared32<NS> &sh, const float (&v)[NV],
                                                 int which, float (&tot)[NV]) {
  static_assert(NV <= NS, "more values than shared slots");
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  float a[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) a[k] = v[k];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int k = 0; k < NV; ++k) a[k] += __shfl_down_sync(0xffffffffu, a[k], o);
  if (l == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) sh.wsum[k][w] = a[k];
  __syncthreads();
  if (w == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) a[k] = l < FG_BATCH_WARPS ? sh.wsum[k][l] : 0.f;
#pragma unroll
    for (int o = FG_BATCH_WARPS / 2; o > 0; o >>= 1)
#pragma unroll
      for (int k = 0; k < NV; ++k) a[k] += __shfl_down_sync(0xffffffffu, a[k], o);
    if (l == 0)
#pragma unroll
      for (int k = 0; k < NV; ++k) sh.slot[which][k] = a[k];
  }
  cluster_sync_acqrel();
  const float *remote = cl.map_shared_rank(&sh.slot[which][0], l < CL ? l : 0);
#pragma unroll
  for (int k = 0; k < NV; ++k) a[k] = l < CL ? remote[k] : 0.f;
#pragma unroll
  for (int o = CL / 2; o > 0; o >>= 1)
#pragma unroll
    for (int k = 0; k < NV; ++k) a[k] += __shfl_down_sync(0xffffffffu, a[k], o);
#pragma unroll
  for (int k = 0; k < NV; ++k) tot[k] = __shfl_sync(0xffffffffu, a[k], 0);
}

// Barrier between a pass that writes vector entries and one that reads other CTAs'
// entries.
__device__ __forceinline__ void cluster_barrier(cgrp::cluster_group &) { cluster_sync_acqrel(); }

// Row i of the SELL-32x4 operator applied to the vector entries get(j): the row's groups
// of four slots lie 128 entries apart, one 16-byte load of columns and one (FP32) or two
// (FP64) of values per group.
template <int U, typename V, typename Get>
__device__ __forceinline__ auto sell_row(const int *__restrict__ sl_ptr, const int *__restrict__ sl_len,
                                         const int *__restrict__ sl_col, const V *__restrict__ val, int64_t i,
                                         Get get) -> decltype(get(0)) {
  using A = decltype(get(0));
  const int s = (int)(i >> 5);
  const int64_t base = (int64_t)sl_ptr[s] + (i & 31) * FG_GROUP;
  const int G = sl_len[s];
  A acc = 0;
#pragma unroll U
  for (int g = 0; g < G; ++g) {
    const int64_t e = base + (int64_t)g * FG_SLICE * FG_GROUP;
    const int4 c = *reinterpret_cast<const int4 *>(sl_col + e);
    if constexpr (std::is_same<V, float>::value) {
      const float4 a = *reinterpret_cast<const float4 *>(val + e);
      acc = fmaf(a.x, get(c.x), acc);
      acc = fmaf(a.y, get(c.y), acc);
      acc = fmaf(a.z, get(c.z), acc);
      acc = fmaf(a.w, get(c.w), acc);
    } else {
      const double2 a0 = *reinterpret_cast<const double2 *>(val + e);
      const double2 a1 = *reinterpret_cast<const double2 *>(val + e + 2);
      acc = fma(a0.x, get(c.x), acc);
      acc = fma(a0.y, get(c.y), acc);
      acc = fma(a1.x, get(c.z), acc);
      acc = fma(a1.y, get(c.w), acc);
    }
  }
  return acc;
}

// FP64 Jacobi-PCG of one problem per cluster.  Each iteration: p = z + beta p (own
// rows), barrier, q = A p with p.q, then x, r, z with r.z and r.r; the scalars come
// from thread 0 of each CTA (the same bits in every CTA) through shared memory.
template <int CL>
__global__ void __launch_bounds__(FG_BATCH_THREADS, 2) k_batch_pcg64(const BatchProb *__restrict__ probs) {
  cgrp::cluster_group cl = cgrp::this_cluster();
  __shared__ BatchShared<2> sh;
  const int rank = (int)cl.block_rank();
  const BatchProb *pp = probs + blockIdx.x / CL;
  const int64_t n = pp->n;
  const int nslices = pp->nslices;
  const int *__restrict__ sl_ptr = pp->sl_ptr;
  const int *__restrict__ sl_len = pp->sl_len;
  const int *__restrict__ sl_col = pp->sl_col;
  const double *__restrict__ val = pp->val;
  const double *__restrict__ dinv = pp->dinv;
  const uint8_t *__restrict__ fixed = pp->fixed;
  double *x = pp->x, *r = pp->r, *z = pp->z, *p = pp->p, *q = pp->q;
  // this CTA's rows: a contiguous run of whole slices
  const int per = (nslices + CL - 1) / CL;
  const int s0 = min(rank * per, nslices), s1 = min(s0 + per, nslices);
  const int64_t i0 = (int64_t)s0 * FG_SLICE, i1 = min((int64_t)s1 * FG_SLICE, n);
  const int maxit = pp->maxit;
  // r = -A x on free rows (the right-hand side is 0), z = D^-1 r, p = 0
  double prz = 0.0, prr = 0.0;
  for (int64_t i = i0 + threadIdx.x; i < i1; i += FG_BATCH_THREADS) {
    double ri = 0.0;
    if (!(fixed && fixed[i])) ri = -sell_row<2>(sl_ptr, sl_len, sl_col, val, i, [&](int j) { return x[j]; });
    const double zi = dinv[i] * ri;
    r[i] = ri;
    z[i] = zi;
    p[i] = 0.0;
    prz = fma(ri, zi, prz);
    prr = fma(ri, ri, prr);
  }
  int which = 0, it = 0, st;
  double tot[2];
  // thread 0's scalar state (the same in every CTA of the cluster)
  double rz = 0.0, rr = 0.0, rr0 = 0.0, tol2 = 0.0;
  {
    const double v[2] = {prz, prr};
    cluster_sums<CL>(cl, sh, v, which, tot);
    which ^= 1;
  }
  if (threadIdx.x == 0) {
    rz = tot[0];
    rr = rr0 = tot[1];
    tol2 = pp->tol2_rel * rr0;
    const int s = !isfinite(rr0) ? 2 : (rr0 == 0.0 ? 0 : (maxit <= 0 ? 1 : -1));
    sh.bc[0] = s;
  }
  __syncthreads();
  st = (int)sh.bc[0];
  double beta = 0.0;
  while (st < 0) {
    // p = z + beta p on this CTA's rows
    for (int64_t i = i0 + threadIdx.x; i < i1; i += FG_BATCH_THREADS)
      p[i] = (fixed && fixed[i]) ? 0.0 : fma(beta, p[i], z[i]);
    cluster_barrier(cl);
    // q = A p, p.q
    double ppq = 0.0;
    for (int64_t i = i0 + threadIdx.x; i < i1; i += FG_BATCH_THREADS) {
      double qi = 0.0;
      if (!(fixed && fixed[i])) qi = sell_row<2>(sl_ptr, sl_len, sl_col, val, i, [&](int j) { return p[j]; });
      q[i] = qi;
      ppq = fma(p[i], qi, ppq);
    }
    {
      const double v[1] = {ppq};
      double t1[1];
      cluster_sums<CL>(cl, sh, v, which, t1);
      which ^= 1;
      if (threadIdx.x == 0) {
        const double pq = t1[0];
        int s = -1;
        if (!(pq > 0.0) || !isfinite(pq)) s = (pq == 0.0) ? 0 : 2;
        sh.bc[0] = s;
        sh.bc[1] = s < 0 ? rz / pq : 0.0;
      }
    }
    __syncthreads();
    st = (int)sh.bc[0];
    if (st >= 0) break;
    const double alpha = sh.bc[1];
    // x += alpha p; r -= alpha q; z = D^-1 r
    prz = 0.0;
    prr = 0.0;
    for (int64_t i = i0 + threadIdx.x; i < i1; i += FG_BATCH_THREADS) {
      x[i] = fma(alpha, p[i], x[i]);
      const double ri = fma(-alpha, q[i], r[i]);
      const double zi = dinv[i] * ri;
      r[i] = ri;
      z[i] = zi;
      prz = fma(ri, zi, prz);
      prr = fma(ri, ri, prr);
    }
    {
      const double v[2] = {prz, prr};
      cluster_sums<CL>(cl, sh, v, which, tot);
      which ^= 1;
    }
    ++it;
    if (threadIdx.x == 0) {
      const double rzn = tot[0];
      rr = tot[1];
      const int s = !isfinite(rr) ? 2 : (rr <= tol2 ? 0 : (it >= maxit ? 1 : -1));
      sh.bc[0] = s;
      sh.bc[1] = rzn / rz;
      rz = rzn;
    }
    __syncthreads();
    st = (int)sh.bc[0];
    beta = sh.bc[1];
  }
  if (rank == 0 && threadIdx.x == 0) {
    *pp->iters = it;
    *pp->relres = rr0 > 0.0 ? sqrt(rr / rr0) : 0.0;
    *pp->status = st;
    *pp->refs = 0;
  }
  cl.sync();  // no CTA leaves while another may still read its shared slots
}

// Mixed precision: FP64 iterative refinement around FP32 Jacobi-PCG, the single-mesh
// solver's scheme (FP64 residual r = -A x, inner FP32 solve of A d = r / ||r|| to
// max(rtol ||r0|| / ||r||, inner_rtol), x += ||r|| d, until ||r|| <= rtol ||r0||) run
// by one cluster per problem.
// The inner solve is Chronopoulos–Gear PCG (one reduction of r.u, w.u, r.r per
// iteration, u = D^-1 r, w = A u) in ONE pass over the rows per iteration: each row's
// state (r, w, s, D^-1) is a float4 in two buffers; a pass reads the old state of its
// rows and of their neighbours and writes the new state of its rows, forming each
// neighbour's new u = D^-1 (r - alpha (w + beta s)) from its old state at the stored
// entry, so w_new = A u_new needs no barrier of its own.  p and d are the row's own.
template <int CL>
__global__ void __launch_bounds__(FG_BATCH_THREADS, 1) k_batch_pcg_mixed(const BatchProb *__restrict__ probs) {
  cgrp::cluster_group cl = cgrp::this_cluster();
  __shared__ BatchShared<1> sh;     // FP64 residual norms
  __shared__ BatchShared32<3> sf;   // inner FP32 sums
  const int rank = (int)cl.block_rank();
  const BatchProb *pp = probs + blockIdx.x / CL;
  const int64_t n = pp->n;
  const int nslices = pp->nslices;
  const int *__restrict__ sl_ptr = pp->sl_ptr;
  const int *__restrict__ sl_len = pp->sl_len;
  const int *__restrict__ sl_col = pp->sl_col;
  const double *__restrict__ val = pp->val;
  const float *__restrict__ val32 = pp->val32;
  const float *__restrict__ dinv32 = pp->dinv32;
  const uint8_t *__restrict__ fixed = pp->fixed;
  double *x = pp->x, *r = pp->r;
  float *pv = pp->p32, *dv = pp->d32;
  const int per = (nslices + CL - 1) / CL;
  const int s0 = min(rank * per, nslices), s1 = min(s0 + per, nslices);
  const int64_t i0 = (int64_t)s0 * FG_SLICE, i1 = min((int64_t)s1 * FG_SLICE, n);
  const int maxit = pp->maxit;
  int which = 0, whichf = 0, it = 0, ref = 0, st = -1;
  // thread 0's FP64 state (the same in every CTA of the cluster)
  double rr0 = -1.0, rrt = 0.0;
  while (true) {
    // FP64 residual r = -A x on the free rows (the right-hand side is 0)
    double prr = 0.0;
    for (int64_t i = i0 + threadIdx.x; i < i1; i += FG_BATCH_THREADS) {
      double ri = 0.0;
      if (!(fixed && fixed[i])) ri = -sell_row<2>(sl_ptr, sl_len, sl_col, val, i, [&](int j) { return x[j]; });
      r[i] = ri;
      prr = fma(ri, ri, prr);
    }
    {
      const double v[1] = {prr};
      double t1[1];
      cluster_sums<CL>(cl, sh, v, which, t1);
      which ^= 1;
      if (threadIdx.x == 0) {
        rrt = t1[0];
        if (rr0 < 0.0) rr0 = rrt;
        const double tol2 = pp->tol2_rel * rr0;
        int s = -1;
        if (!isfinite(rrt)) s = 2;
        else if (rrt <= tol2 || rrt == 0.0) s = 0;
        else if (it >= maxit || ref >= FG_BATCH_MAX_REF) s = 1;
        const double rn = sqrt(rrt);
        const double inner = fmax(sqrt(tol2 / rrt), pp->inner_rtol);
        sh.bc[0] = s;
        sh.bc[1] = s < 0 ? 1.0 / rn : 0.0;
        sh.bc[2] = rn;
        sh.bc[3] = inner * inner;
      }
    }
    __syncthreads();
    st = (int)sh.bc[0];
    if (st >= 0) break;
    const double scale = sh.bc[1], rn = sh.bc[2];
    const float inner2 = (float)sh.bc[3];
    float4 *so = pp->sa32, *sn = pp->sb32;
    // inner start: r0 = r / ||r||, state (r0, 0, 0, D^-1), p = d = 0
    for (int64_t i = i0 + threadIdx.x; i < i1; i += FG_BATCH_THREADS) {
      so[i] = make_float4((float)(r[i] * scale), 0.f, 0.f, dinv32[i]);
      pv[i] = 0.f;
      dv[i] = 0.f;
    }
    cluster_barrier(cl);
    // w0 = A u0 and the first sums (the scalars: every thread holds the same bits)
    float g = 0.f, dl = 0.f, rr = 0.f;
    for (int64_t i = i0 + threadIdx.x; i < i1; i += FG_BATCH_THREADS) {
      const float4 o = so[i];
      float wi = 0.f;
      if (!(fixed && fixed[i]))
        wi = sell_row<4>(sl_ptr, sl_len, sl_col, val32, i, [&](int j) {
          const float4 t = so[j];
          return t.w * t.x;
        });
      const float ui = o.w * o.x;
      sn[i] = make_float4(o.x, wi, 0.f, o.w);
      g = fmaf(o.x, ui, g);
      dl = fmaf(wi, ui, dl);
      rr = fmaf(o.x, o.x, rr);
    }
    float tot[3];
    {
      const float v[3] = {g, dl, rr};
      cluster_sums_f32<CL>(cl, sf, v, whichf, tot);
      whichf ^= 1;
    }
    {
      float4 *t = so;
      so = sn;
      sn = t;
    }
    float gam = tot[0];
    const float itol2 = inner2 * tot[2];
    int ist = -1;
    if (!(tot[2] > 0.f)) ist = 0;
    else if (!(tot[1] > 0.f) || !isfinite(tot[1])) ist = (tot[1] == 0.f) ? 0 : 2;
    float alpha = ist < 0 ? gam / tot[1] : 0.f, beta = 0.f;
    while (ist < 0 && it < maxit) {
      // s = w + beta s; p = u + beta p; d += alpha p; r -= alpha s; u = D^-1 r; w = A u
      g = 0.f;
      dl = 0.f;
      rr = 0.f;
      for (int64_t i = i0 + threadIdx.x; i < i1; i += FG_BATCH_THREADS) {
        const float4 o = so[i];
        const float sk = fmaf(beta, o.z, o.y);
        const float pk = fmaf(beta, pv[i], o.w * o.x);
        dv[i] = fmaf(alpha, pk, dv[i]);
        pv[i] = pk;
        const float rk = fmaf(-alpha, sk, o.x);
        const float uk = o.w * rk;
        float wk = 0.f;
        if (!(fixed && fixed[i]))
          wk = sell_row<4>(sl_ptr, sl_len, sl_col, val32, i, [&](int j) {
            const float4 t = so[j];
            return t.w * fmaf(-alpha, fmaf(beta, t.z, t.y), t.x);
          });
        sn[i] = make_float4(rk, wk, sk, o.w);
        g = fmaf(rk, uk, g);
        dl = fmaf(wk, uk, dl);
        rr = fmaf(rk, rk, rr);
      }
      {
        const float v[3] = {g, dl, rr};
        cluster_sums_f32<CL>(cl, sf, v, whichf, tot);
        whichf ^= 1;
      }
      {
        float4 *t = so;
        so = sn;
        sn = t;
      }
      ++it;
      if (!isfinite(tot[2])) {
        ist = 2;
        break;
      }
      if (tot[2] <= itol2) break;
      const float gn = tot[0];
      beta = gn / gam;
      const float den = tot[1] - beta * gn / alpha;  // p.A p of the next direction
      if (!(den > 0.f) || !isfinite(den)) {
        ist = (den == 0.f) ? 0 : 2;
        break;
      }
      alpha = gn / den;
      gam = gn;
    }
    // x += ||r|| d
    for (int64_t i = i0 + threadIdx.x; i < i1; i += FG_BATCH_THREADS) x[i] = fma(rn, (double)dv[i], x[i]);
    if (ist == 2) {
      st = 2;
      break;
    }
    ++ref;
    cluster_barrier(cl);  // x complete before the next residual reads the neighbours' entries
  }
  if (rank == 0 && threadIdx.x == 0) {
    *pp->iters = it;
    *pp->relres = rr0 > 0.0 ? sqrt(rrt / rr0) : 0.0;
    *pp->status = st;
    *pp->refs = ref;
  }
  cl.sync();  // no CTA leaves while another may still read its shared slots
}

template <int CL>
static const void *batch_fn(bool mixed) {
  return mixed ? reinterpret_cast<const void *>(k_batch_pcg_mixed<CL>)
               : reinterpret_cast<const void *>(k_batch_pcg64<CL>);
}
static const void *batch_kernel(int cl, bool mixed) {
  switch (cl) {
    case 16: return batch_fn<16>(mixed);
    case 8: return batch_fn<8>(mixed);
    case 4: return batch_fn<4>(mixed);
    default: return batch_fn<2>(mixed);
  }
}

extern "C" fg_status fg_batch_magnetostatics_linear(fg_mesh *const *meshes, int32_t count, const double *const *mu,
                                                    const double *const *u_in, const fg_solve_opts *o,
                                                    double *const *u_out, int32_t *iterations,
                                                    fg_batch_stats *s) {
  return fg_guard([&]() -> fg_status {
    FG_REQUIRE(meshes && mu && u_in && u_out && count > 0, FG_BAD_ARG, "fg_batch_magnetostatics_linear: bad arguments");
    fg_solve_opts opts;
    fg_solve_opts_default(&opts);
    if (o) opts = *o;
    FG_REQUIRE(opts.precision == FG_FP64 || opts.precision == FG_MIXED, FG_BAD_ARG,
               "fg_batch_magnetostatics_linear: precision must be FG_FP64 or FG_MIXED");
    const bool mixed = opts.precision == FG_MIXED;
    fg_mesh *m0 = meshes[0];
    FG_REQUIRE(m0 != nullptr, FG_BAD_ARG, "fg_batch_magnetostatics_linear: null mesh");
    std::vector<BatchProb> hp(count);
    for (int k = 0; k < count; ++k) {
      fg_mesh *m = meshes[k];
      FG_REQUIRE(m && mu[k] && u_in[k] && u_out[k], FG_BAD_ARG, "fg_batch_magnetostatics_linear: null entry");
      FG_REQUIRE(m->device == m0->device, FG_BAD_ARG, "fg_batch_magnetostatics_linear: meshes on different devices");
      FG_REQUIRE(m->npe == 4 || m->npe == 3, FG_UNSUPPORTED, "fg_batch_magnetostatics_linear: P1 elements only");
      if (!m->mu_lin) m->mu_lin = dev_alloc<double>(m, (size_t)m->nt);
      FG_CUDA_TRY(cudaMemcpyAsync(m->mu_lin, mu[k], sizeof(double) * (size_t)m->nt, cudaMemcpyHostToDevice, m->stream));
      fg_assemble_operator(m, ASM_STIFF, m->mu_lin, nullptr, nullptr, 0.0, 0.0, 0, OUT_SELL, true, mixed, true);
      for (int j : {7, 0, 1, 2, 3})
        if (!m->v64[j]) m->v64[j] = dev_alloc<double>(m, (size_t)m->nvp);
      // FP32 inner vectors: the fused FP32 CG's row-state buffers (4 nvp floats each)
      // and its x and p vectors (nvp), zeroed when first made as the CG solver makes
      // them; every solve initialises what it reads
      if (mixed)
        for (int j = 0; j < 4; ++j)
          if (!m->v32[j]) {
            const size_t len = (size_t)m->nvp * ((j == 2 || j == 3) ? 4 : 1);
            m->v32[j] = dev_alloc<float>(m, len);
            FG_CUDA_TRY(cudaMemsetAsync(m->v32[j], 0, sizeof(float) * len, m->stream));
          }
      FG_CUDA_TRY(cudaMemcpyAsync(m->v64[7], u_in[k], sizeof(double) * (size_t)m->nv, cudaMemcpyHostToDevice,
                                  m->stream));
      BatchProb &b = hp[k];
      b.n = m->nv;
      b.nslices = m->nslices;
      b.sl_ptr = m->sl_ptr;
      b.sl_len = m->sl_len;
      b.sl_col = m->sl_col;
      b.val = m->val64;
      b.dinv = m->dinv64;
      b.val32 = mixed ? m->val32 : nullptr;
      b.dinv32 = mixed ? m->dinv32 : nullptr;
      b.fixed = m->has_fixed ? m->fixed : nullptr;
      b.x = m->v64[7];
      b.r = m->v64[0];
      b.z = m->v64[1];
      b.p = m->v64[2];
      b.q = m->v64[3];
      b.sa32 = mixed ? reinterpret_cast<float4 *>(m->v32[2]) : nullptr;
      b.sb32 = mixed ? reinterpret_cast<float4 *>(m->v32[3]) : nullptr;
      b.p32 = mixed ? m->v32[1] : nullptr;
      b.d32 = mixed ? m->v32[0] : nullptr;
      b.tol2_rel = opts.rtol * opts.rtol;
      b.inner_rtol = opts.inner_rtol;
      b.maxit = opts.maxiter;
    }
    for (int k = 0; k < count; ++k) {
      fg_sync(meshes[k]);
      for (int j = 0; j < k; ++j)
        FG_REQUIRE(meshes[j] != meshes[k], FG_BAD_ARG, "fg_batch_magnetostatics_linear: a mesh handle appears twice");
    }
    // cluster size per problem from its rows: the largest problem gets the largest
    // cluster the device places (16 where allowed, else 8), the others in proportion
    // to their rows (at least 2 CTAs)
    auto fits = [&](int cl) {
      cudaLaunchConfig_t cfg = {};
      cfg.blockDim = dim3(FG_BATCH_THREADS);
      cfg.gridDim = dim3((unsigned)cl);
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = (unsigned)cl;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      int fit = 0;
      const void *fn = batch_kernel(cl, mixed);
      cudaError_t e = cudaSuccess;
      if (cl == 16) e = cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
      if (e == cudaSuccess) e = cudaOccupancyMaxActiveClusters(&fit, fn, &cfg);
      if (e != cudaSuccess) {
        cudaGetLastError();
        return false;
      }
      return fit > 0;
    };
    const int cl_max = fits(16) ? 16 : 8;
    FG_REQUIRE(fits(8), FG_UNSUPPORTED, "fg_batch_magnetostatics_linear: the device cannot place an 8-CTA cluster");
    int64_t nmax = 1;
    for (int k = 0; k < count; ++k) nmax = std::max(nmax, hp[k].n);
    std::vector<int> clk(count);
    for (int k = 0; k < count; ++k) {
      const double want = (double)cl_max * (double)hp[k].n / (double)nmax;
      int c = 2;
      while (c < cl_max && c < want) c *= 2;
      clk[k] = c;
    }
    // problems ordered by cluster size, then largest first within one size
    std::vector<int> order(count);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
      return clk[a] != clk[b] ? clk[a] > clk[b] : hp[a].n > hp[b].n;
    });
    int *d_out = nullptr;
    BatchProb *d_probs = nullptr;
    double *d_rel = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr, fork = nullptr;
    std::vector<cudaStream_t> side;
    std::vector<cudaEvent_t> joins;
    auto cleanup = [&]() {
      if (exec) cudaGraphExecDestroy(exec);
      if (graph) cudaGraphDestroy(graph);
      if (e0) cudaEventDestroy(e0);
      if (e1) cudaEventDestroy(e1);
      if (fork) cudaEventDestroy(fork);
      for (cudaEvent_t e : joins) cudaEventDestroy(e);
      for (cudaStream_t q : side) cudaStreamDestroy(q);
      cudaFree(d_out);
      cudaFree(d_probs);
      cudaFree(d_rel);
    };
    try {
      FG_CUDA_TRY(cudaMalloc(&d_out, sizeof(int) * 3 * count));
      FG_CUDA_TRY(cudaMalloc(&d_rel, sizeof(double) * count));
      FG_CUDA_TRY(cudaMalloc(&d_probs, sizeof(BatchProb) * count));
      std::vector<BatchProb> sorted(count);
      for (int j = 0; j < count; ++j) {
        sorted[j] = hp[order[j]];
        sorted[j].iters = d_out + j;
        sorted[j].status = d_out + count + j;
        sorted[j].relres = d_rel + j;
        sorted[j].refs = d_out + 2 * count + j;
      }
      cudaStream_t st = m0->stream;
      FG_CUDA_TRY(cudaMemcpyAsync(d_probs, sorted.data(), sizeof(BatchProb) * count, cudaMemcpyHostToDevice, st));
      // one launch per cluster size: [first, first + n) of the sorted problems
      struct Group {
        int cl, first, n;
      };
      std::vector<Group> groups;
      for (int j = 0; j < count;) {
        int e = j;
        while (e < count && clk[order[e]] == clk[order[j]]) ++e;
        groups.push_back(Group{clk[order[j]], j, e - j});
        j = e;
      }
      FG_CUDA_TRY(cudaEventCreate(&e0));
      FG_CUDA_TRY(cudaEventCreate(&e1));
      FG_CUDA_TRY(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
      for (size_t gi = 1; gi < groups.size(); ++gi) {
        cudaStream_t q;
        FG_CUDA_TRY(cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking));
        side.push_back(q);
        cudaEvent_t ev;
        FG_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        joins.push_back(ev);
      }
      auto launch = [&](const Group &g, cudaStream_t q) -> cudaError_t {
        cudaLaunchConfig_t cfg = {};
        cfg.blockDim = dim3(FG_BATCH_THREADS);
        cfg.gridDim = dim3((unsigned)(g.n * g.cl));
        cfg.stream = q;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = (unsigned)g.cl;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        const BatchProb *pp = d_probs + g.first;
        void *args[1] = {&pp};
        return cudaLaunchKernelExC(&cfg, batch_kernel(g.cl, mixed), args);
      };
      FG_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      cudaError_t le = cudaEventRecord(fork, st);
      for (size_t gi = 1; gi < groups.size() && le == cudaSuccess; ++gi) le = cudaStreamWaitEvent(side[gi - 1], fork, 0);
      if (le == cudaSuccess) le = launch(groups[0], st);
      for (size_t gi = 1; gi < groups.size() && le == cudaSuccess; ++gi) {
        le = launch(groups[gi], side[gi - 1]);
        if (le == cudaSuccess) le = cudaEventRecord(joins[gi - 1], side[gi - 1]);
        if (le == cudaSuccess) le = cudaStreamWaitEvent(st, joins[gi - 1], 0);
      }
      cudaError_t ce = cudaStreamEndCapture(st, &graph);
      FG_CUDA_TRY(le);
      FG_CUDA_TRY(ce);
      FG_CUDA_TRY(cudaGraphInstantiate(&exec, graph, 0));
      FG_CUDA_TRY(cudaEventRecord(e0, st));
      FG_CUDA_TRY(cudaGraphLaunch(exec, st));
      FG_CUDA_TRY(cudaEventRecord(e1, st));
      FG_LAUNCHED((long long)groups.size());
      std::vector<int> hout(3 * count);
      std::vector<double> hrel(count);
      FG_CUDA_TRY(cudaMemcpyAsync(hout.data(), d_out, sizeof(int) * 3 * count, cudaMemcpyDeviceToHost, st));
      FG_CUDA_TRY(cudaMemcpyAsync(hrel.data(), d_rel, sizeof(double) * count, cudaMemcpyDeviceToHost, st));
      FG_CUDA_TRY(cudaStreamSynchronize(st));
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      int conv = 0, maxit = 0, nan = 0, maxref = 0;
      long long tot = 0;
      for (int j = 0; j < count; ++j) {
        const int k = order[j];
        if (iterations) iterations[k] = hout[j];
        conv += hout[count + j] == 0;
        nan += hout[count + j] == 2;
        maxit = std::max(maxit, hout[j]);
        maxref = std::max(maxref, hout[2 * count + j]);
        tot += hout[j];
      }
      for (int k = 0; k < count; ++k)
        FG_CUDA_TRY(cudaMemcpyAsync(u_out[k], meshes[k]->v64[7], sizeof(double) * (size_t)meshes[k]->nv,
                                    cudaMemcpyDeviceToHost, st));
      FG_CUDA_TRY(cudaStreamSynchronize(st));
      if (s) {
        s->problems = count;
        s->converged = conv;
        s->max_iterations = maxit;
        s->cluster_ctas = cl_max;
        s->total_iterations = tot;
        s->ms = ms;
        s->max_refinements = maxref;
        s->reserved_ = 0;
      }
      cleanup();
      if (nan) return FG_NAN;
      return conv == count ? FG_OK : FG_NOT_CONVERGED;
    } catch (...) {
      cleanup();
      throw;
    }
  });
}
