// SpMV and Jacobi-preconditioned CG on the SELL-32 operator.
//
// The reference solves with IterativeSolvers.cg (Magnetostatics/2DmagneticField.jl:139,
// Micromagnetics/LL.jl:185, Femeko_jl_C++/Magnetostatics/run.jl:141) or Eigen's
// diagonal-preconditioned ConjugateGradient (magnetostatics.cpp:26-38).  Here one CG
// iteration is two kernels:
//   k_cg_spmv   q = A pn with pn = z + beta p formed on the fly (no separate p pass),
//               p.q reduced in the same launch, alpha computed by the last block;
//   k_cg_update x += alpha pn, r -= alpha q, z = D^-1 r, r.z and r.r reduced, beta and
//               the stopping test computed by the last block.
// Scalars never leave the device; the host reads the "done" flag once per block of
// iterations, and each block can be replayed as a CUDA graph.
//
// Mixed precision: the operator values and the CG vectors are FP32; dot products
// are accumulated with compensated FP32 sums inside a block and FP64 across blocks.
// An FP64 residual b - A x (FP64 operator) drives iterative refinement around the
// FP32 solves.  In the Newton solver the Newton loop itself is that refinement.
#include <cmath>
#include <vector>

#include "fg_common.cuh"

// ------------------------------------------------------------------ reductions
struct ff {
  float hi, lo;
};

__device__ __forceinline__ ff ff_add(ff a, ff b) {
  float s = a.hi + b.hi;
  float bb = s - a.hi;
  float e = (a.hi - (s - bb)) + (b.hi - bb);
  return ff{s, e + a.lo + b.lo};
}

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

// Compensated FP32 block sum of (hi, lo) pairs, returned as double in thread 0.
template <int N>
__device__ __forceinline__ void block_sum_ff(ff (&v)[N], double (&out)[N], ff (*sh)[32]) {
#pragma unroll
  for (int j = 0; j < N; ++j)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      ff other{__shfl_down_sync(0xffffffffu, v[j].hi, o), __shfl_down_sync(0xffffffffu, v[j].lo, o)};
      v[j] = ff_add(v[j], other);
    }
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0)
#pragma unroll
    for (int j = 0; j < N; ++j) sh[j][w] = v[j];
  __syncthreads();
  if (w == 0) {
    int nw = blockDim.x >> 5;
#pragma unroll
    for (int j = 0; j < N; ++j) {
      v[j] = (l < nw) ? sh[j][l] : ff{0.f, 0.f};
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        ff other{__shfl_down_sync(0xffffffffu, v[j].hi, o), __shfl_down_sync(0xffffffffu, v[j].lo, o)};
        v[j] = ff_add(v[j], other);
      }
      out[j] = (double)v[j].hi + (double)v[j].lo;
    }
  }
}

// Block sum of per-thread accumulators; thread 0 gets the totals as doubles.
template <typename S, int N>
__device__ __forceinline__ void block_sum_acc(Acc<S> *a, double (&out)[N]) {
  if (sizeof(S) == 4) {
    __shared__ ff shf[N][32];
    ff v[N];
#pragma unroll
    for (int j = 0; j < N; ++j) v[j] = reinterpret_cast<Acc<float> *>(a)[j].v;
    block_sum_ff<N>(v, out, shf);
  } else {
    __shared__ double shd[N][32];
#pragma unroll
    for (int j = 0; j < N; ++j) out[j] = reinterpret_cast<Acc<double> *>(a)[j].v;
    block_sum<N>(out, shd);
  }
}

// Block partials -> the last block to arrive sums them in block order.  Returns true
// in thread 0 of the last block, with the totals in tot.
template <int N>
__device__ __forceinline__ bool grid_finish(const double (&v)[N], double *partials, unsigned *counter,
                                            double (&tot)[N]) {
  __shared__ bool s_last;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int j = 0; j < N; ++j) partials[(size_t)blockIdx.x * N + j] = v[j];
    __threadfence();
    unsigned prev = atomicAdd(counter, 1u);
    s_last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  // The whole last block loads the partials (independent loads, one pass), then a
  // fixed-shape tree: the order of the sum depends only on the grid size.
  double acc[N];
#pragma unroll
  for (int j = 0; j < N; ++j) acc[j] = 0.0;
  for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x)
#pragma unroll
    for (int j = 0; j < N; ++j) acc[j] += __ldcg(partials + (size_t)b * N + j);
  __shared__ double shfin[N][32];
  block_sum<N>(acc, shfin);
#pragma unroll
  for (int j = 0; j < N; ++j) tot[j] = acc[j];
  if (threadIdx.x == 0) *counter = 0u;
  return threadIdx.x == 0;
}

// ------------------------------------------------------------------ CG kernels
template <typename V, typename S>
__global__ void __launch_bounds__(256) k_cg_spmv(int64_t n, const int *__restrict__ sl_ptr,
                                                 const int *__restrict__ sl_len, const int *__restrict__ col,
                                                 const V *__restrict__ val, const S *__restrict__ z,
                                                 const S *__restrict__ p, S *__restrict__ pn, S *__restrict__ q,
                                                 double *scal, int *ictl, double *partials, unsigned *counter) {
  if (ictl[I_DONE]) return;
  const S beta = (S)scal[S_BETA];
  Acc<S> prod;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    int s = (int)(i >> 5), lane = (int)(i & 31);
    int64_t base = sl_ptr[s] + lane;
    int L = sl_len[s];
    S acc = 0;
#pragma unroll 4
    for (int k = 0; k < L; ++k) {
      int c = __ldg(col + base + (int64_t)k * FG_SLICE);
      S xv = fma(beta, p[c], z[c]);
      acc = fma((S)__ldg(val + base + (int64_t)k * FG_SLICE), xv, acc);
    }
    S pi = fma(beta, p[i], z[i]);
    pn[i] = pi;
    q[i] = acc;
    prod.add(pi * acc);
  }
  double part[1];
  block_sum_acc<S, 1>(&prod, part);
  double tot[1];
  if (grid_finish<1>(part, partials, counter, tot)) {
    scal[S_PQ] = tot[0];
    scal[S_ALPHA] = (tot[0] != 0.0) ? scal[S_RZ] / tot[0] : 0.0;
  }
}

template <typename S>
__global__ void __launch_bounds__(256) k_cg_update(int64_t n, S *__restrict__ x, S *__restrict__ r,
                                                   S *__restrict__ z, const S *__restrict__ pn,
                                                   const S *__restrict__ q, const S *__restrict__ dinv,
                                                   double *scal, int *ictl, double *partials, unsigned *counter) {
  if (ictl[I_DONE]) return;
  const S alpha = (S)scal[S_ALPHA];
  Acc<S> a2[2];
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    S xi = fma(alpha, pn[i], x[i]);
    S ri = fma(-alpha, q[i], r[i]);
    S zi = dinv[i] * ri;
    x[i] = xi;
    r[i] = ri;
    z[i] = zi;
    a2[0].add(ri * zi);
    a2[1].add(ri * ri);
  }
  double part[2];
  block_sum_acc<S, 2>(a2, part);
  double tot[2];
  if (grid_finish<2>(part, partials, counter, tot)) {
    double rzo = scal[S_RZ];
    scal[S_BETA] = (rzo != 0.0) ? tot[0] / rzo : 0.0;
    scal[S_RZ] = tot[0];
    scal[S_RR] = tot[1];
    int it = ictl[I_ITERS] + 1;
    ictl[I_ITERS] = it;
    if (!isfinite(tot[1])) { ictl[I_STATUS] = 2; ictl[I_DONE] = 1; }
    else if (tot[1] <= scal[S_TOL2]) { ictl[I_STATUS] = 0; ictl[I_DONE] = 1; }
    else if (it >= ictl[I_MAXIT]) { ictl[I_STATUS] = 1; ictl[I_DONE] = 1; }
  }
}

// r = scale * rin (FP64 -> S), x = 0, z = D^-1 r, p = 0; reduces r.z and r.r and
// sets the CG scalars.  tol2_rel: stop when r.r <= tol2_rel * r0.r0.
template <typename S>
__global__ void __launch_bounds__(256) k_cg_init(int64_t n, const double *__restrict__ rin, double scale,
                                                 S *__restrict__ x, S *__restrict__ r, S *__restrict__ z,
                                                 S *__restrict__ p, const S *__restrict__ dinv, double tol2_rel,
                                                 int maxit, double *scal, int *ictl, double *partials,
                                                 unsigned *counter) {
  double rz = 0, rr = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    S ri = (S)(scale * rin[i]);
    S zi = dinv[i] * ri;
    x[i] = 0;
    r[i] = ri;
    z[i] = zi;
    p[i] = 0;
    rz += (double)ri * (double)zi;
    rr += (double)ri * (double)ri;
  }
  __shared__ double shd[2][32];
  double part[2] = {rz, rr};
  block_sum<2>(part, shd);
  double tot[2];
  if (grid_finish<2>(part, partials, counter, tot)) {
    scal[S_RZ] = tot[0];
    scal[S_RR] = tot[1];
    scal[S_BETA] = 0.0;
    scal[S_ALPHA] = 0.0;
    scal[S_TOL2] = tol2_rel * tot[1];
    ictl[I_ITERS] = 0;
    ictl[I_MAXIT] = maxit;
    ictl[I_STATUS] = 0;
    ictl[I_DONE] = (tot[1] <= scal[S_TOL2] || tot[1] == 0.0) ? 1 : 0;
  }
}

// ------------------------------------------------------------------ FP64 helpers
// y = A x (SELL FP64); with b != null computes r = b - A x; rows with fixed[i] are
// set to 0 when zero_fixed.  Reduces r.r into scal[slot] when slot >= 0.
template <typename V>
__global__ void __launch_bounds__(256) k_spmv_sell(int64_t n, const int *__restrict__ sl_ptr,
                                                   const int *__restrict__ sl_len, const int *__restrict__ col,
                                                   const V *__restrict__ val, const double *__restrict__ x,
                                                   const double *__restrict__ b, double *__restrict__ y,
                                                   const uint8_t *__restrict__ fixed, int slot, double *scal,
                                                   double *partials, unsigned *counter) {
  double rr = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    int s = (int)(i >> 5), lane = (int)(i & 31);
    int64_t base = sl_ptr[s] + lane;
    int L = sl_len[s];
    double acc = 0.0;
#pragma unroll 4
    for (int k = 0; k < L; ++k)
      acc = fma((double)__ldg(val + base + (int64_t)k * FG_SLICE), x[__ldg(col + base + (int64_t)k * FG_SLICE)], acc);
    double v = b ? b[i] - acc : acc;
    if (fixed && fixed[i]) v = 0.0;
    y[i] = v;
    rr += v * v;
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

// x += scale * d
template <typename S>
__global__ void k_axpy_to64(int64_t n, double scale, const S *__restrict__ d, double *__restrict__ x) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] += scale * (double)d[i];
}

// ------------------------------------------------------------------ host helpers
// Grid of the row-parallel reduction kernels: at most 8 blocks of 256 threads per SM,
// rows visited with a grid-stride loop, so the last block sums a few hundred partials.
static unsigned cg_grid(const fg_mesh *m) {
  unsigned g = grid_for(m->nv, 256);
  unsigned cap = 8u * (unsigned)(m->sm_count > 0 ? m->sm_count : 152);
  return g < cap ? g : cap;
}

static unsigned red_grid(int64_t n) {
  unsigned g = grid_for(n, 256);
  return g > (unsigned)FG_RED_BLOCKS ? (unsigned)FG_RED_BLOCKS : g;
}

double fg_dot_dev(fg_mesh *m, const double *x, const double *y, int64_t n, bool mask_fixed) {
  const int slot = 8;
  k_dot64<<<red_grid(n), 256, 0, m->stream>>>(n, x, y, (mask_fixed && m->has_fixed) ? m->fixed : nullptr, slot,
                                              m->scal, m->red.partials, m->red.counter);
  FG_CUDA_TRY(cudaGetLastError());
  FG_LAUNCHED(1);
  FG_CUDA_TRY(cudaMemcpyAsync(m->hbuf, m->scal + slot, sizeof(double), cudaMemcpyDeviceToHost, m->stream));
  fg_sync(m);
  return m->hbuf[0];
}

double fg_norm2_dev(fg_mesh *m, const double *x, int64_t n, bool mask_fixed) {
  return std::sqrt(fg_dot_dev(m, x, x, n, mask_fixed));
}

void fg_spmv64_dev(fg_mesh *m, const double *x, double *y) {
  FG_REQUIRE(m->val64 != nullptr, FG_BAD_ARG, "no FP64 operator assembled");
  k_spmv_sell<double><<<cg_grid(m), 256, 0, m->stream>>>(m->nv, m->sl_ptr, m->sl_len, m->sl_col, m->val64,
                                                                     x, nullptr, y, nullptr, -1, m->scal,
                                                                     m->red.partials, m->red.counter);
  FG_CUDA_TRY(cudaGetLastError());
  FG_LAUNCHED(1);
}

// CG vectors: FP64 set uses v64[0..5], FP32 set uses v32[0..5]:
// 0 x(correction), 1 r, 2 z, 3 p, 4 pn, 5 q
template <typename S>
static S **cg_vectors(fg_mesh *m);
template <>
double **cg_vectors<double>(fg_mesh *m) {
  for (int j = 0; j < 6; ++j)
    if (!m->v64[j]) m->v64[j] = dev_alloc<double>(m, (size_t)m->nv);
  return m->v64;
}
template <>
float **cg_vectors<float>(fg_mesh *m) {
  for (int j = 0; j < 6; ++j)
    if (!m->v32[j]) m->v32[j] = dev_alloc<float>(m, (size_t)m->nv);
  return m->v32;
}

template <typename V, typename S>
static void launch_iteration(fg_mesh *m, const V *val, const S *dinv, S **v, bool odd) {
  S *p = odd ? v[4] : v[3];
  S *pn = odd ? v[3] : v[4];
  unsigned g = cg_grid(m);
  k_cg_spmv<V, S><<<g, 256, 0, m->stream>>>(m->nv, m->sl_ptr, m->sl_len, m->sl_col, val, v[2], p, pn, v[5], m->scal,
                                            m->ictl, m->red.partials, m->red.counter);
  k_cg_update<S><<<g, 256, 0, m->stream>>>(m->nv, v[0], v[1], v[2], pn, v[5], dinv, m->scal, m->ictl,
                                           m->red.partials, m->red.counter);
}

// Runs inner PCG iterations until the device sets "done".  Returns iterations.
template <typename V, typename S>
static int run_cg(fg_mesh *m, const V *val, const S *dinv, const fg_solve_opts &o, int maxit, int *status) {
  S **v = cg_vectors<S>(m);
  int block = o.check_every > 0 ? o.check_every : 32;
  if (block & 1) ++block;
  int gslot = (sizeof(S) == 4 ? 1 : 0);
  GraphCache &gc = m->graph[gslot];
  const void *key[4] = {val, dinv, v[0], (const void *)(intptr_t)block};
  bool use_graph = o.use_graph != 0;
  if (use_graph) {
    bool match = gc.exec && gc.iters == block;
    for (int j = 0; j < 4 && match; ++j) match = (gc.key[j] == key[j]);
    if (!match) {
      if (gc.exec) { cudaGraphExecDestroy(gc.exec); gc.exec = nullptr; }
      cudaGraph_t graph;
      FG_CUDA_TRY(cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal));
      for (int it = 0; it < block; ++it) launch_iteration<V, S>(m, val, dinv, v, it & 1);
      FG_CUDA_TRY(cudaStreamEndCapture(m->stream, &graph));
      FG_CUDA_TRY(cudaGraphInstantiate(&gc.exec, graph, 0));
      cudaGraphDestroy(graph);
      gc.iters = block;
      for (int j = 0; j < 4; ++j) gc.key[j] = key[j];
    }
  }
  for (;;) {
    if (use_graph) {
      FG_CUDA_TRY(cudaGraphLaunch(gc.exec, m->stream));
      FG_LAUNCHED(2 * block);
    } else {
      for (int it = 0; it < block; ++it) launch_iteration<V, S>(m, val, dinv, v, it & 1);
      FG_CUDA_TRY(cudaGetLastError());
      FG_LAUNCHED(2 * block);
    }
    FG_CUDA_TRY(cudaMemcpyAsync(m->hint, m->ictl, sizeof(int) * 4, cudaMemcpyDeviceToHost, m->stream));
    fg_sync(m);
    if (m->hint[I_DONE]) break;
    (void)maxit;
  }
  if (status) *status = m->hint[I_STATUS];
  return m->hint[I_ITERS];
}

int fg_pcg_solve(fg_mesh *m, const double *d_b, double *d_x, const fg_solve_opts &o, fg_solve_stats *st,
                 bool newton_inner) {
  const bool mixed = o.precision == FG_MIXED;
  FG_REQUIRE(mixed ? m->val32 != nullptr : m->val64 != nullptr, FG_BAD_ARG, "operator not assembled");
  if (!m->v64[6]) m->v64[6] = dev_alloc<double>(m, (size_t)m->nv);
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
      rn = fg_norm2_dev(m, r64, m->nv, true);
    } else {
      FG_REQUIRE(m->val64 != nullptr, FG_BAD_ARG, "refinement needs the FP64 operator");
      k_spmv_sell<double><<<cg_grid(m), 256, 0, m->stream>>>(m->nv, m->sl_ptr, m->sl_len, m->sl_col,
                                                                         m->val64, d_x, d_b, r64, fx, 9, m->scal,
                                                                         m->red.partials, m->red.counter);
      FG_CUDA_TRY(cudaGetLastError());
      FG_LAUNCHED(1);
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
    int maxit = o.maxiter - total;
    int ist = 0, its = 0;
    unsigned g = cg_grid(m);
    if (mixed) {
      float **v = cg_vectors<float>(m);
      k_cg_init<float><<<g, 256, 0, m->stream>>>(m->nv, r64, 1.0 / rn, v[0], v[1], v[2], v[3], m->dinv32,
                                                 inner * inner, maxit, m->scal, m->ictl, m->red.partials,
                                                 m->red.counter);
      FG_CUDA_TRY(cudaGetLastError());
      its = run_cg<float, float>(m, m->val32, m->dinv32, o, maxit, &ist);
      k_axpy_to64<float><<<g, 256, 0, m->stream>>>(m->nv, rn, v[0], d_x);
    } else {
      double **v = cg_vectors<double>(m);
      k_cg_init<double><<<g, 256, 0, m->stream>>>(m->nv, r64, 1.0 / rn, v[0], v[1], v[2], v[3], m->dinv64,
                                                  inner * inner, maxit, m->scal, m->ictl, m->red.partials,
                                                  m->red.counter);
      FG_CUDA_TRY(cudaGetLastError());
      its = run_cg<double, double>(m, m->val64, m->dinv64, o, maxit, &ist);
      k_axpy_to64<double><<<g, 256, 0, m->stream>>>(m->nv, rn, v[0], d_x);
    }
    FG_CUDA_TRY(cudaGetLastError());
    FG_LAUNCHED(2);
    total += its;
    ++refinements;
    if (ist == 2) { status = 2; break; }
    if (newton_inner) { status = ist; break; }
  }
  FG_CUDA_TRY(cudaEventRecord(m->ev1, m->stream));
  fg_sync(m);
  if (st) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, m->ev0, m->ev1);
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
  o->rows_per_warp = 4;
}

// A standalone operator from a symmetric CSC matrix: a handle with the pattern and
// values but no mesh.
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
    FG_CUDA_TRY(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
    FG_CUDA_TRY(cudaEventCreate(&m->ev0));
    FG_CUDA_TRY(cudaEventCreate(&m->ev1));
    m->nv = n;
    m->nnz = nnz;
    m->nslices = (int)((n + FG_SLICE - 1) / FG_SLICE);
    std::vector<int> sl_len(m->nslices), sl_ptr(m->nslices + 1);
    int64_t acc = 0;
    for (int s = 0; s < m->nslices; ++s) {
      int mx = 1;
      for (int64_t r = (int64_t)s * FG_SLICE; r < std::min<int64_t>(n, (int64_t)(s + 1) * FG_SLICE); ++r)
        mx = std::max<int64_t>(mx, colptr[r + 1] - colptr[r]);
      sl_len[s] = mx;
      sl_ptr[s] = (int)acc;
      acc += (int64_t)mx * FG_SLICE;
      FG_REQUIRE(acc < ((int64_t)1 << 31), FG_BAD_ARG, "padded matrix too large");
    }
    sl_ptr[m->nslices] = (int)acc;
    m->nsell = acc;
    std::vector<int> col(acc);
    std::vector<double> val(acc, 0.0);
    std::vector<double> dinv(n, 0.0);
    for (int64_t r = 0; r < n; ++r) {
      int s = (int)(r / FG_SLICE), lane = (int)(r % FG_SLICE);
      int64_t b = colptr[r] - base, e = colptr[r + 1] - base;
      int k = 0;
      for (int64_t q = b; q < e; ++q, ++k) {
        int64_t c = rowval[q] - base;
        FG_REQUIRE(c >= 0 && c < n, FG_BAD_ARG, "row index out of range");
        col[sl_ptr[s] + lane + (int64_t)k * FG_SLICE] = (int)c;
        val[sl_ptr[s] + lane + (int64_t)k * FG_SLICE] = nzval[q];
        if (c == r) dinv[r] += nzval[q];
      }
      for (; k < sl_len[s]; ++k) col[sl_ptr[s] + lane + (int64_t)k * FG_SLICE] = (int)r;
      dinv[r] = dinv[r] != 0.0 ? 1.0 / dinv[r] : 0.0;
    }
    m->sl_ptr = dev_alloc<int>(m, (size_t)m->nslices + 1);
    m->sl_len = dev_alloc<int>(m, (size_t)m->nslices);
    m->sl_col = dev_alloc<int>(m, (size_t)acc);
    m->val64 = dev_alloc<double>(m, (size_t)acc);
    m->dinv64 = dev_alloc<double>(m, (size_t)n);
    FG_CUDA_TRY(cudaMemcpyAsync(m->sl_ptr, sl_ptr.data(), sizeof(int) * (m->nslices + 1), cudaMemcpyHostToDevice, m->stream));
    FG_CUDA_TRY(cudaMemcpyAsync(m->sl_len, sl_len.data(), sizeof(int) * m->nslices, cudaMemcpyHostToDevice, m->stream));
    FG_CUDA_TRY(cudaMemcpyAsync(m->sl_col, col.data(), sizeof(int) * acc, cudaMemcpyHostToDevice, m->stream));
    FG_CUDA_TRY(cudaMemcpyAsync(m->val64, val.data(), sizeof(double) * acc, cudaMemcpyHostToDevice, m->stream));
    FG_CUDA_TRY(cudaMemcpyAsync(m->dinv64, dinv.data(), sizeof(double) * n, cudaMemcpyHostToDevice, m->stream));
    if (want32) {
      std::vector<float> v32(val.begin(), val.end()), d32(dinv.begin(), dinv.end());
      m->val32 = dev_alloc<float>(m, (size_t)acc);
      m->dinv32 = dev_alloc<float>(m, (size_t)n);
      FG_CUDA_TRY(cudaMemcpyAsync(m->val32, v32.data(), sizeof(float) * acc, cudaMemcpyHostToDevice, m->stream));
      FG_CUDA_TRY(cudaMemcpyAsync(m->dinv32, d32.data(), sizeof(float) * n, cudaMemcpyHostToDevice, m->stream));
    }
    m->red.partials = dev_alloc<double>(m, ((size_t)grid_for(n, 256) + FG_RED_BLOCKS) * 4);
    m->red.counter = dev_alloc<unsigned int>(m, 16);
    FG_CUDA_TRY(cudaMemsetAsync(m->red.counter, 0, 16 * sizeof(unsigned int), m->stream));
    m->scal = dev_alloc<double>(m, S_NSCAL);
    m->ictl = dev_alloc<int>(m, I_NINT);
    m->flags = dev_alloc<int>(m, 4);
    FG_CUDA_TRY(cudaMemsetAsync(m->flags, 0, 4 * sizeof(int), m->stream));
    FG_CUDA_TRY(cudaMallocHost(&m->hbuf, 64 * sizeof(double)));
    FG_CUDA_TRY(cudaMallocHost(&m->hint, 16 * sizeof(int)));
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

__global__ void k_fill64(int64_t n, double v, double *__restrict__ x) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] = v;
}

// Average duration of one CG kernel launch on the handle's current operator
// (events on the handle's stream).  Leaves the CG vectors in an unspecified state.
fg_status fg_bench_cg_kernel(fg_mesh *m, int which, int precision, int reps, double *ms_per_launch) {
  const bool mixed = precision == FG_MIXED;
  FG_REQUIRE(mixed ? m->val32 != nullptr : m->val64 != nullptr, FG_BAD_ARG, "operator not assembled");
  unsigned g = cg_grid(m);
  if (!m->v64[6]) m->v64[6] = dev_alloc<double>(m, (size_t)m->nv);
  k_fill64<<<g, 256, 0, m->stream>>>(m->nv, 1.0, m->v64[6]);
  auto body = [&](int n) {
    for (int r = 0; r < n; ++r) {
      if (mixed) {
        float **v = cg_vectors<float>(m);
        if (which == 0)
          k_cg_spmv<float, float><<<g, 256, 0, m->stream>>>(m->nv, m->sl_ptr, m->sl_len, m->sl_col, m->val32, v[2],
                                                            v[3], v[4], v[5], m->scal, m->ictl, m->red.partials,
                                                            m->red.counter);
        else
          k_cg_update<float><<<g, 256, 0, m->stream>>>(m->nv, v[0], v[1], v[2], v[4], v[5], m->dinv32, m->scal,
                                                       m->ictl, m->red.partials, m->red.counter);
      } else {
        double **v = cg_vectors<double>(m);
        if (which == 0)
          k_cg_spmv<double, double><<<g, 256, 0, m->stream>>>(m->nv, m->sl_ptr, m->sl_len, m->sl_col, m->val64,
                                                              v[2], v[3], v[4], v[5], m->scal, m->ictl,
                                                              m->red.partials, m->red.counter);
        else
          k_cg_update<double><<<g, 256, 0, m->stream>>>(m->nv, v[0], v[1], v[2], v[4], v[5], m->dinv64, m->scal,
                                                        m->ictl, m->red.partials, m->red.counter);
      }
    }
    FG_LAUNCHED(n);
  };
  // a CG state that never reports "done": zero vectors, huge iteration cap
  if (mixed) {
    float **v = cg_vectors<float>(m);
    k_cg_init<float><<<g, 256, 0, m->stream>>>(m->nv, m->v64[6], 1.0, v[0], v[1], v[2], v[3], m->dinv32, 0.0,
                                               1 << 30, m->scal, m->ictl, m->red.partials, m->red.counter);
  } else {
    double **v = cg_vectors<double>(m);
    k_cg_init<double><<<g, 256, 0, m->stream>>>(m->nv, m->v64[6], 1.0, v[0], v[1], v[2], v[3], m->dinv64, 0.0,
                                                1 << 30, m->scal, m->ictl, m->red.partials, m->red.counter);
  }
  FG_CUDA_TRY(cudaMemsetAsync(m->ictl, 0, sizeof(int), m->stream));  // clear "done"
  FG_LAUNCHED(1);
  body(3);
  FG_CUDA_TRY(cudaEventRecord(m->ev0, m->stream));
  body(reps);
  FG_CUDA_TRY(cudaEventRecord(m->ev1, m->stream));
  FG_CUDA_TRY(cudaGetLastError());
  fg_sync(m);
  float ms = 0.f;
  FG_CUDA_TRY(cudaEventElapsedTime(&ms, m->ev0, m->ev1));
  *ms_per_launch = ms / reps;
  return FG_OK;
}
