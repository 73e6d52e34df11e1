// A sweep of applied fields on one linear mesh (the hysteresis-loop use of
// Magnetostatics/magneticField.jl:89-132: K(mu) u = 0 on free rows, u = -H0.x on the
// Dirichlet rows, one solve per field) as ONE multi-right-hand-side CG: every
// iteration reads the matrix once for all fields.  Vectors are row-major blocks
// [row][field] (NR fields per row, NR a multiple of 32); one warp handles one row,
// lane l the fields l, l + 32, ...  Each field keeps its own CG scalars (the fields
// are independent systems that share the matrix), so a field whose right-hand side
// is a combination of others is not a breakdown.
// Precision: FP32 matrix and inner CG, FP64 outer residual and solution (iterative
// refinement), FP64 accumulation of every dot product.
#include <algorithm>
#include <cmath>
#include <vector>

#include "fg_common.cuh"

namespace {

constexpr int SW_THREADS = 256;              // 8 warps = 8 rows per pass
constexpr int SW_WARPS = SW_THREADS / 32;

struct SwOp {
  int64_t n;
  const int *sl_ptr, *sl_len, *sl_col;
  const uint8_t *fixed;
};

// Entries of row i: slot q of the row is loaded by lane q (q < 4 G) and broadcast.
template <class V>
__device__ __forceinline__ void row_slot(const SwOp &A, const V *val, int64_t i, int lane, int &G, V &v, int &c) {
  const int s = (int)(i >> 5);
  G = A.sl_len[s];
  v = V(0);
  c = (int)i;
  if (lane < FG_GROUP * G) {
    const int64_t e = sell_pos(A.sl_ptr[s], (int)(i & 31), lane);
    v = val[e];
    c = A.sl_col[e];
  }
}

// Per-field partial sums of a warp, reduced over the block into partials[block][NR].
template <int J>
__device__ __forceinline__ void block_fields_sum(double (&acc)[J], double *sh, double *partials, int NR) {
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
  for (int j = 0; j < J; ++j) sh[w * NR + l + 32 * j] = acc[j];
  __syncthreads();
  for (int c = threadIdx.x; c < NR; c += SW_THREADS) {
    double t = 0.0;
    for (int k = 0; k < SW_WARPS; ++k) t += sh[k * NR + c];
    partials[(int64_t)blockIdx.x * NR + c] = t;
  }
}

// R = -A X on free rows (FP64), per-field r.r partials.
template <int J>
__global__ void __launch_bounds__(SW_THREADS) k_sw_resid64(SwOp A, const double *__restrict__ val,
                                                           const double *__restrict__ X, double *__restrict__ R,
                                                           double *partials) {
  extern __shared__ double sw_sh[];
  constexpr int NR = 32 * J;
  const int lane = threadIdx.x & 31;
  double acc2[J];
#pragma unroll
  for (int j = 0; j < J; ++j) acc2[j] = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * SW_WARPS + (threadIdx.x >> 5); i < A.n; i += (int64_t)gridDim.x * SW_WARPS) {
    int G, c;
    double v;
    row_slot(A, val, i, lane, G, v, c);
    double y[J];
#pragma unroll
    for (int j = 0; j < J; ++j) y[j] = 0.0;
    const bool fx = A.fixed && A.fixed[i];
    if (!fx)
      for (int q = 0; q < FG_GROUP * G; ++q) {
        const double vq = __shfl_sync(0xffffffffu, v, q);
        const int cq = __shfl_sync(0xffffffffu, c, q);
        const double *xr = X + (int64_t)cq * NR + lane;
#pragma unroll
        for (int j = 0; j < J; ++j) y[j] = fma(vq, xr[32 * j], y[j]);
      }
    double *rr = R + i * NR + lane;
#pragma unroll
    for (int j = 0; j < J; ++j) {
      const double r = fx ? 0.0 : -y[j];
      rr[32 * j] = r;
      acc2[j] = fma(r, r, acc2[j]);
    }
  }
  block_fields_sum<J>(acc2, sw_sh, partials, NR);
}

// Sum of the block partials per field: out[c] = sum_b partials[b][c] (threads: 8
// partial lanes x 32 fields per block).
__global__ void k_sw_fieldsum(const double *__restrict__ partials, int nblocks, int NR, double *__restrict__ out) {
  __shared__ double sh[8][33];
  const int c = blockIdx.x * 32 + (threadIdx.x & 31), part = threadIdx.x >> 5;
  double t = 0.0;
  if (c < NR) {
    // four independent partial sums per thread keep four loads in flight
    double t4[4] = {0.0, 0.0, 0.0, 0.0};
    int b = part;
    for (; b + 24 < nblocks; b += 32)
#pragma unroll
      for (int k = 0; k < 4; ++k) t4[k] += partials[(int64_t)(b + 8 * k) * NR + c];
    for (; b < nblocks; b += 8) t4[0] += partials[(int64_t)b * NR + c];
    t = (t4[0] + t4[1]) + (t4[2] + t4[3]);
  }
  sh[part][threadIdx.x & 31] = t;
  __syncthreads();
  if (part == 0 && c < NR) {
    double s = 0.0;
    for (int k = 0; k < 8; ++k) s += sh[k][threadIdx.x & 31];
    out[c] = s;
  }
}

// Start of an inner solve: r = R64 / |R64| per field (FP32), p = x = 0, and the
// per-field partials of r.z with z = D^-1 r.
template <int J>
__global__ void __launch_bounds__(SW_THREADS) k_sw_init32(int64_t n, const double *__restrict__ R,
                                                          const double *__restrict__ rnorm,
                                                          const float *__restrict__ dinv, float *__restrict__ r,
                                                          float *__restrict__ p, float *__restrict__ x,
                                                          double *partials) {
  extern __shared__ double sw_sh[];
  constexpr int NR = 32 * J;
  const int lane = threadIdx.x & 31;
  double inv[J], acc[J];
#pragma unroll
  for (int j = 0; j < J; ++j) {
    const double rn = rnorm[lane + 32 * j];
    inv[j] = rn > 0.0 ? 1.0 / rn : 0.0;
    acc[j] = 0.0;
  }
  for (int64_t i = (int64_t)blockIdx.x * SW_WARPS + (threadIdx.x >> 5); i < n; i += (int64_t)gridDim.x * SW_WARPS) {
    const float d = dinv[i];
#pragma unroll
    for (int j = 0; j < J; ++j) {
      const int64_t e = i * NR + lane + 32 * j;
      const float ri = (float)(R[e] * inv[j]);
      r[e] = ri;
      p[e] = 0.f;
      x[e] = 0.f;
      acc[j] += (double)(ri * (d * ri));
    }
  }
  block_fields_sum<J>(acc, sw_sh, partials, NR);
}

// p_new = z + beta p (z = D^-1 r), q = A p_new with neighbours formed on the fly,
// per-field p.q partials.  Fixed rows stay 0.
template <int J>
__global__ void __launch_bounds__(SW_THREADS) k_sw_spmm32(SwOp A, const float *__restrict__ val,
                                                          const float *__restrict__ dinv,
                                                          const float *__restrict__ r, const float *__restrict__ pold,
                                                          float *__restrict__ pnew, float *__restrict__ q,
                                                          const float *__restrict__ beta, double *partials) {
  extern __shared__ double sw_sh[];
  constexpr int NR = 32 * J;
  const int lane = threadIdx.x & 31;
  float b[J];
  double acc[J];
#pragma unroll
  for (int j = 0; j < J; ++j) {
    b[j] = beta[lane + 32 * j];
    acc[j] = 0.0;
  }
  for (int64_t i = (int64_t)blockIdx.x * SW_WARPS + (threadIdx.x >> 5); i < A.n; i += (int64_t)gridDim.x * SW_WARPS) {
    int G, c;
    float v;
    row_slot(A, val, i, lane, G, v, c);
    float y[J];
#pragma unroll
    for (int j = 0; j < J; ++j) y[j] = 0.f;
    const bool fx = A.fixed && A.fixed[i];
    if (!fx)
      for (int qq = 0; qq < FG_GROUP * G; ++qq) {
        const float vq = __shfl_sync(0xffffffffu, v, qq);
        const int cq = __shfl_sync(0xffffffffu, c, qq);
        const float dq = dinv[cq];
        const float *rr = r + (int64_t)cq * NR + lane;
        const float *pp = pold + (int64_t)cq * NR + lane;
#pragma unroll
        for (int j = 0; j < J; ++j) y[j] = fmaf(vq, fmaf(b[j], pp[32 * j], dq * rr[32 * j]), y[j]);
      }
    const float di = dinv[i];
#pragma unroll
    for (int j = 0; j < J; ++j) {
      const int64_t e = i * NR + lane + 32 * j;
      const float pn = fx ? 0.f : fmaf(b[j], pold[e], di * r[e]);
      pnew[e] = pn;
      q[e] = y[j];
      acc[j] += (double)(pn * y[j]);
    }
  }
  block_fields_sum<J>(acc, sw_sh, partials, NR);
}

// x += alpha p, r -= alpha q; per-field partials of r.z (z = D^-1 r) and r.r.
template <int J>
__global__ void __launch_bounds__(SW_THREADS) k_sw_update32(int64_t n, const float *__restrict__ dinv,
                                                            const float *__restrict__ alpha,
                                                            const float *__restrict__ p, const float *__restrict__ q,
                                                            float *__restrict__ r, float *__restrict__ x,
                                                            double *partials) {
  extern __shared__ double sw_sh[];
  constexpr int NR = 32 * J;
  const int lane = threadIdx.x & 31;
  float a[J];
  double acc[J], acc2[J];
#pragma unroll
  for (int j = 0; j < J; ++j) {
    a[j] = alpha[lane + 32 * j];
    acc[j] = 0.0;
    acc2[j] = 0.0;
  }
  for (int64_t i = (int64_t)blockIdx.x * SW_WARPS + (threadIdx.x >> 5); i < n; i += (int64_t)gridDim.x * SW_WARPS) {
    const float d = dinv[i];
#pragma unroll
    for (int j = 0; j < J; ++j) {
      const int64_t e = i * NR + lane + 32 * j;
      x[e] = fmaf(a[j], p[e], x[e]);
      const float ri = fmaf(-a[j], q[e], r[e]);
      r[e] = ri;
      acc[j] += (double)(ri * (d * ri));
      acc2[j] += (double)(ri * ri);
    }
  }
  block_fields_sum<J>(acc, sw_sh, partials, NR);
  __syncthreads();
  block_fields_sum<J>(acc2, sw_sh, partials + (int64_t)gridDim.x * NR, NR);
}

// Per-field CG scalars.  S holds, per field c: [0] r.z, [1] target r.r, [2] r.r;
// alpha/beta (FP32) feed the next kernels; active[c] = 1 while the field iterates.
// mode 0: after the start (r.z from `sum`); 1: alpha from p.q; 2: beta and
// convergence from r.z (sum) and r.r (sum2).  count[0] receives the active fields.
__global__ void k_sw_scalars(int mode, int NR, int nfield, const double *__restrict__ sum,
                             const double *__restrict__ sum2, double tol2_rel, double *S, float *alpha, float *beta,
                             int *active, int *count) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= NR) return;
  double *s = S + 3 * c;
  if (mode == 0) {
    const double rz = sum[c];
    s[0] = rz;
    s[1] = tol2_rel;  // |r0| = 1 after scaling
    s[2] = 1.0;
    beta[c] = 0.f;
    alpha[c] = 0.f;
    active[c] = (c < nfield && rz > 0.0) ? 1 : 0;
  } else if (mode == 1) {
    const double pq = sum[c];
    const bool on = active[c] && pq > 0.0 && isfinite(pq);
    alpha[c] = on ? (float)(s[0] / pq) : 0.f;
    if (active[c] && !(pq > 0.0 && isfinite(pq))) active[c] = 0;
  } else {
    const double rz = sum[c], rr = sum2[c];
    if (active[c]) {
      s[2] = rr;
      if (!isfinite(rr) || rr <= s[1]) {
        active[c] = 0;
        beta[c] = 0.f;
      } else {
        beta[c] = (float)(rz / s[0]);
        s[0] = rz;
      }
    }
  }
  __syncthreads();
  if (mode != 1 && c == 0) {
    int a = 0;
    for (int k = 0; k < NR; ++k) a += active[k];
    *count = a;
  }
}

// X64 += |R64| x32 per field (the refinement update) on free rows.
template <int J>
__global__ void k_sw_accumulate(int64_t n, const double *__restrict__ rnorm, const float *__restrict__ x,
                                double *__restrict__ X) {
  constexpr int NR = 32 * J;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * NR) return;
  X[e] = fma(rnorm[e % NR], (double)x[e], X[e]);
}

// Initial guess and Dirichlet values: X[i][c] = -H0_c . p_i.
__global__ void k_sw_lift(int64_t n, int NR, int nfield, const double *__restrict__ p, const double *__restrict__ H0,
                          double *__restrict__ X) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * NR) return;
  const int64_t i = e / NR;
  const int c = (int)(e % NR);
  double v = 0.0;
  if (c < nfield)
    v = -(H0[3 * c] * p[3 * i] + H0[3 * c + 1] * p[3 * i + 1] + H0[3 * c + 2] * p[3 * i + 2]);
  X[e] = v;
}

// Transposes one field out of the row-major block into a column-major nv x nfield
// array (the layout of a Julia Matrix{Float64}).
__global__ void k_sw_extract(int64_t n, int NR, int nfield, const double *__restrict__ X, double *__restrict__ U) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * (int64_t)nfield) return;
  const int c = (int)(e / n);
  const int64_t i = e % n;
  U[e] = X[i * NR + c];
}

}  // namespace

// fg_blockcg.cu: the rank-revealing block-CG form of the sweep
fg_status fg_sweep_block(fg_mesh *m, int nfield, const double *H0, const fg_solve_opts &o, double *U,
                         fg_solve_stats *s);

template <int J>
static fg_status sweep_impl(fg_mesh *m, int nfield, const double *H0, const fg_solve_opts &o, double *U,
                            fg_solve_stats *s) {
  constexpr int NR = 32 * J;
  const int64_t n = m->nv;
  const size_t blk = (size_t)n * NR;
  // work space from the stream-ordered pool, released on the stream at the end of the call
  cudaStream_t st = m->stream;
  StreamScratch scratch{st, {}};
  auto alloc = [&](size_t bytes) {
    return static_cast<void *>(scratch.get<unsigned char>(std::max<size_t>(bytes, 16)));
  };
  const int nblocks = std::max(1, std::min<int>(m->sm_count * 8, (int)((n + SW_WARPS - 1) / SW_WARPS)));
  double *X = (double *)alloc(sizeof(double) * blk), *R = (double *)alloc(sizeof(double) * blk);
  float *r = (float *)alloc(sizeof(float) * blk), *p0 = (float *)alloc(sizeof(float) * blk);
  float *p1 = (float *)alloc(sizeof(float) * blk), *q = (float *)alloc(sizeof(float) * blk);
  float *x = (float *)alloc(sizeof(float) * blk);
  double *part = (double *)alloc(sizeof(double) * 2 * nblocks * NR);
  double *sum = (double *)alloc(sizeof(double) * NR), *sum2 = (double *)alloc(sizeof(double) * NR);
  double *rnorm = (double *)alloc(sizeof(double) * NR), *S = (double *)alloc(sizeof(double) * 3 * NR);
  float *alpha = (float *)alloc(sizeof(float) * NR), *beta = (float *)alloc(sizeof(float) * NR);
  int *active = (int *)alloc(sizeof(int) * NR), *count = (int *)alloc(sizeof(int));
  double *dH0 = (double *)alloc(sizeof(double) * 3 * nfield);
  FG_CUDA_TRY(cudaMemcpyAsync(dH0, H0, sizeof(double) * 3 * nfield, cudaMemcpyHostToDevice, st));
  const SwOp A{n, m->sl_ptr, m->sl_len, m->sl_col, m->has_fixed ? m->fixed : nullptr};
  const size_t smem = sizeof(double) * SW_WARPS * NR;
  auto setsmem = [&](auto kern) {
    if (smem > 48 * 1024)
      FG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  };
  setsmem(k_sw_resid64<J>);
  setsmem(k_sw_init32<J>);
  setsmem(k_sw_spmm32<J>);
  setsmem(k_sw_update32<J>);
  const unsigned eg = (unsigned)((blk + 255) / 256);
  const unsigned fg = (unsigned)((NR + 31) / 32);
  cudaEvent_t e0, e1;
  FG_CUDA_TRY(cudaEventCreate(&e0));
  FG_CUDA_TRY(cudaEventCreate(&e1));
  FG_CUDA_TRY(cudaEventRecord(e0, st));
  k_sw_lift<<<eg, 256, 0, st>>>(n, NR, nfield, m->p, dH0, X);
  FG_LAUNCHED(1);
  std::vector<double> hr(NR), hr0(NR);
  int total = 0, refinements = 0;
  bool all_done = false;
  const int check = std::max(2, o.check_every);
  for (int ref = 0; ref < 50 && !all_done; ++ref) {
    // FP64 residual and its norm per field
    k_sw_resid64<J><<<nblocks, SW_THREADS, smem, st>>>(A, m->val64, X, R, part);
    k_sw_fieldsum<<<fg, 256, 0, st>>>(part, nblocks, NR, sum);
    FG_LAUNCHED(2);
    FG_CUDA_TRY(cudaMemcpyAsync(hr.data(), sum, sizeof(double) * NR, cudaMemcpyDeviceToHost, st));
    FG_CUDA_TRY(cudaStreamSynchronize(st));
    all_done = true;
    double worst_rel = 0.0;
    for (int c = 0; c < NR; ++c) {
      hr[c] = std::sqrt(hr[c]);
      if (ref == 0) hr0[c] = hr[c];
      if (c < nfield && hr[c] > o.rtol * hr0[c] && hr[c] > 0.0) {
        all_done = false;
        worst_rel = std::max(worst_rel, hr[c] / hr0[c]);
      }
    }
    if (all_done || total >= o.maxiter) break;
    // fields already at the target get |R| = 0: their inner solve is idle
    for (int c = 0; c < NR; ++c)
      if (c >= nfield || hr[c] <= o.rtol * hr0[c]) hr[c] = 0.0;
    FG_CUDA_TRY(cudaMemcpyAsync(rnorm, hr.data(), sizeof(double) * NR, cudaMemcpyHostToDevice, st));
    const double inner = std::max(o.inner_rtol, o.rtol / std::max(worst_rel, 1e-300));
    k_sw_init32<J><<<nblocks, SW_THREADS, smem, st>>>(n, R, rnorm, m->dinv32, r, p0, x, part);
    k_sw_fieldsum<<<fg, 256, 0, st>>>(part, nblocks, NR, sum);
    k_sw_scalars<<<1, NR, 0, st>>>(0, NR, nfield, sum, nullptr, inner * inner, S, alpha, beta, active, count);
    FG_LAUNCHED(3);
    float *pold = p0, *pnew = p1;
    int it = 0, hc = 1;
    while (hc > 0 && total + it < o.maxiter) {
      for (int k = 0; k < check; ++k) {
        k_sw_spmm32<J><<<nblocks, SW_THREADS, smem, st>>>(A, m->val32, m->dinv32, r, pold, pnew, q, beta, part);
        k_sw_fieldsum<<<fg, 256, 0, st>>>(part, nblocks, NR, sum);
        k_sw_scalars<<<1, NR, 0, st>>>(1, NR, nfield, sum, nullptr, 0.0, S, alpha, beta, active, count);
        k_sw_update32<J><<<nblocks, SW_THREADS, smem, st>>>(n, m->dinv32, alpha, pnew, q, r, x, part);
        k_sw_fieldsum<<<fg, 256, 0, st>>>(part, nblocks, NR, sum);
        k_sw_fieldsum<<<fg, 256, 0, st>>>(part + (size_t)nblocks * NR, nblocks, NR, sum2);
        k_sw_scalars<<<1, NR, 0, st>>>(2, NR, nfield, sum, sum2, 0.0, S, alpha, beta, active, count);
        std::swap(pold, pnew);
      }
      FG_LAUNCHED(7LL * check);
      it += check;
      FG_CUDA_TRY(cudaGetLastError());
      FG_CUDA_TRY(cudaMemcpyAsync(m->hint, count, sizeof(int), cudaMemcpyDeviceToHost, st));
      FG_CUDA_TRY(cudaStreamSynchronize(st));
      hc = m->hint[0];
    }
    total += it;
    ++refinements;
    k_sw_accumulate<J><<<eg, 256, 0, st>>>(n, rnorm, x, X);
    FG_LAUNCHED(1);
  }
  FG_CUDA_TRY(cudaEventRecord(e1, st));
  if (U) {
    double *dU = (double *)alloc(sizeof(double) * (size_t)n * nfield);
    k_sw_extract<<<(unsigned)(((size_t)n * nfield + 255) / 256), 256, 0, st>>>(n, NR, nfield, X, dU);
    FG_LAUNCHED(1);
    FG_CUDA_TRY(cudaMemcpyAsync(U, dU, sizeof(double) * (size_t)n * nfield, cudaMemcpyDeviceToHost, st));
  }
  FG_CUDA_TRY(cudaStreamSynchronize(st));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  double worst = 0.0;
  for (int c = 0; c < nfield; ++c)
    if (hr0[c] > 0.0) worst = std::max(worst, hr[c] / hr0[c]);
  if (s) {
    s->iterations = total;
    s->refinements = refinements;
    s->converged = all_done ? 1 : 0;
    s->pad_ = 0;
    s->relres = worst;
    s->ms = ms;
  }
  return all_done ? FG_OK : FG_NOT_CONVERGED;
}

extern "C" fg_status fg_magnetostatics_sweep(fg_mesh *m, const double *mu, int32_t nfield, const double *H0,
                                             const fg_solve_opts *o, double *U, fg_solve_stats *s) {
  return fg_guard([&]() -> fg_status {
    FG_REQUIRE(m && mu && H0 && nfield > 0, FG_BAD_ARG, "fg_magnetostatics_sweep: bad arguments");
    FG_REQUIRE(m->npe == 4 || m->npe == 3, FG_UNSUPPORTED, "fg_magnetostatics_sweep: P1 elements only");
    fg_solve_opts opts;
    fg_solve_opts_default(&opts);
    if (o) opts = *o;
    FG_REQUIRE(opts.precision == FG_MIXED, FG_UNSUPPORTED, "fg_magnetostatics_sweep: FG_MIXED only");
    FG_REQUIRE(opts.spmv == FG_SWEEP_BLOCK || opts.spmv == FG_SWEEP_PER_FIELD, FG_BAD_ARG,
               "fg_magnetostatics_sweep: o->spmv selects FG_SWEEP_BLOCK (0) or FG_SWEEP_PER_FIELD (1)");
    const bool block = opts.spmv == FG_SWEEP_BLOCK;
    FG_REQUIRE(block || nfield <= 256, FG_BAD_ARG, "fg_magnetostatics_sweep: at most 256 fields per call per field");
    FG_REQUIRE(block || m->maxrow4 <= 32, FG_UNSUPPORTED, "fg_magnetostatics_sweep: rows longer than 32 entries");
    if (!m->mu_lin) m->mu_lin = dev_alloc<double>(m, (size_t)m->nt);
    FG_CUDA_TRY(cudaMemcpyAsync(m->mu_lin, mu, sizeof(double) * (size_t)m->nt, cudaMemcpyHostToDevice, m->stream));
    fg_assemble_operator(m, ASM_STIFF, m->mu_lin, nullptr, nullptr, 0.0, 0.0, 0, OUT_SELL, true, true, true);
    if (block) return fg_sweep_block(m, nfield, H0, opts, U, s);
    const int J = (nfield + 31) / 32;
    switch (J) {
      case 1: return sweep_impl<1>(m, nfield, H0, opts, U, s);
      case 2: return sweep_impl<2>(m, nfield, H0, opts, U, s);
      case 3:
      case 4: return sweep_impl<4>(m, nfield, H0, opts, U, s);
      default: return sweep_impl<8>(m, nfield, H0, opts, U, s);
    }
  });
}
