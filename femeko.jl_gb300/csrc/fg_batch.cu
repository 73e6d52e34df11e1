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
#include <vector>

#include "fg_common.cuh"

namespace cgrp = cooperative_groups;

// Threads per CTA (1024-thread CTAs spilled registers: 64 per thread at most)
constexpr int FG_BATCH_THREADS = 512;

struct BatchProb {
  int64_t n;
  int nslices;
  const int *sl_ptr, *sl_len, *sl_col;
  const double *val, *dinv;
  const uint8_t *fixed;  // may be null
  double *x, *r, *z, *p0, *p1, *q;
  double tol2_rel;
  int maxit;
  int *iters;       // out: iterations
  double *relres;   // out: ||r|| / ||r0||
  int *status;      // out: 0 converged, 1 cap, 2 non-finite / breakdown
};

// Block sum of two values, then the cluster-wide sum of the CTAs' block sums (read
// from every CTA's shared slot in rank order).  slot alternates between calls so a
// slot is rewritten only after the next cluster barrier.
template <int CL>
__device__ __forceinline__ void cluster_sum2(cgrp::cluster_group &cl, double a, double b, double (*slot)[2],
                                             int which, double &ta, double &tb) {
  __shared__ double wsum[2][FG_BATCH_THREADS / 32];
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) { wsum[0][w] = a; wsum[1][w] = b; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double sa = 0.0, sb = 0.0;
    for (int k = 0; k < FG_BATCH_THREADS / 32; ++k) { sa += wsum[0][k]; sb += wsum[1][k]; }
    slot[which][0] = sa;
    slot[which][1] = sb;
    __threadfence();  // this CTA's global vector writes before the cluster barrier
  }
  __threadfence();
  cl.sync();
  double sa = 0.0, sb = 0.0;
#pragma unroll 4
  for (int rank = 0; rank < CL; ++rank) {
    const double *remote = cl.map_shared_rank(&slot[which][0], rank);
    sa += remote[0];
    sb += remote[1];
  }
  ta = sa;
  tb = sb;
}

template <int CL>
__global__ void __launch_bounds__(FG_BATCH_THREADS, 2) k_batch_pcg64(const BatchProb *__restrict__ probs) {
  cgrp::cluster_group cl = cgrp::this_cluster();
  __shared__ double slot[2][2];
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
  double *x = pp->x, *r = pp->r, *z = pp->z, *q = pp->q;
  double *pold = pp->p0, *pnew = pp->p1;
  // this CTA's rows: a contiguous run of whole slices
  const int per = (nslices + CL - 1) / CL;
  const int s0 = min(rank * per, nslices), s1 = min(s0 + per, nslices);
  const int64_t i0 = (int64_t)s0 * FG_SLICE, i1 = min((int64_t)s1 * FG_SLICE, n);
  // r = -A x on free rows (the right-hand side is 0), z = D^-1 r, p = 0
  double prz = 0.0, prr = 0.0;
  for (int64_t i = i0 + threadIdx.x; i < i1; i += FG_BATCH_THREADS) {
    double ri = 0.0;
    if (!(fixed && fixed[i])) {
      const int s = (int)(i >> 5);
      const int64_t base = (int64_t)sl_ptr[s] + (i & 31) * FG_GROUP;
      const int G = sl_len[s];
      double acc = 0.0;
      for (int g = 0; g < G; ++g) {
        const int64_t e = base + (int64_t)g * FG_SLICE * FG_GROUP;
#pragma unroll
        for (int c = 0; c < FG_GROUP; ++c) acc = fma(val[e + c], x[sl_col[e + c]], acc);
      }
      ri = -acc;
    }
    const double zi = dinv[i] * ri;
    r[i] = ri;
    z[i] = zi;
    pold[i] = 0.0;
    pnew[i] = 0.0;
    prz += ri * zi;
    prr += ri * ri;
  }
  int which = 0;
  double rz, rr;
  cluster_sum2<CL>(cl, prz, prr, slot, which, rz, rr);
  which ^= 1;
  const double rr0 = rr, tol2 = pp->tol2_rel * rr0;
  const int maxit = pp->maxit;
  int it = 0, status = (rr0 == 0.0) ? 0 : -1;
  if (!isfinite(rr0)) status = 2;
  double beta = 0.0;
  while (status < 0) {
    if (it >= maxit) { status = 1; break; }
    // p_new = z + beta p_old; q = A p_new (neighbours formed from z and p_old); p.q
    double ppq = 0.0;
    for (int64_t i = i0 + threadIdx.x; i < i1; i += FG_BATCH_THREADS) {
      double qi = 0.0, pi = 0.0;
      if (!(fixed && fixed[i])) {
        const int s = (int)(i >> 5);
        const int64_t base = (int64_t)sl_ptr[s] + (i & 31) * FG_GROUP;
        const int G = sl_len[s];
        for (int g = 0; g < G; ++g) {
          const int64_t e = base + (int64_t)g * FG_SLICE * FG_GROUP;
#pragma unroll
          for (int c = 0; c < FG_GROUP; ++c) {
            const int j = sl_col[e + c];
            qi = fma(val[e + c], fma(beta, pold[j], z[j]), qi);
          }
        }
        pi = fma(beta, pold[i], z[i]);
      }
      pnew[i] = pi;
      q[i] = qi;
      ppq += pi * qi;
    }
    double pq, unused;
    cluster_sum2<CL>(cl, ppq, 0.0, slot, which, pq, unused);
    which ^= 1;
    if (!(pq > 0.0) || !isfinite(pq)) { status = (pq == 0.0) ? 0 : 2; break; }
    const double alpha = rz / pq;
    // x += alpha p; r -= alpha q; z = D^-1 r
    prz = 0.0;
    prr = 0.0;
    for (int64_t i = i0 + threadIdx.x; i < i1; i += FG_BATCH_THREADS) {
      x[i] = fma(alpha, pnew[i], x[i]);
      const double ri = fma(-alpha, q[i], r[i]);
      const double zi = dinv[i] * ri;
      r[i] = ri;
      z[i] = zi;
      prz += ri * zi;
      prr += ri * ri;
    }
    double rzn;
    cluster_sum2<CL>(cl, prz, prr, slot, which, rzn, rr);
    which ^= 1;
    ++it;
    if (!isfinite(rr)) { status = 2; break; }
    if (rr <= tol2) { status = 0; break; }
    beta = rzn / rz;
    rz = rzn;
    double *t = pold;
    pold = pnew;
    pnew = t;
  }
  if (rank == 0 && threadIdx.x == 0) {
    *pp->iters = it;
    *pp->relres = rr0 > 0.0 ? sqrt(rr / rr0) : 0.0;
    *pp->status = status;
  }
  cl.sync();  // no CTA leaves while another may still read its shared slots
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
    FG_REQUIRE(opts.precision == FG_FP64, FG_UNSUPPORTED, "fg_batch_magnetostatics_linear: FP64 only");
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
      fg_assemble_operator(m, ASM_STIFF, m->mu_lin, nullptr, nullptr, 0.0, 0.0, 0, OUT_SELL, true, false, true);
      for (int j : {7, 0, 1, 2, 3, 4, 5})
        if (!m->v64[j]) m->v64[j] = dev_alloc<double>(m, (size_t)m->nvp);
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
      b.fixed = m->has_fixed ? m->fixed : nullptr;
      b.x = m->v64[7];
      b.r = m->v64[0];
      b.z = m->v64[1];
      b.p0 = m->v64[2];
      b.p1 = m->v64[3];
      b.q = m->v64[4];
      b.tol2_rel = opts.rtol * opts.rtol;
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
      cudaError_t e = cudaSuccess;
      if (cl == 16) {
        e = cudaFuncSetAttribute(k_batch_pcg64<16>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveClusters(&fit, k_batch_pcg64<16>, &cfg);
      } else if (cl == 8) {
        e = cudaOccupancyMaxActiveClusters(&fit, k_batch_pcg64<8>, &cfg);
      } else if (cl == 4) {
        e = cudaOccupancyMaxActiveClusters(&fit, k_batch_pcg64<4>, &cfg);
      } else {
        e = cudaOccupancyMaxActiveClusters(&fit, k_batch_pcg64<2>, &cfg);
      }
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
      FG_CUDA_TRY(cudaMalloc(&d_out, sizeof(int) * 2 * count));
      FG_CUDA_TRY(cudaMalloc(&d_rel, sizeof(double) * count));
      FG_CUDA_TRY(cudaMalloc(&d_probs, sizeof(BatchProb) * count));
      std::vector<BatchProb> sorted(count);
      for (int j = 0; j < count; ++j) {
        sorted[j] = hp[order[j]];
        sorted[j].iters = d_out + j;
        sorted[j].status = d_out + count + j;
        sorted[j].relres = d_rel + j;
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
        switch (g.cl) {
          case 16: return cudaLaunchKernelEx(&cfg, k_batch_pcg64<16>, pp);
          case 8: return cudaLaunchKernelEx(&cfg, k_batch_pcg64<8>, pp);
          case 4: return cudaLaunchKernelEx(&cfg, k_batch_pcg64<4>, pp);
          default: return cudaLaunchKernelEx(&cfg, k_batch_pcg64<2>, pp);
        }
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
      std::vector<int> hout(2 * count);
      std::vector<double> hrel(count);
      FG_CUDA_TRY(cudaMemcpyAsync(hout.data(), d_out, sizeof(int) * 2 * count, cudaMemcpyDeviceToHost, st));
      FG_CUDA_TRY(cudaMemcpyAsync(hrel.data(), d_rel, sizeof(double) * count, cudaMemcpyDeviceToHost, st));
      FG_CUDA_TRY(cudaStreamSynchronize(st));
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      int conv = 0, maxit = 0, nan = 0;
      long long tot = 0;
      for (int j = 0; j < count; ++j) {
        const int k = order[j];
        if (iterations) iterations[k] = hout[j];
        conv += hout[count + j] == 0;
        nan += hout[count + j] == 2;
        maxit = std::max(maxit, hout[j]);
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
