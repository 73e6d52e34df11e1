// Backward-Euler heat conduction on P1 tetrahedra (Heat/heat3D.jl:50-90 steps
// T <- (M + dt A) \ (M T)), with a volumetric heat capacity rho_c, per-element
// conductivity kappa and T = 0 on the Dirichlet nodes:
//   (rho_c M + dt K(kappa)) T_{n+1} = rho_c M T_n.
// The operator and the mass matrix are assembled once (FP64, plus FP32 operator when
// mixed); every step forms b = rho_c M T with one SpMV and solves with the previous
// temperature as the initial guess.
#include "fg_common.cuh"

__global__ void k_zero_fixed(int64_t n, const uint8_t *__restrict__ fixed, double *__restrict__ x) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && fixed[i]) x[i] = 0.0;
}

// b = c b on free rows, 0 on the Dirichlet rows (fixed may be NULL).
__global__ void k_scale_free(int64_t n, const uint8_t *__restrict__ fixed, double c, double *__restrict__ b) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (fixed && fixed[i]) ? 0.0 : c * b[i];
}

extern "C" fg_status fg_heat_be(fg_mesh *m, const double *kappa, double rho_c, double dt, int32_t nsteps, double *T,
                                int32_t every, double *snapshots, const fg_solve_opts *o, fg_solve_stats *s) {
  return fg_guard([&]() -> fg_status {
    FG_REQUIRE(m && kappa && T, FG_BAD_ARG, "fg_heat_be: null pointer");
    FG_REQUIRE(m->npe == 4, FG_UNSUPPORTED, "fg_heat_be: P1 tetrahedra only");
    FG_REQUIRE(rho_c > 0.0 && dt > 0.0 && nsteps >= 0, FG_BAD_ARG, "fg_heat_be: need rho_c > 0, dt > 0, nsteps >= 0");
    FG_REQUIRE(!snapshots || every > 0, FG_BAD_ARG, "fg_heat_be: snapshots need every > 0");
    fg_solve_opts opts;
    fg_solve_opts_default(&opts);
    if (o) opts = *o;
    const bool mixed = opts.precision == FG_MIXED;
    const int64_t nv = m->nv, nt = m->nt;
    if (!m->mu_lin) m->mu_lin = dev_alloc<double>(m, (size_t)nt);  // holds kappa here
    for (int j : {7, 9})
      if (!m->v64[j]) m->v64[j] = dev_alloc<double>(m, (size_t)m->nvp);
    double *d_k = m->mu_lin, *d_T = m->v64[7], *d_b = m->v64[9];
    FG_CUDA_TRY(cudaMemcpyAsync(d_k, kappa, sizeof(double) * (size_t)nt, cudaMemcpyHostToDevice, m->stream));
    FG_CUDA_TRY(cudaMemcpyAsync(d_T, T, sizeof(double) * (size_t)nv, cudaMemcpyHostToDevice, m->stream));
    if (m->has_fixed) {
      k_zero_fixed<<<grid_for(nv, 256), 256, 0, m->stream>>>(nv, m->fixed, d_T);
      FG_LAUNCHED(1);
    }
    cudaEvent_t e0, e1;
    FG_CUDA_TRY(cudaEventCreate(&e0));
    FG_CUDA_TRY(cudaEventCreate(&e1));
    FG_CUDA_TRY(cudaEventRecord(e0, m->stream));
    fg_assemble_operator(m, ASM_HEAT, d_k, nullptr, nullptr, rho_c, dt, 0, OUT_SELL, true, mixed, true);
    if (!m->mval) m->mval = dev_alloc<double>(m, (size_t)m->nsell);
    fg_assemble_mass_sell(m, m->mval);
    int iters = 0, refinements = 0, status = 0, snap = 0;
    double relres = 0.0;
    for (int step = 1; step <= nsteps; ++step) {
      // b = rho_c M T (Dirichlet rows 0): one SpMV with the mass matrix
      fg_spmv64_plain(m, m->mval, d_T, d_b);
      k_scale_free<<<grid_for(nv, 256), 256, 0, m->stream>>>(nv, m->has_fixed ? m->fixed : nullptr, rho_c, d_b);
      FG_LAUNCHED(1);
      fg_solve_stats st{};
      const int rc = fg_pcg_solve(m, d_b, d_T, opts, &st, false);
      iters += st.iterations;
      refinements += st.refinements;
      relres = st.relres;
      if (rc != 0) status = rc;
      if (snapshots && step % every == 0) {
        FG_CUDA_TRY(cudaMemcpyAsync(snapshots + (size_t)snap * nv, d_T, sizeof(double) * (size_t)nv,
                                    cudaMemcpyDeviceToHost, m->stream));
        ++snap;
      }
    }
    FG_CUDA_TRY(cudaEventRecord(e1, m->stream));
    FG_CUDA_TRY(cudaMemcpyAsync(T, d_T, sizeof(double) * (size_t)nv, cudaMemcpyDeviceToHost, m->stream));
    fg_sync(m);
    fg_check_flags(m, "fg_heat_be");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (s) {
      s->iterations = iters;
      s->refinements = refinements;
      s->converged = status == 0;
      s->pad_ = 0;
      s->relres = relres;
      s->ms = ms;
    }
    return status == 0 ? FG_OK : FG_NOT_CONVERGED;
  });
}
