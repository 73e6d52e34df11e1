// One-shot entry points shaped like the reference's ccall boundary, and kernel
// timing used by the benchmark's roofline report.
#include <cmath>

#include "fg_common.cuh"

// Femeko_jl_C++/Magnetostatics/magnetostatics.cpp:49-95 (scalarPotential) takes the
// whole mesh from host arrays on every call and writes the potential back.  This is
// the same shape for the nonlinear Newton solve: upload, build the pattern, solve,
// download, release.
extern "C" fg_status fg_scalar_potential_newton(const double *p, int64_t nv, const int32_t *t, int64_t nt,
                                                int32_t index_base, const uint8_t *fixed, const uint8_t *nl,
                                                const double *mu_lin, const double *u0, const fg_newton_opts *o,
                                                double *u, double *H, double *mu, fg_newton_stats *s) {
  fg_mesh *m = nullptr;
  fg_status st = fg_mesh_create(p, nv, t, nt, 4, index_base, &m);
  if (st != FG_OK) return st;
  st = fg_mesh_set_dirichlet(m, fixed);
  if (st == FG_OK) st = fg_newton_magnetostatics(m, nl, mu_lin, u0, o, u, H, mu, s);
  fg_status d = fg_mesh_destroy(m);
  return st != FG_OK ? st : d;
}

// Average device time (CUDA events on the handle's stream) of one launch of a hot
// kernel on the operator currently held by the handle:
//   which = 0: CG SpMV with its dot products (w = A u; the whole iteration for the
//              fused FP32 variants);
//   which = 1: CG vector update (fused FP32 variants: the whole iteration);
//   which = 2: Newton element pass + row gather over all elements at the current
//              potential (residual and Jacobian);
//   which = 3: one whole CG iteration;
//   which = 4: Newton residual on the linear/nonlinear split (FP64 SpMV of the
//              linear elements' operator + the nonlinear elements);
//   which = 5: the same with the Jacobian.
fg_status fg_bench_cg_kernel(fg_mesh *m, int which, int precision, int reps, double *ms_per_launch);

extern "C" fg_status fg_bench_kernel(fg_mesh *m, int32_t which, int32_t precision, int32_t reps,
                                     double *ms_per_launch) {
  return fg_guard([&]() -> fg_status {
    FG_REQUIRE(m && ms_per_launch && reps > 0, FG_BAD_ARG, "fg_bench_kernel: bad argument");
    if (which == 0 || which == 1 || which == 3) return fg_bench_cg_kernel(m, which, precision, reps, ms_per_launch);
    FG_REQUIRE(which == 2 || which == 4 || which == 5, FG_BAD_ARG, "fg_bench_kernel: unknown kernel");
    FG_REQUIRE(m->v64[7] && m->mu, FG_BAD_ARG, "fg_bench_kernel: run a Newton solve on this handle first");
    FG_REQUIRE(which == 2 || m->nl_maps_valid, FG_BAD_ARG, "fg_bench_kernel: run a Newton solve on this handle first");
    if (!m->v64[11]) m->v64[11] = dev_alloc<double>(m, (size_t)m->nv);
    const bool mixed = precision == FG_MIXED;
    auto once = [&]() {
      if (which == 2) fg_newton_assemble(m, m->v64[7], 1.2e6, 500.0, mixed, m->v64[11]);
      else fg_newton_assemble_split(m, m->v64[7], 1.2e6, 500.0, mixed, m->v64[11], which == 5, true);
    };
    once();
    FG_CUDA_TRY(cudaEventRecord(m->ev0, m->stream));
    for (int r = 0; r < reps; ++r) once();
    FG_CUDA_TRY(cudaEventRecord(m->ev1, m->stream));
    fg_sync(m);
    float ms = 0.f;
    FG_CUDA_TRY(cudaEventElapsedTime(&ms, m->ev0, m->ev1));
    *ms_per_launch = ms / reps;
    return FG_OK;
  });
}

extern "C" fg_status fg_mesh_layout(const fg_mesh *m, int64_t *nsell, int64_t *ninc, int32_t *nslices) {
  return fg_guard([&]() -> fg_status {
    FG_REQUIRE(m != nullptr, FG_BAD_ARG, "fg_mesh_layout: null handle");
    if (nsell) *nsell = m->nsell;
    if (ninc) *ninc = m->ninc;
    if (nslices) *nslices = m->nslices;
    return FG_OK;
  });
}
