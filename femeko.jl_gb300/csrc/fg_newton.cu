// Magnetostatic solvers on the P1 tetrahedral operator: the linear solve of
// Magnetostatics/magneticField.jl:89-132 (and the ccall scalarPotential of
// Femeko_jl_C++/Magnetostatics/magnetostatics.cpp:49-95) and the Newton-Raphson
// iteration of Magnetostatics/NewtonRaphson.jl:109-214, both with Dirichlet rows.
//
// Newton step: the residual F = -K(mu(u)) u and the Jacobian K(mu) + At(H, dmu).  The
// linear elements' part of K is assembled once per solve (mu fixed there); a residual
// is that operator's part (K_lin u: one FP64 SpMV at the start, then K_lin u +
// alpha K_lin du per accepted step, one SpMV for K_lin du) plus the nonlinear
// (Froehlich) elements re-evaluated and summed into their rows, and each Jacobian is a
// copy of the linear operator with the nonlinear elements' entries added at their
// slots.  The inner
// increment solve J du = F runs to a relative residual inner_rtol in FP32 (mixed)
// or FP64; F is always FP64, so the Newton loop is the iterative refinement.
// Step control follows src/FEM3D.jl:123-152 (alpha = 1, 0.9, 0.81, ... while the
// residual grows and alpha > min_step), applied either to the frozen secant
// (FG_LS_REFERENCE, the reference's lineSearch) or to the true residual
// (FG_LS_RESIDUAL, up to FG_LS_BATCH steps evaluated per host wait).
#include <cmath>
#include <utility>

#include "fg_common.cuh"

// out = a x + b y elementwise; out may be x or y (in-place updates), so no restrict.
__global__ void k_axpby64(int64_t n, double a, const double *x, double b, const double *y, double *out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = a * x[i] + b * y[i];
}

// One line-search trial point: ut = u + alpha du and, since K_lin is linear, its
// linear elements' part K_lin ut = K_lin u + alpha K_lin du (yt, and F as the start
// of the residual) without another SpMV of the linear operator.
__global__ void k_newton_trial64(int64_t n, double alpha, const double *__restrict__ u, const double *__restrict__ du,
                                 const double *__restrict__ y, const double *__restrict__ z, double *__restrict__ ut,
                                 double *__restrict__ yt, double *__restrict__ F) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  ut[i] = fma(alpha, du[i], u[i]);
  const double v = fma(alpha, z[i], y[i]);
  yt[i] = v;
  F[i] = v;
}

extern "C" void fg_newton_opts_default(fg_newton_opts *o) {
  if (!o) return;
  o->precision = FG_MIXED;
  o->maxit = 100;
  o->tol_update = 1e-8;
  o->inner_rtol = 1e-4;
  o->cg_maxiter = 200000;
  o->line_search = FG_LS_RESIDUAL;
  o->min_step = 1e-4;
  o->Ms = 1.2e6;
  o->Hk = 500.0;
  o->check_every = 32;
  o->use_graph = 1;
  o->forcing = FG_FORCING_EW;
  o->picard_steps = 2;
  // forcing term in [1e-2, 0.3]: near the solution Newton then contracts by about
  // eta_min per step, so after the last step (|alpha du| <= tol_update |u|) the error
  // left is about eta_min x tol_update relative.  Over six jittered 96^3 Froehlich
  // plates (mixed precision) [1e-2, 0.3] took 914-1,030 CG iterations per solve
  // (mean 31.5 ms) with H within 5.5e-11 of a tight FP64 solve; [1e-3, 0.1] took
  // 1,012-1,292 (mean 36.0 ms, H within 3.8e-12).
  o->eta_min = 1e-2;
  o->eta_max = 0.3;
}

static void upload(fg_mesh *m, void *dst, const void *src, size_t bytes) {
  FG_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, m->stream));
}
static void download(fg_mesh *m, void *dst, const void *src, size_t bytes) {
  FG_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, m->stream));
}
static double *vec64(fg_mesh *m, int j) {
  if (!m->v64[j]) m->v64[j] = dev_alloc<double>(m, (size_t)m->nv);
  return m->v64[j];
}

static void ensure_element_state(fg_mesh *m) {
  if (!m->mu) m->mu = dev_alloc<double>(m, (size_t)m->nt);
  if (!m->dmu) m->dmu = dev_alloc<double>(m, (size_t)m->nt);
  if (!m->H) m->H = dev_alloc<double>(m, 3 * (size_t)m->nt);
  if (!m->wdens) m->wdens = dev_alloc<double>(m, (size_t)m->nt);
  if (!m->mu_lin) m->mu_lin = dev_alloc<double>(m, (size_t)m->nt);
  if (!m->nl) m->nl = dev_alloc<uint8_t>(m, (size_t)m->nt);
}

// Device-resident Newton solve; u (device) holds the initial guess and receives the
// solution.  Element state (H, mu, dmu) is left at the solution.
static int newton_dev(fg_mesh *m, double *d_u, const uint8_t *nl_host, const fg_newton_opts &o,
                      fg_newton_stats *st) {
  const bool mixed = o.precision == FG_MIXED;
  double *d_du = vec64(m, 8), *d_F = vec64(m, 9), *d_ut = vec64(m, 10), *d_Ft = vec64(m, 11);
  // residual line search: K_lin u at the current iterate (y: one SpMV at the start,
  // then y + alpha z of each accepted trial), K_lin du (z, one SpMV per step) and
  // K_lin ut (yt), so a trial costs vector updates and the nonlinear elements, not an
  // SpMV, and an accepted step keeps its trial's residual
  const bool incremental = (o.line_search == FG_LS_RESIDUAL || o.line_search == FG_LS_QUADRATIC);
  double *d_y = incremental ? vec64(m, 16) : nullptr, *d_z = incremental ? vec64(m, 17) : nullptr;
  double *d_yt = incremental ? vec64(m, 18) : nullptr;
  // the fixed backtracking alpha <- 0.9 alpha: its trials are evaluated in batches
  const bool batched = (o.line_search == FG_LS_RESIDUAL);
  double uq[3] = {0.0, 0.0, 0.0};  // |u|^2, u.du, |du|^2 of the current step (batched)
  if (batched && !m->ls_out) m->ls_out = dev_alloc<double>(m, FG_LS_QUAD + FG_LS_BATCH);
  double *d_ls = batched ? m->ls_out : nullptr;
  fg_solve_opts so;
  fg_solve_opts_default(&so);
  so.precision = o.precision;
  so.inner_rtol = o.inner_rtol;
  so.maxiter = o.cg_maxiter;
  so.check_every = o.check_every;
  so.use_graph = o.use_graph;
  const int64_t nv = m->nv;
  const unsigned g = grid_for(nv, 256);
  // e0/e1 bracket the solve, e0/es the set-up, ec0/ec1 each inner solve (read after
  // the next host wait, so that timing adds none)
  cudaEvent_t e0, e1, es, ec0, ec1;
  FG_CUDA_TRY(cudaEventCreate(&e0));
  FG_CUDA_TRY(cudaEventCreate(&e1));
  FG_CUDA_TRY(cudaEventCreate(&es));
  FG_CUDA_TRY(cudaEventCreate(&ec0));
  FG_CUDA_TRY(cudaEventCreate(&ec1));
  FG_CUDA_TRY(cudaEventRecord(e0, m->stream));

  // the linear elements' operator once; each residual / Jacobian below re-evaluates
  // only the nonlinear elements on top of it
  fg_nl_setup(m, nl_host, mixed);
  fg_newton_assemble_split(m, d_u, o.Ms, o.Hk, mixed, d_F, true, o.picard_steps <= 0, nullptr, d_y);
  FG_CUDA_TRY(cudaEventRecord(es, m->stream));
  fg_check_flags(m, "fg_newton_magnetostatics");
  double rF = fg_slot_sqrt(m, FG_SLOT_FNORM2);
  float setup_ms = 0.f, cg_ms = 0.f;
  cudaEventElapsedTime(&setup_ms, e0, es);
  int it = 0, cg_total = 0, trials = 0, converged = 0, status = 0;
  double ratio = 0.0, alpha = 0.0;
  double eta = (o.forcing == FG_FORCING_EW) ? o.eta_max : o.inner_rtol, rF_prev = -1.0;
  for (it = 1; it <= o.maxit; ++it) {
    if (rF == 0.0) { converged = 1; ratio = 0.0; break; }
    if (o.forcing == FG_FORCING_EW && rF_prev > 0.0) {
      // Eisenstat & Walker (1996), choice 2 with gamma = 0.9, exponent 2 and their
      // safeguard against a too-fast decrease of eta
      const double gam = 0.9;
      double e = gam * (rF / rF_prev) * (rF / rF_prev);
      const double sg = gam * eta * eta;
      if (sg > 0.1) e = std::max(e, sg);
      eta = std::min(std::max(e, o.eta_min), o.eta_max);
    }
    so.inner_rtol = eta;
    rF_prev = rF;
    // the Jacobian assembled for the next iteration carries the tangent term once the
    // Picard steps are done
    const bool next_tangent = (it >= o.picard_steps);
    FG_CUDA_TRY(cudaMemsetAsync(d_du, 0, sizeof(double) * (size_t)nv, m->stream));
    fg_solve_stats cst{};
    FG_CUDA_TRY(cudaEventRecord(ec0, m->stream));
    fg_pcg_solve(m, d_F, d_du, so, &cst, true, rF);
    FG_CUDA_TRY(cudaEventRecord(ec1, m->stream));
    cg_total += cst.iterations;
    alpha = 1.0;
    bool need_jacobian = false;
    if (o.line_search != FG_LS_REFERENCE) {
      // trials evaluate the residual only; the Jacobian is rebuilt once a step is
      // accepted (and only if the iteration continues)
      const bool trial_jacobian = (o.line_search == FG_LS_NONE);
      need_jacobian = !trial_jacobian;
      const double f0 = rF * rF;
      double rt = 0.0;
      if (incremental) fg_spmv64_vals(m, m->vlin64, d_du, d_z);
      if (batched) {
        // the step sequence of the loop below (alpha, 0.9 alpha, ... until a
        // decrease or alpha <= min_step), FG_LS_BATCH candidates per launch and one
        // host wait per launch: |F(alpha)|^2 is the quadratic in alpha over the rows
        // no nonlinear element touches plus the touched rows evaluated per candidate;
        // the same wait brings |u|^2, u.du and |du|^2 for the update test and the
        // device error flags
        fg_lin_quad_enqueue(m, d_y, d_z, m->nl_rowmask, d_u, d_du, d_ls);
        for (;;) {
          LsCand cand;
          cand.n = 0;
          double a = alpha;
          for (;;) {
            cand.a[cand.n++] = a;
            if (cand.n == FG_LS_BATCH || !(a > o.min_step)) break;
            a *= 0.9;
          }
          fg_newton_trial_batch(m, d_u, d_du, d_y, d_z, cand, o.Ms, o.Hk, d_ls);
          FG_CUDA_TRY(cudaMemcpyAsync(m->hbuf, d_ls, sizeof(double) * (FG_LS_QUAD + (size_t)cand.n),
                                      cudaMemcpyDeviceToHost, m->stream));
          FG_CUDA_TRY(cudaMemcpyAsync(m->hint + 8, m->flags, sizeof(int), cudaMemcpyDeviceToHost, m->stream));
          fg_sync(m);
          fg_raise_flags(m, m->hint[8], "fg_newton_magnetostatics");
          const double qa = m->hbuf[0], qb = m->hbuf[1], qc = m->hbuf[2];
          uq[0] = m->hbuf[3];
          uq[1] = m->hbuf[4];
          uq[2] = m->hbuf[5];
          int stop = -1;
          for (int j = 0; j < cand.n && stop < 0; ++j) {
            ++trials;
            const double aj = cand.a[j];
            rt = std::sqrt(std::max(qa + aj * (2.0 * qb + aj * qc), 0.0) + m->hbuf[FG_LS_QUAD + j]);
            if (!(rt > rF && aj > o.min_step)) stop = j;
          }
          if (stop >= 0) {
            alpha = cand.a[stop];
            break;
          }
          alpha = cand.a[cand.n - 1] * 0.9;
        }
        if (alpha >= o.min_step) {
          // the accepted point, its residual and the element state at it
          k_newton_trial64<<<g, 256, 0, m->stream>>>(nv, alpha, d_u, d_du, d_y, d_z, d_ut, d_yt, d_Ft);
          FG_LAUNCHED(1);
          fg_newton_assemble_split(m, d_ut, o.Ms, o.Hk, mixed, d_Ft, false, next_tangent, d_Ft);
        }
      }
      for (; !batched;) {
        if (incremental) {
          k_newton_trial64<<<g, 256, 0, m->stream>>>(nv, alpha, d_u, d_du, d_y, d_z, d_ut, d_yt, d_Ft);
          FG_LAUNCHED(1);
          fg_newton_assemble_split(m, d_ut, o.Ms, o.Hk, mixed, d_Ft, false, next_tangent, d_Ft);
        } else {
          k_axpby64<<<g, 256, 0, m->stream>>>(nv, 1.0, d_u, alpha, d_du, d_ut);
          FG_LAUNCHED(1);
          fg_newton_assemble_split(m, d_ut, o.Ms, o.Hk, mixed, d_Ft, trial_jacobian, next_tangent);
        }
        rt = fg_slot_sqrt(m, FG_SLOT_FNORM2);
        ++trials;
        if (o.line_search == FG_LS_NONE || !(rt > rF && alpha > o.min_step)) break;
        if (o.line_search == FG_LS_QUADRATIC) {
          // minimiser of the quadratic through f(0) = |F|^2, f'(0) = -2|F|^2 (Newton
          // direction) and f(alpha), kept in [0.1, 0.5] alpha (Dennis & Schnabel,
          // backtracking by quadratic interpolation)
          const double c = (rt * rt - f0 + 2.0 * f0 * alpha) / (alpha * alpha);
          const double anew = (c > 0.0) ? f0 / c : 0.5 * alpha;
          alpha = std::min(std::max(anew, 0.1 * alpha), 0.5 * alpha);
        } else {
          alpha *= 0.9;
        }
      }
      if (alpha < o.min_step) {
        // no decrease: keep u (src/FEM3D.jl:144-147) and restore the state at u
        fg_newton_assemble_split(m, d_u, o.Ms, o.Hk, mixed, d_F, true, it > o.picard_steps, nullptr, d_y);
        status = 1;
        alpha = 0.0;
        break;
      }
      // accept: u <- ut, F <- Ft (copy keeps the caller's u buffer in place)
      FG_CUDA_TRY(cudaMemcpyAsync(d_u, d_ut, sizeof(double) * (size_t)nv, cudaMemcpyDeviceToDevice, m->stream));
      std::swap(m->v64[9], m->v64[11]);
      d_F = m->v64[9];
      d_Ft = m->v64[11];
      if (incremental) {
        std::swap(m->v64[16], m->v64[18]);
        d_y = m->v64[16];
        d_yt = m->v64[18];
      }
      rF = rt;
    } else {
      // reference lineSearch: w = K(mu) du with the secant at the current mu
      double *w = d_Ft;
      fg_apply_operator_vec(m, ASM_STIFF, m->mu, 0.0, 0.0, d_du, w, true);
      double rt = 0.0;
      for (;;) {
        k_axpby64<<<g, 256, 0, m->stream>>>(nv, 1.0, d_F, -alpha, w, d_ut);
        FG_LAUNCHED(1);
        rt = fg_norm2_dev(m, d_ut, nv, true);
        ++trials;
        if (!(rt > rF && alpha > o.min_step)) break;
        alpha *= 0.9;
      }
      if (alpha < o.min_step) { status = 1; alpha = 0.0; break; }
      k_axpby64<<<g, 256, 0, m->stream>>>(nv, 1.0, d_u, alpha, d_du, d_u);
      FG_LAUNCHED(1);
      fg_newton_assemble_split(m, d_u, o.Ms, o.Hk, mixed, d_F, true, next_tangent);
      rF = fg_slot_sqrt(m, FG_SLOT_FNORM2);
    }
    double dn, un;
    if (batched) {
      // |u + alpha du| from the sums the line search read (u is the accepted point)
      dn = alpha * std::sqrt(uq[2]);
      un = std::sqrt(std::max(uq[0] + alpha * (2.0 * uq[1] + alpha * uq[2]), 0.0));
    } else {
      // |du|, |u| and the device error flags in one round trip
      fg_dot_enqueue(m, d_du, d_du, nv, false, 10);
      fg_dot_enqueue(m, d_u, d_u, nv, false, 11);
      FG_CUDA_TRY(cudaMemcpyAsync(m->hbuf, m->scal + 10, 2 * sizeof(double), cudaMemcpyDeviceToHost, m->stream));
      FG_CUDA_TRY(cudaMemcpyAsync(m->hint + 8, m->flags, sizeof(int), cudaMemcpyDeviceToHost, m->stream));
      fg_sync(m);
      fg_raise_flags(m, m->hint[8], "fg_newton_magnetostatics");
      dn = alpha * std::sqrt(m->hbuf[0]);
      un = std::sqrt(m->hbuf[1]);
    }
    {
      float t = 0.f;
      if (cudaEventElapsedTime(&t, ec0, ec1) == cudaSuccess) cg_ms += t;
    }
    ratio = (un > 0.0) ? dn / un : dn;
    if (!std::isfinite(ratio)) throw FgError{FG_NAN, "Newton update is not finite"};
    if (ratio <= o.tol_update) { converged = 1; break; }
    // the accepted trial left F at u (and, on the incremental path, K_lin u in y):
    // only the Jacobian is rebuilt
    if (need_jacobian)
      fg_newton_assemble_split(m, d_u, o.Ms, o.Hk, mixed, incremental ? nullptr : d_F, true, next_tangent);
  }
  // the flags of the last accepted point's element evaluation (the batched path reads
  // them with each step's first line-search wait)
  if (batched) fg_check_flags(m, "fg_newton_magnetostatics");
  fg_energy_dev(m, d_u, o.Ms, o.Hk);
  double energy = fg_dot_dev(m, m->wdens, nullptr, m->nt, false);
  FG_CUDA_TRY(cudaEventRecord(e1, m->stream));
  fg_sync(m);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaEventDestroy(es);
  cudaEventDestroy(ec0);
  cudaEventDestroy(ec1);
  if (st) {
    st->newton_iters = std::min(it, o.maxit);
    st->cg_iters = cg_total;
    st->converged = converged;
    st->trials = trials;
    st->update_ratio = ratio;
    st->residual = rF;
    st->alpha = alpha;
    st->energy = energy;
    st->ms = ms;
    st->setup_ms = setup_ms;
    st->cg_ms = cg_ms;
  }
  (void)status;
  return converged ? 0 : 1;
}

static fg_newton_opts checked_opts(const fg_newton_opts *o) {
  fg_newton_opts opts;
  fg_newton_opts_default(&opts);
  if (o) opts = *o;
  FG_REQUIRE(opts.Hk > 0.0 && opts.tol_update > 0.0 && opts.maxit > 0, FG_BAD_ARG,
             "fg_newton_magnetostatics: bad options");
  return opts;
}

static void set_inputs(fg_mesh *m, const uint8_t *nl, const double *mu_lin, const double *u0) {
  FG_REQUIRE(m && nl && mu_lin && u0, FG_BAD_ARG, "fg_newton_magnetostatics: null pointer");
  FG_REQUIRE(m->npe == 4, FG_UNSUPPORTED, "fg_newton_magnetostatics: P1 tetrahedra only");
  ensure_element_state(m);
  upload(m, m->nl, nl, (size_t)m->nt);
  upload(m, m->mu_lin, mu_lin, sizeof(double) * (size_t)m->nt);
  if (!m->u0dev) m->u0dev = dev_alloc<double>(m, (size_t)m->nv);
  upload(m, m->u0dev, u0, sizeof(double) * (size_t)m->nv);
  fg_set_nl_host(m, nl);
}

// Newton solve from the inputs held on the device; u, H and mu stay on the device.
static int solve_resident(fg_mesh *m, const fg_newton_opts &opts, fg_newton_stats *s) {
  FG_REQUIRE(m->nl_host.size() == (size_t)m->nt, FG_BAD_ARG, "fg_newton_solve_resident: no inputs set");
  double *d_u = vec64(m, 7);
  FG_CUDA_TRY(cudaMemcpyAsync(d_u, m->u0dev, sizeof(double) * (size_t)m->nv, cudaMemcpyDeviceToDevice,
                              m->stream));
  const int rc = newton_dev(m, d_u, m->nl_host.data(), opts, s);
  fg_hfield_dev(m, d_u, m->H);
  fg_sync(m);
  return rc;
}

static void get_outputs(fg_mesh *m, double *u, double *H, double *mu) {
  if (u) download(m, u, m->v64[7], sizeof(double) * (size_t)m->nv);
  if (H) download(m, H, m->H, sizeof(double) * 3 * (size_t)m->nt);
  if (mu) download(m, mu, m->mu, sizeof(double) * (size_t)m->nt);
  fg_sync(m);
}

extern "C" fg_status fg_newton_magnetostatics(fg_mesh *m, const uint8_t *nl, const double *mu_lin, const double *u0,
                                              const fg_newton_opts *o, double *u, double *H, double *mu,
                                              fg_newton_stats *s) {
  return fg_guard([&]() -> fg_status {
    FG_REQUIRE(u != nullptr, FG_BAD_ARG, "fg_newton_magnetostatics: null pointer");
    const fg_newton_opts opts = checked_opts(o);
    set_inputs(m, nl, mu_lin, u0);
    const int rc = solve_resident(m, opts, s);
    get_outputs(m, u, H, mu);
    return rc == 0 ? FG_OK : FG_NOT_CONVERGED;
  });
}

extern "C" fg_status fg_newton_set_inputs(fg_mesh *m, const uint8_t *nl, const double *mu_lin, const double *u0) {
  return fg_guard([&]() -> fg_status {
    set_inputs(m, nl, mu_lin, u0);
    fg_sync(m);
    return FG_OK;
  });
}

extern "C" fg_status fg_newton_solve_resident(fg_mesh *m, const fg_newton_opts *o, fg_newton_stats *s) {
  return fg_guard([&]() -> fg_status {
    FG_REQUIRE(m != nullptr, FG_BAD_ARG, "fg_newton_solve_resident: null handle");
    const fg_newton_opts opts = checked_opts(o);
    return solve_resident(m, opts, s) == 0 ? FG_OK : FG_NOT_CONVERGED;
  });
}

extern "C" fg_status fg_newton_get_outputs(fg_mesh *m, double *u, double *H, double *mu) {
  return fg_guard([&]() -> fg_status {
    FG_REQUIRE(m != nullptr && m->v64[7] && m->H && m->mu, FG_BAD_ARG, "fg_newton_get_outputs: nothing solved");
    get_outputs(m, u, H, mu);
    return FG_OK;
  });
}

extern "C" fg_status fg_magnetostatics_linear(fg_mesh *m, const double *mu, const double *u_in,
                                              const fg_solve_opts *o, double *u, double *H, fg_solve_stats *s) {
  return fg_guard([&]() -> fg_status {
    FG_REQUIRE(m && mu && u_in && u, FG_BAD_ARG, "fg_magnetostatics_linear: null pointer");
    FG_REQUIRE(m->npe == 4 || m->npe == 3, FG_UNSUPPORTED, "fg_magnetostatics_linear: P1 elements only");
    fg_solve_opts opts;
    fg_solve_opts_default(&opts);
    if (o) opts = *o;
    ensure_element_state(m);
    upload(m, m->mu_lin, mu, sizeof(double) * (size_t)m->nt);
    const bool mixed = opts.precision == FG_MIXED;
    fg_assemble_operator(m, ASM_STIFF, m->mu_lin, nullptr, nullptr, 0.0, 0.0, 0, OUT_SELL, true, mixed, true);
    double *d_x = vec64(m, 7), *d_b = vec64(m, 9);
    upload(m, d_x, u_in, sizeof(double) * (size_t)m->nv);
    FG_CUDA_TRY(cudaMemsetAsync(d_b, 0, sizeof(double) * (size_t)m->nv, m->stream));
    int status = fg_pcg_solve(m, d_b, d_x, opts, s, false);
    download(m, u, d_x, sizeof(double) * (size_t)m->nv);
    if (H) {
      FG_REQUIRE(m->npe == 4, FG_UNSUPPORTED, "H output: P1 tetrahedra only");
      fg_hfield_dev(m, d_x, m->H);
      download(m, H, m->H, sizeof(double) * 3 * (size_t)m->nt);
    }
    fg_sync(m);
    fg_check_flags(m, "fg_magnetostatics_linear");
    return status == 0 ? FG_OK : FG_NOT_CONVERGED;
  });
}

// Per-element factor of the stiffness for the caller's element volumes: the stored
// geometry holds VE grad phi_a . grad phi_b with this library's VE, so f = mu VE_in / VE
// gives mu VE_in grad phi_a . grad phi_b (src/FEMc.cpp:74-96 takes VE from the caller).
__global__ void k_mu_caller_ve(int64_t nt, const double *__restrict__ mu, const double *__restrict__ ve_in,
                               const double *__restrict__ geo, int vol_row, double *__restrict__ f) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nt) return;
  const double ve = geo[(int64_t)vol_row * nt + k];
  f[k] = ve != 0.0 ? mu[k] * (ve_in[k] / ve) : 0.0;
}

// Femeko_jl_C++/Magnetostatics/magnetostatics.cpp:5-95 (scalarPotential): the linear
// Neumann problem K(mu) u = -BoundaryIntegral(Hext) on the whole mesh, no Dirichlet
// rows (the system is singular with the constants as null space and consistent:
// the flux of a uniform field through the closed shell is zero), solved by
// Jacobi-PCG from u = 0 like Eigen's ConjugateGradient with its diagonal
// preconditioner (src/FEMc.cpp:26-38 of the caller).  t and surfaceT are 0-based as
// Femeko_jl_C++/Magnetostatics/run.jl:49-52 passes them; surfaceT is 4 x ns (three
// nodes and the boundary id, row 4 compared with shell_id).
extern "C" fg_status fg_scalar_potential(double *u, const double *p, const int32_t *t, const int32_t *surfaceT,
                                         const double *normal, int32_t nv, int32_t nt, int32_t ns, const double *VE,
                                         const double *mu, const double *Hext, int32_t shell_id,
                                         const fg_solve_opts *o, fg_solve_stats *s) {
  fg_mesh *m = nullptr;
  fg_status st = fg_guard([&]() -> fg_status {
    FG_REQUIRE(u && p && t && VE && mu && Hext && (ns == 0 || (surfaceT && normal)), FG_BAD_ARG,
               "fg_scalar_potential: null pointer");
    FG_REQUIRE(nv > 0 && nt > 0 && ns >= 0, FG_BAD_ARG, "fg_scalar_potential: bad sizes");
    return FG_OK;
  });
  if (st != FG_OK) return st;
  st = fg_mesh_create(p, nv, t, nt, 4, 0, &m);
  if (st != FG_OK) return st;
  st = fg_guard([&]() -> fg_status {
    fg_solve_opts opts;
    fg_solve_opts_default(&opts);
    if (o) {
      opts = *o;
    } else {
      opts.precision = FG_MIXED;
      opts.rtol = 1e-12;
    }
    const bool mixed = opts.precision == FG_MIXED;
    ensure_element_state(m);
    double *d_f = m->wdens, *d_b = vec64(m, 9), *d_x = vec64(m, 7);
    upload(m, m->mu_lin, mu, sizeof(double) * (size_t)nt);
    // the caller's volumes, staged through an element-sized buffer of the handle
    double *d_vein = m->dmu;
    upload(m, d_vein, VE, sizeof(double) * (size_t)nt);
    k_mu_caller_ve<<<grid_for(nt, 256), 256, 0, m->stream>>>(nt, m->mu_lin, d_vein, m->geo, m->nvert * m->dim, d_f);
    FG_CUDA_TRY(cudaGetLastError());
    FG_LAUNCHED(1);
    fg_assemble_operator(m, ASM_STIFF, d_f, nullptr, nullptr, 0.0, 0.0, 0, OUT_SELL, true, mixed, true);
    // b = -RHS = BoundaryIntegral(-Hext): the integral is linear in the field
    const double mF[3] = {-Hext[0], -Hext[1], -Hext[2]};
    const int32_t shell = shell_id;
    fg_boundary_rhs_dev(m, surfaceT, ns, 0, normal, nullptr, mF, &shell, 1, d_b);
    FG_CUDA_TRY(cudaMemsetAsync(d_x, 0, sizeof(double) * (size_t)nv, m->stream));
    fg_solve_stats ss{};
    const int rc = fg_pcg_solve(m, d_b, d_x, opts, &ss, false);
    download(m, u, d_x, sizeof(double) * (size_t)nv);
    fg_sync(m);
    fg_check_flags(m, "fg_scalar_potential");
    if (s) *s = ss;
    if (rc != 0) {
      fg_set_error("fg_scalar_potential: CG stopped at the iteration cap before the tolerance");
      return FG_NOT_CONVERGED;
    }
    return FG_OK;
  });
  const fg_status d = fg_mesh_destroy(m);
  return st != FG_OK ? st : d;
}

// The reference's own entry point, same name and arguments (a void C function that
// Julia binds with @ccall ... ::Cvoid, run.jl:66-79).  Nothing throws across it: the
// status is kept for fg_scalar_potential_status() and the message in fg_last_error()
// (empty after a successful call).  u receives the solution (also when the iteration
// cap stopped the solve); on any other error u is left as it was.
static thread_local fg_status g_sp_status = FG_OK;

extern "C" void scalarPotential(double *u_in, double *p_in, int *t_in, int *surfaceT_in, double *normal_in, int nv,
                                int nt, int ns, double *VE, double *mu, double *Hext, int shell_id) {
  fg_set_error("");
  g_sp_status = fg_scalar_potential(u_in, p_in, t_in, surfaceT_in, normal_in, nv, nt, ns, VE, mu, Hext, shell_id,
                                    nullptr, nullptr);
}

extern "C" fg_status fg_scalar_potential_status(void) { return g_sp_status; }

// Adjoint sensitivity of J = volume-weighted mean Hx over the target elements with
// respect to the per-element relative permeability.  Forward: the linear solve of
// Magnetostatics/magneticField.jl:89-132 (nl == NULL) or the Newton solve of
// Magnetostatics/NewtonRaphson.jl:109-214.  Adjoint: op lambda = dJ/du on the free
// rows with op = K(mu) (linear) or the converged Newton Jacobian K(mu) + At (both
// symmetric); then dJ/dmur_k = -mu0 VE_k grad(lambda).grad(u).  The element gradients
// are recomputed from the stored geometry, not kept from the forward pass.
extern "C" fg_status fg_adjoint_dJdmu(fg_mesh *m, const double *mur, const double *u0, const uint8_t *target,
                                      const uint8_t *nl, const fg_newton_opts *o, double rtol, double *J,
                                      double *grad, double *u, fg_adjoint_stats *s) {
  return fg_guard([&]() -> fg_status {
    FG_REQUIRE(m && mur && u0 && target && J && grad, FG_BAD_ARG, "fg_adjoint_dJdmu: null pointer");
    FG_REQUIRE(m->npe == 4, FG_UNSUPPORTED, "fg_adjoint_dJdmu: P1 tetrahedra only");
    FG_REQUIRE(m->has_fixed, FG_BAD_ARG, "fg_adjoint_dJdmu: set Dirichlet nodes first (fg_mesh_set_dirichlet)");
    FG_REQUIRE(rtol > 0.0, FG_BAD_ARG, "fg_adjoint_dJdmu: rtol must be positive");
    fg_newton_opts opts;
    fg_newton_opts_default(&opts);
    if (o) opts = *o;
    const bool mixed = opts.precision == FG_MIXED;
    ensure_element_state(m);
    const int64_t nt = m->nt, nv = m->nv;
    if (!m->target) m->target = dev_alloc<uint8_t>(m, (size_t)nt);
    if (!m->objbuf) m->objbuf = dev_alloc<double>(m, 2 * (size_t)nt);
    upload(m, m->target, target, (size_t)nt);
    upload(m, m->mu_lin, mur, sizeof(double) * (size_t)nt);
    k_axpby64<<<grid_for(nt, 256), 256, 0, m->stream>>>(nt, FG_MU0, m->mu_lin, 0.0, m->mu_lin, m->mu_lin);
    FG_LAUNCHED(1);
    double *d_u = vec64(m, 7), *d_b = vec64(m, 9), *d_g = vec64(m, 13), *d_lam = vec64(m, 14);
    upload(m, d_u, u0, sizeof(double) * (size_t)nv);
    fg_solve_opts so;
    fg_solve_opts_default(&so);
    so.precision = opts.precision;
    so.rtol = rtol;
    so.maxiter = opts.cg_maxiter;
    so.check_every = opts.check_every;
    so.use_graph = opts.use_graph;
    cudaEvent_t e0, e1, e2;
    FG_CUDA_TRY(cudaEventCreate(&e0));
    FG_CUDA_TRY(cudaEventCreate(&e1));
    FG_CUDA_TRY(cudaEventCreate(&e2));
    FG_CUDA_TRY(cudaEventRecord(e0, m->stream));
    int fwd_iters = 0, newton_iters = 0, converged = 1;
    if (!nl) {
      fg_assemble_operator(m, ASM_STIFF, m->mu_lin, nullptr, nullptr, 0.0, 0.0, 0, OUT_SELL, true, mixed, true);
      FG_CUDA_TRY(cudaMemsetAsync(d_b, 0, sizeof(double) * (size_t)nv, m->stream));
      fg_solve_stats fs{};
      converged = fg_pcg_solve(m, d_b, d_u, so, &fs, false) == 0;
      fwd_iters = fs.iterations;
    } else {
      upload(m, m->nl, nl, (size_t)nt);
      fg_newton_stats ns{};
      fg_set_nl_host(m, nl);
      converged = newton_dev(m, d_u, m->nl_host.data(), opts, &ns) == 0;
      fwd_iters = ns.cg_iters;
      newton_iters = ns.newton_iters;
      // the Jacobian at the converged state: FP64 for the refinement residual, FP32
      // for the inner solve when mixed
      fg_newton_assemble(m, d_u, opts.Ms, opts.Hk, false, d_b, true, true);
      if (mixed) fg_newton_assemble(m, d_u, opts.Ms, opts.Hk, true, d_b, true, true);
    }
    FG_CUDA_TRY(cudaEventRecord(e1, m->stream));
    double *pa = m->objbuf, *pv = m->objbuf + nt;
    fg_objective_parts_dev(m, d_u, m->target, pa, pv);
    const double num = fg_dot_dev(m, pa, nullptr, nt, false);
    const double vol = fg_dot_dev(m, pv, nullptr, nt, false);
    FG_REQUIRE(vol > 0.0, FG_BAD_ARG, "fg_adjoint_dJdmu: the target selects no element");
    *J = num / vol;
    fg_objective_rhs_dev(m, m->target, vol, d_g);
    FG_CUDA_TRY(cudaMemsetAsync(d_lam, 0, sizeof(double) * (size_t)nv, m->stream));
    fg_solve_stats as{};
    const bool adj_ok = fg_pcg_solve(m, d_g, d_lam, so, &as, false) == 0;
    fg_adjoint_grad_dev(m, d_lam, d_u, -FG_MU0, pa);
    FG_CUDA_TRY(cudaEventRecord(e2, m->stream));
    download(m, grad, pa, sizeof(double) * (size_t)nt);
    if (u) download(m, u, d_u, sizeof(double) * (size_t)nv);
    fg_sync(m);
    fg_check_flags(m, "fg_adjoint_dJdmu");
    float f_ms = 0.f, a_ms = 0.f;
    cudaEventElapsedTime(&f_ms, e0, e1);
    cudaEventElapsedTime(&a_ms, e1, e2);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaEventDestroy(e2);
    if (s) {
      s->forward_iters = fwd_iters;
      s->adjoint_iters = as.iterations;
      s->newton_iters = newton_iters;
      s->converged = (converged && adj_ok) ? 1 : 0;
      s->forward_ms = f_ms;
      s->adjoint_ms = a_ms;
    }
    return (converged && adj_ok) ? FG_OK : FG_NOT_CONVERGED;
  });
}

// Demagnetising field of Micromagnetics/LL.jl:162-211 (magnetostaticField): the
// stiffness operator of the whole mesh (assembled once and kept while nothing else
// is assembled on the handle: the reference builds A once and calls cg every
// Landau-Lifshitz step), the load vector of the inside elements from the nodal
// magnetisation, the CG solve from zero, H = -grad u and its nodal volume average.
enum { OP_DEMAG64 = 1, OP_DEMAG_MIXED = 2 };

extern "C" fg_status fg_demag_field(fg_mesh *m, const uint8_t *inside, const double *M, const fg_solve_opts *o,
                                    double *Hn, double *u, fg_solve_stats *s) {
  return fg_guard([&]() -> fg_status {
    FG_REQUIRE(m && inside && M && Hn, FG_BAD_ARG, "fg_demag_field: null pointer");
    FG_REQUIRE(m->npe == 4, FG_UNSUPPORTED, "fg_demag_field: P1 tetrahedra only");
    fg_solve_opts opts;
    fg_solve_opts_default(&opts);
    if (o) opts = *o;
    const bool mixed = opts.precision == FG_MIXED;
    const int64_t nv = m->nv, nt = m->nt;
    ensure_element_state(m);
    if (!m->inside) m->inside = dev_alloc<uint8_t>(m, (size_t)nt);
    if (!m->nodal_in) m->nodal_in = dev_alloc<double>(m, 3 * (size_t)nv);
    upload(m, m->inside, inside, (size_t)nt);
    upload(m, m->nodal_in, M, sizeof(double) * 3 * (size_t)nv);
    const int want = mixed ? OP_DEMAG_MIXED : OP_DEMAG64;
    if (m->op_tag != want && m->op_tag != OP_DEMAG_MIXED) {
      fg_assemble_operator(m, ASM_STIFF, nullptr, nullptr, nullptr, 0.0, 0.0, 0, OUT_SELL, true, mixed, true);
      m->op_tag = want;
    }
    double *d_b = vec64(m, 9), *d_u = vec64(m, 7);
    fg_demag_rhs_dev(m, m->inside, m->nodal_in, d_b);
    FG_CUDA_TRY(cudaMemsetAsync(d_u, 0, sizeof(double) * (size_t)nv, m->stream));
    fg_solve_stats st{};
    const int rc = fg_pcg_solve(m, d_b, d_u, opts, &st, false);
    fg_hfield_dev(m, d_u, m->H);
    if (!m->nodal_work) m->nodal_work = dev_alloc<double>(m, 7 * (size_t)nv);  // 4 sums + 3 x nv field
    fg_nodal_average_dev(m, m->inside, m->H, m->nodal_work, m->nodal_work + 4 * nv);
    download(m, Hn, m->nodal_work + 4 * nv, sizeof(double) * 3 * (size_t)nv);
    if (u) download(m, u, d_u, sizeof(double) * (size_t)nv);
    fg_sync(m);
    if (s) *s = st;
    return rc == 0 ? FG_OK : FG_NOT_CONVERGED;
  });
}

extern "C" fg_status fg_hfield(fg_mesh *m, const double *u, double *H) {
  return fg_guard([&]() -> fg_status {
    FG_REQUIRE(m && u && H, FG_BAD_ARG, "fg_hfield: null pointer");
    ensure_element_state(m);
    double *d_u = vec64(m, 7);
    upload(m, d_u, u, sizeof(double) * (size_t)m->nv);
    fg_hfield_dev(m, d_u, m->H);
    download(m, H, m->H, sizeof(double) * 3 * (size_t)m->nt);
    fg_sync(m);
    return FG_OK;
  });
}
