// Nedelec (Whitney) edge elements for the vector-potential magnetostatics of
// Magnetostatics/nedelec3D.jl: the element blocks of src/FEM3D.jl:155-191, the global
// curl-curl and tangential matrices over the edge unknowns (:172-182, src/FEM3D.jl:
// 194-271), the load vector of an applied flux density (:106-139), B per element from
// the edge values (:190-221) and the first (linear) solve A(nu) u = RHS
// (du = cg(A + At, RHS - A u) at :185 with u = 0 and At = 0).  The handle comes from
// fg_edge_mesh_create: its matrix rows are the edges (the reference's
// edge2localMap[t[5:10, k]]), its geometry the P1 vertex tetrahedra.
#include "fg_common.cuh"

#include <cmath>
#include <cstring>
#include <initializer_list>
#include <vector>

namespace {

// Interpolating cubic spline with not-a-knot ends through (x_i, y_i), i < n, n >= 4:
// the function Dierckx's Spline1D(x, y) (FITPACK curfit, k = 3, s = 0, knots at the
// data except the second and the second-to-last) interpolates with.  Returns the
// second derivatives M_i.  Tridiagonal system in M_1..M_{n-2} after eliminating M_0
// and M_{n-1} with the two not-a-knot rows (third derivative continuous at x_1 and
// x_{n-2}).
std::vector<double> not_a_knot(const std::vector<double> &x, const std::vector<double> &y) {
  const int n = (int)x.size();
  std::vector<double> h(n - 1), M(n, 0.0);
  for (int i = 0; i + 1 < n; ++i) h[i] = x[i + 1] - x[i];
  const int k = n - 2;  // unknowns M_1..M_{n-2}
  std::vector<double> a(k, 0.0), b(k, 0.0), c(k, 0.0), r(k, 0.0);
  for (int i = 1; i <= n - 2; ++i) {
    const int q = i - 1;
    a[q] = h[i - 1];
    b[q] = 2.0 * (h[i - 1] + h[i]);
    c[q] = h[i];
    r[q] = 6.0 * ((y[i + 1] - y[i]) / h[i] - (y[i] - y[i - 1]) / h[i - 1]);
  }
  // M_0 = ((h0 + h1) M_1 - h0 M_2) / h1 into the first row
  b[0] += a[0] * (h[0] + h[1]) / h[1];
  if (k > 1) c[0] -= a[0] * h[0] / h[1];
  a[0] = 0.0;
  // M_{n-1} = ((h_{n-2} + h_{n-3}) M_{n-2} - h_{n-2} M_{n-3}) / h_{n-3} into the last row
  const double hl = h[n - 2], hp = h[n - 3];
  b[k - 1] += c[k - 1] * (hl + hp) / hp;
  if (k > 1) a[k - 1] -= c[k - 1] * hl / hp;
  c[k - 1] = 0.0;
  // Thomas algorithm (diagonally dominant for increasing x)
  for (int q = 1; q < k; ++q) {
    const double w = a[q] / b[q - 1];
    b[q] -= w * c[q - 1];
    r[q] -= w * r[q - 1];
  }
  std::vector<double> z(k);
  z[k - 1] = r[k - 1] / b[k - 1];
  for (int q = k - 2; q >= 0; --q) z[q] = (r[q] - c[q] * z[q + 1]) / b[q];
  for (int q = 0; q < k; ++q) M[q + 1] = z[q];
  M[0] = ((h[0] + h[1]) * M[1] - h[0] * M[2]) / h[1];
  M[n - 1] = ((hl + hp) * M[n - 2] - hl * M[n - 3]) / hp;
  return M;
}

// src/FEM.jl:66-92 gradient: one-sided differences at the ends, central inside.
std::vector<double> fd_gradient(const std::vector<double> &x, const std::vector<double> &y) {
  const int n = (int)x.size();
  std::vector<double> z(n);
  z[0] = (y[1] - y[0]) / (x[1] - x[0]);
  z[n - 1] = (y[n - 1] - y[n - 2]) / (x[n - 1] - x[n - 2]);
  for (int i = 1; i + 1 < n; ++i) z[i] = (y[i + 1] - y[i - 1]) / (x[i + 1] - x[i - 1]);
  return z;
}

}  // namespace

// Spline value at b, clamped to the data range (Spline1D's bc = "nearest").
__device__ __forceinline__ double spline_eval(const double *x, const double *y, const double *M, int n, double b) {
  if (b <= x[0]) return y[0];
  if (b >= x[n - 1]) return y[n - 1];
  int lo = 0, hi = n - 1;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (x[mid] <= b) lo = mid; else hi = mid;
  }
  const double h = x[hi] - x[lo], A = x[hi] - b, Bq = b - x[lo];
  return M[lo] * A * A * A / (6.0 * h) + M[hi] * Bq * Bq * Bq / (6.0 * h) + (y[lo] / h - M[lo] * h / 6.0) * A +
         (y[hi] / h - M[hi] * h / 6.0) * Bq;
}

// nu = spl(|B|), dnu = spl_dnu(|B|) on the nonlinear elements (nedelec3D.jl:225-226);
// the others keep nu_lin (1 when null) and dnu = 0.  tab: x, y, M of nu, then y, M of
// the finite-difference derivative (5 n doubles).
__global__ void k_ned_material(int64_t nt, const uint8_t *__restrict__ nonlin, const double *__restrict__ nu_lin,
                               const double *__restrict__ Bn, const double *__restrict__ tab, int n,
                               double *__restrict__ nu, double *__restrict__ dnu, int *flags) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nt) return;
  if (nonlin[k]) {
    const double v = spline_eval(tab, tab + n, tab + 2 * n, n, Bn[k]);
    const double d = spline_eval(tab, tab + 3 * n, tab + 4 * n, n, Bn[k]);
    if (!isfinite(v) || !isfinite(d)) atomicOr(flags, FLAG_NAN);
    nu[k] = v;
    dnu[k] = d;
  } else {
    nu[k] = nu_lin ? nu_lin[k] : 1.0;
    dnu[k] = 0.0;
  }
}

// out = u + a du
__global__ void k_ned_axpy(int64_t n, const double *__restrict__ u, double a, const double *__restrict__ du,
                           double *__restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = u[i] + a * du[i];
}

// max_k |B_k - Bold_k| into *res (non-negative doubles order as their bit patterns);
// then Bold = B.
__global__ void k_ned_maxdiff(int64_t nt, const double *__restrict__ Bn, double *__restrict__ Bold,
                              unsigned long long *res) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double d = 0.0;
  if (k < nt) {
    d = fabs(Bn[k] - Bold[k]);
    if (d != d) d = INFINITY;
    Bold[k] = Bn[k];
  }
  for (int o = 16; o > 0; o >>= 1) d = fmax(d, __shfl_down_sync(0xffffffffu, d, o));
  if ((threadIdx.x & 31) == 0) atomicMax(res, (unsigned long long)__double_as_longlong(d));
}

__global__ void k_fill64_ned(int64_t n, double v, double *__restrict__ x) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = v;
}

__global__ void k_ned_keep_linear(int64_t nt, const uint8_t *__restrict__ nonlin, const double *__restrict__ nu_lin,
                                  double *__restrict__ nu) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < nt && !nonlin[k]) nu[k] = nu_lin[k];
}

namespace {

double *upload_d(fg_mesh *m, const double *h, size_t n) {
  if (!h) return nullptr;
  double *d = nullptr;
  FG_CUDA_TRY(cudaMallocAsync(&d, sizeof(double) * n, m->stream));
  FG_CUDA_TRY(cudaMemcpyAsync(d, h, sizeof(double) * n, cudaMemcpyHostToDevice, m->stream));
  return d;
}

void free_d(fg_mesh *m, std::initializer_list<double *> ps) {
  for (double *p : ps)
    if (p) cudaFreeAsync(p, m->stream);
}

void need_edge(fg_mesh *m, const char *w) {
  FG_REQUIRE(m != nullptr, FG_BAD_ARG, std::string(w) + ": null handle");
  FG_REQUIRE(m->edge, FG_UNSUPPORTED, std::string(w) + ": needs a handle from fg_edge_mesh_create");
}

// The mixed path (FP32 CG inside FP64 refinement) first; on this singular
// (gradient null space) system its FP32 inner iterations can stall short of a tight
// rtol at high permeability contrast, and then FP64 PCG continues from where it
// stopped (the operator holds both precisions).  Iterations of both are counted.
int solve_with_fallback(fg_mesh *m, const double *d_b, double *d_x, const fg_solve_opts &o, fg_solve_stats *st) {
  int rc = fg_pcg_solve(m, d_b, d_x, o, st, false);
  if (rc == 0 || o.precision != FG_MIXED) return rc;
  fg_solve_opts o64 = o;
  o64.precision = FG_FP64;
  fg_solve_stats s2{};
  rc = fg_pcg_solve(m, d_b, d_x, o64, &s2, false);
  st->iterations += s2.iterations;
  st->refinements += 1;
  st->converged = s2.converged;
  st->relres = s2.relres;
  return rc;
}

fg_status export_nz(fg_mesh *m, double *nzval, const char *w) {
  FG_CUDA_TRY(cudaMemcpyAsync(nzval, m->csrval, sizeof(double) * (size_t)m->nnz, cudaMemcpyDeviceToHost, m->stream));
  fg_sync(m);
  fg_check_flags(m, w);
  return FG_OK;
}

}  // namespace

extern "C" fg_status fg_nedelec_local_stiffness(fg_mesh *m, double *Ak) {
  double *d = nullptr;
  fg_status st = fg_guard([&]() -> fg_status {
    need_edge(m, "fg_nedelec_local_stiffness");
    FG_REQUIRE(Ak, FG_BAD_ARG, "fg_nedelec_local_stiffness: null pointer");
    FG_CUDA_TRY(cudaMallocAsync(&d, sizeof(double) * 36 * (size_t)m->nt, m->stream));
    fg_nedelec_local_dev(m, d);
    FG_CUDA_TRY(cudaMemcpyAsync(Ak, d, sizeof(double) * 36 * (size_t)m->nt, cudaMemcpyDeviceToHost, m->stream));
    fg_sync(m);
    return FG_OK;
  });
  if (m && d) free_d(m, {d});
  return st;
}

extern "C" fg_status fg_nedelec_stiffness(fg_mesh *m, const double *nu, double *nzval) {
  double *dn = nullptr;
  fg_status st = fg_guard([&]() -> fg_status {
    need_edge(m, "fg_nedelec_stiffness");
    FG_REQUIRE(nzval, FG_BAD_ARG, "fg_nedelec_stiffness: null pointer");
    dn = upload_d(m, nu, (size_t)m->nt);
    fg_nedelec_operator(m, dn, true, nullptr, nullptr, nullptr, OUT_CSR, false);
    return export_nz(m, nzval, "fg_nedelec_stiffness");
  });
  if (m) free_d(m, {dn});
  return st;
}

extern "C" fg_status fg_nedelec_tangent(fg_mesh *m, const double *dnu, const double *Bfield, const double *B,
                                        double *nzval) {
  double *a = nullptr, *b = nullptr, *c = nullptr;
  fg_status st = fg_guard([&]() -> fg_status {
    need_edge(m, "fg_nedelec_tangent");
    FG_REQUIRE(dnu && Bfield && B && nzval, FG_BAD_ARG, "fg_nedelec_tangent: null pointer");
    a = upload_d(m, dnu, (size_t)m->nt);
    b = upload_d(m, Bfield, 3 * (size_t)m->nt);
    c = upload_d(m, B, (size_t)m->nt);
    fg_nedelec_operator(m, nullptr, false, a, b, c, OUT_CSR, false);
    return export_nz(m, nzval, "fg_nedelec_tangent");
  });
  if (m) free_d(m, {a, b, c});
  return st;
}

extern "C" fg_status fg_nedelec_load(fg_mesh *m, const double *Bext, double *rhs) {
  double *d = nullptr;
  fg_status st = fg_guard([&]() -> fg_status {
    need_edge(m, "fg_nedelec_load");
    FG_REQUIRE(Bext && rhs, FG_BAD_ARG, "fg_nedelec_load: null pointer");
    FG_CUDA_TRY(cudaMallocAsync(&d, sizeof(double) * (size_t)m->nvp, m->stream));
    fg_nedelec_load_dev(m, Bext, d);
    FG_CUDA_TRY(cudaMemcpyAsync(rhs, d, sizeof(double) * (size_t)m->nv, cudaMemcpyDeviceToHost, m->stream));
    fg_sync(m);
    return FG_OK;
  });
  if (m) free_d(m, {d});
  return st;
}

extern "C" fg_status fg_nedelec_bfield(fg_mesh *m, const double *u, double *Bfield, double *B) {
  double *du = nullptr, *dB = nullptr, *dn = nullptr;
  fg_status st = fg_guard([&]() -> fg_status {
    need_edge(m, "fg_nedelec_bfield");
    FG_REQUIRE(u && Bfield, FG_BAD_ARG, "fg_nedelec_bfield: null pointer");
    du = upload_d(m, u, (size_t)m->nv);
    FG_CUDA_TRY(cudaMallocAsync(&dB, sizeof(double) * 3 * (size_t)m->nt, m->stream));
    FG_CUDA_TRY(cudaMallocAsync(&dn, sizeof(double) * (size_t)m->nt, m->stream));
    fg_nedelec_bfield_dev(m, du, dB, dn);
    FG_CUDA_TRY(cudaMemcpyAsync(Bfield, dB, sizeof(double) * 3 * (size_t)m->nt, cudaMemcpyDeviceToHost, m->stream));
    if (B) FG_CUDA_TRY(cudaMemcpyAsync(B, dn, sizeof(double) * (size_t)m->nt, cudaMemcpyDeviceToHost, m->stream));
    fg_sync(m);
    return FG_OK;
  });
  if (m) free_d(m, {du, dB, dn});
  return st;
}

extern "C" fg_status fg_nedelec_linear(fg_mesh *m, const double *nu, const double *Bext, double *u, double *Bfield,
                                       double *B, const fg_solve_opts *o, fg_solve_stats *s) {
  double *dn = nullptr, *drhs = nullptr, *du = nullptr, *dB = nullptr, *dBn = nullptr;
  int rc = 0;
  fg_status st = fg_guard([&]() -> fg_status {
    need_edge(m, "fg_nedelec_linear");
    FG_REQUIRE(Bext && u, FG_BAD_ARG, "fg_nedelec_linear: null pointer");
    fg_solve_opts opts;
    fg_solve_opts_default(&opts);
    if (o) opts = *o;
    const bool mixed = opts.precision == FG_MIXED;
    dn = upload_d(m, nu, (size_t)m->nt);
    FG_CUDA_TRY(cudaMallocAsync(&drhs, sizeof(double) * (size_t)m->nvp, m->stream));
    FG_CUDA_TRY(cudaMallocAsync(&du, sizeof(double) * (size_t)m->nvp, m->stream));
    FG_CUDA_TRY(cudaMemsetAsync(du, 0, sizeof(double) * (size_t)m->nvp, m->stream));
    FG_CUDA_TRY(cudaMemsetAsync(drhs, 0, sizeof(double) * (size_t)m->nvp, m->stream));
    cudaEvent_t e0, e1;
    FG_CUDA_TRY(cudaEventCreate(&e0));
    FG_CUDA_TRY(cudaEventCreate(&e1));
    FG_CUDA_TRY(cudaEventRecord(e0, m->stream));
    fg_nedelec_operator(m, dn, true, nullptr, nullptr, nullptr, OUT_SELL, mixed);
    fg_nedelec_load_dev(m, Bext, drhs);
    fg_solve_stats st0{};
    rc = solve_with_fallback(m, drhs, du, opts, &st0);
    if (Bfield) {
      FG_CUDA_TRY(cudaMallocAsync(&dB, sizeof(double) * 3 * (size_t)m->nt, m->stream));
      FG_CUDA_TRY(cudaMallocAsync(&dBn, sizeof(double) * (size_t)m->nt, m->stream));
      fg_nedelec_bfield_dev(m, du, dB, dBn);
    }
    FG_CUDA_TRY(cudaEventRecord(e1, m->stream));
    FG_CUDA_TRY(cudaMemcpyAsync(u, du, sizeof(double) * (size_t)m->nv, cudaMemcpyDeviceToHost, m->stream));
    if (Bfield) {
      FG_CUDA_TRY(cudaMemcpyAsync(Bfield, dB, sizeof(double) * 3 * (size_t)m->nt, cudaMemcpyDeviceToHost, m->stream));
      if (B) FG_CUDA_TRY(cudaMemcpyAsync(B, dBn, sizeof(double) * (size_t)m->nt, cudaMemcpyDeviceToHost, m->stream));
    }
    fg_sync(m);
    fg_check_flags(m, "fg_nedelec_linear");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (s) {
      *s = st0;
      s->ms = ms;
    }
    return rc == 0 ? FG_OK : FG_NOT_CONVERGED;
  });
  if (m) free_d(m, {dn, drhs, du, dB, dBn});
  return st;
}

extern "C" fg_status fg_nedelec_newton(fg_mesh *m, const double *Bext, const uint8_t *nonlinear,
                                       const double *nu_lin, const double *curve_B, const double *curve_nu,
                                       int32_t ncurve, double tol, int32_t max_newton, double min_step, double *u,
                                       double *Bfield, double *B, double *nu_out, int32_t *newton_iters,
                                       const fg_solve_opts *o, fg_solve_stats *s) {
  double *tab = nullptr, *dnl = nullptr, *dmask_d = nullptr;
  uint8_t *dmask = nullptr;
  unsigned long long *dmax = nullptr;
  int iters_done = 0;
  fg_status st = fg_guard([&]() -> fg_status {
    need_edge(m, "fg_nedelec_newton");
    FG_REQUIRE(Bext && nonlinear && curve_B && curve_nu && u, FG_BAD_ARG, "fg_nedelec_newton: null pointer");
    FG_REQUIRE(ncurve >= 4, FG_BAD_ARG, "fg_nedelec_newton: the B-nu curve needs at least 4 points");
    FG_REQUIRE(max_newton > 0 && tol >= 0.0, FG_BAD_ARG, "fg_nedelec_newton: need max_newton > 0, tol >= 0");
    std::vector<double> x(curve_B, curve_B + ncurve), y(curve_nu, curve_nu + ncurve);
    for (int i = 0; i + 1 < ncurve; ++i)
      FG_REQUIRE(x[i + 1] > x[i], FG_BAD_ARG, "fg_nedelec_newton: curve_B must increase");
    const std::vector<double> M1 = not_a_knot(x, y), yd = fd_gradient(x, y), M2 = not_a_knot(x, yd);
    std::vector<double> htab;
    for (const std::vector<double> *v : std::initializer_list<const std::vector<double> *>{&x, &y, &M1, &yd, &M2})
      htab.insert(htab.end(), v->begin(), v->end());
    fg_solve_opts opts;
    fg_solve_opts_default(&opts);
    if (o) opts = *o;
    const bool mixed = opts.precision == FG_MIXED;
    const int64_t ne = m->nv, nt = m->nt;
    tab = upload_d(m, htab.data(), htab.size());
    dnl = upload_d(m, nu_lin, (size_t)nt);
    FG_CUDA_TRY(cudaMallocAsync(&dmask, (size_t)nt, m->stream));
    FG_CUDA_TRY(cudaMemcpyAsync(dmask, nonlinear, (size_t)nt, cudaMemcpyHostToDevice, m->stream));
    FG_CUDA_TRY(cudaMallocAsync(&dmax, sizeof(unsigned long long), m->stream));
    // work vectors: the BiCGStab slots (unused on edge handles)
    for (int j = 0; j < 10; ++j)
      if (!m->bcg[j]) {
        m->bcg[j] = dev_alloc<double>(m, (size_t)m->nvp);
        FG_CUDA_TRY(cudaMemsetAsync(m->bcg[j], 0, sizeof(double) * (size_t)m->nvp, m->stream));
      }
    double *du_ = m->bcg[0], *r = m->bcg[1], *trial = m->bcg[2], *rhs = m->bcg[3], *uu = m->bcg[4];
    FG_CUDA_TRY(cudaMemsetAsync(uu, 0, sizeof(double) * (size_t)m->nvp, m->stream));
    FG_CUDA_TRY(cudaMemsetAsync(rhs, 0, sizeof(double) * (size_t)m->nvp, m->stream));
    // per-element fields: nu, dnu, B (3 x nt), |B|, |B| of the previous step
    FG_CUDA_TRY(cudaMallocAsync(&dmask_d, sizeof(double) * 7 * (size_t)nt, m->stream));
    double *nu = dmask_d, *dnu = nu + nt, *Bf = dnu + nt, *Bn = Bf + 3 * nt, *Bold = Bn + nt;
    FG_CUDA_TRY(cudaMemsetAsync(dmask_d, 0, sizeof(double) * 7 * (size_t)nt, m->stream));
    k_fill64_ned<<<grid_for(nt, 256), 256, 0, m->stream>>>(nt, 1.0, nu);   // nu = ones(nt) (nedelec3D.jl:142)
    if (dnl) {
      // elements outside the nonlinear set keep their given reluctance from the start
      k_ned_keep_linear<<<grid_for(nt, 256), 256, 0, m->stream>>>(nt, dmask, dnl, nu);
    }
    FG_LAUNCHED(dnl ? 2 : 1);
    if (!m->mval) m->mval = dev_alloc<double>(m, (size_t)m->nsell);
    cudaEvent_t e0, e1;
    FG_CUDA_TRY(cudaEventCreate(&e0));
    FG_CUDA_TRY(cudaEventCreate(&e1));
    FG_CUDA_TRY(cudaEventRecord(e0, m->stream));
    fg_nedelec_load_dev(m, Bext, rhs);
    int cg_iters = 0, status = 0;
    double residue = 0.0, div = INFINITY;
    while (div > tol && iters_done < max_newton) {
      ++iters_done;
      // A(nu) for the residuals, A(nu) + At for the correction (At from the second step)
      fg_nedelec_operator(m, nu, true, nullptr, nullptr, nullptr, OUT_SELL, mixed && iters_done == 1);
      FG_CUDA_TRY(cudaMemcpyAsync(m->mval, m->val64, sizeof(double) * (size_t)m->nsell, cudaMemcpyDeviceToDevice,
                                  m->stream));
      if (iters_done > 1) fg_nedelec_operator(m, nu, true, dnu, Bf, Bn, OUT_SELL, mixed);
      const double res_old = fg_residual_norm(m, m->mval, uu, rhs, r);
      FG_CUDA_TRY(cudaMemsetAsync(du_, 0, sizeof(double) * (size_t)m->nvp, m->stream));
      fg_solve_stats cs{};
      // an inner solve that stops short of rtol still gives a correction (the
      // reference's cg returns what it has as well); it is counted, not fatal
      if (solve_with_fallback(m, r, du_, opts, &cs) != 0) ++status;
      cg_iters += cs.iterations;
      // line search of src/FEM3D.jl:122-151 on ||RHS - A u||
      double alf = 1.0;
      k_ned_axpy<<<grid_for(ne, 256), 256, 0, m->stream>>>(ne, uu, alf, du_, trial);
      FG_LAUNCHED(1);
      residue = fg_residual_norm(m, m->mval, trial, rhs, r);
      while (residue > res_old && alf > min_step) {
        alf *= 0.9;
        k_ned_axpy<<<grid_for(ne, 256), 256, 0, m->stream>>>(ne, uu, alf, du_, trial);
        FG_LAUNCHED(1);
        residue = fg_residual_norm(m, m->mval, trial, rhs, r);
      }
      if (!(alf < min_step))
        FG_CUDA_TRY(cudaMemcpyAsync(uu, trial, sizeof(double) * (size_t)ne, cudaMemcpyDeviceToDevice, m->stream));
      fg_nedelec_bfield_dev(m, uu, Bf, Bn);
      k_ned_material<<<grid_for(nt, 256), 256, 0, m->stream>>>(nt, dmask, dnl, Bn, tab, ncurve, nu, dnu, m->flags);
      FG_CUDA_TRY(cudaMemsetAsync(dmax, 0, sizeof(unsigned long long), m->stream));
      k_ned_maxdiff<<<grid_for(nt, 256), 256, 0, m->stream>>>(nt, Bn, Bold, dmax);
      FG_CUDA_TRY(cudaGetLastError());
      FG_LAUNCHED(2);
      unsigned long long bits = 0;
      FG_CUDA_TRY(cudaMemcpyAsync(&bits, dmax, sizeof(bits), cudaMemcpyDeviceToHost, m->stream));
      fg_sync(m);
      fg_check_flags(m, "fg_nedelec_newton");
      std::memcpy(&div, &bits, sizeof(div));
    }
    FG_CUDA_TRY(cudaEventRecord(e1, m->stream));
    FG_CUDA_TRY(cudaMemcpyAsync(u, uu, sizeof(double) * (size_t)ne, cudaMemcpyDeviceToHost, m->stream));
    if (Bfield) FG_CUDA_TRY(cudaMemcpyAsync(Bfield, Bf, sizeof(double) * 3 * (size_t)nt, cudaMemcpyDeviceToHost, m->stream));
    if (B) FG_CUDA_TRY(cudaMemcpyAsync(B, Bn, sizeof(double) * (size_t)nt, cudaMemcpyDeviceToHost, m->stream));
    if (nu_out) FG_CUDA_TRY(cudaMemcpyAsync(nu_out, nu, sizeof(double) * (size_t)nt, cudaMemcpyDeviceToHost, m->stream));
    fg_sync(m);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (newton_iters) *newton_iters = iters_done;
    const bool conv = div <= tol;
    if (s) {
      s->iterations = cg_iters;
      s->refinements = iters_done;
      s->converged = conv;
      s->pad_ = status;  // inner solves that stopped short of rtol
      s->relres = residue;
      s->ms = ms;
    }
    return conv ? FG_OK : FG_NOT_CONVERGED;
  });
  if (m) {
    free_d(m, {tab, dnl, dmask_d});
    if (dmask) cudaFreeAsync(dmask, m->stream);
    if (dmax) cudaFreeAsync(dmax, m->stream);
  }
  return st;
}
