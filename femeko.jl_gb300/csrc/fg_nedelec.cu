// Nedelec (Whitney) edge elements for the vector-potential magnetostatics of
// Magnetostatics/nedelec3D.jl: the element blocks of src/FEM3D.jl:155-191, the global
// curl-curl and tangential matrices over the edge unknowns (:172-182, src/FEM3D.jl:
// 194-271), the load vector of an applied flux density (:106-139), B per element from
// the edge values (:190-221) and the first (linear) solve A(nu) u = RHS
// (du = cg(A + At, RHS - A u) at :185 with u = 0 and At = 0).  The handle comes from
// fg_edge_mesh_create: its matrix rows are the edges (the reference's
// edge2localMap[t[5:10, k]]), its geometry the P1 vertex tetrahedra.
#include "fg_common.cuh"

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
    rc = fg_pcg_solve(m, drhs, du, opts, &st0, false);
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
