// Heat transport with convection on P2 tetrahedra (Transport/main3D.jl:143-213) and
// P2 triangles (Transport/main2D.jl:150-190, with the 2D matrices of src/FEM2D.jl):
// intake faces carry a penalty boundary mass R (src/FEM3D.jl:300-322), and every step
// solves the backward-Euler system
//   LM T_{n+1} = M T_n,   LM = M(rho_cp) + dt (A(kappa) + R + C(u, rho_cp))
// (main3D.jl:199-204).  M, A and C are the P2 mass, stiffness and convection matrices
// of src/FEM3D.jl:494-648.  LM is constant, so it is assembled once (SELL values and
// Jacobi inverse) with M kept beside it; each step is one SpMV for M T_n and one
// Jacobi-BiCGStab solve from T_n.  The reference solves with a direct factorisation;
// BiCGStab stops at ||M T_n - LM T|| <= rtol ||M T_n||.
#include "fg_common.cuh"

#include <vector>

namespace {

// Host-side incidence of the faces that carry a nonzero factor: the distinct nodes
// they touch (rows) and, per row, its (face << 3 | face-local node) entries in face
// order.  faces is fw x nf column-major, 0-based (fw = 6: P2 triangles of a
// tetrahedral mesh, 3: P2 lines of a triangle mesh).
struct FaceRows {
  std::vector<int> rows, fptr, flist;
};

FaceRows face_rows(const int32_t *faces, int fw, const double *AE, const double *F, int64_t nf, int64_t nv) {
  FaceRows fr;
  std::vector<int> count((size_t)nv, 0), slot((size_t)nv, -1);
  for (int64_t s = 0; s < nf; ++s) {
    if (AE[s] * F[s] == 0.0) continue;
    for (int i = 0; i < fw; ++i) {
      const int64_t v = faces[fw * s + i];
      FG_REQUIRE(v >= 0 && v < nv, FG_BAD_ARG, "boundary faces: node index out of range");
      for (int j = 0; j < i; ++j)
        FG_REQUIRE(faces[fw * s + j] != v, FG_BAD_ARG, "boundary faces: a face repeats a node");
      ++count[(size_t)v];
    }
  }
  fr.fptr.push_back(0);
  for (int64_t v = 0; v < nv; ++v)
    if (count[(size_t)v]) {
      slot[(size_t)v] = (int)fr.rows.size();
      fr.rows.push_back((int)v);
      fr.fptr.push_back(fr.fptr.back() + count[(size_t)v]);
    }
  fr.flist.resize((size_t)fr.fptr.back());
  std::vector<int> cur(fr.fptr.begin(), fr.fptr.end() - 1);
  for (int64_t s = 0; s < nf; ++s) {
    if (AE[s] * F[s] == 0.0) continue;
    FG_REQUIRE(s < (1 << 28), FG_BAD_ARG, "boundary faces: too many faces");
    for (int i = 0; i < fw; ++i) fr.flist[(size_t)cur[(size_t)slot[(size_t)faces[fw * s + i]]]++] = (int)(s << 3 | i);
  }
  return fr;
}

// Uploads the face lists into stream-ordered temporaries (freed with the mesh pool).
struct FaceDev {
  int *rows = nullptr, *fptr = nullptr, *flist = nullptr, *faces = nullptr;
  double *AE = nullptr, *F = nullptr;
  int64_t nrows = 0;
};

template <typename T>
T *upload(fg_mesh *m, const T *h, size_t n) {
  T *d = nullptr;
  FG_CUDA_TRY(cudaMallocAsync(&d, sizeof(T) * (n ? n : 1), m->stream));
  if (n) FG_CUDA_TRY(cudaMemcpyAsync(d, h, sizeof(T) * n, cudaMemcpyHostToDevice, m->stream));
  return d;
}

FaceDev face_upload(fg_mesh *m, const FaceRows &fr, const int32_t *faces, int fw, const double *AE, const double *F,
                    int64_t nf) {
  FaceDev d;
  d.nrows = (int64_t)fr.rows.size();
  d.rows = upload(m, fr.rows.data(), fr.rows.size());
  d.fptr = upload(m, fr.fptr.data(), fr.fptr.size());
  d.flist = upload(m, fr.flist.data(), fr.flist.size());
  d.faces = upload(m, faces, (size_t)fw * (size_t)nf);
  d.AE = upload(m, AE, (size_t)nf);
  d.F = upload(m, F, (size_t)nf);
  return d;
}

void face_free(fg_mesh *m, FaceDev &d) {
  for (void *p : {(void *)d.rows, (void *)d.fptr, (void *)d.flist, (void *)d.faces, (void *)d.AE, (void *)d.F})
    if (p) cudaFreeAsync(p, m->stream);
  d = FaceDev{};
}

}  // namespace

extern "C" fg_status fg_boundary_mass(fg_mesh *m, const int32_t *faces, const double *AE, const double *F,
                                      int64_t nfaces, double *nzval) {
  FaceDev d;
  fg_status st = fg_guard([&]() -> fg_status {
    FG_REQUIRE(m && nzval && (nfaces == 0 || (faces && AE)), FG_BAD_ARG, "fg_boundary_mass: null pointer");
    FG_REQUIRE(!m->edge && (m->npe == 10 || m->npe == 6), FG_UNSUPPORTED,
               "fg_boundary_mass: P2 tetrahedra (src/FEM3D.jl:300-322) or P2 triangles (src/FEM2D.jl:394-419)");
    const int fw = m->npe == 10 ? 6 : 3;
    std::vector<double> ones;
    if (!F) {
      ones.assign((size_t)nfaces, 1.0);
      F = ones.data();
    }
    const FaceRows fr = face_rows(faces, fw, AE, F, nfaces, m->nv);
    if (!m->csrval) m->csrval = dev_alloc<double>(m, (size_t)m->nnz);
    FG_CUDA_TRY(cudaMemsetAsync(m->csrval, 0, sizeof(double) * (size_t)m->nnz, m->stream));
    d = face_upload(m, fr, faces, fw, AE, F, nfaces);
    fg_face_mass(m, false, d.rows, d.nrows, d.fptr, d.flist, d.faces, d.AE, d.F, 1.0);
    FG_CUDA_TRY(cudaMemcpyAsync(nzval, m->csrval, sizeof(double) * (size_t)m->nnz, cudaMemcpyDeviceToHost, m->stream));
    fg_sync(m);
    fg_check_flags(m, "fg_boundary_mass");
    return FG_OK;
  });
  if (m) face_free(m, d);
  return st;
}

extern "C" fg_status fg_transport_be(fg_mesh *m, const double *rho_cp, const double *kappa, const double *vel,
                                     const int32_t *faces, const double *AE, const double *F, int64_t nfaces,
                                     double dt, int32_t nsteps, int32_t full_phi, double *T, int32_t every,
                                     double *snapshots, const fg_solve_opts *o, fg_solve_stats *s) {
  FaceDev fd;
  double *tmp[4] = {nullptr, nullptr, nullptr, nullptr};
  // created outside the guarded body so that the cleanup below also runs when the
  // body leaves early with an error
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  fg_status st = fg_guard([&]() -> fg_status {
    FG_REQUIRE(m && rho_cp && kappa && vel && T, FG_BAD_ARG, "fg_transport_be: null pointer");
    FG_REQUIRE(nfaces == 0 || (faces && AE && F), FG_BAD_ARG, "fg_transport_be: null face arrays");
    FG_REQUIRE(!m->edge && (m->npe == 10 || m->npe == 6), FG_UNSUPPORTED,
               "fg_transport_be: P2 tetrahedra or P2 triangles only");
    const int fw = m->npe == 10 ? 6 : 3;
    FG_REQUIRE(dt > 0.0 && nsteps >= 0 && nfaces >= 0, FG_BAD_ARG, "fg_transport_be: need dt > 0, nsteps >= 0");
    FG_REQUIRE(!snapshots || every > 0, FG_BAD_ARG, "fg_transport_be: snapshots need every > 0");
    fg_solve_opts opts;
    fg_solve_opts_default(&opts);
    if (o) opts = *o;
    const int64_t nv = m->nv, nt = m->nt;
    // per-element factors: rho_cp (M), dt kappa (A), dt rho_cp (C)
    std::vector<double> kdt((size_t)nt), fdt((size_t)nt);
    for (int64_t k = 0; k < nt; ++k) {
      kdt[(size_t)k] = dt * kappa[k];
      fdt[(size_t)k] = dt * rho_cp[k];
    }
    tmp[0] = upload(m, rho_cp, (size_t)nt);
    tmp[1] = upload(m, kdt.data(), (size_t)nt);
    tmp[2] = upload(m, fdt.data(), (size_t)nt);
    tmp[3] = upload(m, vel, 3 * (size_t)nv);
    FG_CUDA_TRY(cudaEventCreate(&e0));
    FG_CUDA_TRY(cudaEventCreate(&e1));
    FG_CUDA_TRY(cudaEventRecord(e0, m->stream));
    fg_transport_operator(m, tmp[0], tmp[1], tmp[3], tmp[2], full_phi);
    if (nfaces > 0) {
      const FaceRows fr = face_rows(faces, fw, AE, F, nfaces, nv);
      fd = face_upload(m, fr, faces, fw, AE, F, nfaces);
      fg_face_mass(m, true, fd.rows, fd.nrows, fd.fptr, fd.flist, fd.faces, fd.AE, fd.F, dt);
    }
    fg_check_flags(m, "fg_transport_be");
    // T lives in the solver's x vector; b = M T in its right-hand side vector
    fg_solve_stats st0{};
    double *d_T = nullptr, *d_b = nullptr;
    {
      // allocate the solver vectors (a zero-iteration call would also do; keep it explicit)
      for (int j = 0; j < 10; ++j)
        if (!m->bcg[j]) {
          m->bcg[j] = dev_alloc<double>(m, (size_t)m->nvp);
          FG_CUDA_TRY(cudaMemsetAsync(m->bcg[j], 0, sizeof(double) * (size_t)m->nvp, m->stream));
        }
      d_T = m->bcg[0];
      d_b = m->bcg[9];
    }
    FG_CUDA_TRY(cudaMemcpyAsync(d_T, T, sizeof(double) * (size_t)nv, cudaMemcpyHostToDevice, m->stream));
    int iters = 0, status = 0, snap = 0;
    double relres = 0.0;
    for (int step = 1; step <= nsteps; ++step) {
      fg_spmv64_plain(m, m->mval, d_T, d_b);
      const int rc = fg_bicgstab_solve(m, d_b, d_T, opts, &st0);
      iters += st0.iterations;
      relres = st0.relres;
      if (rc != 0 && status == 0) status = rc;
      if (snapshots && step % every == 0) {
        FG_CUDA_TRY(cudaMemcpyAsync(snapshots + (size_t)snap * nv, d_T, sizeof(double) * (size_t)nv,
                                    cudaMemcpyDeviceToHost, m->stream));
        ++snap;
      }
    }
    FG_CUDA_TRY(cudaEventRecord(e1, m->stream));
    FG_CUDA_TRY(cudaMemcpyAsync(T, d_T, sizeof(double) * (size_t)nv, cudaMemcpyDeviceToHost, m->stream));
    fg_sync(m);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (s) {
      s->iterations = iters;
      s->refinements = 0;
      s->converged = status == 0;
      s->pad_ = status;
      s->relres = relres;
      s->ms = ms;
    }
    return status == 0 ? FG_OK : FG_NOT_CONVERGED;
  });
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (m) {
    face_free(m, fd);
    for (double *p : tmp)
      if (p) cudaFreeAsync(p, m->stream);
  }
  return st;
}
