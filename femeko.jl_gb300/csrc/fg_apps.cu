// One-shot entry points shaped like the reference's ccall boundary, and kernel
// timing used by the benchmark's roofline report.
#include <algorithm>
#include <cmath>
#include <vector>

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
//   which = 5: the same with the Jacobian;
//   which = 7: P1 stiffness assembly K(mu) at the handle's current permeabilities into
//              the FP64 and FP32 SELL operator with its Jacobi diagonals (one pass,
//              rows gather their elements' entries);
//   which = 8: the same through element records and a row sum (the two-pass form);
//   which = 9: the one-block kernel that finishes the dot products of the
//              split-reduction FP32 variants (which = 0 times their SpMV alone).
fg_status fg_bench_cg_kernel(fg_mesh *m, int which, int precision, int reps, double *ms_per_launch);

extern "C" fg_status fg_bench_kernel(fg_mesh *m, int32_t which, int32_t precision, int32_t reps,
                                     double *ms_per_launch) {
  return fg_guard([&]() -> fg_status {
    FG_REQUIRE(m && ms_per_launch && reps > 0, FG_BAD_ARG, "fg_bench_kernel: bad argument");
    if (which == 0 || which == 1 || which == 3 || which == 6 || which == 9)
      return fg_bench_cg_kernel(m, which, precision, reps, ms_per_launch);
    if (which == 7 || which == 8) {
      FG_REQUIRE(m->npe == 4 && !m->edge && m->mu, FG_BAD_ARG,
                 "fg_bench_kernel: assembly timing needs a P1 tetrahedron handle after a solve");
      m->asm_two_pass = (which == 8);
      auto once = [&]() {
        fg_assemble_operator(m, ASM_STIFF, m->mu, nullptr, nullptr, 0.0, 0.0, 0, OUT_SELL, true, true, true);
      };
      once();
      FG_CUDA_TRY(cudaEventRecord(m->ev0, m->stream));
      for (int r = 0; r < reps; ++r) once();
      FG_CUDA_TRY(cudaEventRecord(m->ev1, m->stream));
      fg_sync(m);
      m->asm_two_pass = false;
      float ms = 0.f;
      FG_CUDA_TRY(cudaEventElapsedTime(&ms, m->ev0, m->ev1));
      *ms_per_launch = ms / reps;
      return FG_OK;
    }
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

// ------------------------------------------------------------------ right-hand sides
// src/FEM3D.jl:274-281 lagrange: C_i = sum over the elements of node i of VE/4, as
// vector records summed per row in a fixed order.
__global__ void k_lagrange_tet4(int64_t nt, const double *__restrict__ geo, const int *__restrict__ recpos,
                                double *__restrict__ rec_r) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nt) return;
  const double q = 0.25 * geo[12 * nt + k];
#pragma unroll
  for (int a = 0; a < 4; ++a) rec_r[recpos[(int64_t)a * nt + k]] = q;
}

extern "C" fg_status fg_lagrange(fg_mesh *m, double *C) {
  return fg_guard([&]() -> fg_status {
    FG_REQUIRE(m && C, FG_BAD_ARG, "fg_lagrange: null pointer");
    FG_REQUIRE(m->npe == 4, FG_UNSUPPORTED, "fg_lagrange: P1 tetrahedra only");
    fg_ensure_records(m);
    k_lagrange_tet4<<<grid_for(m->nt, 256), 256, 0, m->stream>>>(m->nt, m->geo, m->recpos, m->rec_r);
    FG_CUDA_TRY(cudaGetLastError());
    FG_LAUNCHED(1);
    if (!m->v64[15]) m->v64[15] = dev_alloc<double>(m, (size_t)m->nvp);
    fg_vector_gather(m, m->v64[15]);
    FG_CUDA_TRY(cudaMemcpyAsync(C, m->v64[15], sizeof(double) * (size_t)m->nv, cudaMemcpyDeviceToHost, m->stream));
    fg_sync(m);
    return FG_OK;
  });
}

// src/FEM3D.jl:284-297 BoundaryIntegral: RHS[face nodes] += (n . F) AE / 3 over the
// boundary faces whose id is in shell_id.  Per face value, then per node the sum
// over its faces in face order (a node -> face list built on the host).
// With AE == NULL the face area is computed from the node coordinates p (3 x np), as
// areaTriangle does in the C++ reference (src/FEMc.cpp:44-53): |AB x AC| / 2.
__global__ void k_face_flux(int64_t ns, const int *__restrict__ sT, const double *__restrict__ normal,
                            const double *__restrict__ AE, const double *__restrict__ p, double F0, double F1,
                            double F2, const int *__restrict__ shell, int nshell, double *__restrict__ v) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= ns) return;
  const int id = sT[4 * s + 3];
  bool hit = false;
  for (int q = 0; q < nshell; ++q) hit |= (id == shell[q]);
  double area = 0.0;
  if (hit) {
    if (AE) {
      area = AE[s];
    } else {
      const double *a = p + 3 * (int64_t)sT[4 * s], *b = p + 3 * (int64_t)sT[4 * s + 1],
                   *c = p + 3 * (int64_t)sT[4 * s + 2];
      const double ab[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
      const double ac[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
      const double cx = ab[1] * ac[2] - ab[2] * ac[1], cy = ab[2] * ac[0] - ab[0] * ac[2],
                   cz = ab[0] * ac[1] - ab[1] * ac[0];
      area = 0.5 * sqrt(cx * cx + cy * cy + cz * cz);
    }
  }
  v[s] = hit ? (normal[3 * s] * F0 + normal[3 * s + 1] * F1 + normal[3 * s + 2] * F2) * area / 3.0 : 0.0;
}

__global__ void k_node_faces(int64_t nv, const int *__restrict__ ptr, const int *__restrict__ face,
                             const double *__restrict__ v, double *__restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  double acc = 0.0;
  for (int q = ptr[i]; q < ptr[i + 1]; ++q) acc += v[face[q]];
  out[i] = acc;
}

// Device form of the boundary integral: writes all nv entries of d_out (device).
// AE may be NULL: the face areas then come from the mesh's coordinates.
void fg_boundary_rhs_dev(fg_mesh *m, const int32_t *surfaceT, int64_t ns, int32_t index_base, const double *normal,
                         const double *AE, const double *F, const int32_t *shell_id, int32_t nshell,
                         double *d_out) {
  FG_REQUIRE(F && (ns == 0 || (surfaceT && normal)), FG_BAD_ARG, "boundary integral: null pointer");
  FG_REQUIRE(ns >= 0 && nshell >= 0 && (nshell == 0 || shell_id), FG_BAD_ARG, "boundary integral: bad sizes");
  FG_REQUIRE(index_base == 0 || index_base == 1, FG_BAD_ARG, "boundary integral: index_base must be 0 or 1");
  const int64_t nv = m->nv;
  // node -> faces (face order), 0-based copy of the faces
  std::vector<int> st((size_t)4 * ns), cnt((size_t)nv + 1, 0);
  for (int64_t s = 0; s < ns; ++s) {
    for (int a = 0; a < 3; ++a) {
      const int64_t node = (int64_t)surfaceT[4 * s + a] - index_base;
      FG_REQUIRE(node >= 0 && node < nv, FG_BAD_MESH, "boundary integral: face node out of range");
      st[4 * s + a] = (int)node;
      ++cnt[node + 1];
    }
    st[4 * s + 3] = surfaceT[4 * s + 3];
  }
  for (int64_t i = 0; i < nv; ++i) cnt[i + 1] += cnt[i];
  std::vector<int> face((size_t)3 * ns), fill(cnt.begin(), cnt.end() - 1);
  for (int64_t s = 0; s < ns; ++s)
    for (int a = 0; a < 3; ++a) face[fill[st[4 * s + a]]++] = (int)s;
  // device work space for this call, from the stream-ordered pool
  StreamScratch scratch{m->stream, {}};
  auto dmalloc = [&](size_t bytes) {
    return static_cast<void *>(scratch.get<unsigned char>(std::max<size_t>(bytes, 16)));
  };
  int *d_st = (int *)dmalloc(sizeof(int) * st.size()), *d_ptr = (int *)dmalloc(sizeof(int) * cnt.size());
  int *d_face = (int *)dmalloc(sizeof(int) * face.size()), *d_shell = (int *)dmalloc(sizeof(int) * (nshell + 1));
  double *d_n = (double *)dmalloc(sizeof(double) * 3 * ns);
  double *d_ae = AE ? (double *)dmalloc(sizeof(double) * ns) : nullptr;
  double *d_v = (double *)dmalloc(sizeof(double) * ns);
  auto up = [&](void *dst, const void *src, size_t bytes) {
    if (bytes) FG_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, m->stream));
  };
  up(d_st, st.data(), sizeof(int) * st.size());
  up(d_ptr, cnt.data(), sizeof(int) * cnt.size());
  up(d_face, face.data(), sizeof(int) * face.size());
  up(d_shell, shell_id, sizeof(int) * nshell);
  up(d_n, normal, sizeof(double) * 3 * ns);
  if (AE) up(d_ae, AE, sizeof(double) * ns);
  if (ns > 0) {
    k_face_flux<<<grid_for(ns, 256), 256, 0, m->stream>>>(ns, d_st, d_n, d_ae, m->p, F[0], F[1], F[2], d_shell,
                                                          nshell, d_v);
    FG_LAUNCHED(1);
  }
  k_node_faces<<<grid_for(nv, 256), 256, 0, m->stream>>>(nv, d_ptr, d_face, d_v, d_out);
  FG_LAUNCHED(1);
  FG_CUDA_TRY(cudaGetLastError());
}

extern "C" fg_status fg_boundary_integral(fg_mesh *m, const int32_t *surfaceT, int64_t ns, int32_t index_base,
                                          const double *normal, const double *AE, const double *F,
                                          const int32_t *shell_id, int32_t nshell, double *RHS) {
  double *d_out = nullptr;
  fg_status st = fg_guard([&]() -> fg_status {
    FG_REQUIRE(m && RHS && F && (ns == 0 || (surfaceT && normal && AE)), FG_BAD_ARG,
               "fg_boundary_integral: null pointer");
    FG_CUDA_TRY(cudaMalloc(&d_out, sizeof(double) * (size_t)std::max<int64_t>(m->nv, 1)));
    fg_boundary_rhs_dev(m, surfaceT, ns, index_base, normal, AE, F, shell_id, nshell, d_out);
    FG_CUDA_TRY(cudaMemcpyAsync(RHS, d_out, sizeof(double) * m->nv, cudaMemcpyDeviceToHost, m->stream));
    fg_sync(m);
    return FG_OK;
  });
  if (d_out) cudaFree(d_out);
  return st;
}
