/*
 * femeko_gpu.h -- C ABI of libfemeko_gpu.so, the GB300 (sm_103a) engine for
 * Femeko's FEM hot path: P1/P2 tetrahedral and triangle assembly, the nonlinear
 * permeability / Newton-tangent rebuild, and the sparse CG solve.
 *
 * Conventions
 *  - Plain pointers and sizes only.  Host pointers are caller-owned and are read
 *    or written before the call returns.  Device memory is owned by the handle.
 *  - Arrays use Julia's column-major layouts: p is 3 x nv (p[3*i + c]),
 *    t is npe x nt (t[npe*k + a]), H is 3 x nt.  index_base (0 or 1) lets Julia
 *    pass mesh.t (Int32, 1-based) without a copy.
 *  - Sparse matrices are SparseMatrixCSC-compatible: colptr (nv+1), rowval (nnz),
 *    nzval (nnz), rows sorted within each column.  Every matrix here is
 *    symmetric, so the same arrays are also its CSR form.
 *  - Every function returns an fg_status; nothing throws across the ABI.
 *    fg_last_error() describes the last failure on the calling thread.
 *  - One handle per thread; calls on one handle are serialised on its stream.
 *
 * Reference interfaces each entry point replaces are cited as file:line of the
 * Femeko.jl repository.
 */
#ifndef FEMEKO_GPU_H
#define FEMEKO_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum fg_status {
  FG_OK = 0,
  FG_NOT_CONVERGED = 1, /* iteration cap reached; outputs hold the last iterate */
  FG_NAN = 2,           /* a NaN/Inf appeared (Magnetostatics/NewtonRaphson.jl:210-212) */
  FG_BAD_ARG = 3,
  FG_BAD_MESH = 4,      /* node index out of range, degenerate element, row too long */
  FG_CUDA = 5,
  FG_NO_DEVICE = 6,
  FG_UNSUPPORTED = 7
} fg_status;

/* element kinds = nodes per element */
enum { FG_TRI3 = 3, FG_TET4 = 4, FG_TRI6 = 6, FG_TET10 = 10 };
/* precision of a solve */
enum { FG_FP64 = 0, FG_MIXED = 1 };
/* Newton step control */
enum {
  FG_LS_NONE = 0,      /* full step */
  FG_LS_REFERENCE = 1, /* src/FEM3D.jl:123-152: backtracking on ||RHS - A(u+a du)|| with the frozen secant A */
  FG_LS_RESIDUAL = 2,  /* same backtracking rule on the true nonlinear residual */
  FG_LS_QUADRATIC = 3  /* true residual, next step from the minimiser of a quadratic fit
                          of |F(u + a du)|^2, kept in [0.1, 0.5] of the last step */
};
/* FP32 CG iteration kernel: FG_SPMV_AUTO lets the autotuner time the variants on
 * the first mixed solve of a handle and keep the fastest; k = 1..29 forces variant
 * k-1.  One fused kernel per iteration: 1: 4x-unrolled gather loop, 256 threads;
 * 2: all row loads issued first, 256 threads; 3: loop, 128 threads; 4: loop, 512
 * threads; 5: halo staging (the neighbour entries of a block of rows gathered once
 * into shared memory); 6: halo staging, persistent and software-pipelined (bulk
 * copies and asynchronous gathers of the next row blocks).  Two kernels per
 * iteration (vector pass + SpMV): 7: direct gathers; 8: halo staging; 9: direct
 * gathers in a persistent grid (each block walks several row blocks); 10: 9 with
 * programmatic dependent launch between the two kernels; 11: 15 with the matrix
 * values kept in a persisting-L2 window (the process's context sets aside L2 for
 * them while a handle uses this variant); 12-16: 9 with 4, 3, 5, 6 and 7 blocks per
 * SM; 17: plain CG on the symmetrically Jacobi-scaled system D^-1/2 A D^-1/2 (the
 * same iterates as Jacobi-PCG, no preconditioned-residual vector, the same stopping
 * test on the unscaled residual) with the SpMV of 15; 18-20: 9 with 4, 3 and 2
 * blocks per SM and the matrix entries of each block's next 256 rows copied into a
 * second shared-memory stage by the bulk-copy engine while it computes the current
 * ones (available where two stages fit in shared memory); 21: 17 with its scaled
 * values in the persisting-L2 window; 22: 18 with the values in the window;
 * 23, 24: 18 and 19 with each block of the SpMV leaving its partial dot products and
 * a one-block kernel adding them (no arrival chain at the end of the SpMV);
 * 25, 26: pipelined Jacobi-PCG (Ghysels-Vanroose): the dot products of an iteration
 * come from the previous vector pass and one block of the bulk-staged SpMV (4 or 3
 * blocks per SM) finishes their sum while the other blocks multiply, so no kernel
 * ends with a grid-wide reduction.  25 and 26 are timed by the autotuner but never
 * chosen by it (their FP32 recurrences stall above tolerances near 1e-6 and diverge
 * on singular systems): they run only when forced; 27: the iteration of 23 run by ONE
 * persistent cooperative launch for up to 1024 iterations (grid barriers in place of
 * kernel boundaries; the last block at the closing barrier adds the dot products;
 * each block's matrix entries prefetched across the barriers); 28, 29: 23 and 24 with
 * the partials added by the last SpMV block to arrive (one arrival counter) instead of
 * a separate one-block kernel: the same iterates, one launch fewer per iteration.
 * The autotuner times each variant through the solver's own graph loop (64
 * iterations after an untimed run) and keeps the fastest; a variant with an L2
 * window (11, 21, 22), which sets L2 aside for the whole context, only when it is
 * more than 5 % faster than every variant without one; the Jacobi-scaled ones (17,
 * 21) are timed but not kept (in FP32 their iterates need more iterations); within
 * 1.5 % of the fastest, 23, 24, 28 or 29 is kept. */
enum { FG_SPMV_AUTO = 0 };

typedef struct fg_mesh fg_mesh;

typedef struct fg_solve_opts {
  int32_t precision;   /* FG_FP64 or FG_MIXED (FP32 matrix/vectors, FP64 refinement) */
  double rtol;         /* FP64 relative residual target ||b - A x|| <= rtol ||b - A x0|| */
  int32_t maxiter;     /* cap on CG iterations (inner iterations in total) */
  double inner_rtol;   /* mixed: FP32 PCG target per refinement step */
  int32_t check_every; /* iterations between convergence checks (even) */
  int32_t use_graph;   /* 1: the whole CG as one CUDA graph launch (a WHILE node around
                          check_every iterations, the test on the device); 2: a graph of
                          check_every iterations per launch, tested on the host; 0: no graph */
  int32_t spmv;        /* FG_SPMV_AUTO or a forced variant 1..29 */
  int32_t reserved_;
} fg_solve_opts;

typedef struct fg_solve_stats {
  int32_t iterations;  /* CG iterations (all refinement steps) */
  int32_t refinements; /* FP64 refinement steps (mixed) */
  int32_t converged;
  int32_t pad_;
  double relres;       /* final FP64 relative residual */
  double ms;           /* device time of the solve (CUDA events) */
} fg_solve_stats;

typedef struct fg_newton_opts {
  int32_t precision;   /* inner CG precision: FG_FP64 or FG_MIXED */
  int32_t maxit;       /* Newton iteration cap (Magnetostatics/NewtonRaphson.jl:38: 100) */
  double tol_update;   /* stop when ||a du|| <= tol_update ||u|| */
  double inner_rtol;   /* relative residual of each inner (increment) solve */
  int32_t cg_maxiter;  /* inner CG cap per Newton step */
  int32_t line_search; /* FG_LS_* */
  double min_step;     /* smallest accepted step (src/FEM3D.jl:123: 1e-4) */
  double Ms, Hk;       /* Froehlich law mu(H) = mu0 (1 + Ms/(Hk + |H|)) */
  int32_t check_every;
  int32_t use_graph;
  int32_t forcing;     /* inner tolerance: FG_FORCING_FIXED (inner_rtol) or
                          FG_FORCING_EW (Eisenstat-Walker, clamped to [eta_min, eta_max]) */
  int32_t picard_steps; /* first iterations without the tangent term (secant/Picard
                           steps; the reference's first iteration is one,
                           Magnetostatics/NewtonRaphson.jl:164-168) */
  double eta_min, eta_max;  /* defaults 1e-2 and 0.3 */
} fg_newton_opts;

/* inner-tolerance (forcing term) rules of the Newton solver */
enum { FG_FORCING_FIXED = 0, FG_FORCING_EW = 1 };

typedef struct fg_newton_stats {
  int32_t newton_iters;
  int32_t cg_iters;
  int32_t converged;
  int32_t trials;      /* line-search trials in total */
  double update_ratio; /* last ||a du|| / ||u|| */
  double residual;     /* last ||F|| on free rows */
  double alpha;        /* last accepted step */
  double energy;       /* integral of H dB (src/magneticProperties.jl:252-309, closed form) */
  double ms;           /* device time of the solve */
  double setup_ms;     /* of which: the linear elements' operator and the first residual */
  double cg_ms;        /* of which: the inner CG solves */
} fg_newton_stats;

/* Defaults matching the reference behaviour / the published path settings. */
void fg_solve_opts_default(fg_solve_opts *o);
void fg_newton_opts_default(fg_newton_opts *o);

const char *fg_last_error(void);
int32_t fg_version(void);
/* Name and SM count of the current CUDA device. */
fg_status fg_device_info(char *name, int32_t name_len, int32_t *sm_count);

/* ---------------------------------------------------------------------- mesh */
/* Uploads a mesh and builds, once, the structural CSR pattern (all element node
 * pairs, as the single sparse(I,J,V) of Magnetostatics/NewtonRaphson.jl:161),
 * the element-to-slot map and the P1 geometry.  Replaces the index work of
 * Magnetostatics/NewtonRaphson.jl:115-127 and the per-call abcd solves of
 * src/FEM3D.jl:5-17.  nodes_per_elem: 4 (P1 tet), 3 (P1 tri), 10 (P2 tet),
 * 6 (P2 tri).  p is 3 x nv (z ignored for triangles). */
fg_status fg_mesh_create(const double *p, int64_t nv, const int32_t *t, int64_t nt, int32_t nodes_per_elem,
                         int32_t index_base, fg_mesh **out);
/* A handle whose unknowns are the edges of a tetrahedral mesh (Nedelec elements,
 * Magnetostatics/nedelec3D.jl): t (4 x nt) the vertices into the nv points p, edges
 * (6 x nt) each element's edge unknowns 0..ne-1 (the reference's
 * edge2localMap[t[5:10, k]], src/mesh.jl:168-183), local edge e joining local vertices
 * (1,2), (2,3), (3,1), (4,1), (3,4), (2,4) (src/mesh.jl:603-630).  The pattern,
 * records and solvers of the handle run over the ne edges; only the fg_nedelec_*
 * assembly entry points accept it. */
fg_status fg_edge_mesh_create(const double *p, int64_t nv, const int32_t *t, const int32_t *edges, int64_t nt,
                              int64_t ne, int32_t index_base, fg_mesh **out);
fg_status fg_mesh_destroy(fg_mesh *m);
/* nnz of the structural pattern and the longest row. */
fg_status fg_mesh_nnz(const fg_mesh *m, int64_t *nnz, int32_t *max_row);
/* Dirichlet rows (fixed[i] != 0); NULL clears. */
fg_status fg_mesh_set_dirichlet(fg_mesh *m, const uint8_t *fixed);
/* Element volumes (areas for triangles): src/mesh.jl:484-505 elementVolume. */
fg_status fg_mesh_volumes(fg_mesh *m, double *VE);
/* Pattern in SparseMatrixCSC form (colptr nv+1, rowval nnz) with the given base. */
fg_status fg_csc_pattern(const fg_mesh *m, int64_t *colptr, int32_t *rowval, int32_t index_base);

/* ------------------------------------------------------------------ assembly */
/* Values in the order of fg_csc_pattern (nnz doubles). */
/* src/FEM3D.jl:40-56 stiffnessMatrix, src/FEM2D.jl:48-76 stiffnessMatrix2D,
 * src/FEM3D.jl:378-395 quadraticStiffnessMatrix, src/FEM2D.jl:117-137
 * quadraticStiffnessMatrix2D.  f: per-element coefficient (NULL = ones). */
fg_status fg_stiffness(fg_mesh *m, const double *f, double *nzval);
/* src/FEM3D.jl:466-492 massMatrix, src/FEM2D.jl:139-161 massMatrix2D,
 * src/FEM3D.jl:494-561 quadraticMassMatrix (full_phi = 0 reproduces the
 * reference's linear-part-only phi of :529-531, 1 evaluates the full quadratic),
 * src/FEM2D.jl:163-229 quadraticMassMatrix2D.  f: per-element factor or NULL. */
fg_status fg_mass(fg_mesh *m, const double *f, int32_t full_phi, double *nzval);
/* src/FEM3D.jl:563-648 quadraticConvectionMatrix (P2 tetrahedra): vel is the
 * nodal velocity, 3 x nv column-major; f per-element factor or NULL; full_phi as
 * for fg_mass (the reference's phi at :610-613 keeps the linear part only).  The
 * values are those of the reference's C, whose entry (t_i, t_j) sums the local
 * Ck[j, i] (:640-648), in the order of fg_csc_pattern. */
fg_status fg_convection(fg_mesh *m, const double *vel, const double *f, int32_t full_phi, double *nzval);
/* (On a P2 triangle handle fg_convection is src/FEM2D.jl:231-319
 * quadraticConvectionMatrix2D: vel 3 x nv with z unused, interpolated with the P2
 * basis at the 4-point rule; its C[t_i, t_j] = sum w (u . grad phi_j) phi_i; f should
 * be NULL (the 2D reference has no factor); full_phi is ignored.) */
/* src/FEM3D.jl:79-119 tangentialStiffnessMatrix (P1 tet): H is 3 x nt, dmu nt.
 * Where |H| = 0 the stored term is its limit 0. */
fg_status fg_tangent(fg_mesh *m, const double *H, const double *dmu, double *nzval);
/* src/FEM3D.jl:59-76 localStiffnessMatrix: Ak (npe*npe x nt, column k holds the
 * element matrix in column-major order). */
fg_status fg_local_stiffness(fg_mesh *m, const double *f, double *Ak);

/* ------------------------------------------------------------ right-hand sides */
/* src/FEM3D.jl:274-281 lagrange: C (nv) with C_i = sum of VE/4 over the P1
 * tetrahedra of node i (the Lagrange-multiplier row). */
fg_status fg_lagrange(fg_mesh *m, double *C);
/* src/FEM3D.jl:284-297 BoundaryIntegral: RHS (nv) with RHS[face nodes] += (n . F) AE/3
 * over the boundary faces whose id (row 4 of surfaceT, 4 x ns) is one of shell_id
 * (nshell ids); normal 3 x ns, AE ns, F 3; face nodes carry index_base. */
fg_status fg_boundary_integral(fg_mesh *m, const int32_t *surfaceT, int64_t ns, int32_t index_base,
                               const double *normal, const double *AE, const double *F, const int32_t *shell_id,
                               int32_t nshell, double *RHS);

/* ------------------------------------------------------------------- solvers */
/* Drop-in for IterativeSolvers.cg(A, b) (Magnetostatics/2DmagneticField.jl:139,
 * Micromagnetics/LL.jl:185, Femeko_jl_C++/Magnetostatics/run.jl:141) and Eigen's
 * ConjugateGradient (Femeko_jl_C++/Magnetostatics/magnetostatics.cpp:26-38) on a
 * symmetric SparseMatrixCSC{Float64,Int64}: Jacobi-preconditioned CG.
 * x holds the initial guess on entry. */
fg_status fg_cg_csc(int64_t n, const int64_t *colptr, const int64_t *rowval, const double *nzval, int32_t index_base,
                    const double *b, double *x, const fg_solve_opts *o, fg_solve_stats *s);
/* y = A x for the same CSC input (one call = upload + SpMV + download). */
fg_status fg_spmv_csc(int64_t n, const int64_t *colptr, const int64_t *rowval, const double *nzval,
                      int32_t index_base, const double *x, double *y);

/* The fg_cg_csc solve (FP64 Jacobi-PCG, stop at ||r|| <= rtol ||r0||) for a matrix
 * and vectors already in DEVICE memory, allocating nothing: no cudaMalloc/cudaFree
 * and no allocating library routine.  No counterpart in the reference.
 * For callers that cannot allocate: a time loop re-solving a small system every
 * step while other streams work (cudaMalloc/cudaFree may synchronise the device),
 * or a process whose device memory is reserved by its own pool.
 * Work space is one fixed scratch area per device inside the library:
 * n <= FG_NOALLOC_MAX_ROWS rows (6 MiB of vectors); larger n returns FG_BAD_ARG.
 * The first call on each device (with that device current) looks up the scratch
 * address; make that first call before any stream capture.  Calls that overlap on
 * one device would race on the shared scratch: a per-device host lock serialises
 * them.  colptr/rowval/nzval/b/x are managed pointers or pointers to memory of the
 * current device (another device's memory returns FG_BAD_ARG); x holds the initial
 * guess and receives the solution; stream may be NULL (default stream);
 * o->precision must be FG_FP64 (o may be NULL: defaults; o->maxiter <= 0 takes the
 * default cap too); s->ms is host wall time.  A column range or row index outside
 * the matrix, or a zero diagonal entry, returns FG_BAD_ARG (checked on the device
 * before any access); p.q = 0 before the tolerance is met returns FG_NOT_CONVERGED. */
#define FG_NOALLOC_MAX_ROWS ((int64_t)131072)
fg_status fg_cg_csc_noalloc(int64_t n, const int64_t *colptr, const int64_t *rowval, const double *nzval,
                            int32_t index_base, const double *b, double *x, const fg_solve_opts *o, void *stream,
                            fg_solve_stats *s);

/* Linear magnetostatics (Magnetostatics/magneticField.jl:89-132 and
 * Femeko_jl_C++/Magnetostatics/magnetostatics.cpp:49-95 scalarPotential) with the
 * Dirichlet rows set by fg_mesh_set_dirichlet: K(mu) u = 0 on free rows, u fixed
 * to u_in on Dirichlet rows (u_in also seeds the free rows).  mu is absolute
 * permeability per element.  H (3 x nt) may be NULL. */
fg_status fg_magnetostatics_linear(fg_mesh *m, const double *mu, const double *u_in, const fg_solve_opts *o,
                                   double *u, double *H, fg_solve_stats *s);
/* Nonlinear Newton-Raphson magnetostatics (Magnetostatics/NewtonRaphson.jl:109-214):
 * nl[k] != 0 marks Froehlich elements, the others use mu_lin[k]; u0 gives the
 * Dirichlet values and the initial guess.  Outputs u (nv), H (3 x nt), mu (nt);
 * H and mu may be NULL. */
fg_status fg_newton_magnetostatics(fg_mesh *m, const uint8_t *nl, const double *mu_lin, const double *u0,
                                   const fg_newton_opts *o, double *u, double *H, double *mu, fg_newton_stats *s);
/* Backward-Euler heat conduction (Heat/heat3D.jl:50-90: T <- (M + dt A) \ (M T)) on
 * P1 tetrahedra with heat capacity rho_c, per-element conductivity kappa (nt) and
 * T = 0 on the Dirichlet nodes of fg_mesh_set_dirichlet:
 * (rho_c M + dt K(kappa)) T_{n+1} = rho_c M T_n for nsteps steps, each solve started
 * from T_n.  T (nv) holds the initial field and receives the last one; snapshots
 * (may be NULL) receives T after every `every` steps (nsteps/every rows of nv).
 * o->precision: FG_MIXED (FP32 operator and CG inside FP64 refinement) or FG_FP64;
 * stats accumulate over the steps. */
fg_status fg_heat_be(fg_mesh *m, const double *kappa, double rho_c, double dt, int32_t nsteps, double *T,
                     int32_t every, double *snapshots, const fg_solve_opts *o, fg_solve_stats *s);

/* src/FEM3D.jl:300-322 quadraticBoundaryMassMatrix: faces is 6 x nfaces (0-based,
 * column-major; the first six rows of the reference's P2 surfaceT: vertices, then the
 * midpoints of edges 12, 23, 31), AE the face areas, F the per-face factor (NULL =
 * ones).  Entry AE[s] Mk[i,j] F[s] with Mk the P2 triangle mass of :303-308; values in
 * the order of fg_csc_pattern (a face pair outside the pattern is FG_BAD_ARG). */
fg_status fg_boundary_mass(fg_mesh *m, const int32_t *faces, const double *AE, const double *F, int64_t nfaces,
                           double *nzval);
/* (On a P2 triangle handle: src/FEM2D.jl:394-419 quadraticMassMatrix1D, faces 3 x
 * nfaces = the reference's surfaceT rows 1-3 (Gmsh line order: vertex, vertex,
 * midpoint), Mk = (1/30) [4 2 -1; 2 16 2; -1 2 4] by that position, as the
 * reference applies it.) */

/* ------------------------------------------------------------------ Nedelec */
/* Edge-element routines on a handle from fg_edge_mesh_create.  curlN_e =
 * 2 l_e (grad lambda_i x grad lambda_j) in the element's local edge orientation. */
/* src/FEM3D.jl:155-191 nedelecLocalStiffness: Ak 36 x nt (column k = 6 x 6 block). */
fg_status fg_nedelec_local_stiffness(fg_mesh *m, double *Ak);
/* The global matrix sum sparse(edge_i, edge_j, Ak .* nu) of
 * Magnetostatics/nedelec3D.jl:168-178 (nu per element, NULL = ones), values in the
 * order of fg_csc_pattern. */
fg_status fg_nedelec_stiffness(fg_mesh *m, const double *nu, double *nzval);
/* src/FEM3D.jl:194-271 nedelecTangentialStiffness: VE (curlN_i.B)(curlN_j.B) dnu/|B|
 * (Bfield 3 x nt, B = |B| nt); elements with |B| = 0 contribute 0. */
fg_status fg_nedelec_tangent(fg_mesh *m, const double *dnu, const double *Bfield, const double *B, double *nzval);
/* nedelec3D.jl:106-139: rhs[e] = sum over elements of VE Bext.curlN_e (ne values). */
fg_status fg_nedelec_load(fg_mesh *m, const double *Bext, double *rhs);
/* nedelec3D.jl:190-221: B per element (3 x nt) and |B| (nt, may be NULL) from u (ne). */
fg_status fg_nedelec_bfield(fg_mesh *m, const double *u, double *Bfield, double *B);
/* The first Newton step of nedelec3D.jl (u = 0, At = 0): A(nu) u = RHS(Bext) by the
 * Jacobi-PCG of fg_pcg (the curl-curl matrix is singular with a consistent right-hand
 * side: u is one solution, B = curl u is unique); Bfield/B (may be NULL) as in
 * fg_nedelec_bfield.  With o->precision = FG_MIXED a solve whose FP32 inner
 * iterations stall on this singular system (high permeability contrast, tight rtol)
 * is finished by FP64 PCG from where it stopped (refinements + 1). */
fg_status fg_nedelec_linear(fg_mesh *m, const double *nu, const double *Bext, double *u, double *Bfield, double *B,
                            const fg_solve_opts *o, fg_solve_stats *s);

/* The Newton loop of Magnetostatics/nedelec3D.jl:149-231 on the GPU: nu = 1 (nu_lin
 * on the elements outside `nonlinear`, NULL = ones), u = 0; per step A(nu), At (from
 * the second step), du = PCG(A + At, RHS - A u) (o->rtol), the line search of
 * src/FEM3D.jl:122-151 (steps x0.9 down to min_step), B = curl u, then on the
 * `nonlinear` elements nu = spl(|B|), dnu = spl_dnu(|B|), until max |B - B_prev| <= tol
 * or max_newton steps.  spl is the not-a-knot interpolating cubic through
 * (curve_B, curve_nu) (the interpolant of Dierckx's Spline1D(B, nu), s = 0), spl_dnu
 * the same through the finite-difference gradient of src/FEM.jl:66-92; both are held
 * at their end values outside the data (bc = "nearest").  ncurve >= 4, curve_B
 * increasing.  Outputs: u (ne), Bfield (3 x nt), B (nt), nu_out (nt) (each may be NULL
 * but u), newton_iters; stats: iterations = CG iterations in total, refinements =
 * Newton steps, relres = the last line-search residual ||RHS - A u||, pad_ = inner
 * solves that stopped short of o->rtol (their corrections are used, as the
 * reference's cg returns what it has); FG_NOT_CONVERGED when max_newton steps end
 * with max |B - B_prev| > tol. */
fg_status fg_nedelec_newton(fg_mesh *m, const double *Bext, const uint8_t *nonlinear, const double *nu_lin,
                            const double *curve_B, const double *curve_nu, int32_t ncurve, double tol,
                            int32_t max_newton, double min_step, double *u, double *Bfield, double *B,
                            double *nu_out, int32_t *newton_iters, const fg_solve_opts *o, fg_solve_stats *s);

/* Heat transport with convection on P2 tetrahedra (Transport/main3D.jl:143-213;
 * on P2 triangles the same loop of Transport/main2D.jl:150-190 with the 2D matrices
 * and 3-node boundary lines, rho_cp = ones for the reference's unweighted 2D M):
 * LM = M(rho_cp) + dt (A(kappa) + R + C(vel, rho_cp)), then nsteps steps of
 * T <- LM \ (M T) (main3D.jl:199-204), each solved by Jacobi-preconditioned BiCGStab
 * (FP64, started from the previous T) to ||M T_n - LM T|| <= o->rtol ||M T_n||
 * (o->maxiter iterations per step; precision, spmv and graph options are ignored).
 * rho_cp, kappa: nt; vel: 3 x nv column-major; faces/AE/F: the penalty faces and
 * factors of fg_boundary_mass (nfaces may be 0).  full_phi as for fg_mass: the
 * reference's linear-part-only phi (0) gives an operator on which the iteration can
 * fail where the reference's direct solve does not; 1 is the full P2 basis.  T (nv)
 * holds the initial field and receives the last one; snapshots as for fg_heat_be.
 * stats: iterations summed over the steps, the last step's relres, ms the device time
 * from the assembly to the last solve; FG_NOT_CONVERGED if a step stopped short
 * (pad_ = 1 iteration limit, 2 breakdown). */
fg_status fg_transport_be(fg_mesh *m, const double *rho_cp, const double *kappa, const double *vel,
                          const int32_t *faces, const double *AE, const double *F, int64_t nfaces, double dt,
                          int32_t nsteps, int32_t full_phi, double *T, int32_t every, double *snapshots,
                          const fg_solve_opts *o, fg_solve_stats *s);

/* A sweep of applied fields on one linear mesh (the hysteresis-loop use of
 * Magnetostatics/magneticField.jl:89-132): for field c, K(mu) u_c = 0 on the free
 * rows with u_c = -H0_c . x on the Dirichlet rows of fg_mesh_set_dirichlet.
 * o->spmv selects the method:
 *   FG_SWEEP_BLOCK (0, default): the residual block of all fields has the rank r <= 3
 *     of H0 (the problem is linear in the field); its rank-revealing factorisation
 *     H0 = C V^T (V: r orthonormal field directions) reduces the sweep to one block
 *     CG of width r (O'Leary, Jacobi-preconditioned, r x r systems by Cholesky with
 *     dropped dependent directions), and u_c = sum_k C_ck u(v_k).  Any nfield.
 *   FG_SWEEP_PER_FIELD (1): one multi-right-hand-side Jacobi-PCG with a CG per field
 *     that reads the matrix once per iteration for every field; nfield <= 256, rows of
 *     at most 32 entries.
 * Both: FP32 matrix and inner iterations, FP64 residual and solution by iterative
 * refinement until every field's residual is below rtol of its initial one
 * (o->precision must be FG_MIXED).  mu: nt absolute permeabilities; H0: 3 x nfield;
 * U (nv x nfield column-major, may be NULL) receives the potentials.  s->iterations:
 * block (or multi-field) iterations summed over the refinements; with FG_SWEEP_BLOCK
 * s->pad_ is the rank r; s->ms covers the solve and the expansion to all fields. */
#define FG_SWEEP_BLOCK 0
#define FG_SWEEP_PER_FIELD 1
fg_status fg_magnetostatics_sweep(fg_mesh *m, const double *mu, int32_t nfield, const double *H0,
                                  const fg_solve_opts *o, double *U, fg_solve_stats *s);

typedef struct fg_batch_stats {
  int32_t problems;
  int32_t converged;       /* problems that reached rtol */
  int32_t max_iterations;  /* largest CG iteration count of a problem */
  int32_t cluster_ctas;    /* CTAs of the largest problem's cluster (16 or 8; smaller problems get
                              fewer in proportion to their rows, at least 2) */
  int64_t total_iterations;
  double ms;               /* device time of the graph launch */
  int32_t max_refinements; /* FG_MIXED: most FP64 refinement steps of a problem (0 in FP64) */
  int32_t reserved_;
} fg_batch_stats;

/* count independent linear magnetostatic problems (Magnetostatics/magneticField.jl:89-132
 * on each mesh: K(mu) u = 0 on free rows, u = u_in on the Dirichlet rows set by
 * fg_mesh_set_dirichlet) solved by Jacobi-PCG in ONE graph launch: each problem
 * runs its whole solve on its own thread-block cluster, whose size follows the
 * problem's rows (16, 8, 4 or 2 CTAs; one persistent kernel per cluster size, the
 * kernels on parallel branches of the graph).
 * mu[k] (nt_k, absolute permeability), u_in[k] and u_out[k] (nv_k) are host arrays
 * per mesh; iterations (count, may be NULL) receives each problem's CG iterations.
 * o->precision: FG_FP64 (FP64 PCG to rtol) or FG_MIXED (on each cluster, FP64
 * iterative refinement around FP32 PCG solves of inner relative target
 * max(rtol ||r0|| / ||r||, o->inner_rtol), as fg_solve; iterations are then the inner
 * FP32 iterations).  All meshes on the current device. */
fg_status fg_batch_magnetostatics_linear(fg_mesh *const *meshes, int32_t count, const double *const *mu,
                                         const double *const *u_in, const fg_solve_opts *o, double *const *u_out,
                                         int32_t *iterations, fg_batch_stats *s);

typedef struct fg_adjoint_stats {
  int32_t forward_iters;  /* CG iterations of the forward solve (all Newton steps) */
  int32_t adjoint_iters;  /* CG iterations of the adjoint solve */
  int32_t newton_iters;   /* 0 for the linear forward problem */
  int32_t converged;      /* forward and adjoint both converged */
  double forward_ms;      /* device time of the forward solve */
  double adjoint_ms;      /* device time of J, the adjoint solve and the gradient */
} fg_adjoint_stats;

/* Differentiation of J = volume-weighted mean of H_x over the elements with
 * target[k] != 0 (the volume average of Magnetostatics/NewtonRaphson.jl:234-240)
 * with respect to the per-element relative permeability mur (mu = mu0 mur).
 * Forward: linear magnetostatics (Magnetostatics/magneticField.jl:89-132) when
 * nl == NULL, else the Newton solve of fg_newton_magnetostatics (Froehlich elements
 * nl[k] != 0, the others mu0 mur[k]).  Adjoint: the symmetric operator (K(mu), or
 * the converged Newton Jacobian K + At) solved for lambda with right-hand side
 * dJ/du; grad[k] = dJ/dmur_k = -mu0 VE_k grad(lambda).grad(u).  Dirichlet nodes come
 * from fg_mesh_set_dirichlet with values u0; o->precision selects FP32 solves with
 * FP64 refinement (FG_MIXED) or FP64; rtol is the relative residual of the linear
 * forward solve and of the adjoint solve.  u (nv, may be NULL) receives the forward
 * potential.  No counterpart in the reference (which has no derivatives). */
fg_status fg_adjoint_dJdmu(fg_mesh *m, const double *mur, const double *u0, const uint8_t *target,
                           const uint8_t *nl, const fg_newton_opts *o, double rtol, double *J, double *grad,
                           double *u, fg_adjoint_stats *s);
/* The same solve in three steps, for callers that keep the problem on the device
 * and solve it repeatedly: fg_newton_set_inputs uploads nl, mu_lin and u0 once;
 * fg_newton_solve_resident runs the Newton solve from them and leaves u, H and mu
 * on the device; fg_newton_get_outputs downloads them (each may be NULL). */
fg_status fg_newton_set_inputs(fg_mesh *m, const uint8_t *nl, const double *mu_lin, const double *u0);
fg_status fg_newton_solve_resident(fg_mesh *m, const fg_newton_opts *o, fg_newton_stats *s);
fg_status fg_newton_get_outputs(fg_mesh *m, double *u, double *H, double *mu);
/* Demagnetising field of Micromagnetics/LL.jl:162-211 (magnetostaticField), the
 * Poisson solve of every Landau-Lifshitz step: RHS_i = sum over the inside elements
 * (inside[k] != 0) of VE (grad phi_i . mean nodal M), u = PCG(A, RHS) from zero with
 * A the stiffness matrix (assembled on the first call and kept for the next ones;
 * Dirichlet rows of fg_mesh_set_dirichlet apply if set, the reference has none),
 * H = -grad u per element, and Hn (3 x nv) its volume-weighted nodal average over
 * the inside elements (NaN on nodes with no inside element, as the reference's
 * division by a zero node volume).  M is 3 x nv; u (nv) may be NULL. */
fg_status fg_demag_field(fg_mesh *m, const uint8_t *inside, const double *M, const fg_solve_opts *o, double *Hn,
                         double *u, fg_solve_stats *s);
/* H = -sum u_a grad(phi_a) per element (Magnetostatics/magneticField.jl:111-124). */
fg_status fg_hfield(fg_mesh *m, const double *u, double *H);

/* Drop-in for the reference's own ccall entry point
 * Femeko_jl_C++/Magnetostatics/magnetostatics.cpp:49-95 (scalarPotential, bound by
 * Femeko_jl_C++/Magnetostatics/run.jl:66-79 with @ccall ... ::Cvoid): same name, same
 * argument list and meaning.  Solves the linear Neumann problem of magnetostatics()
 * (magnetostatics.cpp:5-38): RHS = BoundaryIntegral(p, surfaceT, normal, Hext,
 * shell_id) (src/FEMc.cpp:170-200: faces whose id, row 4 of surfaceT, equals shell_id;
 * face areas from p), A = stiffnessMatrix(p, t, VE, mu) (src/FEMc.cpp:74-125, with the
 * caller's VE), u = CG(A) \ (-RHS) from u = 0 with the diagonal (Jacobi)
 * preconditioner; the solution is unique up to a constant, and the zero start fixes
 * it as Eigen's does (sum_i A_ii u_i = 0 in exact arithmetic).
 * p 3 x nv, t 4 x nt and surfaceT 4 x ns (0-based, as run.jl:49-52 shifts them),
 * normal 3 x ns, VE and mu nt, Hext 3; u (nv) receives the potential.
 * Solver: FP32 Jacobi-PCG inside FP64 iterative refinement to relative residual
 * 1e-12 (Eigen's default asks for machine epsilon, which its 2n iteration cap
 * rarely reaches).  The reference throws C++ exceptions through this extern "C"
 * function; here nothing is thrown: fg_scalar_potential_status() returns the status of
 * the calling thread's last call and fg_last_error() its message (empty after
 * success).  u is written on FG_OK and FG_NOT_CONVERGED, left as it was otherwise. */
void scalarPotential(double *u_in, double *p_in, int *t_in, int *surfaceT_in, double *normal_in, int nv, int nt,
                     int ns, double *VE, double *mu, double *Hext, int shell_id);
fg_status fg_scalar_potential_status(void);
/* The same solve with a status return, solver options (o may be NULL: the defaults
 * of scalarPotential above) and statistics (s may be NULL). */
fg_status fg_scalar_potential(double *u, const double *p, const int32_t *t, const int32_t *surfaceT,
                              const double *normal, int32_t nv, int32_t nt, int32_t ns, const double *VE,
                              const double *mu, const double *Hext, int32_t shell_id, const fg_solve_opts *o,
                              fg_solve_stats *s);

/* One call from host arrays in the shape of the ccall boundary scalarPotential
 * above, for the nonlinear Dirichlet problem: the Newton solve of
 * Magnetostatics/NewtonRaphson.jl:109-214: uploads the P1 mesh (p 3 x nv, t 4 x nt),
 * builds the pattern, solves, downloads u/H/mu and releases the device memory.
 * fixed marks Dirichlet nodes (u0 holds their values). */
fg_status fg_scalar_potential_newton(const double *p, int64_t nv, const int32_t *t, int64_t nt, int32_t index_base,
                                     const uint8_t *fixed, const uint8_t *nl, const double *mu_lin, const double *u0,
                                     const fg_newton_opts *o, double *u, double *H, double *mu, fg_newton_stats *s);

/* ------------------------------------------------------------- diagnostics */
/* Kernel launches issued by this library so far (graph replays count every node). */
int64_t fg_kernel_launches(void);
/* Average device time of one launch of a hot kernel on the handle's current
 * operator: which = 0 CG SpMV with its dot products (for the fused FP32 iteration
 * variants: the whole iteration), 1 CG vector update, 2 Newton element pass + row
 * gather over all elements, 3 one whole CG iteration, 4 Newton residual on the
 * linear/nonlinear split, 5 the same with the Jacobian (4, 5: after a Newton solve),
 * 6 one whole CG iteration run the way the solver runs it (its graph loop; reps
 * iterations after an untimed run), 7 the P1 stiffness assembly K(mu) at the
 * handle's current permeabilities into the FP64 and FP32 operator (one pass over the
 * rows, after a solve), 8 the same assembly through element records and a row sum,
 * 9 the one-block kernel that adds the SpMV's per-block dot products in the
 * split-reduction FP32 variants (for those, 0 times the SpMV kernel alone).
 * No reference counterpart (used for roofline reporting). */
fg_status fg_bench_kernel(fg_mesh *m, int32_t which, int32_t precision, int32_t reps, double *ms_per_launch);
/* Autotuner: times the CG kernel variants of one precision on the handle's current
 * operator (FG_MIXED: the FP32 iteration variants; FG_FP64: the SpMV with direct
 * gathers, halo staging or a persistent grid of 4 or 8 blocks per SM; assemble one
 * first, e.g. by a solve) and keeps the fastest.
 * variant receives the chosen index (0-based), us_per_variant (n_slots entries, may
 * be NULL) the measured microseconds per launch.  No reference counterpart. */
fg_status fg_autotune(fg_mesh *m, int32_t precision, int32_t *variant, double *us_per_variant, int32_t n_slots);
/* Fixes the CG kernel variant of one precision for the handle (the numbering of
 * fg_solve_opts.spmv: FG_MIXED 1..29, FG_FP64 1..4), or 0 to return to the
 * autotuner's choice at the next solve.  The autotuner's choices are remembered per
 * process for each operator shape (device, rows, padded entries, longest row), so a
 * new handle for a mesh of the same structure does not time the variants again.
 * No reference counterpart (profiling and tuning control). */
fg_status fg_set_cg_variant(fg_mesh *m, int32_t precision, int32_t variant);
/* The CG kernel variant the handle's solves of one precision use (numbering of
 * fg_set_cg_variant), 0 while none is chosen yet.  No reference counterpart. */
fg_status fg_get_cg_variant(const fg_mesh *m, int32_t precision, int32_t *variant);
/* Padded sizes of the device layouts: SELL-32 matrix entries, incidence records, slices. */
fg_status fg_mesh_layout(const fg_mesh *m, int64_t *nsell, int64_t *ninc, int32_t *nslices);

#ifdef __cplusplus
}
#endif
#endif /* FEMEKO_GPU_H */
