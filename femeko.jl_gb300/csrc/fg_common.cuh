// Internal definitions shared by the translation units of libfemeko_gpu.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/femeko_gpu.h"

#define FG_MU0 (3.14159265358979323846 * 4e-7)

// ---------------------------------------------------------------- errors
void fg_set_error(const std::string &msg);

struct FgError {
  fg_status code;
  std::string msg;
};

// The message names the failing call and its source position (file name and line).
static inline const char *fg_basename(const char *path) {
  const char *b = path;
  for (const char *c = path; *c; ++c)
    if (*c == '/') b = c + 1;
  return b;
}
#define FG_CUDA_TRY(call)                                                                    \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess)                                                                   \
      throw FgError{FG_CUDA, std::string(#call) + " at " + fg_basename(__FILE__) + ":" +     \
                                 std::to_string(__LINE__) + ": " + cudaGetErrorString(e_)};  \
  } while (0)

#define FG_REQUIRE(cond, code, msg)                                                          \
  do {                                                                                       \
    if (!(cond)) throw FgError{code, msg};                                                   \
  } while (0)

// Runs body, converting exceptions into a status (nothing crosses the C ABI).
template <class F>
static inline fg_status fg_guard(F &&body) {
  try {
    return body();
  } catch (const FgError &e) {
    fg_set_error(e.msg);
    return e.code;
  } catch (const std::exception &e) {
    fg_set_error(e.what());
    return FG_CUDA;
  } catch (...) {
    fg_set_error("unknown error");
    return FG_CUDA;
  }
}

// ---------------------------------------------------------------- device flags
enum {
  FLAG_BAD_INDEX = 1,   // node index outside [0, nv)
  FLAG_DEGENERATE = 2,  // zero-volume element
  FLAG_ROW_OVERFLOW = 4,// a row longer than the supported maximum
  FLAG_NAN = 8,         // NaN/Inf in a permeability or residual
  FLAG_DUP_NODE = 16,   // an element lists the same node twice
  FLAG_BAD_FACE = 32    // a boundary face pair that is not in the matrix pattern
};

// Longest matrix row the pattern builder accepts (slot positions fit a byte).
constexpr int FG_MAX_ROW = 252;
constexpr int FG_SLICE = 32;  // rows per SELL slice
constexpr int FG_GROUP = 4;   // row slots per 128-bit group

// Position of slot q of the row with lane `lane` in a slice starting at `base`.
__host__ __device__ __forceinline__ int64_t sell_pos(int64_t base, int lane, int q) {
  return base + ((int64_t)(q >> 2) * FG_SLICE + lane) * FG_GROUP + (q & 3);
}
constexpr int FG_RED_BLOCKS = 4096;

// ---------------------------------------------------------------- device scratch
// Scalars of one CG run (device doubles)
enum {
  S_RZ = 0,    // r.z
  S_PQ,        // p.q
  S_ALPHA,
  S_BETA,
  S_RR,        // r.r
  S_BB,        // b.b
  S_TOL2,      // stop when r.r <= TOL2
  S_SCALE,     // mixed: scale applied to the FP64 residual before the FP32 solve
  S_NSCAL = 16
};
// CG control words; I_FAULT is set by a kernel whose asynchronous copy did not
// complete within its bounded wait (the solve stops and reports an error); I_BODIES
// counts the bodies run by a whole-solve loop graph; I_PIPE_FIRST marks the first
// reduction of a pipelined FP32 CG run (it turns the relative tolerance absolute).
enum { I_DONE = 0, I_ITERS, I_MAXIT, I_STATUS, I_FAULT, I_BODIES, I_PIPE_FIRST, I_NINT = 8 };

// Reduction workspace: per-block partials and an arrival counter for the
// "last block finishes the sum" pattern (the sum runs in block order, so results
// do not depend on scheduling).
struct RedWs {
  double *partials;   // FG_RED_BLOCKS * 4
  unsigned int *counter;
};

// A block of CG iterations captured as a CUDA graph; `loop`: the graph is a WHILE
// conditional node around that block, run until the device's done flag is set.
struct GraphCache {
  cudaGraphExec_t exec = nullptr;
  const void *key[8] = {nullptr};
  int iters = 0;
  bool loop = false;
};

struct fg_mesh {
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;

  int64_t nv = 0, nt = 0;
  int npe = 0, dim = 0, nvert = 0;

  // mesh on the device
  double *p = nullptr;       // 3 x nv (AoS, as given)
  int *t = nullptr;          // npe x nt stored SoA: t[a*nt + k]
  // Nedelec handles: t lists the 6 edge unknowns of each tetrahedron (local edges
  // 12, 23, 31, 41, 34, 24), tv its 4 vertices (SoA) into the np points p
  bool edge = false;
  int *tv = nullptr;
  int64_t np = 0;
  uint8_t *fixed = nullptr;  // nv Dirichlet mask (0/1)
  bool has_fixed = false;
  double *geo = nullptr;     // P1: SoA per element, (nvert*dim gradients + volume) x nt
  int ngeo = 0;

  // CSR pattern (structural)
  int *rowptr = nullptr;     // nv+1
  int *colidx = nullptr;     // nnz
  int64_t nnz = 0;
  int maxrow = 0;

  // SELL-32x4 matrix layout (rows in natural order): slice s holds rows 32s..32s+31;
  // its entries are stored in groups of 4 consecutive row slots, group-major, lane
  // within the group, so a thread loads 4 entries of its row with one 128-bit load
  // and a warp's loads are contiguous.  Rows are padded to 4*sl_len[s] slots with
  // the row's own column and value 0.  Entry (row i, slot q) sits at sell_pos().
  int nslices = 0;
  int64_t nvp = 0;           // rows padded to whole slices (vector length)
  int *sl_ptr = nullptr;     // nslices+1 offsets into sl_col / values
  int *sl_len = nullptr;     // nslices: groups of 4 slots per row in the slice
  int *sl_col = nullptr;     // nsell absolute column indices
  int16_t *sl_dcol = nullptr;// nsell column - row, when every |column - row| < 32768
  // Halo staging: rows are taken in blocks of hrows (one CTA each); a block's distinct
  // columns (its halo, sorted) are listed at halo_col[b * hcap ...], halo_len[b] of
  // them, and every entry's column is also stored as its position in that list
  // (sl_lcol), so a CTA gathers each needed vector entry once into shared memory.
  int hrows = 0, hcap = 0, hmax = 0, nhblocks = 0;
  int tmax = 0;       // most matrix entries (padded slots) of one row block
  int tmax256 = 0;    // most matrix entries (padded slots) of one 256-row block
  int bulk_fit = -1;  // resident CTAs per SM of the bulk-staged SpMV (-1: not sized yet)
  int pipe_fit = -1;  // the same for the pipelined CG's SpMV
  int coop_fit = -1;  // the same for the cooperative persistent CG
  unsigned *coop_bar = nullptr;  // its grid barrier: arrivals, generation
  int pipe_grid = 0;  // CTAs of the persistent pipelined iteration (0: not sized yet, -1: does not fit)
  int *halo_col = nullptr, *halo_len = nullptr;
  bool halo_tried = false;   // the halo lists are built at the first variant that needs them
  uint16_t *sl_lcol = nullptr;
  bool use_dcol = false;
  int64_t nsell = 0;
  int maxrow4 = 0;           // longest row rounded up to a multiple of 4
  uint8_t *diagk = nullptr;  // nv: position of the diagonal in its row
  int *rowlen = nullptr;     // nv

  // incidence (node -> element-local slot) in SELL-32 layout
  int *in_ptr = nullptr;     // nslices+1
  int *in_len = nullptr;     // nslices
  int64_t ninc = 0;          // padded count
  uint8_t *in_slot = nullptr;// ninc * npe slot positions (0xFF on pads)
  int *recpos = nullptr;     // nt * npe (SoA: [a*nt + k]) -> incidence position
  int *in_elem = nullptr;    // ninc: 4 k + a of each incidence position, -1 on pads (P1 tetrahedra)
  bool asm_two_pass = false; // P1 stiffness/mass/heat through element records + row sum (timing comparison)
  int maxdeg = 0;

  // records written by the element kernels, summed by the row kernel
  void *rec = nullptr;       // ninc * npe (double or float)
  double *rec_r = nullptr;   // ninc vector records

  // operator values (SELL layout) and Jacobi preconditioner
  double *val64 = nullptr;
  float *val32 = nullptr;
  double *dinv64 = nullptr;
  float *dinv32 = nullptr;
  double *csrval = nullptr;  // nnz, export buffer

  // per-element state (Newton)
  double *mu = nullptr, *dmu = nullptr, *H = nullptr, *wdens = nullptr;
  double *mu_lin = nullptr;
  uint8_t *nl = nullptr;
  // Newton with a few nonlinear elements: the linear elements' operator (with the
  // Dirichlet rows) assembled once per solve, and the maps of the nonlinear ones
  double *vlin64 = nullptr, *dlin64 = nullptr;  // SELL values / Jacobi inverses
  float *vlin32 = nullptr, *dlin32 = nullptr;
  int n_nl = 0, nl_cap = 0, n_nl_slots = 0, n_nl_rows = 0;
  int *nl_elems = nullptr;                       // nonlinear element indices
  int *nl_slot_pos = nullptr, *nl_slot_ptr = nullptr, *nl_slot_src = nullptr, *nl_slot_code = nullptr;
  int *nl_rows = nullptr, *nl_row_ptr = nullptr, *nl_row_src = nullptr;
  double *nl_re = nullptr, *nl_ke = nullptr;     // 4 / 16 per nonlinear element
  // batched line search: rows that nonlinear elements touch (1 per row) and the
  // element residual records of up to FG_LS_BATCH candidate steps
  uint8_t *nl_rowmask = nullptr;
  double *nl_re_cand = nullptr;
  int nl_cand_cap = 0;
  double *ls_out = nullptr;                      // FG_LS_QUAD + FG_LS_BATCH results
  std::vector<int> nl_list_host;                 // the list the maps were built for
  std::vector<uint8_t> nl_host;                  // nonlinear mask of the current Newton inputs
  double *u0dev = nullptr;                       // Dirichlet values / initial guess of the Newton inputs
  bool nl_maps_valid = false;
  bool nl_list_current = false;                  // nl_list_host was built from nl_host as it is now
  uint8_t *target = nullptr;  // nt objective mask (adjoint)
  double *objbuf = nullptr;   // 2 x nt objective scratch (adjoint)

  // vectors
  double *v64[20] = {nullptr};
  // BiCGStab vectors (padded to nvp), the mass values of the transport operator
  // (SELL layout) and the captured iteration graph
  double *bcg[10] = {nullptr};
  double *mval = nullptr;
  cudaGraphExec_t bcg_exec = nullptr;
  bool bcg_dcol = false;
  float *v32[8] = {nullptr};
  float *pv32[3] = {nullptr};  // pipelined FP32 CG: z, n = A m, m = D w

  // reductions and CG control
  RedWs red{};
  double *scal = nullptr;     // S_NSCAL
  int *ictl = nullptr;        // I_NINT
  int *flags = nullptr;       // device error flags
  double *hbuf = nullptr;     // pinned host mirror for small readbacks (64 doubles)
  int *hint = nullptr;        // pinned host ints (16)

  GraphCache graph[4];
  int op_tag = 0;            // what val64/val32 hold when a caller reuses them (0: unknown)
  int64_t op_version = 0;    // incremented whenever val64/val32 are rewritten
  // symmetrically Jacobi-scaled FP32 operator D^-1/2 A D^-1/2 (the scaled CG variant),
  // D^-1/2 and D (the weights of the residual norm) per row
  float *val32s = nullptr, *sdiag32 = nullptr, *diag32 = nullptr;
  int64_t val32s_version = -1;
  uint8_t *inside = nullptr; // nt mask of the magnetic body (demagnetising field)
  double *nodal_in = nullptr;// 3 x nv nodal magnetisation (demagnetising field)
  double *nodal_work = nullptr; // 7 x nv: nodal sums, volumes and the nodal field
  int64_t l2_win_bytes = 0;  // L2 access-policy window on val32 (0: not set up, -1: unavailable)
  float l2_hit_ratio = 0.f;
  int spmv_variant32 = 0;     // FP32 CG iteration variant chosen by the autotuner
  int spmv_variant64 = 0;     // FP64 CG SpMV variant chosen by the autotuner
  bool tuned32 = false, tuned64 = false;
  std::vector<void *> extra;  // stream-ordered allocations released at destroy
  std::vector<void *> extra_sync;  // plain allocations (made before the stream existed)
};

// ---------------------------------------------------------------- helpers
// Device memory of a handle comes from the device's stream-ordered pool on the
// handle's stream (cudaMallocAsync; released with cudaFreeAsync at destroy): a
// one-shot call that creates and destroys a handle reuses the pool's memory instead
// of paying a synchronising cudaMalloc/cudaFree per buffer (fg_setup.cu keeps the
// pool's memory when it is freed).
void fg_pool_init(int device);
// Temporary device buffers from the stream-ordered pool, released on the stream when
// the holder goes out of scope (normally or by an exception).
struct StreamScratch {
  cudaStream_t s;
  std::vector<void *> held;
  template <class T>
  T *get(size_t count) {
    void *q = nullptr;
    FG_CUDA_TRY(cudaMallocAsync(&q, sizeof(T) * std::max<size_t>(count, 1), s));
    held.push_back(q);
    return static_cast<T *>(q);
  }
  ~StreamScratch() {
    for (void *q : held) cudaFreeAsync(q, s);
  }
};
// Pinned host blocks of FG_PINNED_BLOCK bytes for a handle's small read-backs
// (hbuf: 64 doubles, hint: 16 ints after it), recycled across handles:
// cudaMallocHost pins pages and cudaFreeHost waits for the device, both per handle
// otherwise.
constexpr size_t FG_PINNED_BLOCK = 1024;
void *fg_pinned_block_get();
void fg_pinned_block_put(void *block);
template <class T>
static inline T *dev_alloc(fg_mesh *m, size_t count) {
  void *ptr = nullptr;
  if (count == 0) count = 1;
  if (m && m->stream) {
    FG_CUDA_TRY(cudaMallocAsync(&ptr, count * sizeof(T), m->stream));
    m->extra.push_back(ptr);
  } else {
    FG_CUDA_TRY(cudaMalloc(&ptr, count * sizeof(T)));
    if (m) m->extra_sync.push_back(ptr);
  }
  return static_cast<T *>(ptr);
}


static inline unsigned grid_for(int64_t n, int block) { return (unsigned)((n + block - 1) / block); }

// Host-side count of kernel launches issued by this library (graph replays count
// every kernel node).
void fg_count_launch(long long n);
#define FG_LAUNCHED(n) fg_count_launch(n)

void fg_check_flags(fg_mesh *m, const char *where);
// Releases the handle's share of the persisting-L2 set-aside (fg_solve.cu).
void fg_release_l2(fg_mesh *m);
void fg_sync(fg_mesh *m);
// Builds the halo lists and local column indices (needs sl_ptr/sl_len/sl_col, maxrow4).
void fg_build_halo(fg_mesh *m);
// The halo lists, built on first use (not inside a stream capture); false when the
// rows are too long for halo staging.
bool fg_ensure_halo(fg_mesh *m);

// assembly (fg_assemble.cu)
enum AsmKind { ASM_STIFF = 0, ASM_MASS = 1, ASM_TANGENT = 2, ASM_HEAT = 3, ASM_CONV = 4 };
enum OutLayout { OUT_SELL = 0, OUT_CSR = 1 };
void fg_assemble_operator(fg_mesh *m, int kind, const double *d_f, const double *d_H, const double *d_dmu,
                          double c_mass, double c_stiff, int full_phi, int layout, bool want64, bool want32,
                          bool apply_bc);
void fg_ensure_records(fg_mesh *m);
// P1-tetrahedron mass matrix (unit coefficient, no boundary rows) into SELL values.
void fg_assemble_mass_sell(fg_mesh *m, double *out64);
// Element pass + row gather at potential d_u: element state (H, mu, dmu, energy
// density), the residual F = -K(mu(u)) u (FP64) and, when want_jacobian, the
// Jacobian K + At in the operator (FP32 when mixed) with its Jacobi diagonal.
void fg_newton_assemble(fg_mesh *m, const double *d_u, double Ms, double Hk, bool mixed, double *d_F,
                        bool want_jacobian = true, bool tangent = true);
// Newton on the linear/nonlinear split: fg_nl_setup (once per solve, after mu_lin and
// nl are on the device; nl_host is the same mask on the host) assembles the linear
// elements' operator and the nonlinear elements' maps; fg_newton_assemble_split then
// has the contract of fg_newton_assemble.
void fg_nl_setup(fg_mesh *m, const uint8_t *nl_host, bool mixed);
// Stores the nonlinear mask of new Newton inputs in m->nl_host; the element list
// built from it is kept when the mask did not change.
void fg_set_nl_host(fg_mesh *m, const uint8_t *nl);
// Candidate steps of one batched line-search launch.
constexpr int FG_LS_BATCH = 8;
constexpr int FG_LS_QUAD = 6;  // results of fg_lin_quad_enqueue ahead of the candidates'
struct LsCand {
  double a[FG_LS_BATCH];
  int n;
};
// Residual norms of the trial points u + a_c du (c < cand.n) in one launch pair:
// out[FG_LS_QUAD + c] = sum over the rows that nonlinear elements touch of F_i^2, with
// F_i = fma(a_c, z_i, y_i) + the nonlinear elements' records at u + a_c du (the
// arithmetic of k_newton_trial64 + k_elem_newton_nl + k_nl_rows, bit for bit).  The
// rest of |F|^2 is out[0] + 2 a out[1] + a^2 out[2] from fg_lin_quad_enqueue.
void fg_newton_trial_batch(fg_mesh *m, const double *d_u, const double *d_du, const double *d_y, const double *d_z,
                           const LsCand &cand, double Ms, double Hk, double *d_out);
// out[0..2] = (y.y, y.z, z.z) over the rows with mask 0, out[3..5] = (u.u, u.du,
// du.du) over all rows (fixed order).
void fg_lin_quad_enqueue(fg_mesh *m, const double *d_y, const double *d_z, const uint8_t *mask, const double *d_u,
                         const double *d_du, double *d_out);
// lin_in: K_lin u already known (a vector, or d_F itself when it holds it), so the
// linear elements' SpMV is skipped; lin_out: where the SpMV also leaves K_lin u;
// d_F null: the Jacobian alone (element state and operator at u).
void fg_newton_assemble_split(fg_mesh *m, const double *d_u, double Ms, double Hk, bool mixed, double *d_F,
                              bool want_jacobian, bool tangent, const double *lin_in = nullptr,
                              double *lin_out = nullptr);
// d_out[i] = sum of the vector records of row i (P1 tetrahedra), no Dirichlet masking.
void fg_vector_gather(fg_mesh *m, double *d_out);
// src/FEM3D.jl:284-297 / src/FEMc.cpp:170-200 BoundaryIntegral into a device vector
// (nv entries written); AE == NULL takes the face areas from the mesh coordinates.
void fg_boundary_rhs_dev(fg_mesh *m, const int32_t *surfaceT, int64_t ns, int32_t index_base, const double *normal,
                         const double *AE, const double *F, const int32_t *shell_id, int32_t nshell, double *d_out);
// Demagnetising field (Micromagnetics/LL.jl:162-211): load vector of the inside
// elements from the nodal magnetisation, and the nodal volume average of H.
void fg_demag_rhs_dev(fg_mesh *m, const uint8_t *d_inside, const double *d_M, double *d_b);
void fg_nodal_average_dev(fg_mesh *m, const uint8_t *d_inside, const double *d_H, double *d_work, double *d_Hn);
// y = vals x on the handle's pattern (FP64), Dirichlet rows 0.
void fg_spmv64_vals(fg_mesh *m, const double *vals, const double *x, double *y);
void fg_apply_operator_vec(fg_mesh *m, int kind, const double *d_coef, double c_mass, double c_stiff,
                           const double *d_x, double *d_y, bool zero_fixed);
void fg_hfield_dev(fg_mesh *m, const double *d_u, double *d_H);
// Energy density integral times VE per element into m->wdens (from the potential).
void fg_energy_dev(fg_mesh *m, const double *d_u, double Ms, double Hk);
// Objective J = sum_T VE Hx / sum_T VE over the target elements: per-element parts
// VE Hx and VE (zero outside the target) into d_a, d_v (nt each).
void fg_objective_parts_dev(fg_mesh *m, const double *d_u, const uint8_t *d_target, double *d_a, double *d_v);
// dJ/du (zero on Dirichlet rows) into d_g, for a target volume vol.
void fg_objective_rhs_dev(fg_mesh *m, const uint8_t *d_target, double vol, double *d_g);
// grad_k = scale VE_k grad(lambda).grad(u) per element.
void fg_adjoint_grad_dev(fg_mesh *m, const double *d_lam, const double *d_u, double scale, double *d_grad);

// solve (fg_solve.cu)
double fg_norm2_dev(fg_mesh *m, const double *x, int64_t n, bool mask_fixed);
double fg_dot_dev(fg_mesh *m, const double *x, const double *y, int64_t n, bool mask_fixed);
// Enqueues x.y into scal[slot] (slots 10-15 are free for callers) without waiting.
void fg_dot_enqueue(fg_mesh *m, const double *x, const double *y, int64_t n, bool mask_fixed, int slot);
// F <- -F over the handle's rows with |F|^2 left in scal[FG_SLOT_FNORM2]; the square
// root of that slot read back (one host wait).
constexpr int FG_SLOT_FNORM2 = 12;
void fg_negate_norm2_enqueue(fg_mesh *m, double *F);
double fg_slot_sqrt(fg_mesh *m, int slot);
// Throws the error that a device flag word h reports (no-op for 0).
void fg_raise_flags(fg_mesh *m, int h, const char *where);
// Solves A x = b (A = the handle's operator, SELL layout) on free rows.  b, x are FP64
// device vectors; x holds the initial guess.  Returns iterations; stats filled.
// newton_inner: one inner solve from x = 0 (no FP64 refinement), not timed; b_norm,
// when >= 0, is |b| on the free rows, already known to the caller.
int fg_pcg_solve(fg_mesh *m, const double *d_b, double *d_x, const fg_solve_opts &o, fg_solve_stats *st,
                 bool newton_inner, double b_norm = -1.0);
void fg_spmv64_dev(fg_mesh *m, const double *x, double *y);
// r = b - A x with the given SELL values (no Dirichlet masking); returns ||r|| (syncs)
double fg_residual_norm(fg_mesh *m, const double *vals, const double *x, const double *b, double *r);
// y = A x with the given SELL values and no Dirichlet masking
void fg_spmv64_plain(fg_mesh *m, const double *vals, const double *x, double *y);
// Jacobi right-preconditioned BiCGStab on the FP64 operator (val64, dinv64), no
// Dirichlet rows; d_x holds the initial guess and receives the solution.
// Returns 0 converged, 1 iteration limit, 2 breakdown.
int fg_bicgstab_solve(fg_mesh *m, const double *d_b, double *d_x, const fg_solve_opts &o, fg_solve_stats *st);
// Nedelec edge elements (handles from fg_edge_mesh_create): the operator
// nu-weighted curl-curl (with_stiff) plus the tangential term when d_dnu is given, to
// SELL (val64/dinv64, val32/dinv32 when want32) or to csrval; the load vector
// Bext.curlN; B per element from the edge values.
void fg_nedelec_operator(fg_mesh *m, const double *d_nu, bool with_stiff, const double *d_dnu, const double *d_Bf,
                         const double *d_Bn, int layout, bool want32);
void fg_nedelec_load_dev(fg_mesh *m, const double bext[3], double *d_rhs);
void fg_nedelec_bfield_dev(fg_mesh *m, const double *d_u, double *d_Bf, double *d_Bn);
void fg_nedelec_local_dev(fg_mesh *m, double *d_Ak);
// Backward-Euler transport operator of P2 tetrahedra: mval = M(rho_cp) and
// val64/dinv64 = M(rho_cp) + K(kdt) + C^(fdt) (the reference's convection matrix with
// the factor fdt), no boundary conditions.
void fg_transport_operator(fg_mesh *m, const double *d_rhocp, const double *d_kdt, const double *d_vel,
                           const double *d_fdt, int full_phi);
// Adds scale * (the P2 boundary mass of the listed faces) into val64 (refreshing
// dinv64) when sell, else writes it alone into csrval.  Row list rows[0..nrows), each
// row's (face << 3 | face-local node) entries in flist[fptr[i]..fptr[i+1]).
void fg_face_mass(fg_mesh *m, bool sell, const int *d_rows, int64_t nrows, const int *d_fptr, const int *d_flist,
                  const int *d_faces, const double *d_AE, const double *d_F, double scale);
