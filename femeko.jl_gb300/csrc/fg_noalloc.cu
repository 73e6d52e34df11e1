// Jacobi-preconditioned CG on a symmetric CSC matrix held in device memory that
// allocates nothing: no cudaMalloc/cudaFree, no allocating library routine.  The CG
// vectors, reduction partials, scalars and control words live in one fixed scratch
// array per device, compiled into the library (FG_NOALLOC_MAX_ROWS rows at most).
//
// Who cannot allocate: a time loop that solves the same small system every step
// (the demagnetising-field solve of Micromagnetics/LL.jl:162-211 calls cg at :185 on
// every Landau-Lifshitz step) while other work runs on its own streams --
// cudaMalloc/cudaFree may synchronise the whole device, stalling that work -- and
// callers whose device memory is reserved up front by their own pool (a Julia
// CUDA.jl process), where a foreign allocation can fail or evict their cache.
//
// Same iteration as the handle path of fg_cg_csc (Jacobi-PCG, stop when
// ||r|| <= rtol ||r0||), written for small systems: one thread per row over the CSC
// columns (symmetric, so a column is a row), two kernels per iteration.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <mutex>

#include "fg_common.cuh"

namespace {

constexpr int NA_THREADS = 256;
constexpr int NA_MAX_BLOCKS = (int)((FG_NOALLOC_MAX_ROWS + NA_THREADS - 1) / NA_THREADS);
constexpr int NA_MAX_DEVICES = 64;

// Layout of the scratch array (in doubles).
enum { NA_R = 0, NA_Z, NA_P0, NA_P1, NA_Q, NA_DINV, NA_NVEC };
constexpr int64_t NA_PART = (int64_t)NA_NVEC * FG_NOALLOC_MAX_ROWS;  // 2 per block
constexpr int64_t NA_SCAL = NA_PART + 2 * NA_MAX_BLOCKS;             // scalars below
constexpr int64_t NA_CTL = NA_SCAL + 16;                             // 16 x 32-bit words
constexpr int64_t NA_TOTAL = NA_CTL + 8;

enum { SC_RZ = 0, SC_ALPHA, SC_BETA, SC_RR, SC_TOL2, SC_RR0 };
// Control words.  Only C_ARRIVE must be zero when a kernel starts; every call clears
// the whole control block before its first launch, and the last block of each
// reduction puts C_ARRIVE back to zero.
enum { C_ARRIVE = 0, C_DONE, C_ITERS, C_STATUS, C_MAXIT };
enum { ST_RUNNING = 0, ST_CONVERGED = 1, ST_NAN = 2, ST_MAXIT = 3, ST_BAD_INDEX = 4, ST_BAD_DIAG = 5,
       ST_BREAKDOWN = 6 };

}  // namespace

// The scratch: 6 vectors of FG_NOALLOC_MAX_ROWS doubles (6 MiB at 131072 rows) plus
// 8 KiB of partials, scalars and control words.  Zero at module load.
static __device__ __align__(256) double fg_noalloc_scratch[NA_TOTAL];

namespace {

struct NaPtrs {
  double *vec;   // NA_NVEC vectors of FG_NOALLOC_MAX_ROWS
  double *part;
  double *scal;
  unsigned *ctl;
};

__device__ __forceinline__ NaPtrs na_ptrs(double *s) {
  return NaPtrs{s, s + NA_PART, s + NA_SCAL, reinterpret_cast<unsigned *>(s + NA_CTL)};
}

__device__ __forceinline__ double *na_vec(const NaPtrs &P, int which) {
  return P.vec + (int64_t)which * FG_NOALLOC_MAX_ROWS;
}

// Block sums of two values into partials; the last block to arrive adds the
// partials in block order (deterministic) and returns true in thread 0 with tot set.
__device__ bool na_reduce2(double a, double b, const NaPtrs &P, double &tot_a, double &tot_b) {
  __shared__ double sh[2][NA_THREADS / 32];
  __shared__ bool s_last;
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) { sh[0][w] = a; sh[1][w] = b; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double sa = 0.0, sb = 0.0;
    for (int k = 0; k < NA_THREADS / 32; ++k) { sa += sh[0][k]; sb += sh[1][k]; }
    P.part[2 * blockIdx.x] = sa;
    P.part[2 * blockIdx.x + 1] = sb;
    __threadfence();
    s_last = (atomicAdd(P.ctl + C_ARRIVE, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  double ta = 0.0, tb = 0.0;
  for (unsigned k = threadIdx.x; k < gridDim.x; k += NA_THREADS) {
    ta += __ldcg(P.part + 2 * k);
    tb += __ldcg(P.part + 2 * k + 1);
  }
  for (int o = 16; o > 0; o >>= 1) {
    ta += __shfl_down_sync(0xffffffffu, ta, o);
    tb += __shfl_down_sync(0xffffffffu, tb, o);
  }
  __syncthreads();
  if (l == 0) { sh[0][w] = ta; sh[1][w] = tb; }
  __syncthreads();
  if (threadIdx.x != 0) return false;
  tot_a = 0.0;
  tot_b = 0.0;
  for (int k = 0; k < NA_THREADS / 32; ++k) { tot_a += sh[0][k]; tot_b += sh[1][k]; }
  P.ctl[C_ARRIVE] = 0u;
  return true;
}

// Range of column i's entries, checked against nnz; false (and the status set) when
// colptr is not a valid CSC column pointer.
__device__ __forceinline__ bool na_col_range(const int64_t *colptr, int64_t i, int64_t nnz, int base, int64_t &k0,
                                             int64_t &k1, const NaPtrs &P) {
  k0 = colptr[i] - base;
  k1 = colptr[i + 1] - base;
  if (k0 < 0 || k1 < k0 || k1 > nnz) {
    atomicExch(P.ctl + C_STATUS, (unsigned)ST_BAD_INDEX);
    return false;
  }
  return true;
}

// r = b - A x, D^-1 from the diagonal, z = D^-1 r, p = 0; r.z and r.r.
__global__ void __launch_bounds__(NA_THREADS)
    k_na_init(int64_t n, int64_t nnz, const int64_t *__restrict__ colptr, const int64_t *__restrict__ rowval,
              const double *__restrict__ nzval, int base, const double *__restrict__ b,
              const double *__restrict__ x, double rtol2, int maxit, double *scratch) {
  const NaPtrs P = na_ptrs(scratch);
  const int64_t i = (int64_t)blockIdx.x * NA_THREADS + threadIdx.x;
  double rz = 0.0, rr = 0.0;
  if (i < n) {
    double ax = 0.0, diag = 0.0;
    int64_t k0, k1;
    bool bad = true;
    if (na_col_range(colptr, i, nnz, base, k0, k1, P)) {
      bad = false;
      for (int64_t k = k0; k < k1; ++k) {
        const int64_t j = rowval[k] - base;
        if (j < 0 || j >= n) {
          atomicExch(P.ctl + C_STATUS, (unsigned)ST_BAD_INDEX);
          bad = true;
          continue;
        }
        const double a = nzval[k];
        ax = fma(a, x[j], ax);
        if (j == i) diag += a;
      }
    }
    const double r = b[i] - ax;
    // a Jacobi preconditioner needs a nonzero finite diagonal (a symmetric positive
    // definite matrix has a positive one): report the row instead of dividing by zero.
    // A structure error takes precedence (it is written unconditionally, this only
    // over a running status), and a row with a bad index reports only that.
    if (!bad && (!(diag != 0.0) || !isfinite(diag)))
      atomicCAS(P.ctl + C_STATUS, (unsigned)ST_RUNNING, (unsigned)ST_BAD_DIAG);
    const double dinv = (diag != 0.0 && isfinite(diag)) ? 1.0 / diag : 0.0;
    const double z = dinv * r;
    na_vec(P, NA_R)[i] = r;
    na_vec(P, NA_Z)[i] = z;
    na_vec(P, NA_DINV)[i] = dinv;
    na_vec(P, NA_P0)[i] = 0.0;
    na_vec(P, NA_P1)[i] = 0.0;
    rz = r * z;
    rr = r * r;
  }
  double trz, trr;
  if (na_reduce2(rz, rr, P, trz, trr)) {
    P.scal[SC_RZ] = trz;
    P.scal[SC_RR] = trr;
    P.scal[SC_RR0] = trr;
    P.scal[SC_TOL2] = rtol2 * trr;
    P.scal[SC_ALPHA] = 0.0;
    P.scal[SC_BETA] = 0.0;
    P.ctl[C_ITERS] = 0u;
    P.ctl[C_MAXIT] = (unsigned)maxit;
    unsigned st = __ldcg(P.ctl + C_STATUS);  // set by any block before it arrived
    if (st == ST_RUNNING) {
      if (!isfinite(trr) || !isfinite(trz)) st = ST_NAN;
      else if (trr == 0.0) st = ST_CONVERGED;
      else if (maxit <= 0) st = ST_MAXIT;
    }
    P.ctl[C_STATUS] = st;
    P.ctl[C_DONE] = (st != ST_RUNNING) ? 1u : 0u;
  }
}

// p_new = z + beta p_old, q = A p_new (neighbour entries of p_new formed on the fly
// from z and p_old), p_new.q; alpha = r.z / p.q.
__global__ void __launch_bounds__(NA_THREADS)
    k_na_spmv(int64_t n, int64_t nnz, const int64_t *__restrict__ colptr, const int64_t *__restrict__ rowval,
              const double *__restrict__ nzval, int base, int pin, double *scratch) {
  const NaPtrs P = na_ptrs(scratch);
  if (P.ctl[C_DONE]) return;
  const double beta = P.scal[SC_BETA];
  const double *z = na_vec(P, NA_Z);
  const double *po = na_vec(P, pin);
  double *pn = na_vec(P, pin == NA_P0 ? NA_P1 : NA_P0);
  const int64_t i = (int64_t)blockIdx.x * NA_THREADS + threadIdx.x;
  double pq = 0.0;
  if (i < n) {
    double q = 0.0;
    int64_t k0, k1;
    if (na_col_range(colptr, i, nnz, base, k0, k1, P))
      for (int64_t k = k0; k < k1; ++k) {
        const int64_t j = rowval[k] - base;
        if (j < 0 || j >= n) continue;  // reported by k_na_init
        q = fma(nzval[k], fma(beta, po[j], z[j]), q);
      }
    const double p = fma(beta, po[i], z[i]);
    pn[i] = p;
    na_vec(P, NA_Q)[i] = q;
    pq = p * q;
  }
  double tpq, unused;
  if (na_reduce2(pq, 0.0, P, tpq, unused)) {
    if (!isfinite(tpq) || tpq <= 0.0) {
      // p.q = 0 ends the iteration: converged only if the residual already meets the
      // tolerance, a breakdown otherwise; p.q < 0: the matrix is not positive definite
      unsigned stop = ST_NAN;
      if (isfinite(tpq) && tpq == 0.0) stop = (P.scal[SC_RR] <= P.scal[SC_TOL2]) ? ST_CONVERGED : ST_BREAKDOWN;
      P.ctl[C_STATUS] = stop;
      P.ctl[C_DONE] = 1u;
    } else {
      P.scal[SC_ALPHA] = P.scal[SC_RZ] / tpq;
    }
  }
}

// x += alpha p, r -= alpha q, z = D^-1 r; r.z, r.r; beta, convergence.
__global__ void __launch_bounds__(NA_THREADS)
    k_na_update(int64_t n, int pnew, double *__restrict__ x, double *scratch) {
  const NaPtrs P = na_ptrs(scratch);
  if (P.ctl[C_DONE]) return;
  const double alpha = P.scal[SC_ALPHA];
  const int64_t i = (int64_t)blockIdx.x * NA_THREADS + threadIdx.x;
  double rz = 0.0, rr = 0.0;
  if (i < n) {
    x[i] = fma(alpha, na_vec(P, pnew)[i], x[i]);
    const double r = fma(-alpha, na_vec(P, NA_Q)[i], na_vec(P, NA_R)[i]);
    const double z = na_vec(P, NA_DINV)[i] * r;
    na_vec(P, NA_R)[i] = r;
    na_vec(P, NA_Z)[i] = z;
    rz = r * z;
    rr = r * r;
  }
  double trz, trr;
  if (na_reduce2(rz, rr, P, trz, trr)) {
    const unsigned it = P.ctl[C_ITERS] + 1u;
    P.ctl[C_ITERS] = it;
    P.scal[SC_BETA] = trz / P.scal[SC_RZ];
    P.scal[SC_RZ] = trz;
    P.scal[SC_RR] = trr;
    unsigned st = ST_RUNNING;
    if (!isfinite(trr) || !isfinite(trz)) st = ST_NAN;
    else if (trr <= P.scal[SC_TOL2]) st = ST_CONVERGED;
    else if (it >= P.ctl[C_MAXIT]) st = ST_MAXIT;
    if (st != ST_RUNNING) {
      P.ctl[C_STATUS] = st;
      P.ctl[C_DONE] = 1u;
    }
  }
}

// Device address of the scratch, looked up once per device (with that device
// current) and kept; the lock also serialises calls on one device, which would
// otherwise race on the shared scratch.
std::mutex g_na_lock[NA_MAX_DEVICES];
double *g_na_ptr[NA_MAX_DEVICES] = {nullptr};

fg_status na_fail(fg_status code, const char *msg) {
  fg_set_error(msg);
  return code;
}

// True when the kernels, launched on device `dev`, can read and write p: managed
// memory or memory of `dev` itself.  Another device's memory is refused even where
// peer access would reach it: the check stays a pure query of the pointer.
bool na_device_pointer(const void *p, int dev) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (a.type == cudaMemoryTypeManaged) return true;
  return a.type == cudaMemoryTypeDevice && a.device == dev;
}

}  // namespace

extern "C" fg_status fg_cg_csc_noalloc(int64_t n, const int64_t *colptr, const int64_t *rowval,
                                       const double *nzval, int32_t index_base, const double *b, double *x,
                                       const fg_solve_opts *o, void *stream, fg_solve_stats *s) {
  const auto t0 = std::chrono::steady_clock::now();
  if (!colptr || !rowval || !nzval || !b || !x) return na_fail(FG_BAD_ARG, "fg_cg_csc_noalloc: null pointer");
  if (n <= 0) return na_fail(FG_BAD_ARG, "fg_cg_csc_noalloc: n must be positive");
  if (n > FG_NOALLOC_MAX_ROWS) {
    char msg[160];
    snprintf(msg, sizeof msg, "fg_cg_csc_noalloc: %lld rows exceed the fixed scratch of %lld rows", (long long)n,
             (long long)FG_NOALLOC_MAX_ROWS);
    return na_fail(FG_BAD_ARG, msg);
  }
  if (index_base != 0 && index_base != 1) return na_fail(FG_BAD_ARG, "fg_cg_csc_noalloc: index_base must be 0 or 1");
  fg_solve_opts opts;
  fg_solve_opts_default(&opts);
  if (o) opts = *o;
  if (opts.precision != FG_FP64) return na_fail(FG_UNSUPPORTED, "fg_cg_csc_noalloc: FP64 only");
  if (!(opts.rtol >= 0.0)) return na_fail(FG_BAD_ARG, "fg_cg_csc_noalloc: rtol must be >= 0");
  const int check = opts.check_every > 0 ? opts.check_every : 32;
  // maxiter <= 0 means "no cap given": the default of fg_solve_opts_default, as with o == NULL
  fg_solve_opts dflt;
  fg_solve_opts_default(&dflt);
  const int maxit = opts.maxiter > 0 ? opts.maxiter : dflt.maxiter;

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NA_MAX_DEVICES)
    return na_fail(FG_NO_DEVICE, "fg_cg_csc_noalloc: no current CUDA device");
  if (!na_device_pointer(colptr, dev) || !na_device_pointer(rowval, dev) || !na_device_pointer(nzval, dev) ||
      !na_device_pointer(b, dev) || !na_device_pointer(x, dev))
    return na_fail(FG_BAD_ARG,
                   "fg_cg_csc_noalloc: every array must be managed memory or memory of the current device");

  std::lock_guard<std::mutex> guard(g_na_lock[dev]);
  if (!g_na_ptr[dev]) {
    void *ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, fg_noalloc_scratch);
    if (e != cudaSuccess || !ptr) {
      fg_set_error(std::string("fg_cg_csc_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      return FG_CUDA;
    }
    g_na_ptr[dev] = static_cast<double *>(ptr);
  }
  double *scr = g_na_ptr[dev];
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned *ctl = reinterpret_cast<unsigned *>(scr + NA_CTL);

  auto cuda_fail = [&](cudaError_t e, const char *what) {
    fg_set_error(std::string("fg_cg_csc_noalloc: ") + what + ": " + cudaGetErrorString(e));
    return FG_CUDA;
  };
  // nnz from the last column pointer (the kernels check every column range against it)
  int64_t last = 0;
  cudaError_t e = cudaMemcpyAsync(&last, colptr + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "reading colptr[n]");
  const int64_t nnz = last - index_base;
  if (nnz < 0) return na_fail(FG_BAD_ARG, "fg_cg_csc_noalloc: colptr[n] below index_base");

  e = cudaMemsetAsync(ctl, 0, 16 * sizeof(unsigned), st);
  if (e != cudaSuccess) return cuda_fail(e, "clearing the control words");
  const unsigned grid = (unsigned)((n + NA_THREADS - 1) / NA_THREADS);
  k_na_init<<<grid, NA_THREADS, 0, st>>>(n, nnz, colptr, rowval, nzval, index_base, b, x, opts.rtol * opts.rtol,
                                          maxit, scr);
  FG_LAUNCHED(1);
  unsigned hc[8] = {0};
  int64_t launched = 0;
  for (;;) {
    for (int k = 0; k < check; ++k, ++launched) {
      const int pin = (launched & 1) ? NA_P1 : NA_P0;
      const int pnew = (launched & 1) ? NA_P0 : NA_P1;
      k_na_spmv<<<grid, NA_THREADS, 0, st>>>(n, nnz, colptr, rowval, nzval, index_base, pin, scr);
      k_na_update<<<grid, NA_THREADS, 0, st>>>(n, pnew, x, scr);
    }
    FG_LAUNCHED(2LL * check);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(hc, ctl, sizeof hc, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "CG iterations");
    if (hc[C_DONE]) break;
    if (launched > (int64_t)maxit + check) break;  // the device stops at maxit; never reached
  }
  double hs[8] = {0};
  e = cudaMemcpyAsync(hs, scr + NA_SCAL, sizeof hs, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "reading the result");
  const unsigned status = hc[C_STATUS];
  if (s) {
    s->iterations = (int32_t)hc[C_ITERS];
    s->refinements = 0;
    s->converged = status == ST_CONVERGED;
    s->pad_ = 0;
    s->relres = hs[SC_RR0] > 0.0 ? std::sqrt(hs[SC_RR] / hs[SC_RR0]) : 0.0;
    s->ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  switch (status) {
    case ST_CONVERGED: return FG_OK;
    case ST_NAN: return na_fail(FG_NAN, "fg_cg_csc_noalloc: CG produced a non-finite or non-positive curvature");
    case ST_BAD_INDEX: return na_fail(FG_BAD_ARG, "fg_cg_csc_noalloc: colptr/rowval not a valid CSC structure");
    case ST_BAD_DIAG: return na_fail(FG_BAD_ARG, "fg_cg_csc_noalloc: a zero or non-finite diagonal entry");
    case ST_BREAKDOWN:
      return na_fail(FG_NOT_CONVERGED, "fg_cg_csc_noalloc: p.q = 0 before the residual met the tolerance");
    default: return na_fail(FG_NOT_CONVERGED, "fg_cg_csc_noalloc: iteration cap reached");
  }
}
