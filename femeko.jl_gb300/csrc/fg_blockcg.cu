// Block conjugate gradients for a sweep of applied fields (the hysteresis-loop use of
// Magnetostatics/magneticField.jl:89-132: K(mu) u = 0 on free rows, u = -H0.x on the
// Dirichlet rows, for many H0 on one linear mesh).
//
// The right-hand sides are rank-deficient by construction: the lifted residual of
// field c is R0_c = -K(-H0_c . x) = sum_k H0_c,k R0(e_k), so the residual block
// [R0_1 .. R0_m] = [R0(e_x) R0(e_y) R0(e_z)] H0^T has rank r <= 3, the rank of H0.
// A rank-revealing factorisation of the block is therefore that of H0 (m x 3, on
// the host: one-sided Jacobi SVD, directions whose singular value is below 1e-13 of
// the largest dropped): H0 = C V^T with V (3 x r) orthonormal field directions and
// C = H0 V (m x r).  One block CG of width r solves the r direction
// problems together, and every field's potential is the combination
// u_c = sum_k C_c,k u(v_k) (exact: the problem is linear in H0).
//
// Block CG (O'Leary 1980) with the Jacobi preconditioner M = D^-1:
//   Q = A P;  alpha = (P^T Q)^-1 (Z^T R);  X += P alpha;  R -= Q alpha;  Z = M R;
//   beta = (Z_old^T R_old)^-1 (Z^T R);  P = Z + P beta
// The r x r systems are solved in FP64 by a Cholesky factorisation that drops a
// direction whose pivot falls below 1e-12 of the largest diagonal entry (a column
// that has converged or become dependent on the others), so a rank-deficient block
// does not break the iteration.
// Precision: FP32 matrix and inner block CG (compensated FP32 dot products), FP64
// outer residual, solution and Gram matrices (iterative refinement), as the
// per-field sweep.  Every field's residual is checked exactly at each refinement:
// |R_c|^2 = C_c G C_c^T with G the FP64 Gram matrix of the direction residuals.
//
// Layout: row-major blocks of 4 columns per row (float4 / 2 x double2 per row), one
// thread per row over the SELL-32x4 operator; directions beyond r are zero columns.
#include <algorithm>
#include <cmath>
#include <vector>

#include "fg_common.cuh"
#include "fg_reduce.cuh"

namespace {

constexpr int BC_T = 256;
constexpr int BC_SYM = 10;  // upper triangle of a symmetric 4 x 4
__constant__ int c_sym_a[BC_SYM] = {0, 0, 0, 0, 1, 1, 1, 2, 2, 3};
__constant__ int c_sym_b[BC_SYM] = {0, 1, 2, 3, 1, 2, 3, 2, 3, 3};

// Device scalars (doubles): full 4 x 4 matrices, row-major
enum { B_RZ = 0, B_ALPHA = 16, B_BETA = 32, B_TOL2 = 48, B_RR = 52, B_NSCAL = 64 };
// Control words
enum { C_DONE = 0, C_ITERS, C_MAXIT, C_STATUS, C_NCTL = 8 };
enum { BS_RUNNING = 0, BS_CONVERGED = 1, BS_NAN = 2, BS_MAXIT = 3 };

struct BcOp {
  int64_t n;
  const int *sl_ptr, *sl_len, *sl_col;
  const uint8_t *fixed;
};

__device__ __forceinline__ float get(const float4 &v, int k) {
  return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w));
}

// y = v M for a row vector v (4) and M (4 x 4, row-major floats).
__device__ __forceinline__ float4 vecmat(const float4 &v, const float (&M)[16]) {
  float4 y;
  y.x = v.x * M[0] + v.y * M[4] + v.z * M[8] + v.w * M[12];
  y.y = v.x * M[1] + v.y * M[5] + v.z * M[9] + v.w * M[13];
  y.z = v.x * M[2] + v.y * M[6] + v.z * M[10] + v.w * M[14];
  y.w = v.x * M[3] + v.y * M[7] + v.z * M[11] + v.w * M[15];
  return y;
}

// X = S^-1 M for a symmetric positive semi-definite S (4 x 4) by Cholesky; a pivot
// below tol * max(diag S) drops its direction (its rows of X are zero).
// One reciprocal per pivot, multiplications elsewhere: an FP64 division is a long
// instruction sequence on a pipe that runs at 1/64 of the FP32 rate, and this runs in
// one thread at the end of every block iteration.
__device__ void chol_solve_drop(const double *S, const double *M, double *X) {
  double L[4][4] = {{0.0}};
  double inv[4] = {0.0, 0.0, 0.0, 0.0};
  bool keep[4];
  double smax = 0.0;
  for (int j = 0; j < 4; ++j) smax = fmax(smax, S[5 * j]);
  const double tol = 1e-12 * smax;
  for (int j = 0; j < 4; ++j) {
    double d = S[5 * j];
    for (int k = 0; k < j; ++k)
      if (keep[k]) d -= L[j][k] * L[j][k];
    keep[j] = smax > 0.0 && d > tol && isfinite(d);
    if (!keep[j]) continue;
    L[j][j] = sqrt(d);
    inv[j] = 1.0 / L[j][j];
    for (int i = j + 1; i < 4; ++i) {
      double v = S[4 * i + j];
      for (int k = 0; k < j; ++k)
        if (keep[k]) v -= L[i][k] * L[j][k];
      L[i][j] = v * inv[j];
    }
  }
  double Y[4][4];
  for (int i = 0; i < 4; ++i)
    for (int c = 0; c < 4; ++c) {
      if (!keep[i]) { Y[i][c] = 0.0; continue; }
      double v = M[4 * i + c];
      for (int k = 0; k < i; ++k)
        if (keep[k]) v -= L[i][k] * Y[k][c];
      Y[i][c] = v * inv[i];
    }
  for (int i = 3; i >= 0; --i)
    for (int c = 0; c < 4; ++c) {
      if (!keep[i]) { X[4 * i + c] = 0.0; continue; }
      double v = Y[i][c];
      for (int k = i + 1; k < 4; ++k)
        if (keep[k]) v -= L[k][i] * X[4 * k + c];
      X[4 * i + c] = v * inv[i];
    }
}

// Symmetric 4 x 4 from its upper triangle.
__device__ __forceinline__ void unpack_sym(const double (&t)[BC_SYM], double *S) {
  for (int q = 0; q < BC_SYM; ++q) {
    S[4 * c_sym_a[q] + c_sym_b[q]] = t[q];
    S[4 * c_sym_b[q] + c_sym_a[q]] = t[q];
  }
}

__device__ __forceinline__ void add_sym_ff(ff (&acc)[BC_SYM], const float4 &a, const float4 &b) {
#pragma unroll
  for (int q = 0; q < BC_SYM; ++q) {
    const int i = q < 4 ? 0 : (q < 7 ? 1 : (q < 9 ? 2 : 3));
    const int j = q < 4 ? q : (q < 7 ? q - 3 : (q < 9 ? q - 5 : 3));
    // a_i b_j + a_j b_i over 2 (symmetric part; a and b are R and Z or P and Q)
    const float v = i == j ? get(a, i) * get(b, i) : 0.5f * (get(a, i) * get(b, j) + get(a, j) * get(b, i));
    acc[q] = ff_add(acc[q], ff{v, 0.f});
  }
}

// Four per-column factors passed by value.
struct Col4 {
  double v[4];
};

// X64[i][k] = -v_k . p_i (the lifted Dirichlet values and initial guess).
struct Dirs {
  double v[4][3];
};
__global__ void k_bc_lift(int64_t n, const double *__restrict__ p, Dirs d, double *__restrict__ X) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double x = p[3 * i], y = p[3 * i + 1], z = p[3 * i + 2];
#pragma unroll
  for (int k = 0; k < 4; ++k) X[4 * i + k] = -(d.v[k][0] * x + d.v[k][1] * y + d.v[k][2] * z);
}

// R = -A X on free rows (FP64), and the block's partial Gram matrix R^T R (upper
// triangle) into partials[block][10].
__global__ void __launch_bounds__(BC_T) k_bc_resid64(BcOp A, const double *__restrict__ val,
                                                     const double *__restrict__ X, double *__restrict__ R,
                                                     double *__restrict__ partials) {
  __shared__ double sh[BC_SYM][BC_T / 32];
  const int64_t i = (int64_t)blockIdx.x * BC_T + threadIdx.x;
  double g[BC_SYM];
#pragma unroll
  for (int q = 0; q < BC_SYM; ++q) g[q] = 0.0;
  if (i < A.n) {
    double y[4] = {0.0, 0.0, 0.0, 0.0};
    const bool fx = A.fixed && A.fixed[i];
    if (!fx) {
      const int s = (int)(i >> 5), lane = (int)(i & 31);
      const int G = A.sl_len[s];
      const int64_t base = A.sl_ptr[s];
      for (int q = 0; q < FG_GROUP * G; ++q) {
        const int64_t e = sell_pos(base, lane, q);
        const double a = val[e];
        const double2 *xr = reinterpret_cast<const double2 *>(X + 4 * (int64_t)A.sl_col[e]);
        const double2 x01 = xr[0], x23 = xr[1];
        y[0] = fma(a, x01.x, y[0]);
        y[1] = fma(a, x01.y, y[1]);
        y[2] = fma(a, x23.x, y[2]);
        y[3] = fma(a, x23.y, y[3]);
      }
    }
    const double r[4] = {fx ? 0.0 : -y[0], fx ? 0.0 : -y[1], fx ? 0.0 : -y[2], fx ? 0.0 : -y[3]};
    double2 *rr = reinterpret_cast<double2 *>(R + 4 * i);
    rr[0] = make_double2(r[0], r[1]);
    rr[1] = make_double2(r[2], r[3]);
#pragma unroll
    for (int q = 0; q < BC_SYM; ++q) g[q] = r[c_sym_a[q]] * r[c_sym_b[q]];
  }
#pragma unroll
  for (int q = 0; q < BC_SYM; ++q)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) g[q] += __shfl_down_sync(0xffffffffu, g[q], o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0)
#pragma unroll
    for (int q = 0; q < BC_SYM; ++q) sh[q][w] = g[q];
  __syncthreads();
  if (threadIdx.x < BC_SYM) {
    double t = 0.0;
    for (int k = 0; k < BC_T / 32; ++k) t += sh[threadIdx.x][k];
    partials[(int64_t)blockIdx.x * BC_SYM + threadIdx.x] = t;
  }
}

// Gram matrix (full 4 x 4) from the per-block partials, summed in block order.
__global__ void k_bc_gram(const double *__restrict__ partials, int nblocks, double *__restrict__ gram) {
  __shared__ double sh[BC_SYM][32];
  const int q = threadIdx.x >> 5, l = threadIdx.x & 31;  // 10 warps, one entry each
  double t = 0.0;
  for (int b = l; b < nblocks; b += 32) t += partials[(int64_t)b * BC_SYM + q];
  sh[q][l] = t;
  __syncthreads();
  if (l == 0) {
    double s = 0.0;
    for (int k = 0; k < 32; ++k) s += sh[q][k];
    gram[4 * c_sym_a[q] + c_sym_b[q]] = s;
    gram[4 * c_sym_b[q] + c_sym_a[q]] = s;
  }
}

// Start of an inner solve: r = R64 scale (per column), z = D^-1 r, p = x = 0, Z^T R;
// the last block sets the scalars (beta = 0, tolerances, control words).
__global__ void __launch_bounds__(BC_T) k_bc_init32(int64_t n, const double *__restrict__ R, Col4 scale,
                                                    double inner2, int maxit, const float *__restrict__ dinv,
                                                    float4 *__restrict__ r, float4 *__restrict__ z,
                                                    float4 *__restrict__ p, float4 *__restrict__ x,
                                                    double *__restrict__ scal, int *__restrict__ ctl,
                                                    float2 *__restrict__ partials, unsigned *__restrict__ counter) {
  const int64_t i = (int64_t)blockIdx.x * BC_T + threadIdx.x;
  ff acc[BC_SYM];
#pragma unroll
  for (int q = 0; q < BC_SYM; ++q) acc[q] = ff{0.f, 0.f};
  if (i < n) {
    const double2 *rr = reinterpret_cast<const double2 *>(R + 4 * i);
    const double2 a = rr[0], b = rr[1];
    const float4 ri = make_float4((float)(a.x * scale.v[0]), (float)(a.y * scale.v[1]), (float)(b.x * scale.v[2]),
                                  (float)(b.y * scale.v[3]));
    const float d = dinv[i];
    const float4 zi = make_float4(d * ri.x, d * ri.y, d * ri.z, d * ri.w);
    r[i] = ri;
    z[i] = zi;
    p[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    x[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    add_sym_ff(acc, zi, ri);
  }
  __shared__ ff shb[BC_SYM][32];
  block_sum_ff_pair<BC_SYM>(acc, shb);
  double tot[BC_SYM];
  if (grid_finish_ff<BC_SYM>(acc, partials, counter, tot)) {
    unpack_sym(tot, scal + B_RZ);
    const double *sc = scale.v;
    for (int k = 0; k < 16; ++k) {
      scal[B_ALPHA + k] = 0.0;
      scal[B_BETA + k] = 0.0;
    }
    bool any = false;
    for (int k = 0; k < 4; ++k) {
      scal[B_TOL2 + k] = sc[k] > 0.0 ? inner2 : 0.0;  // the scaled residual starts at 1
      scal[B_RR + k] = sc[k] > 0.0 ? 1.0 : 0.0;
      any |= sc[k] > 0.0;
    }
    ctl[C_ITERS] = 0;
    ctl[C_MAXIT] = maxit;
    ctl[C_STATUS] = any ? BS_RUNNING : BS_CONVERGED;
    ctl[C_DONE] = any ? 0 : 1;
  }
}

// p_new = z + p_old beta, q = A p_new (neighbours' p_new formed from their z and
// p_old), P^T Q; the last block solves alpha = (P^T Q)^-1 (Z^T R).
__global__ void __launch_bounds__(BC_T) k_bc_spmm32(BcOp A, const float *__restrict__ val,
                                                    const float4 *__restrict__ z, const float4 *__restrict__ pold,
                                                    float4 *__restrict__ pnew, float4 *__restrict__ q,
                                                    double *__restrict__ scal, int *__restrict__ ctl,
                                                    float2 *__restrict__ partials, unsigned *__restrict__ counter) {
  if (ctl[C_DONE]) return;
  float beta[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) beta[k] = (float)scal[B_BETA + k];
  const int64_t i = (int64_t)blockIdx.x * BC_T + threadIdx.x;
  ff acc[BC_SYM];
#pragma unroll
  for (int k = 0; k < BC_SYM; ++k) acc[k] = ff{0.f, 0.f};
  if (i < A.n) {
    const bool fx = A.fixed && A.fixed[i];
    float4 y = make_float4(0.f, 0.f, 0.f, 0.f);
    if (!fx) {
      const int s = (int)(i >> 5), lane = (int)(i & 31);
      const int G = A.sl_len[s];
      const int64_t base = A.sl_ptr[s];
      for (int g = 0; g < G; ++g) {
        const int64_t e = base + ((int64_t)g * FG_SLICE + lane) * FG_GROUP;
        const float4 a4 = __ldg(reinterpret_cast<const float4 *>(val + e));
        const int4 c4 = __ldg(reinterpret_cast<const int4 *>(A.sl_col + e));
        const int cs[4] = {c4.x, c4.y, c4.z, c4.w};
        const float as[4] = {a4.x, a4.y, a4.z, a4.w};
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          const float4 zj = z[cs[t]], pj = pold[cs[t]];
          const float4 pb = vecmat(pj, beta);
          y.x = fmaf(as[t], zj.x + pb.x, y.x);
          y.y = fmaf(as[t], zj.y + pb.y, y.y);
          y.z = fmaf(as[t], zj.z + pb.z, y.z);
          y.w = fmaf(as[t], zj.w + pb.w, y.w);
        }
      }
    }
    float4 pi = make_float4(0.f, 0.f, 0.f, 0.f);
    if (!fx) {
      const float4 zi = z[i], po = pold[i];
      const float4 pb = vecmat(po, beta);
      pi = make_float4(zi.x + pb.x, zi.y + pb.y, zi.z + pb.z, zi.w + pb.w);
    }
    pnew[i] = pi;
    q[i] = y;
    add_sym_ff(acc, pi, y);
  }
  __shared__ ff shb[BC_SYM][32];
  block_sum_ff_pair<BC_SYM>(acc, shb);
  double tot[BC_SYM];
  if (grid_finish_ff<BC_SYM>(acc, partials, counter, tot)) {
    double PQ[16], al[16];
    unpack_sym(tot, PQ);
    bool fin = true;
    for (int k = 0; k < 16; ++k) fin &= isfinite(PQ[k]);
    if (!fin) {
      ctl[C_STATUS] = BS_NAN;
      ctl[C_DONE] = 1;
      return;
    }
    chol_solve_drop(PQ, scal + B_RZ, al);
    for (int k = 0; k < 16; ++k) scal[B_ALPHA + k] = al[k];
  }
}

// x += p alpha, r -= q alpha, z = D^-1 r; Z^T R and the columns' r.r; the last block
// forms beta = (Z_old^T R_old)^-1 (Z^T R) and tests every column's tolerance.
__global__ void __launch_bounds__(BC_T) k_bc_update32(int64_t n, const float *__restrict__ dinv,
                                                      const float4 *__restrict__ p, const float4 *__restrict__ q,
                                                      float4 *__restrict__ r, float4 *__restrict__ z,
                                                      float4 *__restrict__ x, double *__restrict__ scal,
                                                      int *__restrict__ ctl, float2 *__restrict__ partials,
                                                      unsigned *__restrict__ counter) {
  if (ctl[C_DONE]) return;
  float al[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) al[k] = (float)scal[B_ALPHA + k];
  const int64_t i = (int64_t)blockIdx.x * BC_T + threadIdx.x;
  constexpr int NS = BC_SYM + 4;
  ff acc[NS];
#pragma unroll
  for (int k = 0; k < NS; ++k) acc[k] = ff{0.f, 0.f};
  if (i < n) {
    const float4 pi = p[i], qi = q[i];
    const float4 pa = vecmat(pi, al), qa = vecmat(qi, al);
    float4 xi = x[i], ri = r[i];
    xi.x += pa.x; xi.y += pa.y; xi.z += pa.z; xi.w += pa.w;
    ri.x -= qa.x; ri.y -= qa.y; ri.z -= qa.z; ri.w -= qa.w;
    const float d = dinv[i];
    const float4 zi = make_float4(d * ri.x, d * ri.y, d * ri.z, d * ri.w);
    x[i] = xi;
    r[i] = ri;
    z[i] = zi;
    ff sym[BC_SYM];
#pragma unroll
    for (int k = 0; k < BC_SYM; ++k) sym[k] = acc[k];
    add_sym_ff(sym, zi, ri);
#pragma unroll
    for (int k = 0; k < BC_SYM; ++k) acc[k] = sym[k];
#pragma unroll
    for (int k = 0; k < 4; ++k) acc[BC_SYM + k] = ff_add(acc[BC_SYM + k], ff{get(ri, k) * get(ri, k), 0.f});
  }
  __shared__ ff shb[NS][32];
  block_sum_ff_pair<NS>(acc, shb);
  double tot[NS];
  if (grid_finish_ff<NS>(acc, partials, counter, tot)) {
    double RZn[16], be[16];
    double t10[BC_SYM];
    for (int k = 0; k < BC_SYM; ++k) t10[k] = tot[k];
    unpack_sym(t10, RZn);
    chol_solve_drop(scal + B_RZ, RZn, be);
    const int it = ctl[C_ITERS] + 1;
    ctl[C_ITERS] = it;
    bool fin = true, conv = true;
    for (int k = 0; k < 16; ++k) {
      scal[B_RZ + k] = RZn[k];
      scal[B_BETA + k] = be[k];
      fin &= isfinite(RZn[k]);
    }
    for (int k = 0; k < 4; ++k) {
      const double rr = tot[BC_SYM + k];
      scal[B_RR + k] = rr;
      fin &= isfinite(rr);
      conv &= rr <= scal[B_TOL2 + k];
    }
    int st = BS_RUNNING;
    if (!fin) st = BS_NAN;
    else if (conv) st = BS_CONVERGED;
    else if (it >= ctl[C_MAXIT]) st = BS_MAXIT;
    if (st != BS_RUNNING) {
      ctl[C_STATUS] = st;
      ctl[C_DONE] = 1;
    }
  }
}

// X64 += x32 / scale per column (the refinement update); x32 is 0 on fixed rows.
__global__ void k_bc_accumulate(int64_t n, Col4 inv, const float4 *__restrict__ x, double *__restrict__ X) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 xi = x[i];
  double2 *Xr = reinterpret_cast<double2 *>(X + 4 * i);
  double2 a = Xr[0], b = Xr[1];
  a.x = fma(inv.v[0], (double)xi.x, a.x);
  a.y = fma(inv.v[1], (double)xi.y, a.y);
  b.x = fma(inv.v[2], (double)xi.z, b.x);
  b.y = fma(inv.v[3], (double)xi.w, b.y);
  Xr[0] = a;
  Xr[1] = b;
}

// U[c n + i] = sum_k C[c][k] X[i][k] (column-major nv x nfield, a Julia Matrix).
__global__ void k_bc_expand(int64_t n, int nfield, const double *__restrict__ C, const double *__restrict__ X,
                            double *__restrict__ U) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * (int64_t)nfield) return;
  const int c = (int)(e / n);
  const int64_t i = e - (int64_t)c * n;
  const double2 *Xr = reinterpret_cast<const double2 *>(X + 4 * i);
  const double2 a = Xr[0], b = Xr[1];
  const double *cc = C + 4 * c;
  U[e] = fma(cc[0], a.x, fma(cc[1], a.y, fma(cc[2], b.x, cc[3] * b.y)));
}

// Singular value decomposition of the field block H0 (m x 3, row c = field c) by
// one-sided Jacobi rotations (Hestenes): the three columns are rotated pairwise until
// orthogonal, H0 V = W (columns of W orthogonal), so the singular values are the
// column norms of W and C = W.  Unlike an eigen-decomposition of H0^T H0 this keeps
// small singular values accurate to working precision relative to the largest, so a
// threshold of 1e-13 separates exact rank deficiency from rounding.
void fields_svd(const double *H0, int m, std::vector<double> &W, double V[3][3], double sig[3]) {
  W.assign(H0, H0 + 3 * (size_t)m);  // W[3 c + a]
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) V[a][b] = a == b ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 60; ++sweep) {
    bool rotated = false;
    for (int p = 0; p < 2; ++p)
      for (int q = p + 1; q < 3; ++q) {
        double app = 0.0, aqq = 0.0, apq = 0.0;
        for (int c = 0; c < m; ++c) {
          const double x = W[3 * c + p], y = W[3 * c + q];
          app += x * x;
          aqq += y * y;
          apq += x * y;
        }
        if (apq == 0.0 || std::fabs(apq) <= 1e-15 * std::sqrt(app * aqq)) continue;
        rotated = true;
        const double th = (aqq - app) / (2.0 * apq);
        const double t = (th >= 0.0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
        const double cs = 1.0 / std::sqrt(t * t + 1.0), sn = t * cs;
        for (int c = 0; c < m; ++c) {
          const double x = W[3 * c + p], y = W[3 * c + q];
          W[3 * c + p] = cs * x - sn * y;
          W[3 * c + q] = sn * x + cs * y;
        }
        for (int k = 0; k < 3; ++k) {
          const double x = V[k][p], y = V[k][q];
          V[k][p] = cs * x - sn * y;
          V[k][q] = sn * x + cs * y;
        }
      }
    if (!rotated) break;
  }
  for (int a = 0; a < 3; ++a) {
    double s2 = 0.0;
    for (int c = 0; c < m; ++c) s2 += W[3 * c + a] * W[3 * c + a];
    sig[a] = std::sqrt(s2);
  }
}

}  // namespace

// The block-CG sweep (the operator is assembled by the caller: val64/val32, dinv32).
fg_status fg_sweep_block(fg_mesh *m, int nfield, const double *H0, const fg_solve_opts &o, double *U,
                         fg_solve_stats *s) {
  const int64_t n = m->nv;
  cudaStream_t st = m->stream;
  // rank-revealing factorisation of the field block: H0 V = W, W's columns orthogonal
  std::vector<double> W;
  double V[3][3], sig[3];
  fields_svd(H0, nfield, W, V, sig);
  int order[3] = {0, 1, 2};
  std::sort(order, order + 3, [&](int a, int b) { return sig[a] > sig[b]; });
  const double smax = sig[order[0]];
  int r = 0;
  Dirs dirs{};
  std::vector<double> Cm((size_t)4 * nfield, 0.0);  // C = H0 V_r (nfield x 4, zero beyond r)
  for (int k = 0; k < 3; ++k) {
    const int e = order[k];
    if (!(smax > 0.0) || !(sig[e] > 1e-13 * smax)) continue;  // singular value below 1e-13 of the largest
    for (int a = 0; a < 3; ++a) dirs.v[r][a] = V[a][e];
    for (int c = 0; c < nfield; ++c) Cm[4 * c + r] = W[3 * c + e];
    ++r;
  }

  // work space from the device's stream-ordered pool, released on the stream at exit
  StreamScratch scratch{st, {}};
  auto alloc = [&](size_t bytes) { return static_cast<void *>(scratch.get<unsigned char>(std::max<size_t>(bytes, 16))); };
  const unsigned nb = grid_for(n, BC_T);
  double *X = (double *)alloc(sizeof(double) * 4 * n), *R = (double *)alloc(sizeof(double) * 4 * n);
  float4 *r32 = (float4 *)alloc(sizeof(float4) * n), *z32 = (float4 *)alloc(sizeof(float4) * n);
  float4 *p0 = (float4 *)alloc(sizeof(float4) * n), *p1 = (float4 *)alloc(sizeof(float4) * n);
  float4 *q32 = (float4 *)alloc(sizeof(float4) * n), *x32 = (float4 *)alloc(sizeof(float4) * n);
  double *gpart = (double *)alloc(sizeof(double) * BC_SYM * nb);
  double *gram = (double *)alloc(sizeof(double) * 16);
  float2 *fpart = (float2 *)alloc(sizeof(float2) * (BC_SYM + 4) * ((size_t)nb + FG_ARRIVE_GROUPS));
  unsigned *counter = (unsigned *)alloc(sizeof(unsigned) * 128);  // above FG_LAST1_COUNTER
  double *scal = (double *)alloc(sizeof(double) * B_NSCAL);
  int *ctl = (int *)alloc(sizeof(int) * C_NCTL);
  double *dC = (double *)alloc(sizeof(double) * Cm.size());
  FG_CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(unsigned) * 128, st));
  FG_CUDA_TRY(cudaMemcpyAsync(dC, Cm.data(), sizeof(double) * Cm.size(), cudaMemcpyHostToDevice, st));
  const BcOp A{n, m->sl_ptr, m->sl_len, m->sl_col, m->has_fixed ? m->fixed : nullptr};

  cudaEvent_t e0, e1;
  FG_CUDA_TRY(cudaEventCreate(&e0));
  FG_CUDA_TRY(cudaEventCreate(&e1));
  struct Ev {
    cudaEvent_t a, b;
    ~Ev() {
      cudaEventDestroy(a);
      cudaEventDestroy(b);
    }
  } evs{e0, e1};
  FG_CUDA_TRY(cudaEventRecord(e0, st));
  k_bc_lift<<<nb, BC_T, 0, st>>>(n, m->p, dirs, X);
  FG_LAUNCHED(1);

  // per-field residual norms^2 from a direction Gram matrix
  auto field_rr = [&](const double *Gm, int c) {
    double v = 0.0;
    for (int a = 0; a < 4; ++a)
      for (int b = 0; b < 4; ++b) v += Cm[4 * c + a] * Gm[4 * a + b] * Cm[4 * c + b];
    return std::max(v, 0.0);
  };
  double G[16], G0[16];
  std::vector<double> hist;
  int total = 0, refinements = 0;
  bool all_done = false;
  double worst = 0.0;
  // an even number of iterations per host check: the two direction buffers return
  // to their roles, so one captured graph of `check` iterations serves every check
  const int check = (std::max(4, o.check_every) + 1) & ~1;
  cudaGraphExec_t body = nullptr;
  struct BodyGraph {
    cudaGraphExec_t &g;
    ~BodyGraph() {
      if (g) cudaGraphExecDestroy(g);
    }
  } body_guard{body};
  auto enqueue_body = [&]() {
    float4 *po = p0, *pn = p1;
    for (int k = 0; k < check; ++k) {
      k_bc_spmm32<<<nb, BC_T, 0, st>>>(A, m->val32, z32, po, pn, q32, scal, ctl, fpart, counter);
      k_bc_update32<<<nb, BC_T, 0, st>>>(n, m->dinv32, pn, q32, r32, z32, x32, scal, ctl, fpart, counter);
      std::swap(po, pn);
    }
  };
  for (int ref = 0; ref < 50; ++ref) {
    k_bc_resid64<<<nb, BC_T, 0, st>>>(A, m->val64, X, R, gpart);
    k_bc_gram<<<1, 32 * BC_SYM, 0, st>>>(gpart, (int)nb, gram);
    FG_LAUNCHED(2);
    FG_CUDA_TRY(cudaMemcpyAsync(m->hbuf, gram, sizeof(double) * 16, cudaMemcpyDeviceToHost, st));
    FG_CUDA_TRY(cudaStreamSynchronize(st));
    std::copy(m->hbuf, m->hbuf + 16, G);
    if (ref == 0) std::copy(G, G + 16, G0);
    all_done = true;
    worst = 0.0;
    bool finite = true;
    for (int k = 0; k < 16; ++k) finite &= std::isfinite(G[k]);
    if (!finite) throw FgError{FG_NAN, "fg_magnetostatics_sweep: non-finite residual"};
    for (int c = 0; c < nfield; ++c) {
      const double r0 = field_rr(G0, c), rc = field_rr(G, c);
      if (r0 > 0.0 && rc > o.rtol * o.rtol * r0) {
        all_done = false;
        worst = std::max(worst, std::sqrt(rc / r0));
      }
    }
    if (all_done || total >= o.maxiter) break;
    // stagnation (a residual at the rounding level of the FP64 operator cannot be
    // reduced further): stop when three refinements did not halve the worst field
    hist.push_back(worst);
    if (hist.size() >= 4 && worst > 0.5 * hist[hist.size() - 4]) break;
    double sc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int k = 0; k < r; ++k)
      if (G[5 * k] > 0.0) sc[k] = 1.0 / std::sqrt(G[5 * k]);
    const double inner = std::max(o.inner_rtol, o.rtol / std::max(worst, 1e-300));
    k_bc_init32<<<nb, BC_T, 0, st>>>(n, R, Col4{{sc[0], sc[1], sc[2], sc[3]}}, inner * inner,
                                     o.maxiter - total, m->dinv32, r32, z32, p0, x32, scal, ctl, fpart, counter);
    FG_LAUNCHED(1);
    int it = 0;
    if (!body) {
      // the iterations of one host check as one graph launch
      cudaGraph_t graph = nullptr;
      FG_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      enqueue_body();
      const cudaError_t ce = cudaStreamEndCapture(st, &graph);
      const cudaError_t ie = (ce == cudaSuccess) ? cudaGraphInstantiate(&body, graph, 0) : ce;
      if (graph) cudaGraphDestroy(graph);
      if (ie != cudaSuccess) {
        body = nullptr;
        cudaGetLastError();
      }
    }
    for (;;) {
      if (body) FG_CUDA_TRY(cudaGraphLaunch(body, st));
      else enqueue_body();
      FG_LAUNCHED(2LL * check);
      FG_CUDA_TRY(cudaGetLastError());
      FG_CUDA_TRY(cudaMemcpyAsync(m->hint, ctl, sizeof(int) * 4, cudaMemcpyDeviceToHost, st));
      FG_CUDA_TRY(cudaStreamSynchronize(st));
      it = m->hint[C_ITERS];
      if (m->hint[C_DONE]) break;
    }
    if (m->hint[C_STATUS] == BS_NAN) throw FgError{FG_NAN, "fg_magnetostatics_sweep: block CG breakdown"};
    total += it;
    ++refinements;
    Col4 inv;
    for (int k = 0; k < 4; ++k) inv.v[k] = sc[k] > 0.0 ? 1.0 / sc[k] : 0.0;
    k_bc_accumulate<<<nb, BC_T, 0, st>>>(n, inv, x32, X);
    FG_LAUNCHED(1);
  }
  double *dU = nullptr;
  if (U) {
    dU = (double *)alloc(sizeof(double) * (size_t)n * nfield);
    k_bc_expand<<<grid_for(n * (int64_t)nfield, 256), 256, 0, st>>>(n, nfield, dC, X, dU);
    FG_LAUNCHED(1);
  }
  FG_CUDA_TRY(cudaEventRecord(e1, st));
  if (U) FG_CUDA_TRY(cudaMemcpyAsync(U, dU, sizeof(double) * (size_t)n * nfield, cudaMemcpyDeviceToHost, st));
  FG_CUDA_TRY(cudaStreamSynchronize(st));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  if (s) {
    s->iterations = total;
    s->refinements = refinements;
    s->converged = all_done ? 1 : 0;
    s->pad_ = r;
    s->relres = worst;
    s->ms = ms;
  }
  return all_done ? FG_OK : FG_NOT_CONVERGED;
}
