/*
 * femeko_oracle.c -- CPU FP64 restatement of Femeko's FEM hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle and the timed CPU
 * baseline.  Only the test suite, the smoke check and the benchmark's CPU-baseline
 * leg load it; the GPU library never links or calls it.
 *
 * Parity status: UNPINNED against reference outputs.  The reference is Julia
 * (no `julia` here) and its C++ side needs Eigen (the extern/eigen submodule is
 * empty), so no reference run could produce golden vectors, and the reference
 * ships no tests or fixtures.  The oracle is pinned instead to analytic
 * known answers (single-element matrices, row-sum zero, mass total = volume,
 * linear patch test, symmetry, Froehlich derivative by finite differences,
 * adjoint by finite differences); see tests/golden/.
 *
 * Conventions: indices are 0-based; p is 3 x nv column-major (p[3*i + c]);
 * t is npe x nt column-major (t[npe*k + a]); sparse matrices are CSC with
 * int64 column pointers and int32 row indices (the symmetric ones double as CSR).
 *
 * Every function cites the reference lines it restates (paths relative to the
 * reference repository root).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_MU0 (3.14159265358979323846 * 4e-7)

int or_version(void) { return 3; }

void or_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

int or_get_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------------- */
/* Dense LU with partial pivoting (what Julia's `\` runs on a square Matrix). */
/* A is row-major n x n and is overwritten; b is overwritten with x.           */
static int lu_solve(int n, double *A, double *b) {
  for (int c = 0; c < n; ++c) {
    int piv = c;
    double best = fabs(A[c * n + c]);
    for (int r = c + 1; r < n; ++r) {
      double v = fabs(A[r * n + c]);
      if (v > best) { best = v; piv = r; }
    }
    if (best == 0.0) return -1;
    if (piv != c) {
      for (int k = 0; k < n; ++k) { double tmp = A[c * n + k]; A[c * n + k] = A[piv * n + k]; A[piv * n + k] = tmp; }
      double tb = b[c]; b[c] = b[piv]; b[piv] = tb;
    }
    double inv = 1.0 / A[c * n + c];
    for (int r = c + 1; r < n; ++r) {
      double l = A[r * n + c] * inv;
      A[r * n + c] = l;
      for (int k = c + 1; k < n; ++k) A[r * n + k] -= l * A[c * n + k];
    }
  }
  for (int r = 0; r < n; ++r) {            /* forward: unit lower */
    double s = b[r];
    for (int k = 0; k < r; ++k) s -= A[r * n + k] * b[k];
    b[r] = s;
  }
  for (int r = n - 1; r >= 0; --r) {       /* back: upper */
    double s = b[r];
    for (int k = r + 1; k < n; ++k) s -= A[r * n + k] * b[k];
    b[r] = s / A[r * n + r];
  }
  return 0;
}

/* ------------------------------------------------------------------------- */
/* src/mesh.jl:484-505 elementVolume: |AB . (AC x AD)| / 6                     */
double or_element_volume(const double *p, const int *nds) {
  const double *A = p + 3 * nds[0], *B = p + 3 * nds[1], *C = p + 3 * nds[2], *D = p + 3 * nds[3];
  double ab[3], ac[3], ad[3];
  for (int c = 0; c < 3; ++c) { ab[c] = B[c] - A[c]; ac[c] = C[c] - A[c]; ad[c] = D[c] - A[c]; }
  double cx = ac[1] * ad[2] - ac[2] * ad[1];
  double cy = ac[2] * ad[0] - ac[0] * ad[2];
  double cz = ac[0] * ad[1] - ac[1] * ad[0];
  return fabs(ab[0] * cx + ab[1] * cy + ab[2] * cz) / 6.0;
}

void or_element_volumes(const double *p, const int *t, long nt, double *VE) {
#pragma omp parallel for schedule(static)
  for (long k = 0; k < nt; ++k) VE[k] = or_element_volume(p, t + 4 * k);
}

/* src/mesh.jl:474-481 areaTriangle (3D triangle from the three 2x2 minors). */
double or_area_triangle(const double *p, const int *nds) {
  double x[3], y[3], z[3];
  for (int a = 0; a < 3; ++a) { x[a] = p[3 * nds[a]]; y[a] = p[3 * nds[a] + 1]; z[a] = p[3 * nds[a] + 2]; }
  /* det([u'; v'; 1 1 1]) for the pairs (x,y), (y,z), (z,x) */
#define DET3(u, v) (u[0] * (v[1] - v[2]) - u[1] * (v[0] - v[2]) + u[2] * (v[0] - v[1]))
  double d1 = DET3(x, y), d2 = DET3(y, z), d3 = DET3(z, x);
#undef DET3
  return 0.5 * sqrt(d1 * d1 + d2 * d2 + d3 * d3);
}

/* src/FEM3D.jl:5-17 abcd: coefficients (a,b,c,d) of the P1 basis of node `nd`  */
/* from the 4x4 system [1 x y z] (node nd first, then the others in order).     */
int or_abcd(const double *p, const int *nds, int nd, double *out) {
  int order[4], m = 1;
  order[0] = nd;
  for (int a = 0; a < 4; ++a) if (nds[a] != nd && m < 4) order[m++] = nds[a];
  if (m != 4) return -1;
  double A[16], b[4] = {1.0, 0.0, 0.0, 0.0};
  for (int r = 0; r < 4; ++r) {
    A[4 * r] = 1.0;
    A[4 * r + 1] = p[3 * order[r]];
    A[4 * r + 2] = p[3 * order[r] + 1];
    A[4 * r + 3] = p[3 * order[r] + 2];
  }
  int s = lu_solve(4, A, b);
  for (int c = 0; c < 4; ++c) out[c] = b[c];
  return s;
}

/* src/FEM2D.jl:5-25 abc: P1 triangle basis f = a + b x + c y of node `nd`. */
int or_abc(const double *p, const int *nds, int nd, double *out) {
  int nd1 = -1, nd2 = -1;
  for (int a = 0; a < 3; ++a) {
    if (nds[a] != nd) { if (nd1 < 0) nd1 = nds[a]; else nd2 = nds[a]; }
  }
  if (nd1 < 0 || nd2 < 0) return -1;
  double A[9] = {1.0, p[3 * nd], p[3 * nd + 1], 1.0, p[3 * nd1], p[3 * nd1 + 1], 1.0, p[3 * nd2], p[3 * nd2 + 1]};
  double b[3] = {1.0, 0.0, 0.0};
  int s = lu_solve(3, A, b);
  for (int c = 0; c < 3; ++c) out[c] = b[c];
  return s;
}

/* Gradients of the 4 P1 basis functions of element k through abcd. */
static void p1_grads(const double *p, const int *nds, double g[4][3]) {
  for (int a = 0; a < 4; ++a) {
    double r[4];
    or_abcd(p, nds, nds[a], r);
    g[a][0] = r[1]; g[a][1] = r[2]; g[a][2] = r[3];
  }
}

/* ------------------------------------------------------------------------- */
/* src/FEM3D.jl:59-76 localStiffnessMatrix: Ak[:,k] = VE_k f_k (bb'+cc'+dd').  */
/* Stored per element as 16 values in pass order n = 4*i + j (i row, j col).    */
void or_local_stiffness(const double *p, const int *t, long nt, const double *VE, const double *f, double *Ak) {
#pragma omp parallel for schedule(static)
  for (long k = 0; k < nt; ++k) {
    double g[4][3];
    p1_grads(p, t + 4 * k, g);
    double s = VE[k] * (f ? f[k] : 1.0);
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j)
        Ak[16 * k + 4 * i + j] = s * (g[i][0] * g[j][0] + g[i][1] * g[j][1] + g[i][2] * g[j][2]);
  }
}

/* ------------------------------------------------------------------------- */
/* COO -> CSC with duplicate summation, as SparseArrays.sparse(I,J,V,m,n) does: */
/* rows sorted within each column, duplicates summed in order of appearance.    */
/* Entries are visited in the order (pass n, element k) of src/FEM3D.jl:47-53   */
/* and Magnetostatics/NewtonRaphson.jl:115-127.  drop_zeros=1 removes entries    */
/* whose final value is exactly 0.0 (what the chained sparse `+` of             */
/* src/FEM3D.jl:51 leaves out); drop_zeros=0 keeps the structural pattern of the */
/* single `sparse` call of Magnetostatics/NewtonRaphson.jl:161.                  */
/* The entry list is given implicitly: entry e = n*nt + k has row t[ni*k + I_n], */
/* column t[ni*k + J_n] and value V[nn*k + n] (nn = ni*ni local values).         */
long or_assemble_csc(int nv, long nt, int ni, const int *t, const double *V, int drop_zeros,
                     long *colptr, int *rowval, double *nzval) {
  long nn = (long)ni * ni;
  long m = nn * nt;
  /* pass 1: bucket entries by row, stable */
  long *rptr = (long *)calloc((size_t)nv + 1, sizeof(long));
  for (long n = 0; n < nn; ++n)
    for (long k = 0; k < nt; ++k) rptr[t[ni * k + n / ni] + 1]++;
  for (int i = 0; i < nv; ++i) rptr[i + 1] += rptr[i];
  long *cur = (long *)malloc(sizeof(long) * ((size_t)nv + 1));
  memcpy(cur, rptr, sizeof(long) * ((size_t)nv + 1));
  int64_t *bucket = (int64_t *)malloc(sizeof(int64_t) * (size_t)m);
  for (long n = 0; n < nn; ++n)
    for (long k = 0; k < nt; ++k) bucket[cur[t[ni * k + n / ni]]++] = n * nt + k;
  /* pass 2: walk rows in order and append to columns -> columns sorted by row */
  long *cptr = (long *)calloc((size_t)nv + 1, sizeof(long));
  for (long n = 0; n < nn; ++n)
    for (long k = 0; k < nt; ++k) cptr[t[ni * k + n % ni] + 1]++;
  for (int i = 0; i < nv; ++i) cptr[i + 1] += cptr[i];
  memcpy(cur, cptr, sizeof(long) * ((size_t)nv + 1));
  int *crow = (int *)malloc(sizeof(int) * (size_t)m);
  double *cval = (double *)malloc(sizeof(double) * (size_t)m);
  for (int r = 0; r < nv; ++r) {
    for (long q = rptr[r]; q < rptr[r + 1]; ++q) {
      long e = bucket[q];
      long n = e / nt, k = e % nt;
      int col = t[ni * k + n % ni];
      long pos = cur[col]++;
      crow[pos] = r;
      cval[pos] = V[nn * k + n];
    }
  }
  /* pass 3: combine duplicates per column */
  long nnz = 0;
  colptr[0] = 0;
  for (int c = 0; c < nv; ++c) {
    long q = cptr[c];
    while (q < cptr[c + 1]) {
      int r = crow[q];
      double s = cval[q];
      ++q;
      while (q < cptr[c + 1] && crow[q] == r) { s += cval[q]; ++q; }
      if (!(drop_zeros && s == 0.0)) { rowval[nnz] = r; nzval[nnz] = s; ++nnz; }
    }
    colptr[c + 1] = nnz;
  }
  free(rptr); free(cur); free(bucket); free(cptr); free(crow); free(cval);
  return nnz;
}

/* src/FEM3D.jl:40-56 stiffnessMatrix(mesh, f).  Output buffers hold 16*nt. */
long or_stiffness(const double *p, const int *t, int nv, long nt, const double *VE, const double *f, int drop_zeros,
                  long *colptr, int *rowval, double *nzval) {
  double *Ak = (double *)malloc(sizeof(double) * 16 * (size_t)nt);
  or_local_stiffness(p, t, nt, VE, f, Ak);
  long nnz = or_assemble_csc(nv, nt, 4, t, Ak, drop_zeros, colptr, rowval, nzval);
  free(Ak);
  return nnz;
}

/* src/FEM3D.jl:466-492 massMatrix: VE/20 * [2 on the diagonal, 1 off it]. */
long or_mass(const int *t, int nv, long nt, const double *VE, int drop_zeros, long *colptr, int *rowval, double *nzval) {
  double *Mk = (double *)malloc(sizeof(double) * 16 * (size_t)nt);
  for (long k = 0; k < nt; ++k)
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) Mk[16 * k + 4 * i + j] = VE[k] * (i == j ? 2.0 : 1.0) / 20.0;
  long nnz = or_assemble_csc(nv, nt, 4, t, Mk, drop_zeros, colptr, rowval, nzval);
  free(Mk);
  return nnz;
}

/* src/FEM3D.jl:79-119 tangentialStiffnessMatrix:                              */
/* At_ij = VE dmu/|H| (H.grad phi_i)(H.grad phi_j).  Where |H| = 0 the reference */
/* divides by zero; the term's limit is 0 and that is what is stored here.      */
static void tangent_local(const double *p, const int *nds, double VE, const double *Hv, double dmu, double *out16) {
  double g[4][3];
  p1_grads(p, nds, g);
  double H = sqrt(Hv[0] * Hv[0] + Hv[1] * Hv[1] + Hv[2] * Hv[2]);
  double a[4];
  for (int i = 0; i < 4; ++i) a[i] = Hv[0] * g[i][0] + Hv[1] * g[i][1] + Hv[2] * g[i][2];
  double s = (H > 0.0) ? VE * dmu / H : 0.0;
  for (int i = 0; i < 4; ++i)     /* upper triangle, mirrored (src/FEM3D.jl:96-104) */
    for (int j = i; j < 4; ++j) { out16[4 * i + j] = s * a[i] * a[j]; out16[4 * j + i] = out16[4 * i + j]; }
}

long or_tangent(const double *p, const int *t, int nv, long nt, const double *VE, const double *Hvec, const double *dmu,
                int drop_zeros, long *colptr, int *rowval, double *nzval) {
  double *Ak = (double *)malloc(sizeof(double) * 16 * (size_t)nt);
#pragma omp parallel for schedule(static)
  for (long k = 0; k < nt; ++k) tangent_local(p, t + 4 * k, VE[k], Hvec + 3 * k, dmu[k], Ak + 16 * k);
  long nnz = or_assemble_csc(nv, nt, 4, t, Ak, drop_zeros, colptr, rowval, nzval);
  free(Ak);
  return nnz;
}

/* src/FEM2D.jl:48-76 stiffnessMatrix2D: VE mu (bb' + cc'). */
long or_stiffness2d(const double *p, const int *t, int nv, long nt, const double *VE, const double *f, int drop_zeros,
                    long *colptr, int *rowval, double *nzval) {
  double *Ak = (double *)malloc(sizeof(double) * 9 * (size_t)nt);
#pragma omp parallel for schedule(static)
  for (long k = 0; k < nt; ++k) {
    double g[3][3];
    for (int a = 0; a < 3; ++a) or_abc(p, t + 3 * k, t[3 * k + a], g[a]);
    double s = VE[k] * (f ? f[k] : 1.0);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) Ak[9 * k + 3 * i + j] = s * (g[i][1] * g[j][1] + g[i][2] * g[j][2]);
  }
  long nnz = or_assemble_csc(nv, nt, 3, t, Ak, drop_zeros, colptr, rowval, nzval);
  free(Ak);
  return nnz;
}

/* src/FEM2D.jl:139-161 massMatrix2D: VE/12 * [2 1 1; 1 2 1; 1 1 2]. */
long or_mass2d(const int *t, int nv, long nt, const double *VE, int drop_zeros, long *colptr, int *rowval, double *nzval) {
  double *Mk = (double *)malloc(sizeof(double) * 9 * (size_t)nt);
  for (long k = 0; k < nt; ++k)
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) Mk[9 * k + 3 * i + j] = VE[k] * (i == j ? 2.0 : 1.0) / 12.0;
  long nnz = or_assemble_csc(nv, nt, 3, t, Mk, drop_zeros, colptr, rowval, nzval);
  free(Mk);
  return nnz;
}

/* ------------------------------------------------------------------------- */
/* Second order.  src/FEM3D.jl:21-37 quadraticBasis: 10x10 Vandermonde in       */
/* global coordinates, node nd first.  shift=1 solves the same system in        */
/* coordinates relative to the element's first vertex (better conditioned; the  */
/* basis functions are the same, their monomial coefficients refer to x - x0).  */
static int p2_basis3d(const double *p, const int *nds, int a, const double *x0, double *S) {
  int order[10], m = 1;
  order[0] = nds[a];
  for (int b = 0; b < 10; ++b) if (nds[b] != nds[a] && m < 10) order[m++] = nds[b];
  double A[100];
  for (int r = 0; r < 10; ++r) {
    double x = p[3 * order[r]] - x0[0], y = p[3 * order[r] + 1] - x0[1], z = p[3 * order[r] + 2] - x0[2];
    double row[10] = {1.0, x, y, z, x * x, x * y, x * z, y * y, y * z, z * z};
    memcpy(A + 10 * r, row, sizeof(row));
  }
  for (int c = 0; c < 10; ++c) S[c] = (c == 0) ? 1.0 : 0.0;
  return lu_solve(10, A, S);
}

/* src/FEM3D.jl:324-376 quadraticLocalStiffnessMatrix: equal weights over the   */
/* 10 element nodes, /10, times mu VE.  Ak holds 100 values per element.        */
void or_p2_local_stiffness(const double *p, const int *t, long nt, const double *VE, const double *mu, int shift, double *Ak) {
#pragma omp parallel for schedule(static)
  for (long k = 0; k < nt; ++k) {
    const int *nds = t + 10 * k;
    double x0[3] = {0, 0, 0};
    if (shift) { x0[0] = p[3 * nds[0]]; x0[1] = p[3 * nds[0] + 1]; x0[2] = p[3 * nds[0] + 2]; }
    double S[10][10];
    for (int a = 0; a < 10; ++a) p2_basis3d(p, nds, a, x0, S[a]);
    double d[10][10][3]; /* d[a][node n][xyz] */
    for (int a = 0; a < 10; ++a)
      for (int n = 0; n < 10; ++n) {
        double x = p[3 * nds[n]] - x0[0], y = p[3 * nds[n] + 1] - x0[1], z = p[3 * nds[n] + 2] - x0[2];
        const double *s = S[a];
        d[a][n][0] = s[1] + 2 * s[4] * x + s[5] * y + s[6] * z;
        d[a][n][1] = s[2] + 2 * s[7] * y + s[5] * x + s[8] * z;
        d[a][n][2] = s[3] + 2 * s[9] * z + s[6] * x + s[8] * y;
      }
    double sc = (mu ? mu[k] : 1.0) * VE[k];
    for (int i = 0; i < 10; ++i)
      for (int j = i; j < 10; ++j) {
        double acc = 0.0;
        for (int n = 0; n < 10; ++n) acc += d[i][n][0] * d[j][n][0] + d[i][n][1] * d[j][n][1] + d[i][n][2] * d[j][n][2];
        acc /= 10.0;
        Ak[100 * k + 10 * i + j] = acc * sc;
        Ak[100 * k + 10 * j + i] = acc * sc;
      }
  }
}

long or_p2_stiffness(const double *p, const int *t, int nv, long nt, const double *VE, const double *mu, int shift,
                     long *colptr, int *rowval, double *nzval) {
  double *Ak = (double *)malloc(sizeof(double) * 100 * (size_t)nt);
  or_p2_local_stiffness(p, t, nt, VE, mu, shift, Ak);
  long nnz = or_assemble_csc(nv, nt, 10, t, Ak, 0, colptr, rowval, nzval);
  free(Ak);
  return nnz;
}

/* src/FEM3D.jl:653-755 GaussQuadrature3D(4): the published 15-point degree-5 */
/* rule on the reference tetrahedron (weights sum to 1/6).  Table kept alike. */
static const double GQ3_PTS[15][3] = {
    {0.2500000000000000, 0.2500000000000000, 0.2500000000000000},
    {0.0000000000000000, 0.3333333333333333, 0.3333333333333333},
    {0.3333333333333333, 0.3333333333333333, 0.3333333333333333},
    {0.3333333333333333, 0.3333333333333333, 0.0000000000000000},
    {0.3333333333333333, 0.0000000000000000, 0.3333333333333333},
    {0.7272727272727273, 0.0909090909090909, 0.0909090909090909},
    {0.0909090909090909, 0.0909090909090909, 0.0909090909090909},
    {0.0909090909090909, 0.0909090909090909, 0.7272727272727273},
    {0.0909090909090909, 0.7272727272727273, 0.0909090909090909},
    {0.4334498464263357, 0.0665501535736643, 0.0665501535736643},
    {0.0665501535736643, 0.4334498464263357, 0.0665501535736643},
    {0.0665501535736643, 0.0665501535736643, 0.4334498464263357},
    {0.0665501535736643, 0.4334498464263357, 0.4334498464263357},
    {0.4334498464263357, 0.0665501535736643, 0.4334498464263357},
    {0.4334498464263357, 0.4334498464263357, 0.0665501535736643}};
static const double GQ3_W[15] = {0.1817020685825351, 0.0361607142857143, 0.0361607142857143, 0.0361607142857143,
                                 0.0361607142857143, 0.0698714945161738, 0.0698714945161738, 0.0698714945161738,
                                 0.0698714945161738, 0.0656948493683187, 0.0656948493683187, 0.0656948493683187,
                                 0.0656948493683187, 0.0656948493683187, 0.0656948493683187};

/* src/FEM3D.jl:494-561 quadraticMassMatrix.  The reference's phi expression      */
/* (:529-531) ends its first line with `*z`, so Julia evaluates only the linear   */
/* part S1 + S2 x + S3 y + S4 z of each basis polynomial (global coordinates).    */
/* full_phi=0 reproduces that; full_phi=1 evaluates the whole quadratic.          */
/* The weights are multiplied by VE as in the reference (w = weights[q]*VE).      */
long or_p2_mass(const double *p, const int *t, int nv, long nt, const double *VE, const double *F, int full_phi,
                long *colptr, int *rowval, double *nzval) {
  double *Mk = (double *)malloc(sizeof(double) * 100 * (size_t)nt);
#pragma omp parallel for schedule(static)
  for (long k = 0; k < nt; ++k) {
    const int *nds = t + 10 * k;
    double zero[3] = {0, 0, 0};
    double S[10][10];
    for (int a = 0; a < 10; ++a) p2_basis3d(p, nds, a, zero, S[a]);
    const double *v1 = p + 3 * nds[0], *v2 = p + 3 * nds[1], *v3 = p + 3 * nds[2], *v4 = p + 3 * nds[3];
    double J[3][3];
    for (int r = 0; r < 3; ++r) { J[r][0] = v2[r] - v1[r]; J[r][1] = v3[r] - v1[r]; J[r][2] = v4[r] - v1[r]; }
    double M[100];
    memset(M, 0, sizeof(M));
    double f = F ? F[k] : 1.0;
    for (int q = 0; q < 15; ++q) {
      double xi = GQ3_PTS[q][0], eta = GQ3_PTS[q][1], ze = GQ3_PTS[q][2];
      double x = v1[0] + J[0][0] * xi + J[0][1] * eta + J[0][2] * ze;
      double y = v1[1] + J[1][0] * xi + J[1][1] * eta + J[1][2] * ze;
      double z = v1[2] + J[2][0] * xi + J[2][1] * eta + J[2][2] * ze;
      double phi[10];
      for (int i = 0; i < 10; ++i) {
        const double *s = S[i];
        phi[i] = s[0] + s[1] * x + s[2] * y + s[3] * z;
        if (full_phi) phi[i] += s[4] * x * x + s[5] * x * y + s[6] * x * z + s[7] * y * y + s[8] * y * z + s[9] * z * z;
      }
      double w = GQ3_W[q] / 6.0 * VE[k];
      for (int i = 0; i < 10; ++i)
        for (int j = i; j < 10; ++j) {
          M[10 * i + j] += w * phi[i] * phi[j] * f;
          M[10 * j + i] = M[10 * i + j];
        }
    }
    memcpy(Mk + 100 * k, M, sizeof(M));
  }
  long nnz = or_assemble_csc(nv, nt, 10, t, Mk, 0, colptr, rowval, nzval);
  free(Mk);
  return nnz;
}

/* src/FEM3D.jl:563-648 quadraticConvectionMatrix.  u is the nodal velocity     */
/* (3 x nv, column k at u + 3k); u_avg is the mean over the 4 vertices           */
/* (src/FEM.jl:13-30: ((u1 + u2) + u3) + u4, then /4).  phi as in the mass       */
/* matrix (linear part only unless full_phi, :610-613), gradPhi the full         */
/* quadratic's (:616-618), w = weights[q] VE, Ck[i][j] += w (u_avg . gradPhi_j)   */
/* phi_i F.  The reference flattens Ck column-major (:640) and scatters entry    */
/* n = 10(i-1)+j to (t_i, t_j) (:644-648), so C[t_i, t_j] sums Ck[j][i]: the      */
/* local values below are stored transposed to build that same C.               */
long or_p2_convection(const double *p, const int *t, int nv, long nt, const double *VE, const double *u,
                      const double *F, int full_phi, long *colptr, int *rowval, double *nzval) {
  double *Ck = (double *)malloc(sizeof(double) * 100 * (size_t)nt);
#pragma omp parallel for schedule(static)
  for (long k = 0; k < nt; ++k) {
    const int *nds = t + 10 * k;
    double zero[3] = {0, 0, 0};
    double S[10][10];
    for (int a = 0; a < 10; ++a) p2_basis3d(p, nds, a, zero, S[a]);
    const double *v1 = p + 3 * nds[0], *v2 = p + 3 * nds[1], *v3 = p + 3 * nds[2], *v4 = p + 3 * nds[3];
    double J[3][3];
    for (int r = 0; r < 3; ++r) { J[r][0] = v2[r] - v1[r]; J[r][1] = v3[r] - v1[r]; J[r][2] = v4[r] - v1[r]; }
    double ua[3];
    for (int c = 0; c < 3; ++c)
      ua[c] = (((u[3 * nds[0] + c] + u[3 * nds[1] + c]) + u[3 * nds[2] + c]) + u[3 * nds[3] + c]) / 4.0;
    double C[10][10];
    memset(C, 0, sizeof(C));
    double f = F ? F[k] : 1.0;
    for (int q = 0; q < 15; ++q) {
      double xi = GQ3_PTS[q][0], eta = GQ3_PTS[q][1], ze = GQ3_PTS[q][2];
      double x = v1[0] + J[0][0] * xi + J[0][1] * eta + J[0][2] * ze;
      double y = v1[1] + J[1][0] * xi + J[1][1] * eta + J[1][2] * ze;
      double z = v1[2] + J[2][0] * xi + J[2][1] * eta + J[2][2] * ze;
      double phi[10], gu[10];
      for (int i = 0; i < 10; ++i) {
        const double *s = S[i];
        phi[i] = s[0] + s[1] * x + s[2] * y + s[3] * z;
        if (full_phi) phi[i] += s[4] * x * x + s[5] * x * y + s[6] * x * z + s[7] * y * y + s[8] * y * z + s[9] * z * z;
        double gx = s[1] + 2 * s[4] * x + s[5] * y + s[6] * z;
        double gy = s[2] + 2 * s[7] * y + s[5] * x + s[8] * z;
        double gz = s[3] + 2 * s[9] * z + s[6] * x + s[8] * y;
        gu[i] = ua[0] * gx + ua[1] * gy + ua[2] * gz;
      }
      double w = GQ3_W[q] / 6.0 * VE[k];
      for (int j = 0; j < 10; ++j)
        for (int i = 0; i < 10; ++i) C[i][j] += w * gu[j] * phi[i] * f;
    }
    for (int i = 0; i < 10; ++i)
      for (int j = 0; j < 10; ++j) Ck[100 * k + 10 * i + j] = C[j][i];
  }
  long nnz = or_assemble_csc(nv, nt, 10, t, Ck, 0, colptr, rowval, nzval);
  free(Ck);
  return nnz;
}

/* Nedelec (Whitney) edge elements, src/FEM3D.jl:155-271 and                     */
/* Magnetostatics/nedelec3D.jl:106-221.  abcd (src/FEM3D.jl:5-17) solves           */
/* [1 x y z] r = e1 over the node and the other three (in element order); local    */
/* edge e joins local nodes (1,2), (2,3), (3,1), (4,1), (3,4), (2,4)                */
/* (src/mesh.jl:603-630); curlN_e = 2 |x_j - x_i| (grad_i x grad_j).              */
/* t: 4 (or more) node rows per element, element-major with stride ni.            */
static const int NED_I[6] = {0, 1, 2, 3, 2, 1}, NED_J[6] = {1, 2, 0, 0, 3, 3};

static void ned_curls(const double *p, const int *nds, double cN[6][3]) {
  double g[4][3];
  for (int a = 0; a < 4; ++a) {
    int order[4], m = 1;
    order[0] = nds[a];
    for (int b = 0; b < 4; ++b) if (b != a) order[m++] = nds[b];
    double A[16], r[4] = {1.0, 0.0, 0.0, 0.0};
    for (int q = 0; q < 4; ++q) {
      A[4 * q] = 1.0;
      A[4 * q + 1] = p[3 * order[q]];
      A[4 * q + 2] = p[3 * order[q] + 1];
      A[4 * q + 3] = p[3 * order[q] + 2];
    }
    lu_solve(4, A, r);
    g[a][0] = r[1]; g[a][1] = r[2]; g[a][2] = r[3];
  }
  for (int e = 0; e < 6; ++e) {
    int i = NED_I[e], j = NED_J[e];
    double dx = p[3 * nds[j]] - p[3 * nds[i]], dy = p[3 * nds[j] + 1] - p[3 * nds[i] + 1],
           dz = p[3 * nds[j] + 2] - p[3 * nds[i] + 2];
    double l = sqrt(dx * dx + dy * dy + dz * dz);
    double cx = g[i][1] * g[j][2] - g[i][2] * g[j][1];
    double cy = g[i][2] * g[j][0] - g[i][0] * g[j][2];
    double cz = g[i][0] * g[j][1] - g[i][1] * g[j][0];
    cN[e][0] = 2.0 * l * cx; cN[e][1] = 2.0 * l * cy; cN[e][2] = 2.0 * l * cz;
  }
}

/* Element blocks: mode 0 nedelecLocalStiffness VE curlN_i.curlN_j (times nu when    */
/* given); mode 1 the tangential block VE (curlN_i.B)(curlN_j.B) dnu / |B| of       */
/* src/FEM3D.jl:236-243 (0 where |B| = 0).  Ak[36k + 6i + j].                        */
void or_nedelec_local(const double *p, const int *t, int ni, long nt, const double *VE, const double *nu, int mode,
                      const double *dnu, const double *Bf, const double *Bn, double *Ak) {
#pragma omp parallel for schedule(static)
  for (long k = 0; k < nt; ++k) {
    double cN[6][3];
    ned_curls(p, t + (long)ni * k, cN);
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 6; ++j) {
        double v;
        if (mode == 0) {
          v = VE[k] * (cN[i][0] * cN[j][0] + cN[i][1] * cN[j][1] + cN[i][2] * cN[j][2]);
          if (nu) v *= nu[k];
        } else {
          const double *b = Bf + 3 * k;
          double ci = cN[i][0] * b[0] + cN[i][1] * b[1] + cN[i][2] * b[2];
          double cj = cN[j][0] * b[0] + cN[j][1] * b[1] + cN[j][2] * b[2];
          v = Bn[k] != 0.0 ? VE[k] * ci * cj * dnu[k] / Bn[k] : 0.0;
        }
        Ak[36 * k + 6 * i + j] = v;
      }
  }
}

/* nedelec3D.jl:106-139: RHS[e] += VE Bext.curlN_e, elements then local edges in    */
/* order; edges: 6 x nt element-major edge indices (0-based).                      */
void or_nedelec_load(const double *p, const int *t, int ni, long nt, const double *VE, const int *edges,
                     const double *bext, double *rhs) {
  for (long k = 0; k < nt; ++k) {
    double cN[6][3];
    ned_curls(p, t + (long)ni * k, cN);
    for (int e = 0; e < 6; ++e)
      rhs[edges[6 * k + e]] += VE[k] * (bext[0] * cN[e][0] + bext[1] * cN[e][1] + bext[2] * cN[e][2]);
  }
}

/* nedelec3D.jl:190-221: B_k = sum_e u[edge_e] curlN_e and its norm.               */
void or_nedelec_bfield(const double *p, const int *t, int ni, long nt, const int *edges, const double *u,
                       double *Bf, double *Bn) {
#pragma omp parallel for schedule(static)
  for (long k = 0; k < nt; ++k) {
    double cN[6][3], b[3] = {0.0, 0.0, 0.0};
    ned_curls(p, t + (long)ni * k, cN);
    for (int e = 0; e < 6; ++e)
      for (int c = 0; c < 3; ++c) b[c] += u[edges[6 * k + e]] * cN[e][c];
    for (int c = 0; c < 3; ++c) Bf[3 * k + c] = b[c];
    Bn[k] = sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
  }
}

/* src/FEM2D.jl:28-45 quadraticBasis2D: 6x6 Vandermonde [1 x y x^2 xy y^2]. */
static int p2_basis2d(const double *p, const int *nds, int a, const double *x0, double *S) {
  int order[6], m = 1;
  order[0] = nds[a];
  for (int b = 0; b < 6; ++b) if (nds[b] != nds[a] && m < 6) order[m++] = nds[b];
  double A[36];
  for (int r = 0; r < 6; ++r) {
    double x = p[3 * order[r]] - x0[0], y = p[3 * order[r] + 1] - x0[1];
    double row[6] = {1.0, x, y, x * x, x * y, y * y};
    memcpy(A + 6 * r, row, sizeof(row));
  }
  for (int c = 0; c < 6; ++c) S[c] = (c == 0) ? 1.0 : 0.0;
  return lu_solve(6, A, S);
}

/* src/FEM2D.jl:80-137: 6-node equal-weight rule, /6, times VE, then .* mu. */
long or_p2_stiffness2d(const double *p, const int *t, int nv, long nt, const double *VE, const double *mu, int shift,
                       long *colptr, int *rowval, double *nzval) {
  double *Ak = (double *)malloc(sizeof(double) * 36 * (size_t)nt);
#pragma omp parallel for schedule(static)
  for (long k = 0; k < nt; ++k) {
    const int *nds = t + 6 * k;
    double x0[3] = {0, 0, 0};
    if (shift) { x0[0] = p[3 * nds[0]]; x0[1] = p[3 * nds[0] + 1]; }
    double S[6][6];
    for (int a = 0; a < 6; ++a) p2_basis2d(p, nds, a, x0, S[a]);
    for (int i = 0; i < 6; ++i)
      for (int j = i; j < 6; ++j) {
        double acc = 0.0;
        for (int n = 0; n < 6; ++n) {
          double x = p[3 * nds[n]] - x0[0], y = p[3 * nds[n] + 1] - x0[1];
          double dxi = S[i][1] + 2 * S[i][3] * x + S[i][4] * y, dyi = S[i][2] + S[i][4] * x + 2 * S[i][5] * y;
          double dxj = S[j][1] + 2 * S[j][3] * x + S[j][4] * y, dyj = S[j][2] + S[j][4] * x + 2 * S[j][5] * y;
          acc += dxi * dxj + dyi * dyj;
        }
        acc /= 6.0;
        double v = acc * VE[k] * (mu ? mu[k] : 1.0);
        Ak[36 * k + 6 * i + j] = v;
        Ak[36 * k + 6 * j + i] = v;
      }
  }
  long nnz = or_assemble_csc(nv, nt, 6, t, Ak, 0, colptr, rowval, nzval);
  free(Ak);
  return nnz;
}

/* src/FEM2D.jl:453-506 GaussQuadrature2D(4) (weights sum to 1). */
static const double GQ2_W[6] = {0.223381589678011, 0.223381589678011, 0.223381589678011,
                                0.109951743655322, 0.109951743655322, 0.109951743655322};
static const double GQ2_PTS[6][2] = {{0.445948490915965, 0.445948490915965}, {0.445948490915965, 0.108103018168070},
                                     {0.108103018168070, 0.445948490915965}, {0.091576213509771, 0.091576213509771},
                                     {0.091576213509771, 0.816847572980459}, {0.816847572980459, 0.091576213509771}};

/* src/FEM2D.jl:453-506 GaussQuadrature2D(3): 4 points, weights summing to 1.       */
static const double GQ2C_W[4] = {-27.0 / 48.0, 25.0 / 48.0, 25.0 / 48.0, 25.0 / 48.0};
static const double GQ2C_PTS[4][2] = {{1.0 / 3.0, 1.0 / 3.0}, {0.2, 0.2}, {0.6, 0.2}, {0.2, 0.6}};

/* src/FEM2D.jl:231-319 quadraticConvectionMatrix2D: u (3 x nv, z unused)           */
/* interpolated with the P2 basis at each point, Ck[i][j] += w (gradPhi_i . u)       */
/* phi_j with w = weight * VE; Clocal = vec(Ck) scattered with n = 6(i-1)+j to       */
/* (t_i, t_j), so C[t_i, t_j] sums Ck[j][i].                                       */
long or_p2_convection2d(const double *p, const int *t, int nv, long nt, const double *VE, const double *u,
                        long *colptr, int *rowval, double *nzval) {
  double *Cv = (double *)malloc(sizeof(double) * 36 * (size_t)nt);
#pragma omp parallel for schedule(static)
  for (long k = 0; k < nt; ++k) {
    const int *nds = t + 6 * k;
    double zero[3] = {0, 0, 0};
    double S[6][6];
    for (int a = 0; a < 6; ++a) p2_basis2d(p, nds, a, zero, S[a]);
    const double *v1 = p + 3 * nds[0], *v2 = p + 3 * nds[1], *v3 = p + 3 * nds[2];
    double J11 = v2[0] - v1[0], J12 = v3[0] - v1[0], J21 = v2[1] - v1[1], J22 = v3[1] - v1[1];
    double Ck[6][6];
    memset(Ck, 0, sizeof(Ck));
    for (int q = 0; q < 4; ++q) {
      double xi = GQ2C_PTS[q][0], eta = GQ2C_PTS[q][1];
      double x = v1[0] + J11 * xi + J12 * eta, y = v1[1] + J21 * xi + J22 * eta;
      double phi[6], gx[6], gy[6], ux = 0.0, uy = 0.0;
      for (int i = 0; i < 6; ++i) {
        const double *s = S[i];
        phi[i] = s[0] + s[1] * x + s[2] * y + s[3] * x * x + s[4] * x * y + s[5] * y * y;
        ux += u[3 * nds[i]] * phi[i];
        uy += u[3 * nds[i] + 1] * phi[i];
        gx[i] = s[1] + 2 * s[3] * x + s[4] * y;
        gy[i] = s[2] + 2 * s[5] * y + s[4] * x;
      }
      double w = GQ2C_W[q] * VE[k];
      for (int i = 0; i < 6; ++i) {
        double gi = gx[i] * ux + gy[i] * uy;
        for (int j = 0; j < 6; ++j) Ck[i][j] += w * gi * phi[j];
      }
    }
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 6; ++j) Cv[36 * k + 6 * i + j] = Ck[j][i];
  }
  long nnz = or_assemble_csc(nv, nt, 6, t, Cv, 0, colptr, rowval, nzval);
  free(Cv);
  return nnz;
}

/* src/FEM2D.jl:163-229 quadraticMassMatrix2D (full quadratic phi, w = weight*VE). */
long or_p2_mass2d(const double *p, const int *t, int nv, long nt, const double *VE, long *colptr, int *rowval,
                  double *nzval) {
  double *Mk = (double *)malloc(sizeof(double) * 36 * (size_t)nt);
#pragma omp parallel for schedule(static)
  for (long k = 0; k < nt; ++k) {
    const int *nds = t + 6 * k;
    double zero[3] = {0, 0, 0};
    double S[6][6];
    for (int a = 0; a < 6; ++a) p2_basis2d(p, nds, a, zero, S[a]);
    const double *v1 = p + 3 * nds[0], *v2 = p + 3 * nds[1], *v3 = p + 3 * nds[2];
    double J11 = v2[0] - v1[0], J12 = v3[0] - v1[0], J21 = v2[1] - v1[1], J22 = v3[1] - v1[1];
    double M[36];
    memset(M, 0, sizeof(M));
    for (int q = 0; q < 6; ++q) {
      double xi = GQ2_PTS[q][0], eta = GQ2_PTS[q][1];
      double x = v1[0] + J11 * xi + J12 * eta, y = v1[1] + J21 * xi + J22 * eta;
      double phi[6];
      for (int i = 0; i < 6; ++i)
        phi[i] = S[i][0] + S[i][1] * x + S[i][2] * y + S[i][3] * x * x + S[i][4] * x * y + S[i][5] * y * y;
      double w = GQ2_W[q] * VE[k];
      for (int i = 0; i < 6; ++i)
        for (int j = i; j < 6; ++j) { M[6 * i + j] += w * phi[i] * phi[j]; M[6 * j + i] = M[6 * i + j]; }
    }
    memcpy(Mk + 36 * k, M, sizeof(M));
  }
  long nnz = or_assemble_csc(nv, nt, 6, t, Mk, 0, colptr, rowval, nzval);
  free(Mk);
  return nnz;
}

/* ------------------------------------------------------------------------- */
/* src/FEM3D.jl:274-281 lagrange: C_i += VE/4 for the element's nodes. */
void or_lagrange(const int *t, int nv, long nt, const double *VE, double *C) {
  memset(C, 0, sizeof(double) * (size_t)nv);
  for (long k = 0; k < nt; ++k)
    for (int a = 0; a < 4; ++a) C[t[4 * k + a]] += VE[k] / 4.0;
}

/* src/FEM3D.jl:284-297 BoundaryIntegral: RHS[face nodes] += (n.F) AE / 3 on  */
/* faces whose boundary id (row 4 of surfaceT) is in shell_id.                 */
void or_boundary_integral(const int *surfaceT, long ns, int nv, const double *normal, const double *AE,
                          const double *F, const int *shell_id, int nshell, double *RHS) {
  memset(RHS, 0, sizeof(double) * (size_t)nv);
  for (long s = 0; s < ns; ++s) {
    int id = surfaceT[4 * s + 3], hit = 0;
    for (int q = 0; q < nshell; ++q) hit |= (id == shell_id[q]);
    if (!hit) continue;
    double v = (normal[3 * s] * F[0] + normal[3 * s + 1] * F[1] + normal[3 * s + 2] * F[2]) * AE[s] / 3.0;
    for (int a = 0; a < 3; ++a) RHS[surfaceT[4 * s + a]] += v;
  }
}

/* ------------------------------------------------------------------------- */
/* Sparse kernels on symmetric CSC (= CSR).  fixed[i] != 0 marks a Dirichlet row. */
void or_spmv(int n, const long *cp, const int *ri, const double *v, const double *x, double *y) {
#pragma omp parallel for schedule(static)
  for (int c = 0; c < n; ++c) {
    double s = 0.0;
    for (long q = cp[c]; q < cp[c + 1]; ++q) s += v[q] * x[ri[q]];
    y[c] = s;
  }
}

static double dot_masked(int n, const double *a, const double *b, const unsigned char *fixed) {
  double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (int i = 0; i < n; ++i)
    if (!fixed || !fixed[i]) s += a[i] * b[i];
  return s;
}

/* Jacobi-preconditioned CG on the free rows (the Dirichlet rows/columns are    */
/* eliminated: their entries of x are held).  Stops when ||r|| <= tol ||r0||.    */
/* The reference runs IterativeSolvers.cg (Magnetostatics/2DmagneticField.jl:139, */
/* Micromagnetics/LL.jl:185, Femeko_jl_C++/Magnetostatics/run.jl:141) and Eigen's */
/* diagonal-preconditioned ConjugateGradient (magnetostatics.cpp:26-38).          */
/* Returns the iteration count, or -1 if maxit was reached.                      */
int or_pcg(int n, const long *cp, const int *ri, const double *v, const double *b, double *x,
           const unsigned char *fixed, double tol, int maxit, double *relres_out) {
  double *r = (double *)malloc(sizeof(double) * n), *z = (double *)malloc(sizeof(double) * n);
  double *pp = (double *)malloc(sizeof(double) * n), *q = (double *)malloc(sizeof(double) * n);
  double *dinv = (double *)malloc(sizeof(double) * n);
  for (int c = 0; c < n; ++c) {
    double d = 0.0;
    for (long k = cp[c]; k < cp[c + 1]; ++k) if (ri[k] == c) d += v[k];
    dinv[c] = (fixed && fixed[c]) ? 0.0 : (d != 0.0 ? 1.0 / d : 0.0);
  }
  /* r = b - A x on free rows; the fixed entries of x contribute through A */
  or_spmv(n, cp, ri, v, x, q);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) r[i] = (fixed && fixed[i]) ? 0.0 : b[i] - q[i];
  /* tolerance relative to the initial residual (IterativeSolvers' reltol convention;
     equal to ||b|| for a zero initial guess) */
  double rn = sqrt(dot_masked(n, r, r, fixed));
  double bn = (rn > 0.0) ? rn : 1.0;
  int it = 0;
  double rz = 0.0;
  if (rn <= tol * bn) goto done;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) { z[i] = dinv[i] * r[i]; pp[i] = z[i]; }
  rz = dot_masked(n, r, z, fixed);
  for (it = 1; it <= maxit; ++it) {
    or_spmv(n, cp, ri, v, pp, q);
    double pq = dot_masked(n, pp, q, fixed);
    double alpha = rz / pq;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
      if (fixed && fixed[i]) continue;
      x[i] += alpha * pp[i];
      r[i] -= alpha * q[i];
      z[i] = dinv[i] * r[i];
    }
    double rz_new = dot_masked(n, r, z, fixed);
    rn = sqrt(dot_masked(n, r, r, fixed));
    if (rn <= tol * bn) break;
    double beta = rz_new / rz;
    rz = rz_new;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) pp[i] = (fixed && fixed[i]) ? 0.0 : z[i] + beta * pp[i];
  }
done:
  if (relres_out) *relres_out = rn / bn;
  free(r); free(z); free(pp); free(q); free(dinv);
  return (it > maxit) ? -1 : it;
}

/* ------------------------------------------------------------------------- */
/* H = -sum_a u_a grad phi_a per element (Magnetostatics/magneticField.jl:111-124). */
/* ref_bug_hz=1 reproduces Magnetostatics/NewtonRaphson.jl:189, which subtracts   */
/* the z term into H[2] instead of H[3].                                           */
void or_hfield(const double *p, const int *t, long nt, const double *u, int ref_bug_hz, double *H) {
#pragma omp parallel for schedule(static)
  for (long k = 0; k < nt; ++k) {
    const int *nds = t + 4 * k;
    double hx = 0, hy = 0, hz = 0;
    for (int a = 0; a < 4; ++a) {
      double r[4];
      or_abcd(p, nds, nds[a], r);
      double ua = u[nds[a]];
      hx -= ua * r[1];
      hy -= ua * r[2];
      if (ref_bug_hz) hy -= ua * r[3]; else hz -= ua * r[3];
    }
    H[3 * k] = hx; H[3 * k + 1] = hy; H[3 * k + 2] = hz;
  }
}

/* Froehlich law mu(H) = mu0 (1 + Ms/(Hk + |H|)) and dmu/dH = -mu0 Ms/(Hk + |H|)^2. */
/* It stands in for the Dierckx spline of Magnetostatics/NewtonRaphson.jl:57-63,204-207. */
void or_froehlich(double H, double Ms, double Hk, double *mu, double *dmu) {
  double den = Hk + H;
  *mu = OR_MU0 * (1.0 + Ms / den);
  *dmu = -OR_MU0 * Ms / (den * den);
}

/* Energy density integral of H dB (src/magneticProperties.jl:252-309, FEMM style),    */
/* in closed form: linear elements 0.5 mu H^2; Froehlich elements                       */
/* mu0 [H^2/2 + Ms Hk (ln(1 + H/Hk) + Hk/(Hk+H) - 1)].                                  */
double or_energy(const double *H3, const double *VE, long nt, const unsigned char *nl, const double *mu_lin,
                 double Ms, double Hk) {
  double W = 0.0;
  for (long k = 0; k < nt; ++k) {
    const double *h = H3 + 3 * k;
    double H = sqrt(h[0] * h[0] + h[1] * h[1] + h[2] * h[2]);
    double w;
    if (nl && nl[k]) w = OR_MU0 * (0.5 * H * H + Ms * Hk * (log1p(H / Hk) + Hk / (Hk + H) - 1.0));
    else w = 0.5 * mu_lin[k] * H * H;
    W += w * VE[k];
  }
  return W;
}

/* src/FEM3D.jl:123-152 lineSearch on the secant operator A (no tangent):          */
/* alpha = 1, 0.9, 0.81, ... while ||F - alpha A du|| > ||F|| and alpha > minStep.   */
/* Returns alpha (0 when the step is rejected, as the reference then keeps u).      */
static double line_search(int n, const long *cp, const int *ri, const double *A, const double *F, const double *du,
                          const unsigned char *fixed, double min_step, double *res_out) {
  double *w = (double *)malloc(sizeof(double) * n);
  or_spmv(n, cp, ri, A, du, w);
  double r0 = sqrt(dot_masked(n, F, F, fixed));
  double alf = 1.0;
  double res;
  for (;;) {
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (int i = 0; i < n; ++i) {
      if (fixed && fixed[i]) continue;
      double d = F[i] - alf * w[i];
      s += d * d;
    }
    res = sqrt(s);
    if (!(res > r0 && alf > min_step)) break;
    alf *= 0.9;
  }
  free(w);
  if (res_out) *res_out = res;
  return (alf < min_step) ? 0.0 : alf;
}

/* Field, permeability and secant residual at potential u:                          */
/* H (NewtonRaphson.jl:178-197), mu/dmu (:204-207), A = sparse(Ak .* mu) (:154-161), */
/* F = RHS - A u on free rows with RHS = 0 after the Dirichlet lifting.              */
static void nr_state(const double *p, const int *t, int nv, long nt, const double *Ak, const unsigned char *fixed,
                     const unsigned char *nl, const double *mu_lin, double Ms, double Hk, int ref_bug_hz,
                     const double *u, double *H, double *mu, double *dmu, double *Acsc, long *cp, int *ri, double *Av,
                     double *F) {
  or_hfield(p, t, nt, u, ref_bug_hz, H);
#pragma omp parallel for schedule(static)
  for (long k = 0; k < nt; ++k) {
    if (nl && nl[k]) {
      double h = sqrt(H[3 * k] * H[3 * k] + H[3 * k + 1] * H[3 * k + 1] + H[3 * k + 2] * H[3 * k + 2]);
      or_froehlich(h, Ms, Hk, &mu[k], &dmu[k]);
    } else { mu[k] = mu_lin[k]; dmu[k] = 0.0; }
    for (int n = 0; n < 16; ++n) Acsc[16 * k + n] = Ak[16 * k + n] * mu[k];
  }
  or_assemble_csc(nv, nt, 4, t, Acsc, 0, cp, ri, Av);
  or_spmv(nv, cp, ri, Av, u, F);
  for (int i = 0; i < nv; ++i) F[i] = fixed[i] ? 0.0 : -F[i];
}

/* Newton-Raphson magnetostatics (Magnetostatics/NewtonRaphson.jl:109-214) in the    */
/* Dirichlet form: u = -H0.x on fixed nodes, residual F = -[K(mu(u)) u] on free rows, */
/* Jacobian K + At (src/FEM3D.jl:79-119), Jacobi-PCG for the increment to relative    */
/* residual cg_tol.  ls_mode selects the step control:                               */
/*   0: full step;                                                                   */
/*   1: src/FEM3D.jl:123-152 lineSearch on the frozen secant A (reference behaviour); */
/*   2: the same backtracking (alpha *= 0.9 while the residual grows, alpha >= 1e-4)  */
/*      on the true nonlinear residual ||F(u + alpha du)||;                          */
/*   3: the true residual with quadratic-interpolation backtracking (same acceptance). */
/* Per element: nl[k] != 0 -> Froehlich(Ms, Hk); else mu = mu_lin[k] (absolute).       */
/* Stops when ||alpha du|| <= tol_update ||u|| (2-norms over all nodes).               */
/* Outputs: u (in: initial guess incl. boundary values), H (3 x nt), mu (nt).          */
/* stats[0..5] = newton iterations, total CG iterations, last update norm ratio,       */
/* last residual norm, last alpha, converged flag.                                     */
int or_newton(const double *p, const int *t, int nv, long nt, const double *VE, const unsigned char *fixed,
              const unsigned char *nl, const double *mu_lin, double Ms, double Hk, double tol_update, int maxit,
              double cg_tol, int cg_maxit, int ref_bug_hz, int ls_mode, int forcing, double eta_min,
              double eta_max, int picard_steps, double *u, double *H, double *mu, double *stats) {
  size_t m16 = 16 * (size_t)nt;
  double *Ak = (double *)malloc(sizeof(double) * m16);
  or_local_stiffness(p, t, nt, VE, NULL, Ak);                      /* NewtonRaphson.jl:112 */
  double *Acsc = (double *)malloc(sizeof(double) * m16);
  double *dmu = (double *)malloc(sizeof(double) * (size_t)nt);
  long *cp = (long *)malloc(sizeof(long) * ((size_t)nv + 1));
  int *ri = (int *)malloc(sizeof(int) * m16);
  double *Av = (double *)malloc(sizeof(double) * m16);
  long *cpt = (long *)malloc(sizeof(long) * ((size_t)nv + 1));
  int *rit = (int *)malloc(sizeof(int) * m16);
  double *Atv = (double *)malloc(sizeof(double) * m16);
  double *F = (double *)malloc(sizeof(double) * nv), *du = (double *)malloc(sizeof(double) * nv);
  double *ut = (double *)malloc(sizeof(double) * nv), *Ft = (double *)malloc(sizeof(double) * nv);
  double *Ht = (double *)malloc(sizeof(double) * 3 * (size_t)nt), *mut = (double *)malloc(sizeof(double) * nt);
  double *dmut = (double *)malloc(sizeof(double) * nt);
  long *cpn = (long *)malloc(sizeof(long) * ((size_t)nv + 1));
  int *rin = (int *)malloc(sizeof(int) * m16);
  double *Avn = (double *)malloc(sizeof(double) * m16);
  int total_cg = 0, it, converged = 0;
  double ratio = 0.0, res = 0.0, alf = 0.0;
  nr_state(p, t, nv, nt, Ak, fixed, nl, mu_lin, Ms, Hk, ref_bug_hz, u, H, mu, dmu, Acsc, cp, ri, Av, F);
  double eta = forcing ? eta_max : cg_tol, r_prev = -1.0;
  for (it = 1; it <= maxit; ++it) {
    double r0 = sqrt(dot_masked(nv, F, F, fixed));
    if (forcing && r_prev > 0.0) {
      /* Eisenstat & Walker (1996) choice 2: gamma (|F_k|/|F_k-1|)^2, gamma = 0.9,
         safeguarded by gamma eta^2 when that exceeds 0.1, clamped to [eta_min, eta_max] */
      double e = 0.9 * (r0 / r_prev) * (r0 / r_prev), sg = 0.9 * eta * eta;
      if (sg > 0.1 && sg > e) e = sg;
      eta = e < eta_min ? eta_min : (e > eta_max ? eta_max : e);
    }
    r_prev = r0;
    long nnz = cp[nv];
    if (it > picard_steps) {
      or_tangent(p, t, nv, nt, VE, H, dmu, 0, cpt, rit, Atv);       /* :165 */
      for (long q = 0; q < nnz; ++q) Atv[q] += Av[q];                /* A + At, same pattern */
    } else {
      memcpy(Atv, Av, sizeof(double) * (size_t)nnz);                 /* :167 At = 0 (Picard step) */
    }
    memset(du, 0, sizeof(double) * nv);
    double rr;
    int its = or_pcg(nv, cp, ri, Atv, F, du, fixed, eta, cg_maxit, &rr);  /* :171-172 */
    total_cg += (its < 0) ? cg_maxit : its;
    if (ls_mode == 1) {
      alf = line_search(nv, cp, ri, Av, F, du, fixed, 1e-4, &res);  /* :175 */
      for (int i = 0; i < nv; ++i) u[i] += alf * du[i];
      nr_state(p, t, nv, nt, Ak, fixed, nl, mu_lin, Ms, Hk, ref_bug_hz, u, H, mu, dmu, Acsc, cp, ri, Av, F);
    } else {
      alf = 1.0;
      for (;;) {
        for (int i = 0; i < nv; ++i) ut[i] = u[i] + alf * du[i];
        nr_state(p, t, nv, nt, Ak, fixed, nl, mu_lin, Ms, Hk, ref_bug_hz, ut, Ht, mut, dmut, Acsc, cpn, rin, Avn, Ft);
        res = sqrt(dot_masked(nv, Ft, Ft, fixed));
        if (ls_mode == 0 || !(res > r0 && alf > 1e-4)) break;
        if (ls_mode == 3) {
          /* quadratic interpolation of f(a) = |F(u + a du)|^2 through f(0), f'(0) = -2 f(0)
             and f(alf); next step kept in [0.1, 0.5] alf (Dennis & Schnabel) */
          double f0 = r0 * r0;
          double c = (res * res - f0 + 2.0 * f0 * alf) / (alf * alf);
          double anew = (c > 0.0) ? f0 / c : 0.5 * alf;
          if (anew < 0.1 * alf) anew = 0.1 * alf;
          if (anew > 0.5 * alf) anew = 0.5 * alf;
          alf = anew;
        } else {
          alf *= 0.9;
        }
      }
      if ((ls_mode == 2 || ls_mode == 3) && alf < 1e-4) alf = 0.0;
      if (alf > 0.0) {
        memcpy(u, ut, sizeof(double) * nv); memcpy(F, Ft, sizeof(double) * nv);
        memcpy(H, Ht, sizeof(double) * 3 * (size_t)nt); memcpy(mu, mut, sizeof(double) * nt);
        memcpy(dmu, dmut, sizeof(double) * nt);
        long *tl = cp; cp = cpn; cpn = tl; int *ti = ri; ri = rin; rin = ti; double *tv = Av; Av = Avn; Avn = tv;
      }
    }
    double dn = 0.0, un = 0.0;
    for (int i = 0; i < nv; ++i) { dn += (alf * du[i]) * (alf * du[i]); un += u[i] * u[i]; }
    ratio = sqrt(dn) / sqrt(un);
    if (ratio <= tol_update) { converged = 1; break; }
    if (alf == 0.0) break;
  }
  if (stats) {
    stats[0] = (it > maxit) ? maxit : it; stats[1] = total_cg; stats[2] = ratio;
    stats[3] = res; stats[4] = alf; stats[5] = converged;
  }
  free(Ak); free(Acsc); free(dmu); free(cp); free(ri); free(Av); free(cpt); free(rit); free(Atv); free(F); free(du);
  free(ut); free(Ft); free(Ht); free(mut); free(dmut); free(cpn); free(rin); free(Avn);
  return converged ? 0 : 1;
}

/* Timed pieces of one Newton iteration of or_newton, for a bounded CPU-baseline      */
/* sample: times[0] = field/permeability/secant assembly/residual (nr_state),          */
/* times[1] = tangent assembly + J = A + At, times[2] = `cg_iters` PCG iterations,      */
/* times[3] = PCG iterations actually run.  Wall-clock seconds (OpenMP threads).       */
void or_newton_sample(const double *p, const int *t, int nv, long nt, const double *VE, const unsigned char *fixed,
                      const unsigned char *nl, const double *mu_lin, double Ms, double Hk, const double *u,
                      int cg_iters, double *times) {
  size_t m16 = 16 * (size_t)nt;
  double *Ak = (double *)malloc(sizeof(double) * m16);
  or_local_stiffness(p, t, nt, VE, NULL, Ak);
  double *Acsc = (double *)malloc(sizeof(double) * m16);
  double *H = (double *)malloc(sizeof(double) * 3 * (size_t)nt);
  double *mu = (double *)malloc(sizeof(double) * nt), *dmu = (double *)malloc(sizeof(double) * nt);
  long *cp = (long *)malloc(sizeof(long) * ((size_t)nv + 1));
  int *ri = (int *)malloc(sizeof(int) * m16);
  double *Av = (double *)malloc(sizeof(double) * m16);
  long *cpt = (long *)malloc(sizeof(long) * ((size_t)nv + 1));
  int *rit = (int *)malloc(sizeof(int) * m16);
  double *Atv = (double *)malloc(sizeof(double) * m16);
  double *F = (double *)malloc(sizeof(double) * nv), *du = (double *)calloc((size_t)nv, sizeof(double));
  double t0 = omp_get_wtime();
  nr_state(p, t, nv, nt, Ak, fixed, nl, mu_lin, Ms, Hk, 0, u, H, mu, dmu, Acsc, cp, ri, Av, F);
  double t1 = omp_get_wtime();
  or_tangent(p, t, nv, nt, VE, H, dmu, 0, cpt, rit, Atv);
  for (long q = 0; q < cp[nv]; ++q) Atv[q] += Av[q];
  double t2 = omp_get_wtime();
  double rr;
  int its = or_pcg(nv, cp, ri, Atv, F, du, fixed, 0.0, cg_iters, &rr);
  double t3 = omp_get_wtime();
  times[0] = t1 - t0; times[1] = t2 - t1; times[2] = t3 - t2; times[3] = (its < 0) ? cg_iters : its;
  free(Ak); free(Acsc); free(H); free(mu); free(dmu); free(cp); free(ri); free(Av); free(cpt); free(rit); free(Atv);
  free(F); free(du);
}

/* Linear magnetostatics (Magnetostatics/magneticField.jl:89-132 with Dirichlet        */
/* phi = -H0.x in place of the Neumann flux + Lagrange row): K(mu) u = 0 on free rows.  */
int or_linear_magnetostatics(const double *p, const int *t, int nv, long nt, const double *VE,
                             const unsigned char *fixed, const double *mu, double cg_tol, int cg_maxit,
                             double *u, double *H, int *iters) {
  long *cp = (long *)malloc(sizeof(long) * ((size_t)nv + 1));
  int *ri = (int *)malloc(sizeof(int) * 16 * (size_t)nt);
  double *Av = (double *)malloc(sizeof(double) * 16 * (size_t)nt);
  or_stiffness(p, t, nv, nt, VE, mu, 0, cp, ri, Av);
  double *b = (double *)calloc((size_t)nv, sizeof(double));
  double rr;
  int it = or_pcg(nv, cp, ri, Av, b, u, fixed, cg_tol, cg_maxit, &rr);
  if (iters) *iters = it;
  if (H) or_hfield(p, t, nt, u, 0, H);
  free(cp); free(ri); free(Av); free(b);
  return it < 0 ? 1 : 0;
}

/* Backward-Euler heat (Heat/heat3D.jl:50-90): (M + dt K(k)) T_{n+1} = M T_n with   */
/* T = 0 on fixed nodes, nsteps steps, PCG warm-started from T_n.  T holds the      */
/* initial field on entry; snapshots (nullable) receive T after every `every` steps. */
int or_heat_be(const double *p, const int *t, int nv, long nt, const double *VE, const unsigned char *fixed,
               const double *kappa, double rho_c, double dt, int nsteps, double cg_tol, int cg_maxit, double *T,
               int every, double *snapshots, int *total_iters) {
  long *cp = (long *)malloc(sizeof(long) * ((size_t)nv + 1));
  int *ri = (int *)malloc(sizeof(int) * 16 * (size_t)nt);
  double *Kv = (double *)malloc(sizeof(double) * 16 * (size_t)nt);
  long *cpm = (long *)malloc(sizeof(long) * ((size_t)nv + 1));
  int *rim = (int *)malloc(sizeof(int) * 16 * (size_t)nt);
  double *Mv = (double *)malloc(sizeof(double) * 16 * (size_t)nt);
  or_stiffness(p, t, nv, nt, VE, kappa, 0, cp, ri, Kv);
  or_mass(t, nv, nt, VE, 0, cpm, rim, Mv);
  long nnz = cp[nv];
  double *Av = (double *)malloc(sizeof(double) * (size_t)nnz);
  for (long q = 0; q < nnz; ++q) Av[q] = rho_c * Mv[q] + dt * Kv[q];
  double *b = (double *)malloc(sizeof(double) * nv);
  int tot = 0, bad = 0, snap = 0;
  for (int i = 0; i < nv; ++i) if (fixed[i]) T[i] = 0.0;
  for (int s = 1; s <= nsteps; ++s) {
    or_spmv(nv, cpm, rim, Mv, T, b);
    for (int i = 0; i < nv; ++i) b[i] *= rho_c;
    double rr;
    int it = or_pcg(nv, cp, ri, Av, b, T, fixed, cg_tol, cg_maxit, &rr);
    if (it < 0) { bad = 1; tot += cg_maxit; } else tot += it;
    if (snapshots && every > 0 && s % every == 0) { memcpy(snapshots + (size_t)snap * nv, T, sizeof(double) * nv); ++snap; }
  }
  if (total_iters) *total_iters = tot;
  free(cp); free(ri); free(Kv); free(cpm); free(rim); free(Mv); free(Av); free(b);
  return bad;
}

/* Objective J = volume-weighted mean of H_x over the target elements               */
/* (the volume average of Magnetostatics/NewtonRaphson.jl:234-240).                   */
double or_objective_hx(const double *p, const int *t, long nt, const double *VE, const unsigned char *target,
                       const double *u) {
  double num = 0.0, vol = 0.0;
  for (long k = 0; k < nt; ++k) {
    if (!target[k]) continue;
    const int *nds = t + 4 * k;
    double hx = 0.0;
    for (int a = 0; a < 4; ++a) { double r[4]; or_abcd(p, nds, nds[a], r); hx -= u[nds[a]] * r[1]; }
    num += VE[k] * hx;
    vol += VE[k];
  }
  return num / vol;
}

/* Adjoint of J with respect to the per-element permeability.  The operator is the   */
/* secant K(mu) (linear case) or K(mu) + At (nonlinear, converged Newton tangent,    */
/* when dmu != NULL and H != NULL).  Solves op^T lambda = dJ/du on free rows and      */
/* returns dJ/dmu_k = -VE_k grad(lambda).grad(u) (per unit of absolute permeability). */
int or_adjoint(const double *p, const int *t, int nv, long nt, const double *VE, const unsigned char *fixed,
               const unsigned char *target, const double *mu, const double *H, const double *dmu, const double *u,
               double cg_tol, int cg_maxit, double *lambda, double *grad) {
  long *cp = (long *)malloc(sizeof(long) * ((size_t)nv + 1));
  int *ri = (int *)malloc(sizeof(int) * 16 * (size_t)nt);
  double *Av = (double *)malloc(sizeof(double) * 16 * (size_t)nt);
  or_stiffness(p, t, nv, nt, VE, mu, 0, cp, ri, Av);
  if (dmu && H) {
    long *cpt = (long *)malloc(sizeof(long) * ((size_t)nv + 1));
    int *rit = (int *)malloc(sizeof(int) * 16 * (size_t)nt);
    double *Atv = (double *)malloc(sizeof(double) * 16 * (size_t)nt);
    or_tangent(p, t, nv, nt, VE, H, dmu, 0, cpt, rit, Atv);
    for (long q = 0; q < cp[nv]; ++q) Av[q] += Atv[q];
    free(cpt); free(rit); free(Atv);
  }
  double vol = 0.0;
  for (long k = 0; k < nt; ++k) if (target[k]) vol += VE[k];
  double *g = (double *)calloc((size_t)nv, sizeof(double));
  for (long k = 0; k < nt; ++k) {
    if (!target[k]) continue;
    const int *nds = t + 4 * k;
    for (int a = 0; a < 4; ++a) { double r[4]; or_abcd(p, nds, nds[a], r); g[nds[a]] -= VE[k] * r[1] / vol; }
  }
  for (int i = 0; i < nv; ++i) { if (fixed[i]) g[i] = 0.0; lambda[i] = 0.0; }
  double rr;
  int it = or_pcg(nv, cp, ri, Av, g, lambda, fixed, cg_tol, cg_maxit, &rr);
#pragma omp parallel for schedule(static)
  for (long k = 0; k < nt; ++k) {
    const int *nds = t + 4 * k;
    double gl[3] = {0, 0, 0}, gu[3] = {0, 0, 0};
    for (int a = 0; a < 4; ++a) {
      double r[4];
      or_abcd(p, nds, nds[a], r);
      for (int c = 0; c < 3; ++c) { gl[c] += lambda[nds[a]] * r[1 + c]; gu[c] += u[nds[a]] * r[1 + c]; }
    }
    grad[k] = -VE[k] * (gl[0] * gu[0] + gl[1] * gu[1] + gl[2] * gu[2]);
  }
  free(cp); free(ri); free(Av); free(g);
  return it < 0 ? 1 : 0;
}

/* Demagnetising field of Micromagnetics/LL.jl:162-211 (magnetostaticField): load
 * vector RHS_i = sum over the inside elements of VE (grad phi_i . mean nodal M),
 * u = PCG(A, RHS) with A the stiffness matrix of the whole mesh (no Dirichlet rows;
 * the Neumann problem is consistent), H_k = -grad u per element, and the nodal field
 * sum over the inside elements of VE H_k divided by the node volumes (the sum of VE
 * of the inside elements of the node; 0/0 where a node has none, as the reference).
 * M is 3 x nv (M[3*i + c]); Hn is 3 x nv. */
int or_demag_field(const double *p, const int *t, int nv, long nt, const double *VE, const unsigned char *inside,
                   const double *M, double cg_tol, int cg_maxit, double *u, double *Hn, int *iters) {
  long *cp = (long *)malloc(sizeof(long) * ((size_t)nv + 1));
  int *ri = (int *)malloc(sizeof(int) * 16 * (size_t)nt);
  double *Av = (double *)malloc(sizeof(double) * 16 * (size_t)nt);
  or_stiffness(p, t, nv, nt, VE, NULL, 0, cp, ri, Av);
  double *rhs = (double *)calloc((size_t)nv, sizeof(double));
  double *vol = (double *)calloc((size_t)nv, sizeof(double));
  for (long k = 0; k < nt; ++k) {
    if (!inside[k]) continue;
    const int *nds = t + 4 * k;
    double f[3] = {0, 0, 0};
    for (int a = 0; a < 4; ++a)
      for (int c = 0; c < 3; ++c) f[c] += M[3 * nds[a] + c] / 4.0;
    for (int a = 0; a < 4; ++a) {
      double r[4];
      or_abcd(p, nds, nds[a], r);
      rhs[nds[a]] += VE[k] * (r[1] * f[0] + r[2] * f[1] + r[3] * f[2]);
    }
  }
  for (int i = 0; i < nv; ++i) u[i] = 0.0;
  double rr;
  int it = or_pcg(nv, cp, ri, Av, rhs, u, NULL, cg_tol, cg_maxit, &rr);
  if (iters) *iters = it;
  double *H = (double *)malloc(sizeof(double) * 3 * (size_t)nt);
  or_hfield(p, t, nt, u, 0, H);
  for (int i = 0; i < 3 * nv; ++i) Hn[i] = 0.0;
  for (long k = 0; k < nt; ++k) {
    if (!inside[k]) continue;
    const int *nds = t + 4 * k;
    for (int a = 0; a < 4; ++a) {
      vol[nds[a]] += VE[k];
      for (int c = 0; c < 3; ++c) Hn[3 * nds[a] + c] += VE[k] * H[3 * k + c];
    }
  }
  for (int i = 0; i < nv; ++i)
    for (int c = 0; c < 3; ++c) Hn[3 * i + c] /= vol[i];
  free(cp); free(ri); free(Av); free(rhs); free(vol); free(H);
  return it < 0 ? 1 : 0;
}
