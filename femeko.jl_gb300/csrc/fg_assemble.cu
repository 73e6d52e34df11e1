// Element kernels and the deterministic row gather.
//
// Assembly runs in two passes, neither of which uses atomics:
//   1. an element kernel computes each element's local matrix (and/or a local
//      vector) and writes local row a of element k to incidence position
//      recpos[a][k] -- the incidence records of a node are contiguous per SELL
//      slice, so the second pass reads them coalesced;
//   2. a row kernel (one thread per matrix row) walks its incidence records in
//      (element, local node) order and adds each value into the row slot given by
//      the precomputed slot byte.  The order of every sum is fixed by the mesh, so
//      results are bit-identical from run to run.
//
// Reference formulas (paths relative to the reference repository):
//   P1 stiffness      src/FEM3D.jl:59-76       VE f (grad phi_a . grad phi_b)
//   P1 mass           src/FEM3D.jl:466-492     VE/20 (1 + delta_ab)
//   P1 tangent        src/FEM3D.jl:79-119      VE dmu/|H| (H.grad phi_a)(H.grad phi_b)
//   2D stiffness/mass src/FEM2D.jl:48-76,139-161
//   P2 stiffness      src/FEM3D.jl:324-376, src/FEM2D.jl:80-115 (equal weights at the nodes)
//   P2 mass           src/FEM3D.jl:494-561, src/FEM2D.jl:163-229 (Gauss rules below)
#include <type_traits>

#include <algorithm>
#include <cstring>

#include "fg_common.cuh"

// ------------------------------------------------------------------ helpers
template <int NPE, typename R>
__device__ __forceinline__ void store_row(R *rec, int64_t pos, const R *v) {
#pragma unroll
  for (int j = 0; j < NPE; ++j) rec[pos * NPE + j] = v[j];
}
template <>
__device__ __forceinline__ void store_row<4, double>(double *rec, int64_t pos, const double *v) {
  double2 *d = reinterpret_cast<double2 *>(rec + pos * 4);
  d[0] = make_double2(v[0], v[1]);
  d[1] = make_double2(v[2], v[3]);
}
template <>
__device__ __forceinline__ void store_row<4, float>(float *rec, int64_t pos, const float *v) {
  *reinterpret_cast<float4 *>(rec + pos * 4) = make_float4(v[0], v[1], v[2], v[3]);
}

// ------------------------------------------------------------------ P1 tetrahedra
// kind: ASM_STIFF   Ke = f VE G G^T
//       ASM_MASS    Ke = f VE/20 (1 + delta)
//       ASM_TANGENT Ke = VE dmu/|H| (H.g_a)(H.g_b)
//       ASM_HEAT    Ke = cm VE/20 (1 + delta) + cs f VE G G^T
template <typename R>
__global__ void k_elem_tet4(int kind, int64_t nt, const double *__restrict__ geo, const double *__restrict__ f,
                            const double *__restrict__ H, const double *__restrict__ dmu, double cm, double cs,
                            const int *__restrict__ recpos, R *__restrict__ rec) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nt) return;
  double g[4][3];
#pragma unroll
  for (int c = 0; c < 12; ++c) g[c / 3][c % 3] = geo[(int64_t)c * nt + k];
  double VE = geo[12 * nt + k];
  double fk = f ? f[k] : 1.0;
  double Ke[4][4];
  if (kind == ASM_MASS || kind == ASM_HEAT) {
    double mfac = (kind == ASM_MASS ? fk : cm) * VE / 20.0;
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) Ke[a][b] = mfac * (a == b ? 2.0 : 1.0);
  }
  if (kind == ASM_STIFF || kind == ASM_HEAT) {
    double s = (kind == ASM_STIFF ? fk : cs * fk) * VE;
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = a; b < 4; ++b) {
        double v = s * (g[a][0] * g[b][0] + g[a][1] * g[b][1] + g[a][2] * g[b][2]);
        if (kind == ASM_HEAT) { Ke[a][b] += v; if (b != a) Ke[b][a] += v; }
        else { Ke[a][b] = v; Ke[b][a] = v; }
      }
  }
  if (kind == ASM_TANGENT) {
    double hx = H[3 * k], hy = H[3 * k + 1], hz = H[3 * k + 2];
    double hn = sqrt(hx * hx + hy * hy + hz * hz);
    double s = (hn > 0.0) ? VE * dmu[k] / hn : 0.0;
    double ah[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) ah[a] = hx * g[a][0] + hy * g[a][1] + hz * g[a][2];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = a; b < 4; ++b) { Ke[a][b] = s * ah[a] * ah[b]; Ke[b][a] = Ke[a][b]; }
  }
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    R row[4];
#pragma unroll
    for (int b = 0; b < 4; ++b) row[b] = (R)Ke[a][b];
    store_row<4, R>(rec, recpos[(int64_t)a * nt + k], row);
  }
}

// ------------------------------------------------------------------ P1 triangles
template <typename R>
__global__ void k_elem_tri3(int kind, int64_t nt, const double *__restrict__ geo, const double *__restrict__ f,
                            double cm, double cs, const int *__restrict__ recpos, R *__restrict__ rec) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nt) return;
  double g[3][2];
#pragma unroll
  for (int c = 0; c < 6; ++c) g[c / 2][c % 2] = geo[(int64_t)c * nt + k];
  double VE = geo[6 * nt + k];
  double fk = f ? f[k] : 1.0;
  double Ke[3][3] = {{0}};
  if (kind == ASM_MASS || kind == ASM_HEAT) {
    double mfac = (kind == ASM_MASS ? fk : cm) * VE / 12.0;
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) Ke[a][b] = mfac * (a == b ? 2.0 : 1.0);
  }
  if (kind == ASM_STIFF || kind == ASM_HEAT) {
    double s = (kind == ASM_STIFF ? fk : cs * fk) * VE;
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) Ke[a][b] += s * (g[a][0] * g[b][0] + g[a][1] * g[b][1]);
  }
  for (int a = 0; a < 3; ++a) {
    R row[3];
    for (int b = 0; b < 3; ++b) row[b] = (R)Ke[a][b];
    store_row<3, R>(rec, recpos[(int64_t)a * nt + k], row);
  }
}

// ------------------------------------------------------------------ second order
// The reference builds each P2 basis function by solving the Vandermonde system of
// the element's nodes (src/FEM3D.jl:21-37, src/FEM2D.jl:28-45).  Here the same
// system is inverted once per element with Gauss-Jordan and partial pivoting, in
// coordinates shifted to the first vertex (same basis functions, better
// conditioned).  Column a of the inverse holds the coefficients of node a's basis.
template <int N>
__device__ bool gj_inverse(double *A, double *Inv) {
  for (int r = 0; r < N; ++r)
    for (int c = 0; c < N; ++c) Inv[r * N + c] = (r == c) ? 1.0 : 0.0;
  for (int c = 0; c < N; ++c) {
    int piv = c;
    double best = fabs(A[c * N + c]);
    for (int r = c + 1; r < N; ++r) {
      double v = fabs(A[r * N + c]);
      if (v > best) { best = v; piv = r; }
    }
    if (best == 0.0) return false;
    if (piv != c)
      for (int q = 0; q < N; ++q) {
        double t0 = A[c * N + q]; A[c * N + q] = A[piv * N + q]; A[piv * N + q] = t0;
        double t1 = Inv[c * N + q]; Inv[c * N + q] = Inv[piv * N + q]; Inv[piv * N + q] = t1;
      }
    double inv = 1.0 / A[c * N + c];
    for (int q = 0; q < N; ++q) { A[c * N + q] *= inv; Inv[c * N + q] *= inv; }
    for (int r = 0; r < N; ++r) {
      if (r == c) continue;
      double l = A[r * N + c];
      if (l == 0.0) continue;
      for (int q = 0; q < N; ++q) { A[r * N + q] -= l * A[c * N + q]; Inv[r * N + q] -= l * Inv[c * N + q]; }
    }
  }
  return true;
}

// 15-point rule of src/FEM3D.jl:710-745 (GaussQuadrature3D(4)); the table is the
// published one and is kept alike.  Weights are divided by 6 as in the reference.
__constant__ double c_gq3_pts[15][3] = {
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
__constant__ double c_gq3_w[15] = {0.1817020685825351, 0.0361607142857143, 0.0361607142857143, 0.0361607142857143,
                                   0.0361607142857143, 0.0698714945161738, 0.0698714945161738, 0.0698714945161738,
                                   0.0698714945161738, 0.0656948493683187, 0.0656948493683187, 0.0656948493683187,
                                   0.0656948493683187, 0.0656948493683187, 0.0656948493683187};
// 6-point rule of src/FEM2D.jl:483-497 (GaussQuadrature2D(4)), weights summing to 1.
__constant__ double c_gq2_pts[6][2] = {{0.445948490915965, 0.445948490915965}, {0.445948490915965, 0.108103018168070},
                                       {0.108103018168070, 0.445948490915965}, {0.091576213509771, 0.091576213509771},
                                       {0.091576213509771, 0.816847572980459}, {0.816847572980459, 0.091576213509771}};
__constant__ double c_gq2_w[6] = {0.223381589678011, 0.223381589678011, 0.223381589678011,
                                  0.109951743655322, 0.109951743655322, 0.109951743655322};

// P2 tetrahedron (10 nodes).  ASM_STIFF: equal-weight rule over the 10 nodes, /10
// (src/FEM3D.jl:344-364).  ASM_MASS: 15-point rule, w = W_q/6 * VE * F
// (src/FEM3D.jl:518-541); full_phi = 0 evaluates only S1 + S2 x + S3 y + S4 z of
// each basis polynomial in global coordinates, as the reference's line break at
// :529-531 makes Julia do.  ASM_CONV: the convection matrix of
// src/FEM3D.jl:563-648, C_ij = sum_q w (u_avg . grad phi_j) phi_i F with u_avg the
// mean of the nodal velocity vel (3 x nv) over the 4 vertices, the same rule and the
// same phi (truncated at :610-613 unless full_phi), grad phi the full quadratic's.
// The reference flattens Ck column-major (:640) but scatters entry n = 10(i-1)+j to
// (t_i, t_j) (:644-648), so its global C[t_i, t_j] sums Ck[j, i].  The row gather of
// untransposed records therefore builds C^T, whose rows are C's CSC columns (the
// export); transpose = 1 records Ck^T, giving the rows of C itself for a solve.
__global__ void k_elem_tet10(int kind, int full_phi, int64_t nt, const double *__restrict__ p,
                             const int *__restrict__ t, const double *__restrict__ geo, const double *__restrict__ f,
                             const double *__restrict__ vel, int transpose, int accumulate,
                             const int *__restrict__ recpos, double *__restrict__ rec, int *flags) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nt) return;
  int nds[10];
  for (int a = 0; a < 10; ++a) nds[a] = t[(int64_t)a * nt + k];
  double x0 = p[3 * nds[0]], y0 = p[3 * nds[0] + 1], z0 = p[3 * nds[0] + 2];
  double X[10], Y[10], Z[10];
  double V[100], S[100];
  for (int r = 0; r < 10; ++r) {
    X[r] = p[3 * nds[r]] - x0; Y[r] = p[3 * nds[r] + 1] - y0; Z[r] = p[3 * nds[r] + 2] - z0;
    double row[10] = {1.0, X[r], Y[r], Z[r], X[r] * X[r], X[r] * Y[r], X[r] * Z[r], Y[r] * Y[r], Y[r] * Z[r], Z[r] * Z[r]};
    for (int c = 0; c < 10; ++c) V[r * 10 + c] = row[c];
  }
  if (!gj_inverse<10>(V, S)) { atomicOr(flags, FLAG_DEGENERATE); return; }
  // S[c*10 + a] = coefficient c of node a's basis (shifted coordinates)
  double VE = geo[12 * nt + k];
  double fk = f ? f[k] : 1.0;
  double Ke[10][10];
  for (int i = 0; i < 10; ++i)
    for (int j = 0; j < 10; ++j) Ke[i][j] = 0.0;
  if (kind == ASM_STIFF) {
    for (int n = 0; n < 10; ++n) {
      double dx[10], dy[10], dz[10];
      for (int a = 0; a < 10; ++a) {
        const double s1 = S[10 + a], s2 = S[20 + a], s3 = S[30 + a], s4 = S[40 + a], s5 = S[50 + a],
                     s6 = S[60 + a], s7 = S[70 + a], s8 = S[80 + a], s9 = S[90 + a];
        dx[a] = s1 + 2 * s4 * X[n] + s5 * Y[n] + s6 * Z[n];
        dy[a] = s2 + 2 * s7 * Y[n] + s5 * X[n] + s8 * Z[n];
        dz[a] = s3 + 2 * s9 * Z[n] + s6 * X[n] + s8 * Y[n];
      }
      for (int i = 0; i < 10; ++i)
        for (int j = i; j < 10; ++j) Ke[i][j] += dx[i] * dx[j] + dy[i] * dy[j] + dz[i] * dz[j];
    }
    for (int i = 0; i < 10; ++i)
      for (int j = i; j < 10; ++j) { Ke[i][j] = Ke[i][j] / 10.0 * fk * VE; Ke[j][i] = Ke[i][j]; }
  } else if (kind == ASM_CONV) {
    double ua[3];
    for (int c = 0; c < 3; ++c)
      ua[c] = 0.25 * (vel[3 * nds[0] + c] + vel[3 * nds[1] + c] + vel[3 * nds[2] + c] + vel[3 * nds[3] + c]);
    double e1 = p[3 * nds[1]] - x0, e2 = p[3 * nds[2]] - x0, e3 = p[3 * nds[3]] - x0;
    double f1 = p[3 * nds[1] + 1] - y0, f2 = p[3 * nds[2] + 1] - y0, f3 = p[3 * nds[3] + 1] - y0;
    double g1 = p[3 * nds[1] + 2] - z0, g2 = p[3 * nds[2] + 2] - z0, g3 = p[3 * nds[3] + 2] - z0;
    for (int q = 0; q < 15; ++q) {
      const double xi = c_gq3_pts[q][0], eta = c_gq3_pts[q][1], ze = c_gq3_pts[q][2];
      const double Xq = e1 * xi + e2 * eta + e3 * ze, Yq = f1 * xi + f2 * eta + f3 * ze,
                   Zq = g1 * xi + g2 * eta + g3 * ze;
      double phi[10], gu[10];
      for (int a = 0; a < 10; ++a) {
        const double s0 = S[a], s1 = S[10 + a], s2 = S[20 + a], s3 = S[30 + a], s4 = S[40 + a], s5 = S[50 + a],
                     s6 = S[60 + a], s7 = S[70 + a], s8 = S[80 + a], s9 = S[90 + a];
        if (full_phi) {
          phi[a] = s0 + s1 * Xq + s2 * Yq + s3 * Zq + s4 * Xq * Xq + s5 * Xq * Yq + s6 * Xq * Zq + s7 * Yq * Yq +
                   s8 * Yq * Zq + s9 * Zq * Zq;
        } else {
          // the constant and linear coefficients of the polynomial in global
          // coordinates (value and gradient at the origin), evaluated at x_q
          const double ox = -x0, oy = -y0, oz = -z0;
          const double c0 = s0 + s1 * ox + s2 * oy + s3 * oz + s4 * ox * ox + s5 * ox * oy + s6 * ox * oz +
                            s7 * oy * oy + s8 * oy * oz + s9 * oz * oz;
          const double cx = s1 + 2 * s4 * ox + s5 * oy + s6 * oz, cy = s2 + 2 * s7 * oy + s5 * ox + s8 * oz,
                       cz = s3 + 2 * s9 * oz + s6 * ox + s8 * oy;
          phi[a] = c0 + cx * (Xq + x0) + cy * (Yq + y0) + cz * (Zq + z0);
        }
        const double gx = s1 + 2 * s4 * Xq + s5 * Yq + s6 * Zq, gy = s2 + 2 * s7 * Yq + s5 * Xq + s8 * Zq,
                     gz = s3 + 2 * s9 * Zq + s6 * Xq + s8 * Yq;
        gu[a] = ua[0] * gx + ua[1] * gy + ua[2] * gz;
      }
      const double w = c_gq3_w[q] / 6.0 * VE;
      for (int i = 0; i < 10; ++i)
        for (int j = 0; j < 10; ++j) Ke[i][j] += w * gu[j] * phi[i] * fk;
    }
    if (transpose)
      for (int i = 0; i < 10; ++i)
        for (int j = i + 1; j < 10; ++j) {
          const double tmp = Ke[i][j];
          Ke[i][j] = Ke[j][i];
          Ke[j][i] = tmp;
        }
  } else {
    // global-coordinate constant and linear coefficients (value and gradient at the origin)
    double e1 = p[3 * nds[1]] - x0, e2 = p[3 * nds[2]] - x0, e3 = p[3 * nds[3]] - x0;
    double f1 = p[3 * nds[1] + 1] - y0, f2 = p[3 * nds[2] + 1] - y0, f3 = p[3 * nds[3] + 1] - y0;
    double g1 = p[3 * nds[1] + 2] - z0, g2 = p[3 * nds[2] + 2] - z0, g3 = p[3 * nds[3] + 2] - z0;
    double lin[10][4];
    if (!full_phi) {
      double ox = -x0, oy = -y0, oz = -z0;
      for (int a = 0; a < 10; ++a) {
        const double *c = S;
        double s0 = c[a], s1 = c[10 + a], s2 = c[20 + a], s3 = c[30 + a], s4 = c[40 + a], s5 = c[50 + a],
               s6 = c[60 + a], s7 = c[70 + a], s8 = c[80 + a], s9 = c[90 + a];
        lin[a][0] = s0 + s1 * ox + s2 * oy + s3 * oz + s4 * ox * ox + s5 * ox * oy + s6 * ox * oz + s7 * oy * oy +
                    s8 * oy * oz + s9 * oz * oz;
        lin[a][1] = s1 + 2 * s4 * ox + s5 * oy + s6 * oz;
        lin[a][2] = s2 + 2 * s7 * oy + s5 * ox + s8 * oz;
        lin[a][3] = s3 + 2 * s9 * oz + s6 * ox + s8 * oy;
      }
    }
    for (int q = 0; q < 15; ++q) {
      double xi = c_gq3_pts[q][0], eta = c_gq3_pts[q][1], ze = c_gq3_pts[q][2];
      double Xq = e1 * xi + e2 * eta + e3 * ze, Yq = f1 * xi + f2 * eta + f3 * ze, Zq = g1 * xi + g2 * eta + g3 * ze;
      double phi[10];
      for (int a = 0; a < 10; ++a) {
        if (full_phi) {
          phi[a] = S[a] + S[10 + a] * Xq + S[20 + a] * Yq + S[30 + a] * Zq + S[40 + a] * Xq * Xq +
                   S[50 + a] * Xq * Yq + S[60 + a] * Xq * Zq + S[70 + a] * Yq * Yq + S[80 + a] * Yq * Zq +
                   S[90 + a] * Zq * Zq;
        } else {
          phi[a] = lin[a][0] + lin[a][1] * (Xq + x0) + lin[a][2] * (Yq + y0) + lin[a][3] * (Zq + z0);
        }
      }
      double w = c_gq3_w[q] / 6.0 * VE;
      for (int i = 0; i < 10; ++i)
        for (int j = i; j < 10; ++j) Ke[i][j] += w * phi[i] * phi[j] * fk;
    }
    for (int i = 0; i < 10; ++i)
      for (int j = i + 1; j < 10; ++j) Ke[j][i] = Ke[i][j];
  }
  if (accumulate) {
    for (int a = 0; a < 10; ++a) {
      double *r = rec + (int64_t)recpos[(int64_t)a * nt + k] * 10;
      for (int j = 0; j < 10; ++j) r[j] += Ke[a][j];
    }
  } else {
    for (int a = 0; a < 10; ++a) store_row<10, double>(rec, recpos[(int64_t)a * nt + k], Ke[a]);
  }
}

// 4-point rule of src/FEM2D.jl:477-484 (GaussQuadrature2D(3)), weights summing to 1.
__constant__ double c_gq2c_pts[4][2] = {{1.0 / 3.0, 1.0 / 3.0}, {0.2, 0.2}, {0.6, 0.2}, {0.2, 0.6}};
__constant__ double c_gq2c_w[4] = {-27.0 / 48.0, 25.0 / 48.0, 25.0 / 48.0, 25.0 / 48.0};

// P2 triangle (6 nodes).  ASM_STIFF: 6-node equal-weight rule, /6
// (src/FEM2D.jl:95-107).  ASM_MASS: 6-point rule, w = weight * VE (src/FEM2D.jl:192-212).
// ASM_CONV: src/FEM2D.jl:231-319, the velocity (vel, 3 x nv, z unused) interpolated
// with the P2 basis at each point of the 4-point rule, w = weight * VE; the reference's
// Ck[i,j] = w (grad phi_i . u) phi_j scattered from its column-major flattening gives
// C[t_i, t_j] = sum w (u . grad phi_j) phi_i, whose rows are recorded here
// (transpose = 1 records the rows of C^T, the CSC export).
__global__ void k_elem_tri6(int kind, int64_t nt, const double *__restrict__ p, const int *__restrict__ t,
                            const double *__restrict__ geo, const double *__restrict__ f,
                            const double *__restrict__ vel, int transpose, int accumulate,
                            const int *__restrict__ recpos, double *__restrict__ rec, int *flags) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nt) return;
  int nds[6];
  for (int a = 0; a < 6; ++a) nds[a] = t[(int64_t)a * nt + k];
  double x0 = p[3 * nds[0]], y0 = p[3 * nds[0] + 1];
  double X[6], Y[6], V[36], S[36];
  for (int r = 0; r < 6; ++r) {
    X[r] = p[3 * nds[r]] - x0; Y[r] = p[3 * nds[r] + 1] - y0;
    double row[6] = {1.0, X[r], Y[r], X[r] * X[r], X[r] * Y[r], Y[r] * Y[r]};
    for (int c = 0; c < 6; ++c) V[r * 6 + c] = row[c];
  }
  if (!gj_inverse<6>(V, S)) { atomicOr(flags, FLAG_DEGENERATE); return; }
  double VE = geo[6 * nt + k];
  double fk = f ? f[k] : 1.0;
  double Ke[6][6];
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) Ke[i][j] = 0.0;
  if (kind == ASM_STIFF) {
    for (int n = 0; n < 6; ++n) {
      double dx[6], dy[6];
      for (int a = 0; a < 6; ++a) {
        dx[a] = S[6 + a] + 2 * S[18 + a] * X[n] + S[24 + a] * Y[n];
        dy[a] = S[12 + a] + S[24 + a] * X[n] + 2 * S[30 + a] * Y[n];
      }
      for (int i = 0; i < 6; ++i)
        for (int j = i; j < 6; ++j) Ke[i][j] += dx[i] * dx[j] + dy[i] * dy[j];
    }
    for (int i = 0; i < 6; ++i)
      for (int j = i; j < 6; ++j) { Ke[i][j] = Ke[i][j] / 6.0 * VE * fk; Ke[j][i] = Ke[i][j]; }
  } else if (kind == ASM_CONV) {
    const double e1 = p[3 * nds[1]] - x0, e2 = p[3 * nds[2]] - x0;
    const double f1 = p[3 * nds[1] + 1] - y0, f2 = p[3 * nds[2] + 1] - y0;
    for (int q = 0; q < 4; ++q) {
      const double xi = c_gq2c_pts[q][0], eta = c_gq2c_pts[q][1];
      const double Xq = e1 * xi + e2 * eta, Yq = f1 * xi + f2 * eta;
      double phi[6], gx[6], gy[6], ux = 0.0, uy = 0.0;
      for (int a = 0; a < 6; ++a) {
        phi[a] = S[a] + S[6 + a] * Xq + S[12 + a] * Yq + S[18 + a] * Xq * Xq + S[24 + a] * Xq * Yq + S[30 + a] * Yq * Yq;
        ux += vel[3 * nds[a]] * phi[a];
        uy += vel[3 * nds[a] + 1] * phi[a];
        gx[a] = S[6 + a] + 2 * S[18 + a] * Xq + S[24 + a] * Yq;
        gy[a] = S[12 + a] + 2 * S[30 + a] * Yq + S[24 + a] * Xq;
      }
      const double w = c_gq2c_w[q] * VE;
      for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) Ke[i][j] += w * (gx[j] * ux + gy[j] * uy) * phi[i] * fk;
    }
    if (transpose)
      for (int i = 0; i < 6; ++i)
        for (int j = i + 1; j < 6; ++j) {
          const double tmp = Ke[i][j];
          Ke[i][j] = Ke[j][i];
          Ke[j][i] = tmp;
        }
  } else {
    double e1 = p[3 * nds[1]] - x0, e2 = p[3 * nds[2]] - x0;
    double f1 = p[3 * nds[1] + 1] - y0, f2 = p[3 * nds[2] + 1] - y0;
    for (int q = 0; q < 6; ++q) {
      double xi = c_gq2_pts[q][0], eta = c_gq2_pts[q][1];
      double Xq = e1 * xi + e2 * eta, Yq = f1 * xi + f2 * eta;
      double phi[6];
      for (int a = 0; a < 6; ++a)
        phi[a] = S[a] + S[6 + a] * Xq + S[12 + a] * Yq + S[18 + a] * Xq * Xq + S[24 + a] * Xq * Yq + S[30 + a] * Yq * Yq;
      double w = c_gq2_w[q] * VE;
      for (int i = 0; i < 6; ++i)
        for (int j = i; j < 6; ++j) Ke[i][j] += w * phi[i] * phi[j] * fk;
    }
    for (int i = 0; i < 6; ++i)
      for (int j = i + 1; j < 6; ++j) Ke[j][i] = Ke[i][j];
  }
  if (accumulate) {
    for (int a = 0; a < 6; ++a) {
      double *r = rec + (int64_t)recpos[(int64_t)a * nt + k] * 6;
      for (int j = 0; j < 6; ++j) r[j] += Ke[a][j];
    }
  } else {
    for (int a = 0; a < 6; ++a) store_row<6, double>(rec, recpos[(int64_t)a * nt + k], Ke[a]);
  }
}

// ------------------------------------------------------------------ Newton element pass
// |x|^-1/2 and 1/x in FP64 by Newton-Raphson refinement of the FP32 hardware
// estimate (rsqrtf / __frcp_rn): y <- y (3 - x y^2) / 2 and r <- r (2 - x r), two
// steps each.  Each step squares the relative error, so two steps take the ~1e-7 FP32
// estimate below FP64 rounding.  On GB300 an FP64 operation is ~64x dearer than an
// FP32 one, and these replace the FP64 square root and division of the element pass.
// Arguments outside the FP32 normal range take the FP64 library path.
__device__ __forceinline__ double rsqrt_nr(double x) {
  if (!(x > 1e-30 && x < 1e30)) return (x > 0.0) ? 1.0 / sqrt(x) : 0.0;
  double y = (double)rsqrtf((float)x);
  y = y * fma(-0.5 * x * y, y, 1.5);
  y = y * fma(-0.5 * x * y, y, 1.5);
  return y;
}
__device__ __forceinline__ double rcp_nr(double x) {
  if (!(fabs(x) > 1e-30 && fabs(x) < 1e30)) return 1.0 / x;
  double r = (double)__frcp_rn((float)x);
  r = fma(r, fma(-x, r, 1.0), r);
  r = fma(r, fma(-x, r, 1.0), r);
  return r;
}

// From the potential u (Magnetostatics/NewtonRaphson.jl:154-207, src/FEM3D.jl:79-119),
// with the element Gram matrix G_ab = grad(phi_a).grad(phi_b) precomputed per mesh:
//   w_a = (G u)_a = -H.grad(phi_a), evaluated on u - u_0 (G's rows sum to zero),
//   |H|^2 = u.w,  mu and dmu (Froehlich law for nl elements, mu_lin otherwise),
//   residual records (K_e u_e)_a = VE mu w_a,
//   Jacobian records J_ab = VE mu G_ab + VE dmu/|H| w_a w_b.
// The Jacobian records are skipped when rec is null (line-search trials) and are
// formed in FP32 when R is float (they feed the FP32 operator only); the residual,
// |H| and mu stay FP64.
template <typename R>
__global__ void __launch_bounds__(128) k_elem_newton(int64_t nt, const double *__restrict__ geo,
                                                     const int *__restrict__ t, const double *__restrict__ u,
                                                     const uint8_t *__restrict__ nl,
                                                     const double *__restrict__ mu_lin, double Ms, double Hk,
                                                     const int *__restrict__ recpos, R *__restrict__ rec,
                                                     double *__restrict__ rec_r, double *__restrict__ mu_out,
                                                     double *__restrict__ dmu_out, int tangent, int *flags) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nt) return;
  double G[10];
#pragma unroll
  for (int c = 0; c < 10; ++c) G[c] = geo[(int64_t)(13 + c) * nt + k];
  const double VE = geo[12 * nt + k];
  double uu[4];
#pragma unroll
  for (int a = 0; a < 4; ++a) uu[a] = u[t[(int64_t)a * nt + k]];
  const double d1 = uu[1] - uu[0], d2 = uu[2] - uu[0], d3 = uu[3] - uu[0];
  // G upper triangle: 0:00 1:01 2:02 3:03 4:11 5:12 6:13 7:22 8:23 9:33
  double w[4];
  w[0] = G[1] * d1 + G[2] * d2 + G[3] * d3;
  w[1] = G[4] * d1 + G[5] * d2 + G[6] * d3;
  w[2] = G[5] * d1 + G[7] * d2 + G[8] * d3;
  w[3] = G[6] * d1 + G[8] * d2 + G[9] * d3;
  // |H| only matters where mu depends on it (linear elements skip it: dmu = 0)
  double mu, dmu, ih = 0.0;
  if (nl[k]) {
    const double h2 = fmax(d1 * w[1] + d2 * w[2] + d3 * w[3], 0.0);
    ih = rsqrt_nr(h2);  // 1/|H| (0 when H = 0)
    const double h = h2 * ih;
    const double inv = rcp_nr(Hk + h);
    mu = FG_MU0 * fma(Ms, inv, 1.0);
    dmu = -FG_MU0 * Ms * inv * inv;
  } else {
    mu = mu_lin[k];
    dmu = 0.0;
  }
  if (!isfinite(mu) || !isfinite(dmu)) atomicOr(flags, FLAG_NAN);
  mu_out[k] = mu;
  dmu_out[k] = dmu;
  const double vm = VE * mu;
  int pos[4];
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    pos[a] = recpos[(int64_t)a * nt + k];
    rec_r[pos[a]] = vm * w[a];
  }
  if (rec == nullptr) return;  // residual-only pass (line-search trial)
  const double ct = tangent ? VE * dmu * ih : 0.0;  // 0: secant (Picard) Jacobian
  if (std::is_same<R, float>::value) {
    float Gf[10], wf[4];
#pragma unroll
    for (int c = 0; c < 10; ++c) Gf[c] = (float)G[c];
#pragma unroll
    for (int a = 0; a < 4; ++a) wf[a] = (float)w[a];
    const float vmf = (float)vm, ctf = (float)ct;
    const int idx[4][4] = {{0, 1, 2, 3}, {1, 4, 5, 6}, {2, 5, 7, 8}, {3, 6, 8, 9}};
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      R row[4];
      const float ca = ctf * wf[a];
#pragma unroll
      for (int b = 0; b < 4; ++b) row[b] = (R)fmaf(ca, wf[b], vmf * Gf[idx[a][b]]);
      store_row<4, R>(rec, pos[a], row);
    }
  } else {
    const int idx[4][4] = {{0, 1, 2, 3}, {1, 4, 5, 6}, {2, 5, 7, 8}, {3, 6, 8, 9}};
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      R row[4];
      const double ca = ct * w[a];
#pragma unroll
      for (int b = 0; b < 4; ++b) row[b] = (R)fma(ca, w[b], vm * G[idx[a][b]]);
      store_row<4, R>(rec, pos[a], row);
    }
  }
}

// ---------------------------------------------------------------- nonlinear subset
// Newton on a mesh whose elements are mostly linear: the linear elements' part of the
// operator does not change between Newton iterations, so it is assembled once per
// solve and only the nonlinear (Froehlich) elements are re-evaluated.  These kernels
// work on the list of nonlinear elements.

// For nonlinear element e (mesh element k = list[e]) and local nodes a, b: the SELL
// position of the entry (t[a], t[b]) and the row t[a].
__global__ void k_nl_map(int n_nl, const int *__restrict__ list, int64_t nt, const int *__restrict__ t,
                         const int *__restrict__ recpos, const uint8_t *__restrict__ in_slot,
                         const int *__restrict__ sl_ptr, int *__restrict__ pos_out, int *__restrict__ row_out) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_nl) return;
  const int64_t k = list[e];
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const int row = t[(int64_t)a * nt + k];
    const int64_t ip = recpos[(int64_t)a * nt + k];
    row_out[4 * e + a] = row;
#pragma unroll
    for (int b = 0; b < 4; ++b)
      pos_out[16 * e + 4 * a + b] = (int)sell_pos(sl_ptr[row / FG_SLICE], row % FG_SLICE, in_slot[ip * 4 + b]);
  }
}

// The Froehlich elements of k_elem_newton: mu, dmu, the local residual VE mu G d
// (re, 4 per element) and, when ke != null, the local Jacobian VE mu G + ct w w^T
// (16 per element), all FP64.
// One Froehlich element at nodal potentials uu: w = the Gram matrix times the
// potential differences (w_a = grad phi_a . sum_b u_b grad phi_b), |H|^2 = u . w, the
// permeability mu(|H|) and its derivative, and 1/|H|.
__device__ __forceinline__ void nl_elem_eval(const double (&G)[10], const double (&uu)[4], double Ms, double Hk,
                                             double (&w)[4], double &mu, double &dmu, double &ih) {
  const double d1 = uu[1] - uu[0], d2 = uu[2] - uu[0], d3 = uu[3] - uu[0];
  w[0] = G[1] * d1 + G[2] * d2 + G[3] * d3;
  w[1] = G[4] * d1 + G[5] * d2 + G[6] * d3;
  w[2] = G[5] * d1 + G[7] * d2 + G[8] * d3;
  w[3] = G[6] * d1 + G[8] * d2 + G[9] * d3;
  const double h2 = fmax(d1 * w[1] + d2 * w[2] + d3 * w[3], 0.0);
  ih = rsqrt_nr(h2);
  const double h = h2 * ih;
  const double inv = rcp_nr(Hk + h);
  mu = FG_MU0 * fma(Ms, inv, 1.0);
  dmu = -FG_MU0 * Ms * inv * inv;
}

__global__ void __launch_bounds__(128) k_elem_newton_nl(int n_nl, const int *__restrict__ list, int64_t nt,
                                                        const double *__restrict__ geo, const int *__restrict__ t,
                                                        const double *__restrict__ u, double Ms, double Hk,
                                                        double *__restrict__ mu_out, double *__restrict__ dmu_out,
                                                        double *__restrict__ re, double *__restrict__ ke, int tangent,
                                                        int *flags) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_nl) return;
  const int64_t k = list[e];
  double G[10];
#pragma unroll
  for (int c = 0; c < 10; ++c) G[c] = geo[(int64_t)(13 + c) * nt + k];
  const double VE = geo[12 * nt + k];
  double uu[4];
#pragma unroll
  for (int a = 0; a < 4; ++a) uu[a] = u[t[(int64_t)a * nt + k]];
  double w[4], mu, dmu, ih;
  nl_elem_eval(G, uu, Ms, Hk, w, mu, dmu, ih);
  if (!isfinite(mu) || !isfinite(dmu)) atomicOr(flags, FLAG_NAN);
  mu_out[k] = mu;
  dmu_out[k] = dmu;
  const double vm = VE * mu;
#pragma unroll
  for (int a = 0; a < 4; ++a) re[4 * e + a] = vm * w[a];
  if (ke == nullptr) return;
  const double ct = tangent ? VE * dmu * ih : 0.0;
  const int idx[4][4] = {{0, 1, 2, 3}, {1, 4, 5, 6}, {2, 5, 7, 8}, {3, 6, 8, 9}};
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) ke[16 * e + 4 * a + b] = fma(ct * w[a], w[b], vm * G[idx[a][b]]);
}

// The residual records of every nonlinear element at the candidate points
// u + a_c du (thread per (candidate, element)): the trial point of k_newton_trial64
// and the arithmetic of k_elem_newton_nl, without the element state writes.
__global__ void __launch_bounds__(128) k_elem_newton_nl_cand(LsCand cand, int n_nl, const int *__restrict__ list,
                                                             int64_t nt, const double *__restrict__ geo,
                                                             const int *__restrict__ t, const double *__restrict__ u,
                                                             const double *__restrict__ du, double Ms, double Hk,
                                                             double *__restrict__ re) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (int64_t)cand.n * n_nl) return;
  const int c = (int)(q / n_nl), e = (int)(q - (int64_t)c * n_nl);
  const double alpha = cand.a[c];
  const int64_t k = list[e];
  double G[10];
#pragma unroll
  for (int j = 0; j < 10; ++j) G[j] = geo[(int64_t)(13 + j) * nt + k];
  const double VE = geo[12 * nt + k];
  double uu[4];
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const int node = t[(int64_t)a * nt + k];
    uu[a] = fma(alpha, du[node], u[node]);
  }
  double w[4], mu, dmu, ih;
  nl_elem_eval(G, uu, Ms, Hk, w, mu, dmu, ih);
  const double vm = VE * mu;
#pragma unroll
  for (int a = 0; a < 4; ++a) re[(int64_t)c * 4 * n_nl + 4 * e + a] = vm * w[a];
}

// Per candidate (one block each): the sum over the rows that nonlinear elements touch
// of (fma(a_c, z_i, y_i) + the row's records at that candidate)^2, the records added
// in the order of k_nl_rows; Dirichlet rows are 0.  Thread-strided rows, then a fixed
// shuffle and shared-memory tree.
__global__ void __launch_bounds__(1024) k_nl_rows_cand_norm(LsCand cand, int n_rows, int n_nl,
                                                           const int *__restrict__ rows, const int *__restrict__ ptr,
                                                           const int *__restrict__ src, const double *__restrict__ re,
                                                           const double *__restrict__ y, const double *__restrict__ z,
                                                           const uint8_t *__restrict__ fixed, double *__restrict__ out) {
  const int c = blockIdx.x;
  if (c >= cand.n) return;
  const double alpha = cand.a[c];
  const double *rc = re + (int64_t)c * 4 * n_nl;
  double acc = 0.0;
  for (int r = threadIdx.x; r < n_rows; r += blockDim.x) {
    const int i = rows[r];
    if (fixed && fixed[i]) continue;
    double s = 0.0;
    for (int q = ptr[r]; q < ptr[r + 1]; ++q) s += rc[src[q]];
    const double v = fma(alpha, z[i], y[i]) + s;
    acc = fma(v, v, acc);
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  __shared__ double sh[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) sh[warp] = acc;
  __syncthreads();
  if (warp == 0) {
    acc = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) out[FG_LS_QUAD + c] = acc;
  }
}

// Rows that nonlinear elements touch, as a 0/1 mask.
__global__ void k_mark_rows(int n_rows, const int *__restrict__ rows, uint8_t *__restrict__ mask) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < n_rows) mask[rows[r]] = 1;
}

// y[row] += the nonlinear elements' residual records of the row, in a fixed order
// (rows listed once; Dirichlet rows untouched).
__global__ void k_nl_rows(int n_rows, const int *__restrict__ rows, const int *__restrict__ ptr,
                          const int *__restrict__ src, const double *__restrict__ re,
                          const uint8_t *__restrict__ fixed, double *__restrict__ y) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_rows) return;
  const int i = rows[r];
  if (fixed && fixed[i]) return;
  double s = 0.0;
  for (int q = ptr[r]; q < ptr[r + 1]; ++q) s += re[src[q]];
  y[i] += s;
}

// val[pos] = lin[pos] + the nonlinear elements' entries at that position (fixed
// order); on the diagonal also the Jacobi inverse.  code >= 0: the row of an
// off-diagonal slot; code < 0: ~row of a diagonal slot.  Dirichlet rows keep their
// identity rows.
template <typename T>
__global__ void k_nl_slots(int n_slots, const int *__restrict__ pos, const int *__restrict__ ptr,
                           const int *__restrict__ src, const int *__restrict__ code, const double *__restrict__ lin,
                           const double *__restrict__ ke, const uint8_t *__restrict__ fixed, T *__restrict__ val,
                           T *__restrict__ dinv) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n_slots) return;
  const int c = code[q];
  const int row = c >= 0 ? c : ~c;
  if (fixed && fixed[row]) return;
  const int p = pos[q];
  double v = lin[p];
  for (int j = ptr[q]; j < ptr[q + 1]; ++j) v += ke[src[j]];
  val[p] = (T)v;
  if (c < 0) dinv[row] = (T)(v != 0.0 ? 1.0 / v : 0.0);
}
template __global__ void k_nl_slots<float>(int, const int *, const int *, const int *, const int *, const double *,
                                           const double *, const uint8_t *, float *, float *);
template __global__ void k_nl_slots<double>(int, const int *, const int *, const int *, const int *, const double *,
                                            const double *, const uint8_t *, double *, double *);

// Energy density integral of H dB times VE (src/magneticProperties.jl:252-309, FEMM
// style) in closed form: linear elements mu |H|^2 / 2, Froehlich elements
// mu0 [|H|^2/2 + Ms Hk (ln(1 + |H|/Hk) + Hk/(Hk + |H|) - 1)].
__global__ void k_energy_tet4(int64_t nt, const double *__restrict__ geo, const int *__restrict__ t,
                              const double *__restrict__ u, const uint8_t *__restrict__ nl,
                              const double *__restrict__ mu_lin, double Ms, double Hk, double *__restrict__ wout) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nt) return;
  double hx = 0, hy = 0, hz = 0;
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    double ua = u[t[(int64_t)a * nt + k]];
    hx -= ua * geo[(int64_t)(3 * a) * nt + k];
    hy -= ua * geo[(int64_t)(3 * a + 1) * nt + k];
    hz -= ua * geo[(int64_t)(3 * a + 2) * nt + k];
  }
  double h2 = hx * hx + hy * hy + hz * hz, h = sqrt(h2), wd;
  if (nl[k]) wd = FG_MU0 * (0.5 * h2 + Ms * Hk * (log1p(h / Hk) + Hk / (Hk + h) - 1.0));
  else wd = 0.5 * mu_lin[k] * h2;
  wout[k] = wd * geo[12 * nt + k];
}

// Objective of the adjoint: J = sum_T VE Hx / sum_T VE over the target elements, the
// volume-weighted mean of Magnetostatics/NewtonRaphson.jl:234-240 with
// Hx = -sum_a u_a dphi_a/dx (Magnetostatics/magneticField.jl:111-124).
__global__ void k_objective_tet4(int64_t nt, const double *__restrict__ geo, const int *__restrict__ t,
                                 const double *__restrict__ u, const uint8_t *__restrict__ target,
                                 double *__restrict__ a_out, double *__restrict__ v_out) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nt) return;
  double a = 0.0, v = 0.0;
  if (target[k]) {
    double hx = 0.0;
#pragma unroll
    for (int q = 0; q < 4; ++q) hx = fma(-u[t[(int64_t)q * nt + k]], geo[(int64_t)(3 * q) * nt + k], hx);
    v = geo[12 * nt + k];
    a = v * hx;
  }
  a_out[k] = a;
  v_out[k] = v;
}

// Demagnetising-field load vector of Micromagnetics/LL.jl:169-181: for an inside
// element, VE (grad phi_a . f) with f the mean of the nodal magnetisation M (3 x nv,
// M[3 i + c]); outside elements write 0.
__global__ void k_demag_rhs_tet4(int64_t nt, const double *__restrict__ geo, const int *__restrict__ t,
                                 const uint8_t *__restrict__ inside, const double *__restrict__ M,
                                 const int *__restrict__ recpos, double *__restrict__ rec_r) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nt) return;
  double f[3] = {0.0, 0.0, 0.0};
  const bool in = inside[k] != 0;
  if (in)
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const int node = t[(int64_t)a * nt + k];
#pragma unroll
      for (int c = 0; c < 3; ++c) f[c] += 0.25 * M[3 * (int64_t)node + c];
    }
  const double VE = geo[12 * nt + k];
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    double v = 0.0;
    if (in)
      v = VE * (geo[(int64_t)(3 * a) * nt + k] * f[0] + geo[(int64_t)(3 * a + 1) * nt + k] * f[1] +
                geo[(int64_t)(3 * a + 2) * nt + k] * f[2]);
    rec_r[recpos[(int64_t)a * nt + k]] = v;
  }
}

// VE x_k on the 4 records of every inside element (x = component c of H (3 x nt), or
// 1 when H is null: the node volumes); outside elements write 0.
__global__ void k_inside_weighted_tet4(int64_t nt, const double *__restrict__ geo, const uint8_t *__restrict__ inside,
                                       const double *__restrict__ H, int c, const int *__restrict__ recpos,
                                       double *__restrict__ rec_r) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nt) return;
  const double v = inside[k] ? geo[12 * nt + k] * (H ? H[3 * k + c] : 1.0) : 0.0;
#pragma unroll
  for (int a = 0; a < 4; ++a) rec_r[recpos[(int64_t)a * nt + k]] = v;
}

__global__ void k_nodal_average(int64_t nv, const double *__restrict__ sx, const double *__restrict__ sy,
                                const double *__restrict__ sz, const double *__restrict__ vol, double *__restrict__ Hn) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  // plain division, 0/0 = NaN on nodes without an inside element (as the reference)
  Hn[3 * i] = sx[i] / vol[i];
  Hn[3 * i + 1] = sy[i] / vol[i];
  Hn[3 * i + 2] = sz[i] / vol[i];
}

// dJ/du_a = -sum_{T owns a} VE dphi_a/dx / vol as vector records (every element writes
// its 4 records; zero outside the target).
__global__ void k_objective_rhs_tet4(int64_t nt, const double *__restrict__ geo,
                                     const uint8_t *__restrict__ target, double inv_vol,
                                     const int *__restrict__ recpos, double *__restrict__ rec_r) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nt) return;
  const double s = target[k] ? -geo[12 * nt + k] * inv_vol : 0.0;
#pragma unroll
  for (int q = 0; q < 4; ++q) rec_r[recpos[(int64_t)q * nt + k]] = s * geo[(int64_t)(3 * q) * nt + k];
}

// dJ/dmu_k = -lambda^T (dK/dmu_k) u = -VE_k grad(lambda).grad(u); scale carries the
// sign and the unit (mu0 for a gradient per relative permeability).
__global__ void k_adjoint_grad_tet4(int64_t nt, const double *__restrict__ geo, const int *__restrict__ t,
                                    const double *__restrict__ lam, const double *__restrict__ u, double scale,
                                    double *__restrict__ grad) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nt) return;
  double gl[3] = {0.0, 0.0, 0.0}, gu[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int node = t[(int64_t)q * nt + k];
    const double lq = lam[node], uq = u[node];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const double g = geo[(int64_t)(3 * q + c) * nt + k];
      gl[c] = fma(lq, g, gl[c]);
      gu[c] = fma(uq, g, gu[c]);
    }
  }
  grad[k] = scale * geo[12 * nt + k] * (gl[0] * gu[0] + gl[1] * gu[1] + gl[2] * gu[2]);
}

// (K_e x_e)_a for the stiffness (coef * VE G G^T) or mass (coef VE/20 (1+delta)) or
// both (heat: cm M + cs K).  Vector records only.
__global__ void k_elem_apply_tet4(int kind, int64_t nt, const double *__restrict__ geo, const int *__restrict__ t,
                                  const double *__restrict__ coef, double cm, double cs, const double *__restrict__ x,
                                  const int *__restrict__ recpos, double *__restrict__ rec_r) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nt) return;
  double VE = geo[12 * nt + k];
  double xx[4];
#pragma unroll
  for (int a = 0; a < 4; ++a) xx[a] = x[t[(int64_t)a * nt + k]];
  double ck = coef ? coef[k] : 1.0;
  double out[4] = {0, 0, 0, 0};
  if (kind == ASM_STIFF || kind == ASM_HEAT) {
    double g[4][3];
#pragma unroll
    for (int c = 0; c < 12; ++c) g[c / 3][c % 3] = geo[(int64_t)c * nt + k];
    double gx = 0, gy = 0, gz = 0;
#pragma unroll
    for (int a = 0; a < 4; ++a) { gx += xx[a] * g[a][0]; gy += xx[a] * g[a][1]; gz += xx[a] * g[a][2]; }
    double s = (kind == ASM_STIFF ? ck : cs * ck) * VE;
#pragma unroll
    for (int a = 0; a < 4; ++a) out[a] = s * (g[a][0] * gx + g[a][1] * gy + g[a][2] * gz);
  }
  if (kind == ASM_MASS || kind == ASM_HEAT) {
    double mfac = (kind == ASM_MASS ? ck : cm) * VE / 20.0;
    double sum = xx[0] + xx[1] + xx[2] + xx[3];
#pragma unroll
    for (int a = 0; a < 4; ++a) out[a] += mfac * (sum + xx[a]);
  }
#pragma unroll
  for (int a = 0; a < 4; ++a) rec_r[recpos[(int64_t)a * nt + k]] = out[a];
}

__global__ void k_hfield_tet4(int64_t nt, const double *__restrict__ geo, const int *__restrict__ t,
                              const double *__restrict__ u, double *__restrict__ H) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nt) return;
  double hx = 0, hy = 0, hz = 0;
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    double ua = u[t[(int64_t)a * nt + k]];
    hx -= ua * geo[(int64_t)(3 * a) * nt + k];
    hy -= ua * geo[(int64_t)(3 * a + 1) * nt + k];
    hz -= ua * geo[(int64_t)(3 * a + 2) * nt + k];
  }
  H[3 * k] = hx; H[3 * k + 1] = hy; H[3 * k + 2] = hz;
}

// ------------------------------------------------------------------ row gather
// The assembled row of one thread (slot accumulators acc[q * bs]) to the outputs:
// SELL FP64 / FP32 values, CSR order, and the Jacobi inverse diagonal; a Dirichlet
// row (bc) becomes an identity row with a zero inverse diagonal.
template <typename A>
__device__ __forceinline__ void row_store(int64_t i, int lane, int L, int bs, A *acc, int dk, bool bc, int64_t sb,
                                          const int *__restrict__ rowptr, double *__restrict__ out64,
                                          float *__restrict__ out32, double *__restrict__ outcsr,
                                          double *__restrict__ dinv64, float *__restrict__ dinv32) {
  if (bc)
    for (int q = 0; q < L; ++q) acc[q * bs] = (q == dk) ? (A)1 : (A)0;
  if (out64)
    for (int q = 0; q < L; q += 2) {
      int64_t p0 = sell_pos(sb, lane, q);
      *reinterpret_cast<double2 *>(out64 + p0) = make_double2((double)acc[q * bs], (double)acc[(q + 1) * bs]);
    }
  if (out32)
    for (int q = 0; q < L; q += 4) {
      int64_t p0 = sell_pos(sb, lane, q);
      *reinterpret_cast<float4 *>(out32 + p0) = make_float4((float)acc[q * bs], (float)acc[(q + 1) * bs],
                                                            (float)acc[(q + 2) * bs], (float)acc[(q + 3) * bs]);
    }
  if (outcsr) {
    int rb = rowptr[i], len = rowptr[i + 1] - rb;
    for (int q = 0; q < len; ++q) outcsr[rb + q] = (double)acc[q * bs];
  }
  double d = (double)acc[dk * bs];
  double di = bc ? 0.0 : (d != 0.0 ? 1.0 / d : 0.0);
  if (dinv64) dinv64[i] = di;
  if (dinv32) dinv32[i] = (float)di;
}

// One thread per row.  Walks the row's incidence records (SELL layout, pads marked
// 0xFF) and accumulates into a per-thread slot array in shared memory, then writes
// the row once: SELL (FP64 and/or FP32), or CSR order for export.  Dirichlet rows
// become identity rows when apply_bc is set.  Also writes the Jacobi inverse
// diagonal and the vector-record sum (scaled by vsign, zeroed on Dirichlet rows).
template <int NPE, typename R, typename A>
__global__ void k_row_sum(int64_t nv, const int *__restrict__ in_ptr, const int *__restrict__ in_len,
                          const uint8_t *__restrict__ in_slot, const R *__restrict__ rec,
                          const double *__restrict__ rec_r, const int *__restrict__ sl_ptr,
                          const int *__restrict__ sl_len, const int *__restrict__ rowptr,
                          const uint8_t *__restrict__ diagk, const uint8_t *__restrict__ fixed, int apply_bc,
                          double *__restrict__ out64, float *__restrict__ out32, double *__restrict__ outcsr,
                          double *__restrict__ dinv64, float *__restrict__ dinv32, double *__restrict__ vout,
                          double vsign, int zero_fixed_vec) {
  extern __shared__ unsigned char smem_raw[];
  A *acc = reinterpret_cast<A *>(smem_raw) + threadIdx.x;
  const int bs = blockDim.x;
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  int s = (int)(i / FG_SLICE), lane = (int)(i % FG_SLICE);
  int L = FG_GROUP * sl_len[s];
  const bool want_mat = (rec != nullptr);
  if (want_mat)
    for (int q = 0; q < L; ++q) acc[q * bs] = (A)0;
  double vacc = 0.0;
  int64_t base = in_ptr[s] + lane;
  int ilen = in_len[s];
  for (int mm = 0; mm < ilen; ++mm) {
    int64_t pos = base + (int64_t)mm * FG_SLICE;
    uint8_t sl[NPE];
    if (NPE == 4) {
      uint32_t w = reinterpret_cast<const uint32_t *>(in_slot)[pos];
      sl[0] = w & 0xFF; sl[1] = (w >> 8) & 0xFF; sl[2] = (w >> 16) & 0xFF; sl[3] = (w >> 24) & 0xFF;
    } else {
#pragma unroll
      for (int j = 0; j < NPE; ++j) sl[j] = in_slot[pos * NPE + j];
    }
    if (sl[0] == 0xFF) continue;  // pad
    if (rec_r) vacc += rec_r[pos];
    if (want_mat) {
      if (NPE == 4 && sizeof(R) == 8) {
        const double2 *d = reinterpret_cast<const double2 *>(rec + pos * 4);
        double2 v01 = d[0], v23 = d[1];
        acc[sl[0] * bs] += (A)v01.x; acc[sl[1] * bs] += (A)v01.y;
        acc[sl[2] * bs] += (A)v23.x; acc[sl[3] * bs] += (A)v23.y;
      } else if (NPE == 4 && sizeof(R) == 4) {
        float4 v = *reinterpret_cast<const float4 *>(rec + pos * 4);
        acc[sl[0] * bs] += (A)v.x; acc[sl[1] * bs] += (A)v.y;
        acc[sl[2] * bs] += (A)v.z; acc[sl[3] * bs] += (A)v.w;
      } else {
#pragma unroll
        for (int j = 0; j < NPE; ++j) acc[sl[j] * bs] += (A)rec[pos * NPE + j];
      }
    }
  }
  const bool fx = fixed && fixed[i];
  if (vout) vout[i] = (zero_fixed_vec && fx) ? 0.0 : vsign * vacc;
  if (!want_mat) return;
  row_store<A>(i, lane, L, bs, acc, diagk[i], apply_bc && fx, sl_ptr[s], rowptr, out64, out32, outcsr, dinv64, dinv32);
}

// The element of each incidence position, 4 k + a (element k, local node a), -1 on
// pads: the inverse of recpos, built once per handle.
__global__ void k_inc_elem(int64_t nt, const int *__restrict__ recpos, int *__restrict__ in_elem) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;  // e = a nt + k
  if (e >= 4 * nt) return;
  const int a = (int)(e / nt);
  const int64_t k = e - (int64_t)a * nt;
  in_elem[recpos[e]] = (int)(4 * k + a);
}

// P1 tetrahedra, one pass without element records: one thread per row walks the
// row's incidences (element k, local node a) in the order the two-pass form sums
// its records, and adds each element entry Ke[a][b] straight from the stored
// geometry into the row's slot accumulators (FP64 fused multiply-adds, fixed order,
// no atomics):
//   ASM_STIFF  f_k VE_k G_k[a][b]                       (src/FEM3D.jl:59-76)
//   ASM_MASS   f_k VE_k / 20 (1 + delta_ab)              (src/FEM3D.jl:466-492)
//   ASM_HEAT   cm VE_k / 20 (1 + delta_ab) + cs f_k VE_k G_k[a][b]
// G_k = grad phi_a . grad phi_b is the Gram matrix kept with the element geometry.
// Each element's data is read by its four rows; they run at nearly the same time,
// so the repeats are served from L2.
template <int KIND>
__global__ void __launch_bounds__(128) k_asm_rows_tet4(int64_t nv, int64_t nt, const int *__restrict__ in_ptr,
                                                       const int *__restrict__ in_len,
                                                       const uint8_t *__restrict__ in_slot,
                                                       const int *__restrict__ in_elem, const double *__restrict__ geo,
                                                       const double *__restrict__ f, double cm, double cs,
                                                       const int *__restrict__ sl_ptr, const int *__restrict__ sl_len,
                                                       const int *__restrict__ rowptr, const uint8_t *__restrict__ diagk,
                                                       const uint8_t *__restrict__ fixed, int apply_bc,
                                                       double *__restrict__ out64, float *__restrict__ out32,
                                                       double *__restrict__ outcsr, double *__restrict__ dinv64,
                                                       float *__restrict__ dinv32) {
  extern __shared__ unsigned char smem_raw[];
  double *acc = reinterpret_cast<double *>(smem_raw) + threadIdx.x;
  const int bs = blockDim.x;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  const int s = (int)(i / FG_SLICE), lane = (int)(i % FG_SLICE);
  const int L = FG_GROUP * sl_len[s];
  for (int q = 0; q < L; ++q) acc[q * bs] = 0.0;
  const int64_t base = in_ptr[s] + lane;
  const int ilen = in_len[s];
  const double *VE = geo + 12 * nt;
  const uint32_t *slot4 = reinterpret_cast<const uint32_t *>(in_slot);
  // four incidences at a time: their element codes and slot bytes, then all their
  // element data, are loaded before any of it is used, so that a thread keeps some
  // twenty independent loads in flight instead of two dependent ones
  constexpr int U = 4;
  for (int m0 = 0; m0 < ilen; m0 += U) {
    int code[U];
    uint32_t w[U];
#pragma unroll
    for (int j = 0; j < U; ++j) {
      const int64_t pos = base + (int64_t)(m0 + j) * FG_SLICE;
      code[j] = (m0 + j < ilen) ? in_elem[pos] : -1;
      w[j] = (m0 + j < ilen) ? slot4[pos] : 0u;
    }
    double sk[U], mk[U], g[U][4];
    int aj[U];
#pragma unroll
    for (int j = 0; j < U; ++j) {
      sk[j] = 0.0;
      mk[j] = 0.0;
      aj[j] = code[j] & 3;
#pragma unroll
      for (int b = 0; b < 4; ++b) g[j][b] = 0.0;
      if (code[j] < 0) continue;  // pad
      const int64_t k = code[j] >> 2;
      const int a = aj[j];
      const double fk = f ? f[k] : 1.0;
      const double ve = VE[k];
      if (KIND == ASM_STIFF || KIND == ASM_HEAT) {
        sk[j] = (KIND == ASM_STIFF ? fk : cs * fk) * ve;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          // position of G_ab in the stored upper triangle: lo (9 - lo) / 2 + hi - lo
          const int lo = a < b ? a : b, hi = a < b ? b : a;
          g[j][b] = geo[(int64_t)(13 + (lo * (9 - lo)) / 2 + hi - lo) * nt + k];
        }
      }
      // times 1/20 rather than a division: an FP64 division is a long instruction
      // sequence on a pipe that runs at 1/64 of the FP32 rate (the product differs from
      // the quotient by at most an ulp)
      if (KIND == ASM_MASS || KIND == ASM_HEAT) mk[j] = (KIND == ASM_MASS ? fk : cm) * ve * 0.05;
    }
#pragma unroll
    for (int j = 0; j < U; ++j) {
      if (code[j] < 0) continue;
      const int sl[4] = {(int)(w[j] & 0xFF), (int)((w[j] >> 8) & 0xFF), (int)((w[j] >> 16) & 0xFF), (int)(w[j] >> 24)};
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        double v = acc[sl[b] * bs];
        if (KIND == ASM_MASS || KIND == ASM_HEAT) v += (b == aj[j]) ? 2.0 * mk[j] : mk[j];
        if (KIND == ASM_STIFF || KIND == ASM_HEAT) v = fma(sk[j], g[j][b], v);
        acc[sl[b] * bs] = v;
      }
    }
  }
  const bool fx = fixed && fixed[i];
  row_store<double>(i, lane, L, bs, acc, diagk[i], apply_bc && fx, sl_ptr[s], rowptr, out64, out32, outcsr, dinv64,
                    dinv32);
}

// ------------------------------------------------------------------ host side
void fg_ensure_records(fg_mesh *m) {
  if (!m->rec) m->rec = dev_alloc<double>(m, (size_t)m->ninc * m->npe);
  if (!m->rec_r) m->rec_r = dev_alloc<double>(m, (size_t)m->ninc);
}

static void ensure_operator(fg_mesh *m, bool want64, bool want32) {
  if (want64 && !m->val64) m->val64 = dev_alloc<double>(m, (size_t)m->nsell);
  if (want32 && !m->val32) m->val32 = dev_alloc<float>(m, (size_t)m->nsell);
  // the Jacobi diagonals are read 4 rows at a time: padded rows stay 0
  if (!m->dinv64) {
    m->dinv64 = dev_alloc<double>(m, (size_t)m->nvp);
    FG_CUDA_TRY(cudaMemsetAsync(m->dinv64, 0, sizeof(double) * (size_t)m->nvp, m->stream));
  }
  if (!m->dinv32) {
    m->dinv32 = dev_alloc<float>(m, (size_t)m->nvp);
    FG_CUDA_TRY(cudaMemsetAsync(m->dinv32, 0, sizeof(float) * (size_t)m->nvp, m->stream));
  }
}

template <int NPE, typename R, typename A>
static void launch_row(fg_mesh *m, const R *rec, const double *rec_r, int apply_bc, double *out64, float *out32,
                       double *outcsr, double *dinv64, float *dinv32, double *vout, double vsign, int zero_fixed_vec) {
  int L = std::max(m->maxrow4, FG_GROUP);
  int block = (L * (int)sizeof(A) * 128 <= 48 * 1024) ? 128 : 64;
  size_t smem = (size_t)block * L * sizeof(A);
  auto kern = k_row_sum<NPE, R, A>;
  if (smem > 48 * 1024) FG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  kern<<<grid_for(m->nv, block), block, smem, m->stream>>>(
      m->nv, m->in_ptr, m->in_len, m->in_slot, rec, rec_r, m->sl_ptr, m->sl_len, m->rowptr, m->diagk,
      m->has_fixed ? m->fixed : nullptr, apply_bc, out64, out32, outcsr, dinv64, dinv32, vout, vsign, zero_fixed_vec);
  FG_CUDA_TRY(cudaGetLastError());
  FG_LAUNCHED(1);
}

template <typename R, typename A>
static void launch_row_any(fg_mesh *m, const R *rec, const double *rec_r, int apply_bc, double *out64, float *out32,
                           double *outcsr, double *dinv64, float *dinv32, double *vout, double vsign,
                           int zero_fixed_vec) {
  switch (m->npe) {
    case 3: launch_row<3, R, A>(m, rec, rec_r, apply_bc, out64, out32, outcsr, dinv64, dinv32, vout, vsign, zero_fixed_vec); break;
    case 4: launch_row<4, R, A>(m, rec, rec_r, apply_bc, out64, out32, outcsr, dinv64, dinv32, vout, vsign, zero_fixed_vec); break;
    case 6: launch_row<6, R, A>(m, rec, rec_r, apply_bc, out64, out32, outcsr, dinv64, dinv32, vout, vsign, zero_fixed_vec); break;
    default: launch_row<10, R, A>(m, rec, rec_r, apply_bc, out64, out32, outcsr, dinv64, dinv32, vout, vsign, zero_fixed_vec); break;
  }
}

// Element pass (FP64 records) for the given kind.
static void launch_elem(fg_mesh *m, int kind, const double *d_f, const double *d_H, const double *d_dmu, double cm,
                        double cs, int full_phi, bool transpose) {
  FG_REQUIRE(!m->edge, FG_UNSUPPORTED, "nodal element matrices on a Nedelec (edge) handle");
  fg_ensure_records(m);
  double *rec = static_cast<double *>(m->rec);
  unsigned g = grid_for(m->nt, 128);
  switch (m->npe) {
    case 4: k_elem_tet4<double><<<g, 128, 0, m->stream>>>(kind, m->nt, m->geo, d_f, d_H, d_dmu, cm, cs, m->recpos, rec); break;
    case 3:
      FG_REQUIRE(kind != ASM_TANGENT, FG_UNSUPPORTED, "tangent stiffness is defined for tetrahedra");
      k_elem_tri3<double><<<g, 128, 0, m->stream>>>(kind, m->nt, m->geo, d_f, cm, cs, m->recpos, rec);
      break;
    case 10:
      FG_REQUIRE(kind == ASM_STIFF || kind == ASM_MASS || kind == ASM_CONV, FG_UNSUPPORTED,
                 "P2 tetrahedra: stiffness, mass and convection only");
      k_elem_tet10<<<grid_for(m->nt, 64), 64, 0, m->stream>>>(kind, full_phi, m->nt, m->p, m->t, m->geo, d_f,
                                                               kind == ASM_CONV ? d_H : nullptr, transpose ? 1 : 0,
                                                               0, m->recpos, rec, m->flags);
      break;
    default:
      FG_REQUIRE(kind == ASM_STIFF || kind == ASM_MASS || kind == ASM_CONV, FG_UNSUPPORTED,
                 "P2 triangles: stiffness, mass and convection only");
      k_elem_tri6<<<grid_for(m->nt, 64), 64, 0, m->stream>>>(kind, m->nt, m->p, m->t, m->geo, d_f,
                                                              kind == ASM_CONV ? d_H : nullptr, transpose ? 1 : 0, 0,
                                                              m->recpos, rec, m->flags);
      break;
  }
  FG_CUDA_TRY(cudaGetLastError());
  FG_LAUNCHED(1);
}

// One-pass P1-tetrahedron assembly (k_asm_rows_tet4) of stiffness, mass or heat.
static void launch_rows_tet4(fg_mesh *m, int kind, const double *d_f, double cm, double cs, int apply_bc,
                             double *out64, float *out32, double *outcsr, double *dinv64, float *dinv32) {
  if (!m->in_elem) {
    m->in_elem = dev_alloc<int>(m, (size_t)m->ninc);
    FG_CUDA_TRY(cudaMemsetAsync(m->in_elem, 0xFF, sizeof(int) * (size_t)m->ninc, m->stream));
    k_inc_elem<<<grid_for(4 * m->nt, 256), 256, 0, m->stream>>>(m->nt, m->recpos, m->in_elem);
    FG_CUDA_TRY(cudaGetLastError());
    FG_LAUNCHED(1);
  }
  const int L = std::max(m->maxrow4, FG_GROUP);
  const int block = 128;
  const size_t smem = (size_t)block * L * sizeof(double);
  auto go = [&](auto kern) {
    if (smem > 48 * 1024) FG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<grid_for(m->nv, block), block, smem, m->stream>>>(
        m->nv, m->nt, m->in_ptr, m->in_len, m->in_slot, m->in_elem, m->geo, d_f, cm, cs, m->sl_ptr, m->sl_len,
        m->rowptr, m->diagk, m->has_fixed ? m->fixed : nullptr, apply_bc, out64, out32, outcsr, dinv64, dinv32);
  };
  if (kind == ASM_STIFF) go(k_asm_rows_tet4<ASM_STIFF>);
  else if (kind == ASM_MASS) go(k_asm_rows_tet4<ASM_MASS>);
  else go(k_asm_rows_tet4<ASM_HEAT>);
  FG_CUDA_TRY(cudaGetLastError());
  FG_LAUNCHED(1);
}

// The P1-tetrahedron mass matrix (unit coefficient) into SELL values out64, no
// boundary rows applied: for products M x repeated with one matrix.
void fg_assemble_mass_sell(fg_mesh *m, double *out64) {
  FG_REQUIRE(m->npe == 4 && !m->edge, FG_UNSUPPORTED, "mass operator: P1 tetrahedra only");
  launch_rows_tet4(m, ASM_MASS, nullptr, 0.0, 0.0, 0, out64, nullptr, nullptr, nullptr, nullptr);
}

void fg_assemble_operator(fg_mesh *m, int kind, const double *d_f, const double *d_H, const double *d_dmu,
                          double c_mass, double c_stiff, int full_phi, int layout, bool want64, bool want32,
                          bool apply_bc) {
  if (layout != OUT_CSR) { m->op_tag = 0; ++m->op_version; }
  if (m->npe == 4 && !m->edge && !m->asm_two_pass && (kind == ASM_STIFF || kind == ASM_MASS || kind == ASM_HEAT)) {
    if (layout != OUT_CSR) ensure_operator(m, want64, want32);
    else if (!m->csrval) m->csrval = dev_alloc<double>(m, (size_t)m->nnz);
    launch_rows_tet4(m, kind, d_f, c_mass, c_stiff, layout == OUT_CSR ? 0 : (apply_bc ? 1 : 0),
                     layout == OUT_CSR ? nullptr : (want64 ? m->val64 : nullptr),
                     layout == OUT_CSR ? nullptr : (want32 ? m->val32 : nullptr),
                     layout == OUT_CSR ? m->csrval : nullptr, layout == OUT_CSR ? nullptr : m->dinv64,
                     layout == OUT_CSR ? nullptr : m->dinv32);
    return;
  }
  // convection: the 3D records are the rows of the reference's C^T, the 2D records
  // the rows of its C (see the element kernels); transpose to what the layout needs
  const bool tr = kind == ASM_CONV && ((m->npe == 10) == (layout != OUT_CSR));
  launch_elem(m, kind, d_f, d_H, d_dmu, c_mass, c_stiff, full_phi, tr);
  const double *rec = static_cast<const double *>(m->rec);
  if (layout == OUT_CSR) {
    if (!m->csrval) m->csrval = dev_alloc<double>(m, (size_t)m->nnz);
    launch_row_any<double, double>(m, rec, nullptr, 0, nullptr, nullptr, m->csrval, nullptr, nullptr, nullptr, 0.0, 0);
  } else {
    ensure_operator(m, want64, want32);
    launch_row_any<double, double>(m, rec, nullptr, apply_bc ? 1 : 0, want64 ? m->val64 : nullptr,
                                   want32 ? m->val32 : nullptr, nullptr, m->dinv64, m->dinv32, nullptr, 0.0, 0);
  }
}

// ------------------------------------------------------------------ Nedelec edge elements
// Whitney edge elements on P1 tetrahedra (src/FEM3D.jl:155-271,
// Magnetostatics/nedelec3D.jl:106-221).  Local edge e joins local vertices
// (i_e, j_e) = (1,2), (2,3), (3,1), (4,1), (3,4), (2,4) (src/mesh.jl:603-630, Gmsh's
// order) and curl N_e = 2 l_e (grad lambda_i x grad lambda_j) with l_e = |x_j - x_i|,
// in the element's local orientation as the reference uses it.
__constant__ int c_ned_i[6] = {0, 1, 2, 3, 2, 1};
__constant__ int c_ned_j[6] = {1, 2, 0, 0, 3, 3};

__device__ __forceinline__ void ned_curls(int64_t k, int64_t nt, const double *__restrict__ p,
                                          const int *__restrict__ tv, const double *__restrict__ geo,
                                          double (&cN)[6][3]) {
  int v[4];
  for (int a = 0; a < 4; ++a) v[a] = tv[(int64_t)a * nt + k];
  for (int e = 0; e < 6; ++e) {
    const int i = c_ned_i[e], j = c_ned_j[e];
    const double dx = p[3 * v[j]] - p[3 * v[i]], dy = p[3 * v[j] + 1] - p[3 * v[i] + 1],
                 dz = p[3 * v[j] + 2] - p[3 * v[i] + 2];
    const double l2 = 2.0 * sqrt(dx * dx + dy * dy + dz * dz);
    const double gix = geo[(int64_t)(3 * i) * nt + k], giy = geo[(int64_t)(3 * i + 1) * nt + k],
                 giz = geo[(int64_t)(3 * i + 2) * nt + k];
    const double gjx = geo[(int64_t)(3 * j) * nt + k], gjy = geo[(int64_t)(3 * j + 1) * nt + k],
                 gjz = geo[(int64_t)(3 * j + 2) * nt + k];
    cN[e][0] = l2 * (giy * gjz - giz * gjy);
    cN[e][1] = l2 * (giz * gjx - gix * gjz);
    cN[e][2] = l2 * (gix * gjy - giy * gjx);
  }
}

__device__ __forceinline__ double dot3(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// Element records: nu VE curlN_i.curlN_j (nu = 1 when null; src/FEM3D.jl:155-191 and the
// `.*nu` of nedelec3D.jl:172) plus, with dnu, the tangential term
// VE (curlN_i.B)(curlN_j.B) dnu / |B| of src/FEM3D.jl:194-271 (0 where |B| = 0).
// With bext, the load VE Bext.curlN_e of nedelec3D.jl:109-139 in the vector records.
__global__ void k_elem_ned(int64_t nt, const double *__restrict__ p, const int *__restrict__ tv,
                           const double *__restrict__ geo, const double *__restrict__ nu, int with_stiff,
                           const double *__restrict__ dnu, const double *__restrict__ Bf, const double *__restrict__ Bn,
                           double bx, double by, double bz, int with_load, const int *__restrict__ recpos,
                           double *__restrict__ rec, double *__restrict__ rec_r) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nt) return;
  double cN[6][3];
  ned_curls(k, nt, p, tv, geo, cN);
  const double VE = geo[12 * nt + k];
  if (with_load) {
    const double be[3] = {bx, by, bz};
    for (int e = 0; e < 6; ++e) rec_r[recpos[(int64_t)e * nt + k]] = VE * dot3(be, cN[e]);
  }
  if (!rec) return;
  double Ke[6][6];
  const double nk = nu ? nu[k] : 1.0;
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) Ke[i][j] = with_stiff ? VE * dot3(cN[i], cN[j]) * nk : 0.0;
  if (dnu) {
    const double b[3] = {Bf[3 * k], Bf[3 * k + 1], Bf[3 * k + 2]};
    const double bn = Bn[k];
    if (bn != 0.0) {
      double cb[6];
      for (int e = 0; e < 6; ++e) cb[e] = dot3(cN[e], b);
      for (int i = 0; i < 6; ++i)
        for (int j = i; j < 6; ++j) {
          const double a = VE * cb[i] * cb[j] * dnu[k] / bn;
          Ke[i][j] += a;
          if (j != i) Ke[j][i] += a;
        }
    }
  }
  for (int e = 0; e < 6; ++e) store_row<6, double>(rec, recpos[(int64_t)e * nt + k], Ke[e]);
}

// Element blocks Ak (36 x nt, column k = the 6 x 6 matrix row-major) of
// src/FEM3D.jl:155-191 nedelecLocalStiffness.
__global__ void k_ned_local(int64_t nt, const double *__restrict__ p, const int *__restrict__ tv,
                            const double *__restrict__ geo, double *__restrict__ Ak) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nt) return;
  double cN[6][3];
  ned_curls(k, nt, p, tv, geo, cN);
  const double VE = geo[12 * nt + k];
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) Ak[36 * k + 6 * i + j] = VE * dot3(cN[i], cN[j]);
}

// B on each element: sum_e u[edge_e] curlN_e and its norm (nedelec3D.jl:190-221).
__global__ void k_ned_bfield(int64_t nt, const double *__restrict__ p, const int *__restrict__ tv,
                             const double *__restrict__ geo, const int *__restrict__ t, const double *__restrict__ u,
                             double *__restrict__ Bf, double *__restrict__ Bn) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nt) return;
  double cN[6][3];
  ned_curls(k, nt, p, tv, geo, cN);
  double b[3] = {0.0, 0.0, 0.0};
  for (int e = 0; e < 6; ++e) {
    const double ue = u[t[(int64_t)e * nt + k]];
    for (int c = 0; c < 3; ++c) b[c] += ue * cN[e][c];
  }
  for (int c = 0; c < 3; ++c) Bf[3 * k + c] = b[c];
  if (Bn) Bn[k] = sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
}

void fg_nedelec_operator(fg_mesh *m, const double *d_nu, bool with_stiff, const double *d_dnu, const double *d_Bf,
                         const double *d_Bn, int layout, bool want32) {
  FG_REQUIRE(m->edge, FG_UNSUPPORTED, "Nedelec operator: needs a handle from fg_edge_mesh_create");
  if (layout != OUT_CSR) { m->op_tag = 0; ++m->op_version; }
  fg_ensure_records(m);
  double *rec = static_cast<double *>(m->rec);
  k_elem_ned<<<grid_for(m->nt, 128), 128, 0, m->stream>>>(m->nt, m->p, m->tv, m->geo, d_nu, with_stiff ? 1 : 0,
                                                           d_dnu, d_Bf, d_Bn, 0.0, 0.0, 0.0, 0, m->recpos, rec,
                                                           nullptr);
  FG_CUDA_TRY(cudaGetLastError());
  FG_LAUNCHED(1);
  if (layout == OUT_CSR) {
    if (!m->csrval) m->csrval = dev_alloc<double>(m, (size_t)m->nnz);
    launch_row_any<double, double>(m, rec, nullptr, 0, nullptr, nullptr, m->csrval, nullptr, nullptr, nullptr, 0.0, 0);
  } else {
    ensure_operator(m, true, want32);
    launch_row_any<double, double>(m, rec, nullptr, 0, m->val64, want32 ? m->val32 : nullptr, nullptr, m->dinv64,
                                   want32 ? m->dinv32 : nullptr, nullptr, 0.0, 0);
  }
}

void fg_nedelec_load_dev(fg_mesh *m, const double bext[3], double *d_rhs) {
  FG_REQUIRE(m->edge, FG_UNSUPPORTED, "Nedelec load: needs a handle from fg_edge_mesh_create");
  fg_ensure_records(m);
  k_elem_ned<<<grid_for(m->nt, 128), 128, 0, m->stream>>>(m->nt, m->p, m->tv, m->geo, nullptr, 0, nullptr, nullptr,
                                                           nullptr, bext[0], bext[1], bext[2], 1, m->recpos, nullptr,
                                                           m->rec_r);
  FG_CUDA_TRY(cudaGetLastError());
  FG_LAUNCHED(1);
  launch_row<6, double, double>(m, nullptr, m->rec_r, 0, nullptr, nullptr, nullptr, nullptr, nullptr, d_rhs, 1.0, 0);
}

void fg_nedelec_bfield_dev(fg_mesh *m, const double *d_u, double *d_Bf, double *d_Bn) {
  FG_REQUIRE(m->edge, FG_UNSUPPORTED, "Nedelec B field: needs a handle from fg_edge_mesh_create");
  k_ned_bfield<<<grid_for(m->nt, 128), 128, 0, m->stream>>>(m->nt, m->p, m->tv, m->geo, m->t, d_u, d_Bf, d_Bn);
  FG_CUDA_TRY(cudaGetLastError());
  FG_LAUNCHED(1);
}

void fg_nedelec_local_dev(fg_mesh *m, double *d_Ak) {
  FG_REQUIRE(m->edge, FG_UNSUPPORTED, "Nedelec local stiffness: needs a handle from fg_edge_mesh_create");
  k_ned_local<<<grid_for(m->nt, 128), 128, 0, m->stream>>>(m->nt, m->p, m->tv, m->geo, d_Ak);
  FG_CUDA_TRY(cudaGetLastError());
  FG_LAUNCHED(1);
}

void fg_transport_operator(fg_mesh *m, const double *d_rhocp, const double *d_kdt, const double *d_vel,
                           const double *d_fdt, int full_phi) {
  FG_REQUIRE(!m->edge && (m->npe == 10 || m->npe == 6), FG_UNSUPPORTED,
             "transport operator: P2 tetrahedra or P2 triangles only");
  m->op_tag = 0;
  ++m->op_version;
  fg_ensure_records(m);
  ensure_operator(m, true, false);
  if (!m->mval) m->mval = dev_alloc<double>(m, (size_t)m->nsell);
  double *rec = static_cast<double *>(m->rec);
  const unsigned g = grid_for(m->nt, 64);
  // records: M; gathered alone into mval, then + K + C on the same records (the rows
  // of the reference's C: transposed records in 3D, as they come in 2D)
  auto elem = [&](int kind, const double *f, const double *vel, int acc) {
    if (m->npe == 10)
      k_elem_tet10<<<g, 64, 0, m->stream>>>(kind, full_phi, m->nt, m->p, m->t, m->geo, f, vel, kind == ASM_CONV ? 1 : 0,
                                            acc, m->recpos, rec, m->flags);
    else
      k_elem_tri6<<<g, 64, 0, m->stream>>>(kind, m->nt, m->p, m->t, m->geo, f, vel, 0, acc, m->recpos, rec, m->flags);
    FG_CUDA_TRY(cudaGetLastError());
  };
  elem(ASM_MASS, d_rhocp, nullptr, 0);
  launch_row_any<double, double>(m, rec, nullptr, 0, m->mval, nullptr, nullptr, nullptr, nullptr, nullptr, 0.0, 0);
  elem(ASM_STIFF, d_kdt, nullptr, 1);
  elem(ASM_CONV, d_fdt, d_vel, 1);
  FG_LAUNCHED(3);
  launch_row_any<double, double>(m, rec, nullptr, 0, m->val64, nullptr, nullptr, m->dinv64, nullptr, nullptr, 0.0, 0);
}

// src/FEM3D.jl:300-322 quadraticBoundaryMassMatrix: face-local matrix (1/180) c_ij
// with c = 6 on the vertex diagonal, -1 between vertices, -4 between a vertex and
// the midpoint of the opposite edge, 0 between a vertex and an adjacent midpoint,
// 32 on the midpoint diagonal and 16 between midpoints; face nodes ordered
// (v1, v2, v3, m12, m23, m31); entry AE[s] Mk[i,j] F[s].
__device__ __forceinline__ double face_mass_coef(int i, int j) {
  if (i < 3 && j < 3) return i == j ? 6.0 : -1.0;
  if (i >= 3 && j >= 3) return i == j ? 32.0 : 16.0;
  const int v = i < 3 ? i : j, e = (i < 3 ? j : i) - 3;
  return ((e + 2) % 3 == v) ? -4.0 : 0.0;
}

// src/FEM2D.jl:394-419 quadraticMassMatrix1D: (1/30) [4 2 -1; 2 16 2; -1 2 4] by the
// position of the node in the face's three surfaceT rows, entry AE[s] Mk[i,j] h[s].
__device__ __forceinline__ double line_mass_coef(int i, int j) {
  if (i == 1 && j == 1) return 16.0;
  if (i == j) return 4.0;
  if (i == 1 || j == 1) return 2.0;
  return -1.0;
}

// One thread per listed row: adds its faces' entries, in face order, into the row
// (SELL values, then the Jacobi inverse from the row's diagonal slot; or CSR values).
__global__ void k_face_mass(int64_t nrows, const int *__restrict__ rows, const int *__restrict__ fptr,
                            const int *__restrict__ flist, const int *__restrict__ faces, int fw,
                            const double *__restrict__ AE, const double *__restrict__ F, double scale,
                            const int *__restrict__ sl_ptr, const int *__restrict__ sl_col,
                            const int16_t *__restrict__ sl_dcol, const int *__restrict__ rowlen,
                            const uint8_t *__restrict__ diagk, double *__restrict__ val, double *__restrict__ dinv,
                            const int *__restrict__ rowptr, const int *__restrict__ colidx, double *__restrict__ csr,
                            int *flags) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nrows) return;
  const int r = rows[idx];
  const int s = r >> 5, lane = r & 31;
  for (int e = fptr[idx]; e < fptr[idx + 1]; ++e) {
    const int face = flist[e] >> 3, li = flist[e] & 7;
    for (int j = 0; j < fw; ++j) {
      const double c = fw == 6 ? face_mass_coef(li, j) : line_mass_coef(li, j);
      if (c == 0.0) continue;
      const double mk = fw == 6 ? (1.0 / 180.0) * c : (1.0 / 30.0) * c;
      const double v = scale * (AE[face] * mk * F[face]);
      const int col = faces[fw * (int64_t)face + j];
      int64_t pos = -1;
      if (csr) {
        for (int q = rowptr[r]; q < rowptr[r + 1]; ++q)
          if (colidx[q] == col) { pos = q; break; }
      } else {
        for (int q = 0; q < rowlen[r]; ++q) {
          const int64_t sp = sell_pos(sl_ptr[s], lane, q);
          const int cq = sl_col ? sl_col[sp] : r + (int)sl_dcol[sp];
          if (cq == col) { pos = sp; break; }
        }
      }
      if (pos < 0) { atomicOr(flags, FLAG_BAD_FACE); continue; }
      if (csr) csr[pos] += v; else val[pos] += v;
    }
  }
  if (!csr) dinv[r] = 1.0 / val[sell_pos(sl_ptr[s], lane, diagk[r])];
}

void fg_face_mass(fg_mesh *m, bool sell, const int *d_rows, int64_t nrows, const int *d_fptr, const int *d_flist,
                  const int *d_faces, const double *d_AE, const double *d_F, double scale) {
  const int fw = m->npe == 10 ? 6 : 3;
  if (nrows == 0) return;
  FG_REQUIRE(!sell || m->val64, FG_BAD_ARG, "boundary mass: no FP64 operator assembled");
  if (!sell && !m->csrval) m->csrval = dev_alloc<double>(m, (size_t)m->nnz);
  k_face_mass<<<grid_for(nrows, 128), 128, 0, m->stream>>>(
      nrows, d_rows, d_fptr, d_flist, d_faces, fw, d_AE, d_F, scale, m->sl_ptr, m->use_dcol ? nullptr : m->sl_col,
      m->sl_dcol, m->rowlen, m->diagk, m->val64, m->dinv64, m->rowptr, m->colidx, sell ? nullptr : m->csrval,
      m->flags);
  FG_CUDA_TRY(cudaGetLastError());
  FG_LAUNCHED(1);
}

void fg_newton_assemble(fg_mesh *m, const double *d_u, double Ms, double Hk, bool mixed, double *d_F,
                        bool want_jacobian, bool tangent) {
  const int tg = tangent ? 1 : 0;
  FG_REQUIRE(m->npe == 4, FG_UNSUPPORTED, "Newton magnetostatics needs P1 tetrahedra");
  if (want_jacobian) { m->op_tag = 0; ++m->op_version; }
  fg_ensure_records(m);
  ensure_operator(m, !mixed, mixed);
  unsigned g = grid_for(m->nt, 128);
  if (!want_jacobian) {
    // element state + residual only: the row pass sums the vector records
    k_elem_newton<double><<<g, 128, 0, m->stream>>>(m->nt, m->geo, m->t, d_u, m->nl, m->mu_lin, Ms, Hk, m->recpos,
                                                    nullptr, m->rec_r, m->mu, m->dmu, tg, m->flags);
    FG_CUDA_TRY(cudaGetLastError());
    FG_LAUNCHED(1);
    launch_row<4, double, double>(m, nullptr, m->rec_r, 0, nullptr, nullptr, nullptr, nullptr, nullptr, d_F, -1.0, 1);
    return;
  }
  if (mixed) {
    float *rec = static_cast<float *>(m->rec);
    k_elem_newton<float><<<g, 128, 0, m->stream>>>(m->nt, m->geo, m->t, d_u, m->nl, m->mu_lin, Ms, Hk, m->recpos, rec,
                                                   m->rec_r, m->mu, m->dmu, tg, m->flags);
    FG_CUDA_TRY(cudaGetLastError());
    FG_LAUNCHED(1);
    launch_row<4, float, float>(m, rec, m->rec_r, 1, nullptr, m->val32, nullptr, nullptr, m->dinv32, d_F, -1.0, 1);
  } else {
    double *rec = static_cast<double *>(m->rec);
    k_elem_newton<double><<<g, 128, 0, m->stream>>>(m->nt, m->geo, m->t, d_u, m->nl, m->mu_lin, Ms, Hk, m->recpos,
                                                    rec, m->rec_r, m->mu, m->dmu, tg, m->flags);
    FG_CUDA_TRY(cudaGetLastError());
    FG_LAUNCHED(1);
    launch_row<4, double, double>(m, rec, m->rec_r, 1, m->val64, nullptr, nullptr, m->dinv64, nullptr, d_F, -1.0, 1);
  }
}

__global__ void k_linear_coef(int64_t nt, const double *__restrict__ mu_lin, const uint8_t *__restrict__ nl,
                              double *__restrict__ coef, double *__restrict__ mu, double *__restrict__ dmu) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nt) return;
  coef[k] = nl[k] ? 0.0 : mu_lin[k];
  mu[k] = mu_lin[k];
  dmu[k] = 0.0;
}

void fg_set_nl_host(fg_mesh *m, const uint8_t *nl) {
  const size_t nt = (size_t)m->nt;
  if (m->nl_host.size() == nt && std::memcmp(m->nl_host.data(), nl, nt) == 0) return;
  m->nl_host.assign(nl, nl + nt);
  m->nl_list_current = false;
}

// The nonlinear element list of a mask and, when it differs from the list the maps
// were built for, the slot and row maps of the split residual / Jacobian.
// Indices 0..n-1 ordered by key (non-negative), equal keys in index order: an LSD
// radix sort on 11-bit digits (a stable comparison sort of the ~16 entries per
// nonlinear element took milliseconds on the host with the device idle).
static std::vector<int> order_by_key(const std::vector<int> &key) {
  const size_t n = key.size();
  std::vector<int> ord(n), tmp(n);
  for (size_t q = 0; q < n; ++q) ord[q] = (int)q;
  int kmax = 0;
  for (int k : key) kmax = std::max(kmax, k);
  std::vector<size_t> count(2049);
  for (int shift = 0; shift < 31 && (kmax >> shift) > 0; shift += 11) {
    std::fill(count.begin(), count.end(), 0);
    for (size_t q = 0; q < n; ++q) ++count[1 + ((key[ord[q]] >> shift) & 2047)];
    for (int d = 0; d < 2048; ++d) count[d + 1] += count[d];
    for (size_t q = 0; q < n; ++q) tmp[count[(key[ord[q]] >> shift) & 2047]++] = ord[q];
    ord.swap(tmp);
  }
  return ord;
}

static void nl_maps(fg_mesh *m, const uint8_t *nl_host) {
  const int64_t nt = m->nt;
  // eight mask bytes per test: a sparse mask (a few nonlinear parts in a large
  // mesh) is scanned at memory speed
  std::vector<int> list;
  int64_t k = 0;
  for (; k + 8 <= nt; k += 8) {
    uint64_t word;
    std::memcpy(&word, nl_host + k, sizeof(word));
    if (!word) continue;
    for (int b = 0; b < 8; ++b)
      if (nl_host[k + b]) list.push_back((int)(k + b));
  }
  for (; k < nt; ++k)
    if (nl_host[k]) list.push_back((int)k);
  if (!m->nl_maps_valid || list != m->nl_list_host) {
    const int n = (int)list.size();
    if (n > m->nl_cap) {
      const int cap = std::max(n, 64);
      m->nl_elems = dev_alloc<int>(m, (size_t)cap);
      m->nl_re = dev_alloc<double>(m, 4 * (size_t)cap);
      m->nl_ke = dev_alloc<double>(m, 16 * (size_t)cap);
      m->nl_slot_pos = dev_alloc<int>(m, 16 * (size_t)cap);
      m->nl_slot_ptr = dev_alloc<int>(m, 16 * (size_t)cap + 1);
      m->nl_slot_src = dev_alloc<int>(m, 16 * (size_t)cap);
      m->nl_slot_code = dev_alloc<int>(m, 16 * (size_t)cap);
      m->nl_rows = dev_alloc<int>(m, 4 * (size_t)cap);
      m->nl_row_ptr = dev_alloc<int>(m, 4 * (size_t)cap + 1);
      m->nl_row_src = dev_alloc<int>(m, 4 * (size_t)cap);
      m->nl_cap = cap;
    }
    m->n_nl = n;
    m->n_nl_slots = m->n_nl_rows = 0;
    if (n > 0) {
      FG_CUDA_TRY(cudaMemcpyAsync(m->nl_elems, list.data(), sizeof(int) * n, cudaMemcpyHostToDevice, m->stream));
      // positions and rows into the (not yet used) CSR buffers, then grouped on the host
      k_nl_map<<<grid_for(n, 128), 128, 0, m->stream>>>(n, m->nl_elems, nt, m->t, m->recpos, m->in_slot, m->sl_ptr,
                                                         m->nl_slot_src, m->nl_row_src);
      FG_CUDA_TRY(cudaGetLastError());
      FG_LAUNCHED(1);
      std::vector<int> pos(16 * (size_t)n), rows(4 * (size_t)n);
      FG_CUDA_TRY(cudaMemcpyAsync(pos.data(), m->nl_slot_src, sizeof(int) * pos.size(), cudaMemcpyDeviceToHost,
                                  m->stream));
      FG_CUDA_TRY(cudaMemcpyAsync(rows.data(), m->nl_row_src, sizeof(int) * rows.size(), cudaMemcpyDeviceToHost,
                                  m->stream));
      fg_sync(m);
      // slots: sources (e, a, b) grouped by position, in source order within a position
      const std::vector<int> ord = order_by_key(pos);
      std::vector<int> spos, sptr, scode, ssrc(ord.size());
      for (size_t q = 0; q < ord.size(); ++q) {
        const int src = ord[q];
        ssrc[q] = src;
        if (q == 0 || pos[src] != pos[ord[q - 1]]) {
          const int e = src / 16, a = (src / 4) % 4, b = src % 4;
          const int row = rows[4 * e + a];
          spos.push_back(pos[src]);
          sptr.push_back((int)q);
          scode.push_back(a == b ? ~row : row);
        }
      }
      sptr.push_back((int)ord.size());
      // rows: sources (e, a) grouped by row
      const std::vector<int> rord = order_by_key(rows);
      std::vector<int> rlist, rptr;
      for (size_t q = 0; q < rord.size(); ++q)
        if (q == 0 || rows[rord[q]] != rows[rord[q - 1]]) {
          rlist.push_back(rows[rord[q]]);
          rptr.push_back((int)q);
        }
      rptr.push_back((int)rord.size());
      m->n_nl_slots = (int)spos.size();
      m->n_nl_rows = (int)rlist.size();
      auto up = [&](int *dst, const std::vector<int> &v) {
        FG_CUDA_TRY(cudaMemcpyAsync(dst, v.data(), sizeof(int) * v.size(), cudaMemcpyHostToDevice, m->stream));
      };
      up(m->nl_slot_pos, spos);
      up(m->nl_slot_ptr, sptr);
      up(m->nl_slot_code, scode);
      up(m->nl_slot_src, ssrc);
      up(m->nl_rows, rlist);
      up(m->nl_row_ptr, rptr);
      up(m->nl_row_src, rord);
      fg_sync(m);
    }
    // the rows the nonlinear elements touch, for the batched line search
    if (!m->nl_rowmask) m->nl_rowmask = dev_alloc<uint8_t>(m, (size_t)m->nv);
    FG_CUDA_TRY(cudaMemsetAsync(m->nl_rowmask, 0, (size_t)m->nv, m->stream));
    if (m->n_nl_rows > 0) {
      k_mark_rows<<<grid_for(m->n_nl_rows, 256), 256, 0, m->stream>>>(m->n_nl_rows, m->nl_rows, m->nl_rowmask);
      FG_CUDA_TRY(cudaGetLastError());
      FG_LAUNCHED(1);
    }
    m->nl_list_host = list;
    m->nl_maps_valid = true;
  }
}

void fg_newton_trial_batch(fg_mesh *m, const double *d_u, const double *d_du, const double *d_y, const double *d_z,
                           const LsCand &cand, double Ms, double Hk, double *d_out) {
  FG_REQUIRE(m->nl_maps_valid && m->nl_rowmask, FG_BAD_ARG, "Newton split: no nonlinear maps");
  FG_REQUIRE(cand.n >= 1 && cand.n <= FG_LS_BATCH, FG_BAD_ARG, "batched line search: bad candidate count");
  const int n = m->n_nl;
  if (n > 0) {
    if (n > m->nl_cand_cap) {
      m->nl_re_cand = dev_alloc<double>(m, (size_t)FG_LS_BATCH * 4 * (size_t)n);
      m->nl_cand_cap = n;
    }
    k_elem_newton_nl_cand<<<grid_for((int64_t)cand.n * n, 128), 128, 0, m->stream>>>(
        cand, n, m->nl_elems, m->nt, m->geo, m->t, d_u, d_du, Ms, Hk, m->nl_re_cand);
    FG_LAUNCHED(1);
  }
  // a block per candidate also when no row is touched (the sums are then 0)
  k_nl_rows_cand_norm<<<cand.n, 1024, 0, m->stream>>>(cand, m->n_nl_rows, n, m->nl_rows, m->nl_row_ptr, m->nl_row_src,
                                                    m->nl_re_cand, d_y, d_z, m->has_fixed ? m->fixed : nullptr, d_out);
  FG_CUDA_TRY(cudaGetLastError());
  FG_LAUNCHED(1);
}

void fg_nl_setup(fg_mesh *m, const uint8_t *nl_host, bool mixed) {
  FG_REQUIRE(m->npe == 4, FG_UNSUPPORTED, "Newton magnetostatics needs P1 tetrahedra");
  // no incidence records: the linear operator is assembled in one pass and the
  // nonlinear elements keep their own blocks (nl_re, nl_ke)
  const int64_t nt = m->nt;
  // the linear elements' operator (nonlinear elements contribute 0), Dirichlet rows
  // applied; element state starts at the linear values.  Enqueued before the host
  // builds the nonlinear element list below, so that the device assembles while the
  // host scans the mask.
  double *coef = m->objbuf ? m->objbuf : (m->objbuf = dev_alloc<double>(m, 2 * (size_t)nt));
  k_linear_coef<<<grid_for(nt, 256), 256, 0, m->stream>>>(nt, m->mu_lin, m->nl, coef, m->mu, m->dmu);
  FG_LAUNCHED(1);
  fg_assemble_operator(m, ASM_STIFF, coef, nullptr, nullptr, 0.0, 0.0, 0, OUT_SELL, true, mixed, true);
  if (!m->vlin64) m->vlin64 = dev_alloc<double>(m, (size_t)m->nsell);
  if (!m->dlin64) m->dlin64 = dev_alloc<double>(m, (size_t)m->nvp);
  FG_CUDA_TRY(cudaMemcpyAsync(m->vlin64, m->val64, sizeof(double) * (size_t)m->nsell, cudaMemcpyDeviceToDevice,
                              m->stream));
  FG_CUDA_TRY(cudaMemcpyAsync(m->dlin64, m->dinv64, sizeof(double) * (size_t)m->nvp, cudaMemcpyDeviceToDevice,
                              m->stream));
  if (mixed) {
    if (!m->vlin32) m->vlin32 = dev_alloc<float>(m, (size_t)m->nsell);
    if (!m->dlin32) m->dlin32 = dev_alloc<float>(m, (size_t)m->nvp);
    FG_CUDA_TRY(cudaMemcpyAsync(m->vlin32, m->val32, sizeof(float) * (size_t)m->nsell, cudaMemcpyDeviceToDevice,
                                m->stream));
    FG_CUDA_TRY(cudaMemcpyAsync(m->dlin32, m->dinv32, sizeof(float) * (size_t)m->nvp, cudaMemcpyDeviceToDevice,
                                m->stream));
  }
  // the mask of the handle's inputs, unchanged since its list was built, needs no
  // scan (a scan of millions of elements takes a millisecond on the host)
  const bool own = (nl_host == m->nl_host.data());
  if (!(own && m->nl_list_current && m->nl_maps_valid)) {
    nl_maps(m, nl_host);
    if (own) m->nl_list_current = true;
  }
}

void fg_newton_assemble_split(fg_mesh *m, const double *d_u, double Ms, double Hk, bool mixed, double *d_F,
                              bool want_jacobian, bool tangent, const double *lin_in, double *lin_out) {
  FG_REQUIRE(m->vlin64 != nullptr && m->nl_maps_valid, FG_BAD_ARG, "Newton split: no linear operator");
  const int n = m->n_nl;
  const uint8_t *fx = m->has_fixed ? m->fixed : nullptr;
  // F = -(K_lin u + the nonlinear elements' K_e(mu(u)) u_e), Dirichlet rows 0; with
  // d_F null only the Jacobian (the residual at u is known already)
  if (!d_F) {
    FG_REQUIRE(want_jacobian, FG_BAD_ARG, "Newton split: nothing to assemble");
  } else if (lin_in) {
    if (lin_in != d_F)
      FG_CUDA_TRY(cudaMemcpyAsync(d_F, lin_in, sizeof(double) * (size_t)m->nv, cudaMemcpyDeviceToDevice, m->stream));
  } else if (lin_out) {
    fg_spmv64_vals(m, m->vlin64, d_u, lin_out);
    FG_CUDA_TRY(cudaMemcpyAsync(d_F, lin_out, sizeof(double) * (size_t)m->nv, cudaMemcpyDeviceToDevice, m->stream));
  } else {
    fg_spmv64_vals(m, m->vlin64, d_u, d_F);
  }
  if (n > 0) {
    k_elem_newton_nl<<<grid_for(n, 128), 128, 0, m->stream>>>(n, m->nl_elems, m->nt, m->geo, m->t, d_u, Ms, Hk,
                                                              m->mu, m->dmu, m->nl_re,
                                                              want_jacobian ? m->nl_ke : nullptr, tangent ? 1 : 0,
                                                              m->flags);
    FG_LAUNCHED(1);
    if (d_F) {
      k_nl_rows<<<grid_for(m->n_nl_rows, 128), 128, 0, m->stream>>>(m->n_nl_rows, m->nl_rows, m->nl_row_ptr,
                                                                    m->nl_row_src, m->nl_re, fx, d_F);
      FG_LAUNCHED(1);
    }
  }
  // F <- -F, with |F|^2 in scal[FG_SLOT_FNORM2] (the Dirichlet rows are 0)
  if (d_F) fg_negate_norm2_enqueue(m, d_F);
  if (!want_jacobian) return;
  m->op_tag = 0;
  ++m->op_version;
  const unsigned gs = grid_for(std::max(m->n_nl_slots, 1), 128);
  if (mixed) {
    FG_CUDA_TRY(cudaMemcpyAsync(m->val32, m->vlin32, sizeof(float) * (size_t)m->nsell, cudaMemcpyDeviceToDevice,
                                m->stream));
    FG_CUDA_TRY(cudaMemcpyAsync(m->dinv32, m->dlin32, sizeof(float) * (size_t)m->nvp, cudaMemcpyDeviceToDevice,
                                m->stream));
    if (n > 0)
      k_nl_slots<float><<<gs, 128, 0, m->stream>>>(m->n_nl_slots, m->nl_slot_pos, m->nl_slot_ptr, m->nl_slot_src,
                                                   m->nl_slot_code, m->vlin64, m->nl_ke, fx, m->val32, m->dinv32);
  } else {
    FG_CUDA_TRY(cudaMemcpyAsync(m->val64, m->vlin64, sizeof(double) * (size_t)m->nsell, cudaMemcpyDeviceToDevice,
                                m->stream));
    FG_CUDA_TRY(cudaMemcpyAsync(m->dinv64, m->dlin64, sizeof(double) * (size_t)m->nvp, cudaMemcpyDeviceToDevice,
                                m->stream));
    if (n > 0)
      k_nl_slots<double><<<gs, 128, 0, m->stream>>>(m->n_nl_slots, m->nl_slot_pos, m->nl_slot_ptr, m->nl_slot_src,
                                                    m->nl_slot_code, m->vlin64, m->nl_ke, fx, m->val64, m->dinv64);
  }
  FG_CUDA_TRY(cudaGetLastError());
  if (n > 0) FG_LAUNCHED(1);
}

void fg_apply_operator_vec(fg_mesh *m, int kind, const double *d_coef, double c_mass, double c_stiff,
                           const double *d_x, double *d_y, bool zero_fixed) {
  FG_REQUIRE(m->npe == 4, FG_UNSUPPORTED, "matrix-free apply needs P1 tetrahedra");
  fg_ensure_records(m);
  k_elem_apply_tet4<<<grid_for(m->nt, 128), 128, 0, m->stream>>>(kind, m->nt, m->geo, m->t, d_coef, c_mass, c_stiff,
                                                                  d_x, m->recpos, m->rec_r);
  FG_CUDA_TRY(cudaGetLastError());
  FG_LAUNCHED(1);
  launch_row<4, double, double>(m, nullptr, m->rec_r, 0, nullptr, nullptr, nullptr, nullptr, nullptr, d_y, 1.0,
                                zero_fixed ? 1 : 0);
}

void fg_energy_dev(fg_mesh *m, const double *d_u, double Ms, double Hk) {
  k_energy_tet4<<<grid_for(m->nt, 256), 256, 0, m->stream>>>(m->nt, m->geo, m->t, d_u, m->nl, m->mu_lin, Ms, Hk,
                                                              m->wdens);
  FG_CUDA_TRY(cudaGetLastError());
  FG_LAUNCHED(1);
}

void fg_hfield_dev(fg_mesh *m, const double *d_u, double *d_H) {
  FG_REQUIRE(m->npe == 4, FG_UNSUPPORTED, "H field needs P1 tetrahedra");
  k_hfield_tet4<<<grid_for(m->nt, 256), 256, 0, m->stream>>>(m->nt, m->geo, m->t, d_u, d_H);
  FG_CUDA_TRY(cudaGetLastError());
  FG_LAUNCHED(1);
}

void fg_demag_rhs_dev(fg_mesh *m, const uint8_t *d_inside, const double *d_M, double *d_b) {
  FG_REQUIRE(m->npe == 4, FG_UNSUPPORTED, "demagnetising field: P1 tetrahedra only");
  fg_ensure_records(m);
  k_demag_rhs_tet4<<<grid_for(m->nt, 256), 256, 0, m->stream>>>(m->nt, m->geo, m->t, d_inside, d_M, m->recpos,
                                                                 m->rec_r);
  FG_CUDA_TRY(cudaGetLastError());
  FG_LAUNCHED(1);
  launch_row<4, double, double>(m, nullptr, m->rec_r, 0, nullptr, nullptr, nullptr, nullptr, nullptr, d_b, 1.0, 1);
}

// Nodal field: sum over the inside elements of VE H_k at each node over the node volume.
void fg_nodal_average_dev(fg_mesh *m, const uint8_t *d_inside, const double *d_H, double *d_work, double *d_Hn) {
  fg_ensure_records(m);
  const int64_t nv = m->nv;
  for (int c = 0; c < 4; ++c) {
    k_inside_weighted_tet4<<<grid_for(m->nt, 256), 256, 0, m->stream>>>(m->nt, m->geo, d_inside,
                                                                       c < 3 ? d_H : nullptr, c % 3, m->recpos,
                                                                       m->rec_r);
    FG_CUDA_TRY(cudaGetLastError());
    FG_LAUNCHED(1);
    launch_row<4, double, double>(m, nullptr, m->rec_r, 0, nullptr, nullptr, nullptr, nullptr, nullptr,
                                  d_work + c * nv, 1.0, 0);
  }
  k_nodal_average<<<grid_for(nv, 256), 256, 0, m->stream>>>(nv, d_work, d_work + nv, d_work + 2 * nv,
                                                            d_work + 3 * nv, d_Hn);
  FG_CUDA_TRY(cudaGetLastError());
  FG_LAUNCHED(1);
}

void fg_vector_gather(fg_mesh *m, double *d_out) {
  FG_REQUIRE(m->npe == 4, FG_UNSUPPORTED, "vector gather: P1 tetrahedra only");
  launch_row<4, double, double>(m, nullptr, m->rec_r, 0, nullptr, nullptr, nullptr, nullptr, nullptr, d_out, 1.0, 0);
}

void fg_objective_parts_dev(fg_mesh *m, const double *d_u, const uint8_t *d_target, double *d_a, double *d_v) {
  FG_REQUIRE(m->npe == 4, FG_UNSUPPORTED, "objective needs P1 tetrahedra");
  k_objective_tet4<<<grid_for(m->nt, 256), 256, 0, m->stream>>>(m->nt, m->geo, m->t, d_u, d_target, d_a, d_v);
  FG_CUDA_TRY(cudaGetLastError());
  FG_LAUNCHED(1);
}

void fg_objective_rhs_dev(fg_mesh *m, const uint8_t *d_target, double vol, double *d_g) {
  FG_REQUIRE(m->npe == 4, FG_UNSUPPORTED, "objective needs P1 tetrahedra");
  fg_ensure_records(m);
  k_objective_rhs_tet4<<<grid_for(m->nt, 256), 256, 0, m->stream>>>(m->nt, m->geo, d_target, 1.0 / vol, m->recpos,
                                                                     m->rec_r);
  FG_CUDA_TRY(cudaGetLastError());
  FG_LAUNCHED(1);
  launch_row<4, double, double>(m, nullptr, m->rec_r, 0, nullptr, nullptr, nullptr, nullptr, nullptr, d_g, 1.0, 1);
}

void fg_adjoint_grad_dev(fg_mesh *m, const double *d_lam, const double *d_u, double scale, double *d_grad) {
  FG_REQUIRE(m->npe == 4, FG_UNSUPPORTED, "adjoint gradient needs P1 tetrahedra");
  k_adjoint_grad_tet4<<<grid_for(m->nt, 256), 256, 0, m->stream>>>(m->nt, m->geo, m->t, d_lam, d_u, scale, d_grad);
  FG_CUDA_TRY(cudaGetLastError());
  FG_LAUNCHED(1);
}

// ------------------------------------------------------------------ C ABI
static double *upload_opt(fg_mesh *m, const double *h, size_t n, double *&tmp) {
  if (!h) return nullptr;
  FG_CUDA_TRY(cudaMalloc(&tmp, sizeof(double) * n));
  FG_CUDA_TRY(cudaMemcpyAsync(tmp, h, sizeof(double) * n, cudaMemcpyHostToDevice, m->stream));
  return tmp;
}

static fg_status export_csr(fg_mesh *m, double *nzval, const char *where) {
  FG_CUDA_TRY(cudaMemcpyAsync(nzval, m->csrval, sizeof(double) * (size_t)m->nnz, cudaMemcpyDeviceToHost, m->stream));
  fg_sync(m);
  fg_check_flags(m, where);
  return FG_OK;
}

extern "C" fg_status fg_stiffness(fg_mesh *m, const double *f, double *nzval) {
  double *tf = nullptr;
  fg_status st = fg_guard([&]() -> fg_status {
    FG_REQUIRE(m && nzval, FG_BAD_ARG, "fg_stiffness: null pointer");
    double *df = upload_opt(m, f, (size_t)m->nt, tf);
    fg_assemble_operator(m, ASM_STIFF, df, nullptr, nullptr, 0.0, 0.0, 0, OUT_CSR, false, false, false);
    return export_csr(m, nzval, "fg_stiffness");
  });
  if (tf) cudaFree(tf);
  return st;
}

extern "C" fg_status fg_mass(fg_mesh *m, const double *f, int32_t full_phi, double *nzval) {
  double *tf = nullptr;
  fg_status st = fg_guard([&]() -> fg_status {
    FG_REQUIRE(m && nzval, FG_BAD_ARG, "fg_mass: null pointer");
    double *df = upload_opt(m, f, (size_t)m->nt, tf);
    fg_assemble_operator(m, ASM_MASS, df, nullptr, nullptr, 0.0, 0.0, full_phi, OUT_CSR, false, false, false);
    return export_csr(m, nzval, "fg_mass");
  });
  if (tf) cudaFree(tf);
  return st;
}

extern "C" fg_status fg_convection(fg_mesh *m, const double *vel, const double *f, int32_t full_phi,
                                   double *nzval) {
  double *tf = nullptr, *tv = nullptr;
  fg_status st = fg_guard([&]() -> fg_status {
    FG_REQUIRE(m && vel && nzval, FG_BAD_ARG, "fg_convection: null pointer");
    FG_REQUIRE(!m->edge && (m->npe == 10 || m->npe == 6), FG_UNSUPPORTED,
               "fg_convection: P2 tetrahedra (src/FEM3D.jl:563-648) or P2 triangles (src/FEM2D.jl:231-319)");
    double *df = upload_opt(m, f, (size_t)m->nt, tf);
    double *dv = upload_opt(m, vel, 3 * (size_t)m->nv, tv);
    fg_assemble_operator(m, ASM_CONV, df, dv, nullptr, 0.0, 0.0, full_phi, OUT_CSR, false, false, false);
    return export_csr(m, nzval, "fg_convection");
  });
  if (tf) cudaFree(tf);
  if (tv) cudaFree(tv);
  return st;
}

extern "C" fg_status fg_tangent(fg_mesh *m, const double *H, const double *dmu, double *nzval) {
  double *tH = nullptr, *td = nullptr;
  fg_status st = fg_guard([&]() -> fg_status {
    FG_REQUIRE(m && H && dmu && nzval, FG_BAD_ARG, "fg_tangent: null pointer");
    FG_REQUIRE(m->npe == 4, FG_UNSUPPORTED, "fg_tangent: P1 tetrahedra only (src/FEM3D.jl:79-119)");
    double *dH = upload_opt(m, H, 3 * (size_t)m->nt, tH);
    double *dd = upload_opt(m, dmu, (size_t)m->nt, td);
    fg_assemble_operator(m, ASM_TANGENT, nullptr, dH, dd, 0.0, 0.0, 0, OUT_CSR, false, false, false);
    return export_csr(m, nzval, "fg_tangent");
  });
  if (tH) cudaFree(tH);
  if (td) cudaFree(td);
  return st;
}

__global__ void k_local_tet4(int64_t nt, const double *__restrict__ geo, const double *__restrict__ f,
                             double *__restrict__ Ak) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nt) return;
  double g[4][3];
  for (int c = 0; c < 12; ++c) g[c / 3][c % 3] = geo[(int64_t)c * nt + k];
  double s = (f ? f[k] : 1.0) * geo[12 * nt + k];
  for (int b = 0; b < 4; ++b)
    for (int a = 0; a < 4; ++a) Ak[16 * k + 4 * b + a] = s * (g[a][0] * g[b][0] + g[a][1] * g[b][1] + g[a][2] * g[b][2]);
}

extern "C" fg_status fg_local_stiffness(fg_mesh *m, const double *f, double *Ak) {
  double *tf = nullptr, *dA = nullptr;
  fg_status st = fg_guard([&]() -> fg_status {
    FG_REQUIRE(m && Ak, FG_BAD_ARG, "fg_local_stiffness: null pointer");
    FG_REQUIRE(m->npe == 4, FG_UNSUPPORTED, "fg_local_stiffness: P1 tetrahedra only");
    double *df = upload_opt(m, f, (size_t)m->nt, tf);
    FG_CUDA_TRY(cudaMalloc(&dA, sizeof(double) * 16 * (size_t)m->nt));
    k_local_tet4<<<grid_for(m->nt, 256), 256, 0, m->stream>>>(m->nt, m->geo, df, dA);
    FG_CUDA_TRY(cudaGetLastError());
    FG_CUDA_TRY(cudaMemcpyAsync(Ak, dA, sizeof(double) * 16 * (size_t)m->nt, cudaMemcpyDeviceToHost, m->stream));
    fg_sync(m);
    return FG_OK;
  });
  if (tf) cudaFree(tf);
  if (dA) cudaFree(dA);
  return st;
}
