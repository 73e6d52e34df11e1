// Mesh upload, structural pattern, element-to-slot map and P1 geometry.
//
// The reference rebuilds its sparse structure on every assembly: 16 (36, 100)
// COO->CSC passes in src/FEM3D.jl:47-53 and one sparse(I,J,V) per Newton step in
// Magnetostatics/NewtonRaphson.jl:115-161.  Here the pattern is built once per mesh
// on the GPU and every later assembly writes values straight into it:
//
//   * incidence lists node -> (element, local node), sorted by (element, local);
//   * the structural CSR pattern (all element node pairs, rows sorted, the pattern
//     sparse(I,J,V) keeps), plus the same rows in SELL-32 layout (slices of 32 rows
//     stored column-major, so a warp reads 32 consecutive entries);
//   * for every incidence, the position of each element node inside the row
//     (one byte per node) and, per (element, local node), the incidence position
//     the element kernels write their local row to;
//   * per element the gradients of the P1 (barycentric) basis and the volume,
//     computed once in FP64 from the inverse Jacobian.  The reference solves a
//     4x4 (3x3) Vandermonde system per node instead (src/FEM3D.jl:5-17,
//     src/FEM2D.jl:5-25); the coefficients are the same functions.
#include <algorithm>
#include <climits>
#include <cstring>
#include <mutex>

#include "fg_common.cuh"

#include <atomic>
static std::atomic<long long> g_launches{0};
void fg_count_launch(long long n) { g_launches += n; }
extern "C" int64_t fg_kernel_launches(void) { return g_launches.load(); }

static thread_local std::string g_err;
void fg_set_error(const std::string &msg) { g_err = msg; }

extern "C" const char *fg_last_error(void) { return g_err.c_str(); }
extern "C" int32_t fg_version(void) { return 10; }

extern "C" fg_status fg_device_info(char *name, int32_t name_len, int32_t *sm_count) {
  return fg_guard([&]() -> fg_status {
    int dev = 0;
    FG_CUDA_TRY(cudaGetDevice(&dev));
    cudaDeviceProp prop;
    FG_CUDA_TRY(cudaGetDeviceProperties(&prop, dev));
    if (name && name_len > 0) {
      strncpy(name, prop.name, (size_t)name_len - 1);
      name[name_len - 1] = 0;
    }
    if (sm_count) *sm_count = prop.multiProcessorCount;
    return FG_OK;
  });
}

void fg_sync(fg_mesh *m) { FG_CUDA_TRY(cudaStreamSynchronize(m->stream)); }

void fg_check_flags(fg_mesh *m, const char *where) {
  int h = 0;
  FG_CUDA_TRY(cudaMemcpyAsync(&h, m->flags, sizeof(int), cudaMemcpyDeviceToHost, m->stream));
  fg_sync(m);
  fg_raise_flags(m, h, where);
}

void fg_raise_flags(fg_mesh *m, int h, const char *where) {
  if (!h) return;
  FG_CUDA_TRY(cudaMemsetAsync(m->flags, 0, sizeof(int), m->stream));
  std::string w(where);
  if (h & FLAG_BAD_INDEX) throw FgError{FG_BAD_MESH, w + ": node index out of range"};
  if (h & FLAG_DUP_NODE) throw FgError{FG_BAD_MESH, w + ": an element repeats a node"};
  if (h & FLAG_DEGENERATE) throw FgError{FG_BAD_MESH, w + ": degenerate (zero-volume) element"};
  if (h & FLAG_ROW_OVERFLOW) throw FgError{FG_BAD_MESH, w + ": a matrix row exceeds 255 entries"};
  if (h & FLAG_NAN) throw FgError{FG_NAN, w + ": NaN/Inf in permeability or residual"};
  if (h & FLAG_BAD_FACE) throw FgError{FG_BAD_ARG, w + ": a boundary face is not a face of an element"};
  throw FgError{FG_BAD_MESH, w + ": device error flag"};
}

// ------------------------------------------------------------------ kernels
// t (npe x nt, column-major, index_base) -> SoA 0-based, with range checks.
__global__ void k_convert_t(const int32_t *__restrict__ traw, int *__restrict__ t, int64_t nt, int npe, int64_t nv,
                            int base, int *flags) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nt) return;
  int nodes[10];
  int bad = 0;
  for (int a = 0; a < npe; ++a) {
    int v = traw[k * npe + a] - base;
    if (v < 0 || v >= nv) { bad |= FLAG_BAD_INDEX; v = 0; }
    nodes[a] = v;
    t[(int64_t)a * nt + k] = v;
  }
  for (int a = 0; a < npe; ++a)
    for (int b = a + 1; b < npe; ++b)
      if (nodes[a] == nodes[b]) bad |= FLAG_DUP_NODE;
  if (bad) atomicOr(flags, bad);
}

__global__ void k_count_deg(const int *__restrict__ t, int64_t nt, int npe, int *__restrict__ deg) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nt) return;
  for (int a = 0; a < npe; ++a) atomicAdd(&deg[t[(int64_t)a * nt + k]], 1);
}

__global__ void k_fill_inc(const int *__restrict__ t, int64_t nt, int npe, const int *__restrict__ iptr,
                           int *__restrict__ cursor, int *__restrict__ inc) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nt) return;
  for (int a = 0; a < npe; ++a) {
    int v = t[(int64_t)a * nt + k];
    int pos = iptr[v] + atomicAdd(&cursor[v], 1);
    inc[pos] = (int)(k * npe + a);
  }
}

// Sort each node's incidence list by (element, local) so that every later pass
// visits contributions in one fixed order (deterministic sums).
// Lists of up to 64 incidences are sorted in a thread-local array (one read and one
// write of the list in global memory instead of a dependent global round trip per
// shift); longer ones in place.
__global__ void k_sort_inc(const int *__restrict__ iptr, int *__restrict__ inc, int64_t nv) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  const int b = iptr[i], e = iptr[i + 1];
  constexpr int CAP = 64;
  if (e - b <= CAP) {
    int loc[CAP];
    const int n = e - b;
    for (int q = 0; q < n; ++q) loc[q] = inc[b + q];
    for (int q = 1; q < n; ++q) {
      const int key = loc[q];
      int r = q - 1;
      while (r >= 0 && loc[r] > key) { loc[r + 1] = loc[r]; --r; }
      loc[r + 1] = key;
    }
    for (int q = 0; q < n; ++q) inc[b + q] = loc[q];
    return;
  }
  for (int q = b + 1; q < e; ++q) {
    int key = inc[q];
    int r = q - 1;
    while (r >= b && inc[r] > key) { inc[r + 1] = inc[r]; --r; }
    inc[r + 1] = key;
  }
}

// Sorted unique neighbour set of node i (the nodes of its incident elements).
template <int CAP>
__device__ int gather_row(int64_t i, const int *__restrict__ iptr, const int *__restrict__ inc,
                          const int *__restrict__ t, int64_t nt, int npe, int *nb, int *flags) {
  int len = 0;
  for (int q = iptr[i]; q < iptr[i + 1]; ++q) {
    int key = inc[q];
    int64_t k = key / npe;
    for (int a = 0; a < npe; ++a) {
      int v = t[(int64_t)a * nt + k];
      // binary search for v in nb[0, len)
      int lo = 0, hi = len;
      while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (nb[mid] < v) lo = mid + 1; else hi = mid;
      }
      if (lo < len && nb[lo] == v) continue;
      if (len >= CAP) { atomicOr(flags, FLAG_ROW_OVERFLOW); return len; }
      for (int r = len; r > lo; --r) nb[r] = nb[r - 1];
      nb[lo] = v;
      ++len;
    }
  }
  return len;
}

template <int CAP>
__global__ void k_row_count(const int *__restrict__ iptr, const int *__restrict__ inc, const int *__restrict__ t,
                            int64_t nt, int npe, int64_t nv, int *__restrict__ rowlen, int *flags) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  int nb[CAP];
  rowlen[i] = gather_row<CAP>(i, iptr, inc, t, nt, npe, nb, flags);
}

template <int CAP>
__global__ void k_row_fill(const int *__restrict__ iptr, const int *__restrict__ inc, const int *__restrict__ t,
                           int64_t nt, int npe, int64_t nv, const int *__restrict__ rowptr,
                           const int *__restrict__ sl_ptr, const int *__restrict__ sl_len, int *__restrict__ colidx,
                           int *__restrict__ sl_col, int16_t *__restrict__ sl_dcol, uint8_t *__restrict__ diagk,
                           int *flags) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  int nb[CAP];
  int len = gather_row<CAP>(i, iptr, inc, t, nt, npe, nb, flags);
  int rb = rowptr[i];
  int s = (int)(i / FG_SLICE), lane = (int)(i % FG_SLICE);
  int64_t sb = sl_ptr[s];
  int slots = FG_GROUP * sl_len[s];
  int dk = 0;
  bool wide = false;
  for (int k = 0; k < slots; ++k) {
    int c = (k < len) ? nb[k] : (int)i;  // pads point at the row itself (value 0)
    if (k < len) colidx[rb + k] = c;
    int64_t pos = sell_pos(sb, lane, k);
    sl_col[pos] = c;
    int d = c - (int)i;
    if (d < -32768 || d > 32767) { wide = true; d = 0; }
    sl_dcol[pos] = (int16_t)d;
    if (c == (int)i && k < len) dk = k;
  }
  if (wide) atomicOr(flags + 1, 1);
  diagk[i] = (uint8_t)dk;
}

// Halo of a block of hrows rows: the sorted distinct columns of the block's entries
// (pads included: they point at their own row), written to halo_col[b*cap ...], and
// each entry's position in it (sl_lcol).  One CTA of 512 threads per block; the keys
// are sorted in shared memory with a bitonic network (P2 = power of two >= keys).
constexpr int FG_HALO_THREADS = 512;

__global__ void __launch_bounds__(FG_HALO_THREADS)
    k_build_halo(int64_t nv, int hrows, int slots, int P2, const int *__restrict__ sl_ptr,
                 const int *__restrict__ sl_len, const int *__restrict__ sl_col, int cap, int *__restrict__ halo_col,
                 int *__restrict__ halo_len, uint16_t *__restrict__ sl_lcol, int *flags) {
  extern __shared__ int shk[];
  int *key = shk;        // P2 sorted keys
  int *uniq = shk + P2;  // distinct keys
  __shared__ int wsum[FG_HALO_THREADS / 32];
  const int tid = threadIdx.x, nth = blockDim.x;
  const int64_t r0 = (int64_t)blockIdx.x * hrows;
  const int nkeys = hrows * slots;
  for (int e = tid; e < P2; e += nth) {
    int k = INT_MAX;
    if (e < nkeys) {
      const int64_t row = r0 + e / slots;
      const int q = e % slots;
      if (row < nv) {
        const int s = (int)(row / FG_SLICE), lane = (int)(row % FG_SLICE);
        if (q < FG_GROUP * sl_len[s]) k = sl_col[sell_pos(sl_ptr[s], lane, q)];
      }
    }
    key[e] = k;
  }
  __syncthreads();
  for (int size = 2; size <= P2; size <<= 1)
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int e = tid; e < P2; e += nth) {
        const int partner = e ^ stride;
        if (partner > e) {
          const bool up = ((e & size) == 0);
          const int a = key[e], b = key[partner];
          if ((a > b) == up) { key[e] = b; key[partner] = a; }
        }
      }
      __syncthreads();
    }
  // distinct keys: each thread owns a contiguous chunk, counts, then a block scan
  const int chunk = P2 / nth;  // P2 is a multiple of nth
  const int e0 = tid * chunk;
  int cnt = 0;
  for (int e = e0; e < e0 + chunk; ++e)
    if (key[e] != INT_MAX && (e == 0 || key[e] != key[e - 1])) ++cnt;
  int incl = cnt;
  for (int o = 1; o < 32; o <<= 1) {
    int v = __shfl_up_sync(0xffffffffu, incl, o);
    if ((tid & 31) >= o) incl += v;
  }
  if ((tid & 31) == 31) wsum[tid >> 5] = incl;
  __syncthreads();
  if (tid < 32) {
    int v = (tid < nth / 32) ? wsum[tid] : 0, w = v;
    for (int o = 1; o < 32; o <<= 1) {
      int u = __shfl_up_sync(0xffffffffu, w, o);
      if (tid >= o) w += u;
    }
    if (tid < nth / 32) wsum[tid] = w - v;  // exclusive warp offsets
  }
  __syncthreads();
  int pos = wsum[tid >> 5] + incl - cnt;
  for (int e = e0; e < e0 + chunk; ++e)
    if (key[e] != INT_MAX && (e == 0 || key[e] != key[e - 1])) {
      uniq[pos] = key[e];
      halo_col[(int64_t)blockIdx.x * cap + pos] = key[e];
      ++pos;
    }
  __shared__ int s_hl;
  if (tid == nth - 1) s_hl = pos;  // the last chunk ends at the total count
  __syncthreads();
  const int hlen = s_hl;
  if (tid == 0) {
    halo_len[blockIdx.x] = hlen;
    if (hlen > 65535) atomicOr(flags, FLAG_ROW_OVERFLOW);
  }
  // local index of every entry
  for (int e = tid; e < nkeys; e += nth) {
    const int64_t row = r0 + e / slots;
    const int q = e % slots;
    if (row >= nv) continue;
    const int s = (int)(row / FG_SLICE), lane = (int)(row % FG_SLICE);
    if (q >= FG_GROUP * sl_len[s]) continue;
    const int64_t p = sell_pos(sl_ptr[s], lane, q);
    const int c = sl_col[p];
    int lo = 0, hi = hlen;
    while (lo < hi) {
      int mid = (lo + hi) >> 1;
      if (uniq[mid] < c) lo = mid + 1; else hi = mid;
    }
    sl_lcol[p] = (uint16_t)lo;
  }
}

bool fg_ensure_halo(fg_mesh *m) {
  if (!m->halo_tried) {
    m->halo_tried = true;
    if (m->maxrow4 <= FG_MAX_ROW) {
      try {
        fg_build_halo(m);
      } catch (const FgError &e) {
        if (e.code != FG_BAD_MESH) throw;  // rows too long for staging: no halo variants
        m->halo_col = nullptr;
      }
    }
  }
  return m->halo_col != nullptr;
}

void fg_build_halo(fg_mesh *m) {
  const int slots = std::max(m->maxrow4, FG_GROUP);
  // rows per CTA: the largest power of two in [32, 512] whose keys fit 8192 slots
  int hrows = 512;
  while (hrows > FG_SLICE && hrows * slots > 8192) hrows >>= 1;
  const int nkeys = hrows * slots;
  int P2 = FG_HALO_THREADS;
  while (P2 < nkeys) P2 <<= 1;
  FG_REQUIRE(P2 <= 16384, FG_BAD_MESH, "matrix rows too long for halo staging");
  m->hrows = hrows;
  m->hcap = nkeys;
  m->nhblocks = (int)((m->nv + hrows - 1) / hrows);
  m->halo_col = dev_alloc<int>(m, (size_t)m->nhblocks * m->hcap);
  m->halo_len = dev_alloc<int>(m, (size_t)m->nhblocks);
  m->sl_lcol = dev_alloc<uint16_t>(m, (size_t)m->nsell);
  FG_CUDA_TRY(cudaMemsetAsync(m->sl_lcol, 0, sizeof(uint16_t) * (size_t)m->nsell, m->stream));
  const size_t smem = 2 * (size_t)P2 * sizeof(int);
  FG_CUDA_TRY(cudaFuncSetAttribute(k_build_halo, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_build_halo<<<m->nhblocks, FG_HALO_THREADS, smem, m->stream>>>(m->nv, hrows, slots, P2, m->sl_ptr, m->sl_len,
                                                                   m->sl_col, m->hcap, m->halo_col, m->halo_len,
                                                                   m->sl_lcol, m->flags);
  FG_CUDA_TRY(cudaGetLastError());
  FG_LAUNCHED(1);
  std::vector<int> hl(m->nhblocks);
  FG_CUDA_TRY(cudaMemcpyAsync(hl.data(), m->halo_len, sizeof(int) * m->nhblocks, cudaMemcpyDeviceToHost, m->stream));
  fg_sync(m);
  fg_check_flags(m, "halo staging");
  m->hmax = *std::max_element(hl.begin(), hl.end());
  // largest row block in matrix entries (the pipelined iteration stages one block)
  std::vector<int> sp(m->nslices + 1);
  FG_CUDA_TRY(cudaMemcpy(sp.data(), m->sl_ptr, sizeof(int) * (m->nslices + 1), cudaMemcpyDeviceToHost));
  const int spt = hrows / FG_SLICE;
  m->tmax = 0;
  for (int b = 0; b < m->nhblocks; ++b) {
    const int s0 = b * spt, s1 = std::min(s0 + spt, m->nslices);
    m->tmax = std::max(m->tmax, sp[s1] - sp[s0]);
  }
  m->pipe_grid = 0;
}

// Incidence in SELL layout: record position per (element, local node) and the
// slot (position in the row) of each node of the element.
__global__ void k_slots(const int *__restrict__ iptr, const int *__restrict__ inc, const int *__restrict__ t,
                        int64_t nt, int npe, int64_t nv, const int *__restrict__ rowptr,
                        const int *__restrict__ colidx, const int *__restrict__ in_ptr, const int *__restrict__ in_len,
                        int *__restrict__ recpos, uint8_t *__restrict__ in_slot) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  int s = (int)(i / FG_SLICE), lane = (int)(i % FG_SLICE);
  int base = in_ptr[s] + lane, ilen = in_len[s];
  int rb = rowptr[i], re = rowptr[i + 1];
  int deg = iptr[i + 1] - iptr[i];
  for (int m = 0; m < ilen; ++m) {
    int64_t pos = base + (int64_t)m * FG_SLICE;
    if (m >= deg) {
      for (int j = 0; j < npe; ++j) in_slot[pos * npe + j] = 0xFF;
      continue;
    }
    int key = inc[iptr[i] + m];
    int64_t k = key / npe;
    int a = key % npe;
    recpos[(int64_t)a * nt + k] = (int)pos;
    for (int j = 0; j < npe; ++j) {
      int v = t[(int64_t)j * nt + k];
      int lo = rb, hi = re;
      while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (colidx[mid] < v) lo = mid + 1; else hi = mid;
      }
      in_slot[pos * npe + j] = (uint8_t)(lo - rb);
    }
  }
}

// P1 tetrahedron geometry from the inverse Jacobian (FP64): gradients of the four
// barycentric functions (12 values) and the volume |det J| / 6
// (src/mesh.jl:484-505).  SoA: geo[c*nt + k], c = 3*a + d for gradients, 12 = volume.
__global__ void k_geom_tet(const double *__restrict__ p, const int *__restrict__ t, int64_t nt,
                           double *__restrict__ geo, int *flags) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nt) return;
  int n0 = t[k], n1 = t[nt + k], n2 = t[2 * nt + k], n3 = t[3 * nt + k];
  double x0 = p[3 * n0], y0 = p[3 * n0 + 1], z0 = p[3 * n0 + 2];
  double a1 = p[3 * n1] - x0, a2 = p[3 * n2] - x0, a3 = p[3 * n3] - x0;
  double b1 = p[3 * n1 + 1] - y0, b2 = p[3 * n2 + 1] - y0, b3 = p[3 * n3 + 1] - y0;
  double c1 = p[3 * n1 + 2] - z0, c2 = p[3 * n2 + 2] - z0, c3 = p[3 * n3 + 2] - z0;
  // J = [a1 a2 a3; b1 b2 b3; c1 c2 c3] (columns = edges); rows of J^-1 are the
  // gradients of lambda_1..3.
  double C11 = b2 * c3 - b3 * c2, C12 = b3 * c1 - b1 * c3, C13 = b1 * c2 - b2 * c1;
  double C21 = a3 * c2 - a2 * c3, C22 = a1 * c3 - a3 * c1, C23 = a2 * c1 - a1 * c2;
  double C31 = a2 * b3 - a3 * b2, C32 = a3 * b1 - a1 * b3, C33 = a1 * b2 - a2 * b1;
  double det = a1 * C11 + a2 * C12 + a3 * C13;
  if (det == 0.0) { atomicOr(flags, FLAG_DEGENERATE); det = 1.0; }
  double inv = 1.0 / det;
  // grad lambda_1 = (C11, C21, C31)/det, lambda_2 = (C12, C22, C32)/det, lambda_3 = (C13, C23, C33)/det
  double g1x = C11 * inv, g1y = C21 * inv, g1z = C31 * inv;
  double g2x = C12 * inv, g2y = C22 * inv, g2z = C32 * inv;
  double g3x = C13 * inv, g3y = C23 * inv, g3z = C33 * inv;
  geo[0 * nt + k] = -(g1x + g2x + g3x);
  geo[1 * nt + k] = -(g1y + g2y + g3y);
  geo[2 * nt + k] = -(g1z + g2z + g3z);
  geo[3 * nt + k] = g1x; geo[4 * nt + k] = g1y; geo[5 * nt + k] = g1z;
  geo[6 * nt + k] = g2x; geo[7 * nt + k] = g2y; geo[8 * nt + k] = g2z;
  geo[9 * nt + k] = g3x; geo[10 * nt + k] = g3y; geo[11 * nt + k] = g3z;
  geo[12 * nt + k] = fabs(det) / 6.0;
  // Gram matrix G_ab = grad(phi_a).grad(phi_b), upper triangle row by row (10 values):
  // VE * G is the element stiffness for unit coefficient, the matrix the reference
  // computes once per mesh as Ak (Magnetostatics/NewtonRaphson.jl:112).
  double g[4][3] = {{-(g1x + g2x + g3x), -(g1y + g2y + g3y), -(g1z + g2z + g3z)},
                    {g1x, g1y, g1z}, {g2x, g2y, g2z}, {g3x, g3y, g3z}};
  int c = 13;
  for (int a = 0; a < 4; ++a)
    for (int b = a; b < 4; ++b) geo[(int64_t)(c++) * nt + k] = g[a][0] * g[b][0] + g[a][1] * g[b][1] + g[a][2] * g[b][2];
}

// P1 triangle geometry: gradients of the three barycentric functions (6 values)
// and the area |det J| / 2.  geo[c*nt + k], c = 2*a + d, 6 = area.
__global__ void k_geom_tri(const double *__restrict__ p, const int *__restrict__ t, int64_t nt,
                           double *__restrict__ geo, int *flags) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nt) return;
  int n0 = t[k], n1 = t[nt + k], n2 = t[2 * nt + k];
  double x0 = p[3 * n0], y0 = p[3 * n0 + 1];
  double a1 = p[3 * n1] - x0, a2 = p[3 * n2] - x0;
  double b1 = p[3 * n1 + 1] - y0, b2 = p[3 * n2 + 1] - y0;
  double det = a1 * b2 - a2 * b1;
  if (det == 0.0) { atomicOr(flags, FLAG_DEGENERATE); det = 1.0; }
  double inv = 1.0 / det;
  double g1x = b2 * inv, g1y = -a2 * inv;
  double g2x = -b1 * inv, g2y = a1 * inv;
  geo[0 * nt + k] = -(g1x + g2x);
  geo[1 * nt + k] = -(g1y + g2y);
  geo[2 * nt + k] = g1x; geo[3 * nt + k] = g1y;
  geo[4 * nt + k] = g2x; geo[5 * nt + k] = g2y;
  geo[6 * nt + k] = 0.5 * fabs(det);
}

// ------------------------------------------------------------------ pattern sizes
// Exclusive scans of int arrays on the device (three passes: 1024-element block
// scans, one block over the block totals, the offsets written back as int32 with the
// total at out[n]); the int64 total is left on the device for the host to check
// against 2^31 before anything uses the offsets.
__device__ __forceinline__ int64_t block_incl_scan_1024(int64_t v, int64_t *ws) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int64_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int64_t w = ws[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    ws[lane] = w;
  }
  __syncthreads();
  const int64_t r = x + (wid > 0 ? ws[wid - 1] : 0);
  __syncthreads();  // ws is reused by the next call
  return r;
}

__global__ void __launch_bounds__(1024) k_scan_local(const int *__restrict__ in, int64_t n, int64_t *__restrict__ tmp,
                                                     int64_t *__restrict__ bsum) {
  __shared__ int64_t ws[32];
  const int64_t i = (int64_t)blockIdx.x * 1024 + threadIdx.x;
  const int64_t v = (i < n) ? (int64_t)in[i] : 0;
  const int64_t incl = block_incl_scan_1024(v, ws);
  if (i < n) tmp[i] = incl - v;
  if (threadIdx.x == 1023) bsum[blockIdx.x] = incl;
}

__global__ void __launch_bounds__(1024) k_scan_bsum(int64_t *__restrict__ bsum, int nb, int64_t *__restrict__ total) {
  __shared__ int64_t ws[32];
  __shared__ int64_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nb; base += 1024) {
    const int j = base + (int)threadIdx.x;
    const int64_t v = (j < nb) ? bsum[j] : 0;
    const int64_t incl = block_incl_scan_1024(v, ws);
    const int64_t c = carry;
    if (j < nb) bsum[j] = c + incl - v;
    __syncthreads();
    if (threadIdx.x == 1023) carry = c + incl;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void k_scan_apply(const int64_t *__restrict__ tmp, const int64_t *__restrict__ bsum, int64_t n,
                             const int64_t *__restrict__ total, int *__restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (int)(tmp[i] + bsum[i / 1024]);
  if (i == 0) out[n] = (int)*total;
}

// Per SELL slice of 32 rows: its groups of 4 slots (longest row), its incidence
// depth (largest node degree), their padded sizes for the offset scans, and the
// longest row and degree overall.
__global__ void k_slice_meta(const int *__restrict__ rowlen, const int *__restrict__ deg, int64_t nv, int nslices,
                             int *__restrict__ sl_len, int *__restrict__ in_len, int *__restrict__ slsize,
                             int *__restrict__ insize, int64_t *__restrict__ meta) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nslices) return;
  int mx = 0, md = 0;
  const int64_t r1 = nv < (int64_t)(s + 1) * FG_SLICE ? nv : (int64_t)(s + 1) * FG_SLICE;
  for (int64_t r = (int64_t)s * FG_SLICE; r < r1; ++r) {
    mx = max(mx, rowlen[r]);
    md = max(md, deg[r]);
  }
  const int groups = max(1, (mx + FG_GROUP - 1) / FG_GROUP);
  sl_len[s] = groups;
  in_len[s] = md;
  slsize[s] = groups * FG_GROUP * FG_SLICE;
  insize[s] = md * FG_SLICE;
  atomicMax(reinterpret_cast<unsigned long long *>(meta + 3), (unsigned long long)mx);
  atomicMax(reinterpret_cast<unsigned long long *>(meta + 4), (unsigned long long)md);
}

// The most padded entries of one 256-row block (the bulk-staged SpMV stages one).
__global__ void k_tmax256(const int *__restrict__ sl_ptr, int nslices, int64_t *__restrict__ meta) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  const int s0 = b * (256 / FG_SLICE);
  if (s0 >= nslices) return;
  const int s1 = min(s0 + 256 / FG_SLICE, nslices);
  atomicMax(reinterpret_cast<unsigned long long *>(meta + 5), (unsigned long long)(sl_ptr[s1] - sl_ptr[s0]));
}

// ------------------------------------------------------------------ host side

// The default memory pool of a device keeps the memory freed to it (no release
// threshold) for the next handle; set once per device for this process.
void fg_pool_init(int device) {
  static std::mutex lock;
  static bool done[64] = {false};
  if (device < 0 || device >= 64) return;
  std::lock_guard<std::mutex> g(lock);
  if (done[device]) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  cudaGetLastError();
  done[device] = true;
}

static std::mutex g_pinned_lock;
static std::vector<void *> g_pinned_free;

void *fg_pinned_block_get() {
  {
    std::lock_guard<std::mutex> g(g_pinned_lock);
    if (!g_pinned_free.empty()) {
      void *b = g_pinned_free.back();
      g_pinned_free.pop_back();
      return b;
    }
  }
  void *b = nullptr;
  FG_CUDA_TRY(cudaMallocHost(&b, FG_PINNED_BLOCK));
  return b;
}

void fg_pinned_block_put(void *block) {
  if (!block) return;
  std::lock_guard<std::mutex> g(g_pinned_lock);
  g_pinned_free.push_back(block);
}

static void free_mesh(fg_mesh *m) {
  if (!m) return;
  for (int g = 0; g < 4; ++g)
    if (m->graph[g].exec) cudaGraphExecDestroy(m->graph[g].exec);
  if (m->bcg_exec) cudaGraphExecDestroy(m->bcg_exec);
  if (m->stream) {
    for (void *ptr : m->extra) cudaFreeAsync(ptr, m->stream);
    cudaStreamSynchronize(m->stream);
  }
  for (void *ptr : m->extra_sync) cudaFree(ptr);
  fg_pinned_block_put(m->hbuf);  // hint lives in the same block
  if (m->ev0) cudaEventDestroy(m->ev0);
  if (m->ev1) cudaEventDestroy(m->ev1);
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
}

// Builds a handle whose matrix rows are the nv degrees of freedom listed by t
// (nodes_per_elem x nt).  With tv (4 x nt vertex indices into the np points p) the
// degrees of freedom are the 6 edges of each tetrahedron (Nedelec elements) and the
// geometry comes from tv; otherwise they are the nodes themselves (np = nv).
static fg_status create_impl(const double *p, int64_t np, const int32_t *t, int64_t nt, int32_t nodes_per_elem,
                             int64_t nv, const int32_t *tv, int32_t index_base, fg_mesh **out) {
  fg_mesh *m = nullptr;
  fg_status st = fg_guard([&]() -> fg_status {
    FG_REQUIRE(out != nullptr && p != nullptr && t != nullptr, FG_BAD_ARG, "fg_mesh_create: null pointer");
    *out = nullptr;
    int npe = nodes_per_elem;
    FG_REQUIRE(npe == 3 || npe == 4 || npe == 6 || npe == 10, FG_BAD_ARG,
               "fg_mesh_create: nodes_per_elem must be 3, 4, 6 or 10");
    FG_REQUIRE(!tv || npe == 6, FG_BAD_ARG, "fg_edge_mesh_create: six edges per tetrahedron");
    FG_REQUIRE(np > 0 && np < (int64_t)1 << 30, FG_BAD_ARG, "fg_mesh_create: bad point count");
    FG_REQUIRE(index_base == 0 || index_base == 1, FG_BAD_ARG, "fg_mesh_create: index_base must be 0 or 1");
    FG_REQUIRE(nv > 0 && nt > 0, FG_BAD_ARG, "fg_mesh_create: empty mesh");
    FG_REQUIRE(nv < (int64_t)1 << 30 && nt * npe < (int64_t)1 << 31, FG_BAD_ARG, "fg_mesh_create: mesh too large");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) throw FgError{FG_NO_DEVICE, "no CUDA device"};
    m = new fg_mesh();
    FG_CUDA_TRY(cudaGetDevice(&m->device));
    FG_CUDA_TRY(cudaDeviceGetAttribute(&m->sm_count, cudaDevAttrMultiProcessorCount, m->device));
    fg_pool_init(m->device);
    FG_CUDA_TRY(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
    FG_CUDA_TRY(cudaEventCreate(&m->ev0));
    FG_CUDA_TRY(cudaEventCreate(&m->ev1));
    m->nv = nv;
    m->nt = nt;
    m->npe = npe;
    m->edge = tv != nullptr;
    m->dim = ((npe == 3 || npe == 6) && !m->edge) ? 2 : 3;
    m->nvert = m->dim + 1;
    m->np = np;
    cudaStream_t s = m->stream;

    m->flags = dev_alloc<int>(m, 4);
    FG_CUDA_TRY(cudaMemsetAsync(m->flags, 0, 4 * sizeof(int), s));
    m->p = dev_alloc<double>(m, 3 * (size_t)np);
    FG_CUDA_TRY(cudaMemcpyAsync(m->p, p, sizeof(double) * 3 * (size_t)np, cudaMemcpyHostToDevice, s));
    if (tv) {
      int32_t *tvraw = nullptr;
      FG_CUDA_TRY(cudaMallocAsync(&tvraw, sizeof(int32_t) * (size_t)nt * 4, s));
      FG_CUDA_TRY(cudaMemcpyAsync(tvraw, tv, sizeof(int32_t) * (size_t)nt * 4, cudaMemcpyHostToDevice, s));
      m->tv = dev_alloc<int>(m, (size_t)nt * 4);
      k_convert_t<<<grid_for(nt, 256), 256, 0, s>>>(tvraw, m->tv, nt, 4, np, index_base, m->flags);
      FG_CUDA_TRY(cudaGetLastError());
      cudaFreeAsync(tvraw, s);
    }
    int32_t *traw = nullptr;
    FG_CUDA_TRY(cudaMallocAsync(&traw, sizeof(int32_t) * (size_t)nt * npe, s));
    FG_CUDA_TRY(cudaMemcpyAsync(traw, t, sizeof(int32_t) * (size_t)nt * npe, cudaMemcpyHostToDevice, s));
    m->t = dev_alloc<int>(m, (size_t)nt * npe);
    k_convert_t<<<grid_for(nt, 256), 256, 0, s>>>(traw, m->t, nt, npe, nv, index_base, m->flags);
    FG_CUDA_TRY(cudaGetLastError());
    fg_check_flags(m, "fg_mesh_create");
    cudaFreeAsync(traw, s);

    // incidence lists
    m->hbuf = static_cast<double *>(fg_pinned_block_get());
    m->hint = reinterpret_cast<int *>(m->hbuf + 64);
    m->nslices = (int)((nv + FG_SLICE - 1) / FG_SLICE);
    const int nsl = m->nslices;
    // work space of the pattern build, released on the stream when this scope ends
    // (also when it ends by an error)
    StreamScratch scratch{s, {}};
    int *deg = scratch.get<int>((size_t)nv);
    int *iptr = scratch.get<int>((size_t)nv + 1);
    int *inc = scratch.get<int>((size_t)nt * npe);
    int *slsize = scratch.get<int>((size_t)nsl);
    int *insize = scratch.get<int>((size_t)nsl);
    int64_t *scan_tmp = scratch.get<int64_t>((size_t)nv);
    int64_t *scan_bsum = scratch.get<int64_t>((size_t)((nv + 1023) / 1024));
    // meta: totals of the scans (0 incidences, 1 nnz, 2 padded entries, 6 incidence
    // slots) and maxima (3 longest row, 4 largest degree, 5 entries of a 256-row block)
    int64_t *meta = scratch.get<int64_t>(8);
    FG_CUDA_TRY(cudaMemsetAsync(meta, 0, sizeof(int64_t) * 8, s));
    auto scan = [&](const int *in, int64_t n, int *out, int64_t *total) {
      const int nb = (int)((n + 1023) / 1024);
      k_scan_local<<<nb, 1024, 0, s>>>(in, n, scan_tmp, scan_bsum);
      k_scan_bsum<<<1, 1024, 0, s>>>(scan_bsum, nb, total);
      k_scan_apply<<<grid_for(n, 256), 256, 0, s>>>(scan_tmp, scan_bsum, n, total, out);
    };
    FG_CUDA_TRY(cudaMemsetAsync(deg, 0, sizeof(int) * (size_t)nv, s));
    k_count_deg<<<grid_for(nt, 256), 256, 0, s>>>(m->t, nt, npe, deg);
    scan(deg, nv, iptr, meta + 0);
    // the fill counts each node's list up from 0 again: deg ends as it was
    FG_CUDA_TRY(cudaMemsetAsync(deg, 0, sizeof(int) * (size_t)nv, s));
    k_fill_inc<<<grid_for(nt, 256), 256, 0, s>>>(m->t, nt, npe, iptr, deg, inc);
    k_sort_inc<<<grid_for(nv, 128), 128, 0, s>>>(iptr, inc, nv);
    FG_CUDA_TRY(cudaGetLastError());

    // row lengths of the structural pattern, the SELL-32 slices of the matrix and of
    // the incidence records, and their offsets, all on the device; the host reads the
    // sizes back once (rows longer than 128 entries: once more, with the long-row
    // kernel)
    m->rowlen = dev_alloc<int>(m, (size_t)nv);
    m->rowptr = dev_alloc<int>(m, (size_t)nv + 1);
    m->sl_ptr = dev_alloc<int>(m, (size_t)nsl + 1);
    m->sl_len = dev_alloc<int>(m, (size_t)nsl);
    m->in_ptr = dev_alloc<int>(m, (size_t)nsl + 1);
    m->in_len = dev_alloc<int>(m, (size_t)nsl);
    bool big = false;
    int64_t hm[8];
    for (;;) {
      FG_CUDA_TRY(cudaMemsetAsync(meta + 1, 0, sizeof(int64_t) * 7, s));
      if (big)
        k_row_count<FG_MAX_ROW><<<grid_for(nv, 64), 64, 0, s>>>(iptr, inc, m->t, nt, npe, nv, m->rowlen, m->flags);
      else
        k_row_count<128><<<grid_for(nv, 128), 128, 0, s>>>(iptr, inc, m->t, nt, npe, nv, m->rowlen, m->flags);
      scan(m->rowlen, nv, m->rowptr, meta + 1);
      k_slice_meta<<<grid_for(nsl, 128), 128, 0, s>>>(m->rowlen, deg, nv, nsl, m->sl_len, m->in_len, slsize, insize,
                                                      meta);
      scan(slsize, nsl, m->sl_ptr, meta + 2);
      scan(insize, nsl, m->in_ptr, meta + 6);
      k_tmax256<<<grid_for((nsl + 256 / FG_SLICE - 1) / (256 / FG_SLICE), 128), 128, 0, s>>>(m->sl_ptr, nsl, meta);
      FG_CUDA_TRY(cudaGetLastError());
      FG_CUDA_TRY(cudaMemcpyAsync(m->hbuf, meta, sizeof(int64_t) * 8, cudaMemcpyDeviceToHost, s));
      FG_CUDA_TRY(cudaMemcpyAsync(m->hint, m->flags, sizeof(int), cudaMemcpyDeviceToHost, s));
      fg_sync(m);
      std::memcpy(hm, m->hbuf, sizeof hm);
      const int h = m->hint[0];
      if ((h & FLAG_ROW_OVERFLOW) && !big && (h & ~FLAG_ROW_OVERFLOW) == 0) {
        FG_CUDA_TRY(cudaMemsetAsync(m->flags, 0, sizeof(int), s));
        big = true;
        continue;
      }
      fg_raise_flags(m, h, "fg_mesh_create");
      break;
    }
    m->nnz = hm[1];
    m->nsell = hm[2];
    m->maxrow = (int)hm[3];
    m->maxdeg = (int)hm[4];
    m->tmax256 = (int)hm[5];
    m->ninc = hm[6];
    FG_REQUIRE(m->nnz < ((int64_t)1 << 31), FG_BAD_ARG, "fg_mesh_create: pattern too large");
    FG_REQUIRE(m->nsell < ((int64_t)1 << 31) && m->ninc * npe < ((int64_t)1 << 31), FG_BAD_ARG,
               "fg_mesh_create: padded layout too large");

    m->colidx = dev_alloc<int>(m, (size_t)m->nnz);
    m->sl_col = dev_alloc<int>(m, (size_t)m->nsell);
    m->sl_dcol = dev_alloc<int16_t>(m, (size_t)m->nsell);
    m->nvp = (int64_t)nsl * FG_SLICE;
    m->maxrow4 = (m->maxrow + FG_GROUP - 1) / FG_GROUP * FG_GROUP;
    m->diagk = dev_alloc<uint8_t>(m, (size_t)nv);
    m->in_slot = dev_alloc<uint8_t>(m, (size_t)m->ninc * npe);
    m->recpos = dev_alloc<int>(m, (size_t)nt * npe);
    if (big)
      k_row_fill<FG_MAX_ROW><<<grid_for(nv, 64), 64, 0, s>>>(iptr, inc, m->t, nt, npe, nv, m->rowptr, m->sl_ptr,
                                                             m->sl_len, m->colidx, m->sl_col, m->sl_dcol, m->diagk,
                                                             m->flags);
    else
      k_row_fill<128><<<grid_for(nv, 128), 128, 0, s>>>(iptr, inc, m->t, nt, npe, nv, m->rowptr, m->sl_ptr,
                                                         m->sl_len, m->colidx, m->sl_col, m->sl_dcol, m->diagk,
                                                         m->flags);
    k_slots<<<grid_for(nv, 128), 128, 0, s>>>(iptr, inc, m->t, nt, npe, nv, m->rowptr, m->colidx, m->in_ptr,
                                              m->in_len, m->recpos, m->in_slot);
    FG_CUDA_TRY(cudaGetLastError());

    // geometry of the vertex simplex
    m->ngeo = (m->dim == 3) ? 23 : 7;
    m->geo = dev_alloc<double>(m, (size_t)m->ngeo * nt);
    if (m->dim == 3)
      k_geom_tet<<<grid_for(nt, 256), 256, 0, s>>>(m->p, m->edge ? m->tv : m->t, nt, m->geo, m->flags);
    else
      k_geom_tri<<<grid_for(nt, 256), 256, 0, s>>>(m->p, m->t, nt, m->geo, m->flags);
    FG_CUDA_TRY(cudaGetLastError());

    // control and reduction workspace
    // one slot of 4 per CTA of any row kernel (CTAs of 32 rows or more)
    m->red.partials = dev_alloc<double>(m, ((size_t)grid_for(nv, FG_SLICE) + FG_RED_BLOCKS) * 4);
    m->red.counter = dev_alloc<unsigned int>(m, 128);   // two-level arrival counters
    FG_CUDA_TRY(cudaMemsetAsync(m->red.counter, 0, 128 * sizeof(unsigned int), s));
    m->scal = dev_alloc<double>(m, S_NSCAL);
    m->ictl = dev_alloc<int>(m, I_NINT);
    // the error flags of the fill and geometry kernels, and whether some column is
    // more than 32767 rows from its row (then 32-bit columns), in the last round trip
    FG_CUDA_TRY(cudaMemcpyAsync(m->hint, m->flags, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
    fg_sync(m);
    fg_raise_flags(m, m->hint[0], "fg_mesh_create");
    m->use_dcol = (m->hint[1] == 0);  // 16-bit column offsets when the bandwidth allows
    *out = m;
    m = nullptr;
    return FG_OK;
  });
  if (m) free_mesh(m);
  return st;
}

extern "C" fg_status fg_mesh_create(const double *p, int64_t nv, const int32_t *t, int64_t nt,
                                    int32_t nodes_per_elem, int32_t index_base, fg_mesh **out) {
  return create_impl(p, nv, t, nt, nodes_per_elem, nv, nullptr, index_base, out);
}

extern "C" fg_status fg_edge_mesh_create(const double *p, int64_t nv, const int32_t *t, const int32_t *edges,
                                         int64_t nt, int64_t ne, int32_t index_base, fg_mesh **out) {
  if (!t || !edges || ne <= 0 || ne >= (int64_t)1 << 30) {
    if (out) *out = nullptr;
    return fg_guard([&]() -> fg_status {
      throw FgError{FG_BAD_ARG, "fg_edge_mesh_create: need t, edges and 0 < ne < 2^30"};
    });
  }
  return create_impl(p, nv, edges, nt, 6, ne, t, index_base, out);
}

extern "C" fg_status fg_mesh_destroy(fg_mesh *m) {
  return fg_guard([&]() -> fg_status {
    if (!m) return FG_OK;
    cudaStreamSynchronize(m->stream);
    fg_release_l2(m);
    free_mesh(m);
    return FG_OK;
  });
}

extern "C" fg_status fg_mesh_nnz(const fg_mesh *m, int64_t *nnz, int32_t *max_row) {
  return fg_guard([&]() -> fg_status {
    FG_REQUIRE(m != nullptr, FG_BAD_ARG, "fg_mesh_nnz: null handle");
    if (nnz) *nnz = m->nnz;
    if (max_row) *max_row = m->maxrow;
    return FG_OK;
  });
}

extern "C" fg_status fg_mesh_set_dirichlet(fg_mesh *m, const uint8_t *fixed) {
  return fg_guard([&]() -> fg_status {
    FG_REQUIRE(m != nullptr, FG_BAD_ARG, "fg_mesh_set_dirichlet: null handle");
    m->op_tag = 0;  // an operator kept on the handle has the old Dirichlet rows
    if (!m->fixed) m->fixed = dev_alloc<uint8_t>(m, (size_t)m->nv);
    if (fixed) {
      FG_CUDA_TRY(cudaMemcpyAsync(m->fixed, fixed, (size_t)m->nv, cudaMemcpyHostToDevice, m->stream));
      m->has_fixed = true;
    } else {
      FG_CUDA_TRY(cudaMemsetAsync(m->fixed, 0, (size_t)m->nv, m->stream));
      m->has_fixed = false;
    }
    fg_sync(m);
    return FG_OK;
  });
}

extern "C" fg_status fg_mesh_volumes(fg_mesh *m, double *VE) {
  return fg_guard([&]() -> fg_status {
    FG_REQUIRE(m != nullptr && VE != nullptr, FG_BAD_ARG, "fg_mesh_volumes: null pointer");
    int c = (m->dim == 3) ? 12 : 6;
    FG_CUDA_TRY(cudaMemcpyAsync(VE, m->geo + (size_t)c * m->nt, sizeof(double) * (size_t)m->nt,
                                cudaMemcpyDeviceToHost, m->stream));
    fg_sync(m);
    return FG_OK;
  });
}

extern "C" fg_status fg_csc_pattern(const fg_mesh *mc, int64_t *colptr, int32_t *rowval, int32_t index_base) {
  return fg_guard([&]() -> fg_status {
    fg_mesh *m = const_cast<fg_mesh *>(mc);
    FG_REQUIRE(m != nullptr && colptr != nullptr && rowval != nullptr, FG_BAD_ARG, "fg_csc_pattern: null pointer");
    FG_REQUIRE(index_base == 0 || index_base == 1, FG_BAD_ARG, "fg_csc_pattern: index_base must be 0 or 1");
    std::vector<int> rp(m->nv + 1);
    FG_CUDA_TRY(cudaMemcpyAsync(rp.data(), m->rowptr, sizeof(int) * (size_t)(m->nv + 1), cudaMemcpyDeviceToHost,
                                m->stream));
    FG_CUDA_TRY(cudaMemcpyAsync(rowval, m->colidx, sizeof(int) * (size_t)m->nnz, cudaMemcpyDeviceToHost, m->stream));
    fg_sync(m);
    for (int64_t i = 0; i <= m->nv; ++i) colptr[i] = rp[i] + index_base;
    if (index_base)
      for (int64_t q = 0; q < m->nnz; ++q) rowval[q] += 1;
    return FG_OK;
  });
}
