// K0 -- observation preparation: cell binning (counting sort by cell), per-cell ordering by
// observation index, gather of the per-observation scalars and transpose of HSf into
// observation-major rows.
//
// The reference tests every observation against every zone (assimilation.F90:3745-3757) and
// packs the relevant rows of HSf in ascending index order (rrsqrt.F90:397-404). Here the
// observations are binned once into a regular cell grid (the role ndgrid.F90:1489-1586
// `setupgrid` plays for `near`), so a zone only visits the cells that can hold observations
// within its maxLength; within a cell observations stay in ascending index order.
//
// HBM layout produced (q = cell-sorted position):
//   u[q], v[q]        coordinates the metric uses           (8 B each)
//   innov[q]          yo - Hxf                              (8 B)
//   r[q]              R diagonal                            (8 B)
//   HSt[q*N + k]      HSf(perm[q], k), one 8*N-byte row per observation
#include <cuda_runtime.h>

#include "oakg_internal.cuh"

namespace oakg {

namespace {

constexpr int kScanThreads = 1024;

__device__ __forceinline__ double warp_min(double x) {
  for (int o = 16; o > 0; o >>= 1) x = fmin(x, __shfl_xor_sync(0xffffffffu, x, o));
  return x;
}
__device__ __forceinline__ double warp_max(double x) {
  for (int o = 16; o > 0; o >>= 1) x = fmax(x, __shfl_xor_sync(0xffffffffu, x, o));
  return x;
}

// One block: min/max of u and v (v may be null).
__global__ void k_bounds(const double* __restrict__ u, const double* __restrict__ v, int64_t m,
                         double* __restrict__ out) {
  double umin = INFINITY, umax = -INFINITY, vmin = INFINITY, vmax = -INFINITY;
  for (int64_t j = threadIdx.x; j < m; j += blockDim.x) {
    double a = u[j];
    umin = fmin(umin, a);
    umax = fmax(umax, a);
    double b = v ? v[j] : 0.0;
    vmin = fmin(vmin, b);
    vmax = fmax(vmax, b);
  }
  __shared__ double s[4][32];
  umin = warp_min(umin);
  umax = warp_max(umax);
  vmin = warp_min(vmin);
  vmax = warp_max(vmax);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    s[0][w] = umin;
    s[1][w] = umax;
    s[2][w] = vmin;
    s[3][w] = vmax;
  }
  __syncthreads();
  if (w == 0) {
    int nw = blockDim.x >> 5;
    umin = l < nw ? s[0][l] : INFINITY;
    umax = l < nw ? s[1][l] : -INFINITY;
    vmin = l < nw ? s[2][l] : INFINITY;
    vmax = l < nw ? s[3][l] : -INFINITY;
    umin = warp_min(umin);
    umax = warp_max(umax);
    vmin = warp_min(vmin);
    vmax = warp_max(vmax);
    if (l == 0) {
      out[0] = umin;
      out[1] = umax;
      out[2] = vmin;
      out[3] = vmax;
    }
  }
}

__device__ __forceinline__ int32_t cell_of(const CellGrid& g, double u, double v) {
  double uu = u;
  if (g.periodic_u) uu = u - 360.0 * floor(u / 360.0);
  double fu = floor((uu - g.u0) / g.csu);
  double fv = floor((v - g.v0) / g.csv);
  int32_t cu = (int32_t)fmin(fmax(fu, 0.0), (double)(g.nu - 1));
  int32_t cv = (int32_t)fmin(fmax(fv, 0.0), (double)(g.nv - 1));
  return cu + g.nu * cv;
}

__global__ void k_cell_id(CellGrid g, int64_t m, const double* __restrict__ u,
                          const double* __restrict__ v, int32_t* __restrict__ cell,
                          int32_t* __restrict__ count) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m;
       j += (int64_t)gridDim.x * blockDim.x) {
    int32_t c = cell_of(g, u[j], v ? v[j] : 0.0);
    cell[j] = c;
    atomicAdd(&count[c], 1);
  }
}

// Exclusive scan of in[0..n) into out[0..n] (out[n] = total), one block, chunked with carry.
template <typename TI, typename TO>
__global__ void k_scan_single(const TI* __restrict__ in, int64_t n, TO* __restrict__ out,
                              int32_t* __restrict__ max_out) {
  __shared__ TO s[kScanThreads];
  __shared__ TO carry;
  __shared__ int32_t smax[32];
  if (threadIdx.x == 0) carry = 0;
  int32_t mymax = 0;
  __syncthreads();
  for (int64_t base = 0; base < n; base += kScanThreads) {
    int64_t i = base + threadIdx.x;
    TO x = (i < n) ? (TO)in[i] : (TO)0;
    if (i < n && (int32_t)in[i] > mymax) mymax = (int32_t)in[i];
    s[threadIdx.x] = x;
    __syncthreads();
    for (int off = 1; off < kScanThreads; off <<= 1) {
      TO t = (threadIdx.x >= off) ? s[threadIdx.x - off] : (TO)0;
      __syncthreads();
      s[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < n) out[i] = carry + s[threadIdx.x] - x;
    __syncthreads();
    if (threadIdx.x == kScanThreads - 1) carry += s[threadIdx.x];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[n] = carry;
  if (max_out) {
    for (int o = 16; o > 0; o >>= 1) {
      int32_t t = __shfl_xor_sync(0xffffffffu, mymax, o);
      mymax = t > mymax ? t : mymax;
    }
    if ((threadIdx.x & 31) == 0) smax[threadIdx.x >> 5] = mymax;
    __syncthreads();
    if (threadIdx.x == 0) {
      int32_t mx = 0;
      for (int w = 0; w < kScanThreads / 32; w++) mx = smax[w] > mx ? smax[w] : mx;
      *max_out = mx;
    }
  }
}

__global__ void k_scatter(int64_t m, const int32_t* __restrict__ cell,
                          const int32_t* __restrict__ cell_start, int32_t* __restrict__ cursor,
                          int32_t* __restrict__ perm) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m;
       j += (int64_t)gridDim.x * blockDim.x) {
    int32_t c = cell[j];
    int32_t p = cell_start[c] + atomicAdd(&cursor[c], 1);
    perm[p] = (int32_t)j;
  }
}

// Ascending order of observation indices inside each cell (bitonic sort in shared memory),
// so that the sorted order, and hence every summation order downstream, is deterministic.
constexpr int kCellSortMax = 4096;
__global__ void k_cell_sort(int32_t ncells, const int32_t* __restrict__ cell_start,
                            int32_t* __restrict__ perm, int32_t* __restrict__ oversize) {
  __shared__ int32_t s[kCellSortMax];
  for (int32_t c = blockIdx.x; c < ncells; c += gridDim.x) {
    int32_t a = cell_start[c], b = cell_start[c + 1], len = b - a;
    if (len <= 1) continue;
    if (len > kCellSortMax) {
      if (threadIdx.x == 0) atomicAdd(oversize, 1);
      continue;
    }
    int P = 1;
    while (P < len) P <<= 1;
    for (int i = threadIdx.x; i < P; i += blockDim.x) s[i] = (i < len) ? perm[a + i] : INT32_MAX;
    __syncthreads();
    for (int k = 2; k <= P; k <<= 1) {
      for (int j = k >> 1; j > 0; j >>= 1) {
        for (int i = threadIdx.x; i < P; i += blockDim.x) {
          int ij = i ^ j;
          if (ij > i) {
            bool up = ((i & k) == 0);
            int32_t x = s[i], y = s[ij];
            if ((x > y) == up) {
              s[i] = y;
              s[ij] = x;
            }
          }
        }
        __syncthreads();
      }
    }
    for (int i = threadIdx.x; i < len; i += blockDim.x) perm[a + i] = s[i];
    __syncthreads();
  }
}

// Oversized cells (more than kCellSortMax observations) are ordered by one thread each
// with an in-place insertion sort; only reached for very dense clusters.
__global__ void k_cell_sort_large(int32_t ncells, const int32_t* __restrict__ cell_start,
                                  int32_t* __restrict__ perm) {
  for (int32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < ncells;
       c += gridDim.x * blockDim.x) {
    int32_t a = cell_start[c], b = cell_start[c + 1];
    if (b - a <= kCellSortMax) continue;
    for (int32_t i = a + 1; i < b; i++) {
      int32_t x = perm[i];
      int32_t k = i - 1;
      while (k >= a && perm[k] > x) {
        perm[k + 1] = perm[k];
        k--;
      }
      perm[k + 1] = x;
    }
  }
}

__global__ void k_gather_scalars(CellGrid g, int64_t m, const int32_t* __restrict__ perm,
                                 const double* __restrict__ u_src,
                                 const double* __restrict__ v_src,
                                 const double* __restrict__ yo, const double* __restrict__ Hxf,
                                 const double* __restrict__ r, int32_t* __restrict__ pos,
                                 double* __restrict__ u, double* __restrict__ v,
                                 double* __restrict__ innov, double* __restrict__ rs,
                                 int32_t* __restrict__ cu, float* __restrict__ ru,
                                 float* __restrict__ rv) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < m;
       q += (int64_t)gridDim.x * blockDim.x) {
    int32_t j = perm[q];
    pos[j] = (int32_t)q;
    const double uj = u_src[j], vj = v_src ? v_src[j] : 0.0;
    u[q] = uj;
    v[q] = vj;
    innov[q] = yo[j] - Hxf[j];
    rs[q] = r[j];
    // the cell the observation was binned into and its offsets inside it
    const int32_t c = cell_of(g, uj, vj);
    const int32_t ci = c % g.nu, cj = c / g.nu;
    const double uw = g.periodic_u ? uj - 360.0 * floor(uj / 360.0) : uj;  // as cell_of
    cu[q] = ci;
    ru[q] = (float)(uw - (g.u0 + ci * g.csu));
    rv[q] = (float)(vj - (g.v0 + cj * g.csv));
  }
}

// HSt[pos[j]*N + k] = HSf[j + k*ldH]: 32 x 32 tiles, coalesced reads along j, rows of HSt
// written as contiguous 32-element segments. HSf in FP64 or FP32 (FP32 storage at the
// boundary); the rows are FP64 (exact widening).
template <typename TIn>
__global__ void k_transpose_rows(int64_t m, int N, const TIn* __restrict__ HSf, int64_t ldH,
                                 const int32_t* __restrict__ pos, double* __restrict__ HSt) {
  __shared__ double tile[32][33];
  int64_t j0 = (int64_t)blockIdx.x * 32;
  int k0 = blockIdx.y * 32;
  int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  for (int kk = ty; kk < 32; kk += 8) {
    int64_t j = j0 + tx;
    int k = k0 + kk;
    tile[kk][tx] = (j < m && k < N) ? (double)HSf[j + (int64_t)k * ldH] : 0.0;
  }
  __syncthreads();
  for (int jj = ty; jj < 32; jj += 8) {
    int64_t j = j0 + jj;
    int k = k0 + tx;
    if (j < m && k < N) HSt[(int64_t)pos[j] * N + k] = tile[tx][jj];
  }
}

inline int grid_for(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  if (b > 152 * 32) b = 152 * 32;
  return (int)(b < 1 ? 1 : b);
}

}  // namespace

cudaError_t obs_bounds(const double* u, const double* v, int64_t m, double* d_out4,
                       cudaStream_t st) {
  k_bounds<<<1, 1024, 0, st>>>(u, v, m, d_out4);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t obs_bin_and_sort(const CellGrid& g, int64_t m, int N, const double* u_src,
                             const double* v_src, const double* yo, const double* Hxf,
                             const double* r, const double* HSf, const float* HSf32,
                             int64_t ldH, int32_t* d_cell, int32_t* d_count,
                             int32_t* d_cell_start, int32_t* d_pos, int32_t* d_perm,
                             double* d_u, double* d_v, double* d_innov, double* d_r,
                             double* d_HSt, int32_t* d_cu, float* d_ru, float* d_rv,
                             cudaStream_t st) {
  const int64_t ncells = (int64_t)g.nu * g.nv;
  cudaError_t e = cudaMemsetAsync(d_count, 0, (ncells + 1) * sizeof(int32_t), st);
  if (e != cudaSuccess) return e;
  if (m > 0) {
    k_cell_id<<<grid_for(m, 256), 256, 0, st>>>(g, m, u_src, v_src, d_cell, d_count);
  }
  k_scan_single<int32_t, int32_t><<<1, kScanThreads, 0, st>>>(d_count, ncells, d_cell_start,
                                                              nullptr);
  e = cudaMemsetAsync(d_count, 0, (ncells + 1) * sizeof(int32_t), st);
  if (e != cudaSuccess) return e;
  if (m > 0) {
    k_scatter<<<grid_for(m, 256), 256, 0, st>>>(m, d_cell, d_cell_start, d_count, d_perm);
    // d_count[ncells] is scratch here: number of cells above the shared-memory sort size
    k_cell_sort<<<(int)(ncells < 152 * 8 ? (ncells < 1 ? 1 : ncells) : 152 * 8), 256, 0, st>>>(
        (int32_t)ncells, d_cell_start, d_perm, d_count + ncells);
    k_cell_sort_large<<<grid_for(ncells, 128), 128, 0, st>>>((int32_t)ncells, d_cell_start,
                                                             d_perm);
    k_gather_scalars<<<grid_for(m, 256), 256, 0, st>>>(g, m, d_perm, u_src, v_src, yo, Hxf, r,
                                                       d_pos, d_u, d_v, d_innov, d_r, d_cu,
                                                       d_ru, d_rv);
    dim3 tb(32, 8), tg((unsigned)((m + 31) / 32), (unsigned)((N + 31) / 32));
    if (HSf32)
      k_transpose_rows<float><<<tg, tb, 0, st>>>(m, N, HSf32, ldH, d_pos, d_HSt);
    else
      k_transpose_rows<double><<<tg, tb, 0, st>>>(m, N, HSf, ldH, d_pos, d_HSt);
  }
  count_launches(m > 0 ? 7 : 1);
  return cudaGetLastError();
}

cudaError_t scan_exclusive_i32(const int32_t* d_in, int64_t n, int32_t* d_out, cudaStream_t st) {
  k_scan_single<int32_t, int32_t><<<1, kScanThreads, 0, st>>>(d_in, n, d_out, nullptr);
  count_launches(1);
  return cudaGetLastError();
}

__global__ void k_to_fp32(const double* __restrict__ src, float* __restrict__ dst, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (float)src[i];
}

cudaError_t rows_to_fp32(const double* src, float* dst, int64_t count, cudaStream_t st) {
  if (count <= 0) return cudaSuccess;
  k_to_fp32<<<grid_for(count, 256), 256, 0, st>>>(src, dst, count);
  count_launches(1);
  return cudaGetLastError();
}

__global__ void k_to_fp64(const float* __restrict__ src, double* __restrict__ dst, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (double)src[i];
}

cudaError_t rows_to_fp64(const float* src, double* dst, int64_t count, cudaStream_t st) {
  if (count <= 0) return cudaSuccess;
  k_to_fp64<<<grid_for(count, 256), 256, 0, st>>>(src, dst, count);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t zone_offsets(const int32_t* zone_size, int32_t Z, int64_t* d_zone_start,
                         int32_t* d_zone_max, cudaStream_t st) {
  k_scan_single<int32_t, int64_t><<<1, kScanThreads, 0, st>>>(zone_size, Z, d_zone_start,
                                                              d_zone_max);
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace oakg
