// State and observation layout builders (the host preprocessing of the reference, on the GPU):
//
// * zone_layout -- initPartition (assimilation.F90:578-641): from the partition vector
//   (zone number of every state element, 1..Z) the zone sizes, zoneIndex (sorted position ->
//   element; each zone contiguous, elements in ascending order inside a zone) and its
//   inverse. A least-significant-digit radix sort of the zone numbers (8-bit digits, one
//   histogram and one stable scatter per digit, ranks inside a tile from warp matching), so the
//   order inside a zone is the element order whatever the zone sizes. As in the reference, a
//   zone number outside 1..Z or an empty zone is an error.
// * permute_rows -- Y(i, :) = X(index(i), :) for the columns of an ensemble (into or out of the
//   zone order).
// * sea_index -- packed index of the unmasked grid points (the reference removes land points:
//   ObsML%removeLandPoints), -1 for masked ones.
// * rectilinear_oper -- genObservationOper (assimilation.F90:2471-2656) with cinterp
//   (ndgrid.F90:1183-1257) for a rectilinear grid of 1 to 4 dimensions: the grid cell holding
//   the observation (binary search per axis), its 2^n corners (any masked corner: the
//   observation is out, as in cinterp), then interp_cube (:636-665): the first simplex of the
//   cell's split (split, :353-440: every face recursively split around its centroid, the cell
//   centroid shared) whose barycentric coordinates lie in [-1e-8, 1 + 1e-8]; the corner weights
//   are the simplex's corner combinations applied to them (interp_tetrahedron, :464-629: the
//   (n+1) x (n+1) system [1; X - xc] c = [1; xi - xc], |det| > 1e-8). Rows of the operator: 2^n
//   (index, weight) pairs, index = offset + packed index of the corner; an observation outside
//   the grid gets index -1 and weight 0 in every pair (the reference's out-of-domain entry).
#include <cuda_runtime.h>
#include <math.h>

#include "oakg_internal.cuh"

namespace oakg {

namespace {

constexpr int kThreads = 256;

inline unsigned grid_for(int64_t n) {
  int64_t b = (n + kThreads - 1) / kThreads;
  if (b > 152 * 32) b = 152 * 32;
  return (unsigned)(b < 1 ? 1 : b);
}

__global__ void k_zone_keys(int64_t n, const int32_t* __restrict__ partition,
                            int32_t* __restrict__ key) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n;
       j += (int64_t)gridDim.x * blockDim.x)
    key[j] = partition[j] - 1;
}

__global__ void k_key_count_i32(int64_t n, const int32_t* __restrict__ key, int32_t nb,
                                int32_t* __restrict__ count, int32_t* __restrict__ bad) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n;
       j += (int64_t)gridDim.x * blockDim.x) {
    const int32_t k = key[j];
    if (k < 0 || k >= nb)
      atomicOr(bad, 1);
    else
      atomicAdd(&count[k], 1);
  }
}

__global__ void k_zone_sizes(int32_t Z, const int32_t* __restrict__ start,
                             int32_t* __restrict__ zone_size, int32_t* __restrict__ bad) {
  for (int32_t z = blockIdx.x * blockDim.x + threadIdx.x; z < Z; z += gridDim.x * blockDim.x) {
    const int32_t s = start[z + 1] - start[z];
    zone_size[z] = s;
    if (s == 0) atomicOr(bad, 2);
  }
}

// ---- stable LSD radix sort of int32 keys (8-bit digits) carrying int32 values
constexpr int kRadixItems = 16;
constexpr int kRadixTile = kThreads * kRadixItems;  // elements per block
static_assert(kThreads == 256, "one thread per digit value");

// hist[d * ntiles + t]: elements of tile t with digit d (digit-major, so that the exclusive scan
// of hist gives every (digit, tile) its first output position in stable order)
__global__ void k_radix_hist(int64_t n, const int32_t* __restrict__ key, int shift,
                             int32_t* __restrict__ hist, int64_t ntiles) {
  __shared__ int32_t h[kThreads];
  h[threadIdx.x] = 0;
  __syncthreads();
  const int64_t tb = (int64_t)blockIdx.x * kRadixTile;
#pragma unroll 4
  for (int r = 0; r < kRadixItems; r++) {
    const int64_t e = tb + (int64_t)r * kThreads + threadIdx.x;
    if (e < n) atomicAdd(&h[(key[e] >> shift) & 255], 1);
  }
  __syncthreads();
  hist[(int64_t)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter of one tile: elements go in rounds of kThreads (element order = round, warp,
// lane); inside a warp the rank among equal digits comes from __match_any_sync, across warps
// from the per-warp digit counts of the round.
__global__ void k_radix_scatter(int64_t n, const int32_t* __restrict__ key_in,
                                const int32_t* __restrict__ val_in, int shift,
                                const int32_t* __restrict__ offs, int64_t ntiles,
                                int32_t* __restrict__ key_out, int32_t* __restrict__ val_out) {
  constexpr int W = kThreads / 32;
  __shared__ int32_t base[kThreads];
  __shared__ int32_t wcnt[W][kThreads];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  base[threadIdx.x] = offs[(int64_t)threadIdx.x * ntiles + blockIdx.x];
#pragma unroll
  for (int q = 0; q < W; q++) wcnt[q][threadIdx.x] = 0;
  __syncthreads();
  const int64_t tb = (int64_t)blockIdx.x * kRadixTile;
  for (int r = 0; r < kRadixItems; r++) {
    const int64_t e = tb + (int64_t)r * kThreads + threadIdx.x;
    const bool valid = e < n;
    const int32_t k = valid ? key_in[e] : 0;
    const int32_t v = valid ? (val_in ? val_in[e] : (int32_t)e) : 0;
    // invalid lanes (the tail of the last tile) get distinct non-digit values
    const int d = valid ? (k >> shift) & 255 : 256 + lane;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int rank = __popc(peers & ((1u << lane) - 1u));
    if (valid && rank == 0) wcnt[w][d] = __popc(peers);
    __syncthreads();
    if (valid) {
      int32_t pos = base[d] + rank;
      for (int q = 0; q < w; q++) pos += wcnt[q][d];
      if (key_out) key_out[pos] = k;
      val_out[pos] = v;
    }
    __syncthreads();
    int32_t add = 0;
#pragma unroll
    for (int q = 0; q < W; q++) {
      add += wcnt[q][threadIdx.x];
      wcnt[q][threadIdx.x] = 0;
    }
    base[threadIdx.x] += add;
    __syncthreads();
  }
}

__global__ void k_invert(int64_t n, const int32_t* __restrict__ index, int32_t* __restrict__ inv) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n;
       s += (int64_t)gridDim.x * blockDim.x)
    inv[index[s]] = (int32_t)s;
}

__global__ void k_remap_index(int64_t count, int64_t* __restrict__ index,
                              const int32_t* __restrict__ inv, int64_t n,
                              int32_t* __restrict__ bad) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < count;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = index[t];
    if (r < 0) continue;
    if (r >= n) {
      atomicOr(bad, 1);
      continue;
    }
    index[t] = inv[r];
  }
}

__global__ void k_permute_rows(int64_t n, int ncols, const int32_t* __restrict__ index,
                               const double* __restrict__ X, int64_t ldX, double* __restrict__ Y,
                               int64_t ldY, int32_t* __restrict__ bad) {
  const int64_t total = n * ncols;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = t / n, i = t - c * n;
    const int32_t r = index[i];
    if (r < 0 || r >= n) {  // not a permutation index: flagged, row left as 0
      atomicOr(bad, 1);
      Y[i + c * ldY] = 0.0;
      continue;
    }
    Y[i + c * ldY] = X[(int64_t)r + c * ldX];
  }
}

struct RectGrid {
  int32_t shape[4];
  int64_t coff[4];     // offset of axis k's coordinates in the concatenated array
  int64_t ioffset[4];  // linear-index stride of axis k (first axis fastest)
};

// interp_tetrahedron (ndgrid.F90:464-629) on simplex l of the cell: 3 and the corner weights
// wc when xi lies in it (barycentric coordinates in [-tol, 1 + tol]), 0 when it does not, 2
// when the simplex is degenerate (|det| <= tol)
template <int ND>
__device__ __forceinline__ int solve_simplex(int l, const double* __restrict__ T,
                                             const double (&clo)[ND], const double (&chi)[ND],
                                             const double (&xi)[ND], double (&wc)[1 << ND]) {
  constexpr int K = 1 << ND, NV = ND + 1;
  const double tol = 1e-8;
  // Tl[v * K + c]: corner c's share of vertex v; Ul[k * NV + v]: the share of the corners
  // on the upper side of axis k (the shares of a vertex sum to 1), so that the vertex
  // X(k, v) = sum_c px(k, c) T(c, v) = clo(k) + (chi(k) - clo(k)) U(k, v)
  const double* Tl = T + (int64_t)l * (NV * K + ND * NV);
  const double* Ul = Tl + NV * K;
  double M[NV][NV + 1];
  double xc[ND];
#pragma unroll
  for (int k = 0; k < ND; k++) {
    xc[k] = 0.0;
#pragma unroll
    for (int v = 0; v < NV; v++) {
      const double a = fma(chi[k] - clo[k], Ul[k * NV + v], clo[k]);
      M[1 + k][v] = a;
      xc[k] += a;
    }
  }
#pragma unroll
  for (int v = 0; v < NV; v++) M[0][v] = 1.0;
  M[0][NV] = 1.0;
#pragma unroll
  for (int k = 0; k < ND; k++) {
    xc[k] /= NV;
#pragma unroll
    for (int v = 0; v < NV; v++) M[1 + k][v] -= xc[k];
    M[1 + k][NV] = xi[k] - xc[k];
  }
  // [1; X - xc] c = [1; xi - xc] by Gaussian elimination with partial pivoting
  double det = 1.0;
#pragma unroll
  for (int col = 0; col < NV; col++) {
    int piv = col;
    double best = fabs(M[col][col]);
#pragma unroll
    for (int r = col + 1; r < NV; r++)
      if (fabs(M[r][col]) > best) {
        best = fabs(M[r][col]);
        piv = r;
      }
#pragma unroll
    for (int r = col + 1; r < NV; r++)
      if (r == piv) {
        det = -det;
#pragma unroll
        for (int q = 0; q <= NV; q++) {
          const double t = M[col][q];
          M[col][q] = M[r][q];
          M[r][q] = t;
        }
      }
    det *= M[col][col];
    const double inv = M[col][col] != 0.0 ? 1.0 / M[col][col] : 0.0;
#pragma unroll
    for (int r = col + 1; r < NV; r++) {
      const double f = M[r][col] * inv;
#pragma unroll
      for (int q = col; q <= NV; q++) M[r][q] = fma(-f, M[col][q], M[r][q]);
    }
  }
  if (!(fabs(det) > tol)) return 2;  // every simplex of a rectilinear cell has the same |det|
  double cb[NV];
#pragma unroll
  for (int r = NV - 1; r >= 0; r--) {
    double s = M[r][NV];
#pragma unroll
    for (int q = r + 1; q < NV; q++) s = fma(-M[r][q], cb[q], s);
    cb[r] = s / M[r][r];
  }
  bool inside = true;
#pragma unroll
  for (int v = 0; v < NV; v++) inside = inside && (cb[v] >= -tol) && (cb[v] <= 1.0 + tol);
  if (!inside) return 0;
#pragma unroll
  for (int cc = 0; cc < K; cc++) {
    double a = 0.0;
#pragma unroll
    for (int v = 0; v < NV; v++) a = fma(Tl[v * K + cc], cb[v], a);
    wc[cc] = a;
  }
  return 3;
}

// The simplex of the cell's split holding xi, found directly instead of by trying the
// simplices in turn: in coordinates normalised to the cell ([0, 1] per axis), the pyramid of
// split's first level that holds a point is the one over the face its ray from the centroid
// leaves through (the free axis of largest |p - 1/2|, side p > 1/2); inside it, the simplex is
// the cone over the face simplex holding the point's projection from the centroid onto that
// face, so the same choice repeats on the face. Simplex numbering follows split: per level,
// blocks of (subn - 1)! 2^(subn - 2) simplices in (free axis ascending, side 0 then 1) order.
// Ties go to the lower block, the one split tries first.
template <int ND>
__device__ __forceinline__ int locate_simplex(const double (&clo)[ND], const double (&chi)[ND],
                                              const double (&xi)[ND]) {
  double p[ND];
#pragma unroll
  for (int k = 0; k < ND; k++) p[k] = (xi[k] - clo[k]) / (chi[k] - clo[k]);
  unsigned fixed = 0;
  int l = 0;
#pragma unroll
  for (int subn = ND; subn > 1; subn--) {
    int sub = 1;
    for (int f = 2; f < subn; f++) sub *= f;
    sub <<= (subn - 2);
    int best = 0, best_rank = 0, rank = 0;
    double dev = -1.0;
#pragma unroll
    for (int k = 0; k < ND; k++) {
      if ((fixed >> k) & 1u) continue;
      const double d = fabs(p[k] - 0.5);
      if (d > dev) {
        dev = d;
        best = k;
        best_rank = rank;
      }
      rank++;
    }
    const int side = p[best] > 0.5 ? 1 : 0;
    l += (2 * best_rank + side) * sub;
    if (dev > 0.0) {
      const double t = 0.5 / dev;
#pragma unroll
      for (int k = 0; k < ND; k++)
        if (!((fixed >> k) & 1u) && k != best) p[k] = fma(p[k] - 0.5, t, 0.5);
    }
    p[best] = (double)side;
    fixed |= 1u << best;
  }
  return l;
}

template <int ND>
__global__ void k_rect_oper(RectGrid gr, const double* __restrict__ coords,
                            const int64_t* __restrict__ sea, const double* __restrict__ T,
                            int nsimplex, int64_t m, const double* __restrict__ pos,
                            int64_t offset, int64_t* __restrict__ index,
                            double* __restrict__ weight) {
  constexpr int K = 1 << ND, NV = ND + 1;
  const double tol = 1e-8;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m;
       j += (int64_t)gridDim.x * blockDim.x) {
    double xi[ND], clo[ND], chi[ND];
    int64_t lin0 = 0;
    bool out = false;
#pragma unroll
    for (int k = 0; k < ND; k++) {
      const double x = pos[(int64_t)k * m + j];
      const double* c = coords + gr.coff[k];
      const int32_t nk = gr.shape[k];
      const bool asc = c[nk - 1] > c[0];
      const double cmin = asc ? c[0] : c[nk - 1], cmax = asc ? c[nk - 1] : c[0];
      xi[k] = x;
      int32_t lo = 0;
      if (!(x >= cmin && x <= cmax)) {
        out = true;  // also NaN coordinates
      } else {
        // the cell [c(lo), c(lo+1)] holding x: the largest lo <= nk - 2 with c(lo) on the
        // lower side of x
        int32_t hi = nk - 1;
        while (hi - lo > 1) {
          const int32_t mid = (lo + hi) >> 1;
          if (asc ? (c[mid] <= x) : (c[mid] >= x))
            lo = mid;
          else
            hi = mid;
        }
      }
      clo[k] = c[lo];
      chi[k] = c[lo + 1];
      lin0 += (int64_t)lo * gr.ioffset[k];
    }
    int64_t cidx[K];
#pragma unroll
    for (int cc = 0; cc < K; cc++) {
      int64_t lin = lin0;
#pragma unroll
      for (int k = 0; k < ND; k++)
        if ((cc >> k) & 1) lin += gr.ioffset[k];
      int64_t s = lin;
      if (!out && sea) {
        s = sea[lin];
        if (s < 0) out = true;  // a masked corner (cinterp: out = any(pmasked))
      }
      cidx[cc] = s;
    }
    int status = out ? 1 : 0;  // 0 searching, 1 outside / masked, 2 degenerate cell, 3 found
    double wc[K];
    if (status == 0) {
      const int l0 = locate_simplex<ND>(clo, chi, xi);
      status = solve_simplex<ND>(l0, T, clo, chi, xi, wc);
      // a point on a shared face that rounding put outside the located simplex: split's
      // order, as interp_cube tries the simplices
      for (int l = 0; l < nsimplex && status == 0; l++)
        if (l != l0) status = solve_simplex<ND>(l, T, clo, chi, xi, wc);
    }
#pragma unroll
    for (int cc = 0; cc < K; cc++) {
      index[j * K + cc] = status == 3 ? offset + cidx[cc] : (status == 2 ? -2 : -1);
      weight[j * K + cc] = status == 3 ? wc[cc] : 0.0;
    }
  }
}

// Packed index of the unmasked points: a tile of kScanTile points per block, kPerThread
// consecutive points per thread. Pass 1 counts the tile, the tile counts are scanned, pass 2
// writes the indices.
constexpr int kPerThread = 16;
constexpr int kScanTile = kThreads * kPerThread;

__device__ __forceinline__ int block_excl_scan(int v, int* total) {
  __shared__ int warp_sum[kThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sum[w] = x;
  __syncthreads();
  int before = 0, all = 0;
#pragma unroll
  for (int q = 0; q < kThreads / 32; q++) {
    const int s = warp_sum[q];
    before += q < w ? s : 0;
    all += s;
  }
  __syncthreads();
  *total = all;
  return before + x - v;
}

__global__ void k_sea_tile_count(int64_t npts, const uint8_t* __restrict__ mask,
                                 int32_t* __restrict__ tile_count) {
  const int64_t t0 = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kPerThread;
  int cnt = 0;
#pragma unroll
  for (int q = 0; q < kPerThread; q++) cnt += (t0 + q < npts && !mask[t0 + q]) ? 1 : 0;
  int total;
  block_excl_scan(cnt, &total);
  if (threadIdx.x == 0) tile_count[blockIdx.x] = total;
}

__global__ void k_sea_tile_write(int64_t npts, const uint8_t* __restrict__ mask,
                                 const int32_t* __restrict__ tile_start,
                                 int64_t* __restrict__ sea) {
  const int64_t t0 = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kPerThread;
  uint8_t mk[kPerThread];
  int cnt = 0;
#pragma unroll
  for (int q = 0; q < kPerThread; q++) {
    mk[q] = t0 + q < npts ? mask[t0 + q] : 1;
    cnt += mk[q] ? 0 : 1;
  }
  int total;
  int64_t s = (int64_t)tile_start[blockIdx.x] + block_excl_scan(cnt, &total);
#pragma unroll
  for (int q = 0; q < kPerThread; q++)
    if (t0 + q < npts) {
      sea[t0 + q] = mk[q] ? -1 : s;
      s += mk[q] ? 0 : 1;
    }
}

// exclusive scan of int32 values in tiles of kScanTile (kPerThread consecutive values per
// thread): tile sums, a scan of the sums, then each tile's values from its start
__global__ void k_tile_sum_i32(int64_t n, const int32_t* __restrict__ in,
                               int32_t* __restrict__ tile_sum) {
  const int64_t t0 = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kPerThread;
  int s = 0;
#pragma unroll
  for (int q = 0; q < kPerThread; q++) s += t0 + q < n ? in[t0 + q] : 0;
  int total;
  block_excl_scan(s, &total);
  if (threadIdx.x == 0) tile_sum[blockIdx.x] = total;
}

__global__ void k_tile_scan_i32(int64_t n, const int32_t* __restrict__ in,
                                const int32_t* __restrict__ tile_start,
                                int32_t* __restrict__ out) {
  const int64_t t0 = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kPerThread;
  int v[kPerThread];
  int s = 0;
#pragma unroll
  for (int q = 0; q < kPerThread; q++) {
    v[q] = t0 + q < n ? in[t0 + q] : 0;
    s += v[q];
  }
  int total;
  int32_t run = tile_start[blockIdx.x] + block_excl_scan(s, &total);
#pragma unroll
  for (int q = 0; q < kPerThread; q++)
    if (t0 + q < n) {
      out[t0 + q] = run;
      run += v[q];
      if (t0 + q == n - 1) out[n] = run;
    }
}

// element indices in the stable order of the low 8 * passes bits of key (as unsigned digits)
__global__ void k_flag_new(int64_t n, const int32_t* __restrict__ sorted,
                           int32_t* __restrict__ flag) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n;
       s += (int64_t)gridDim.x * blockDim.x)
    flag[s] = (s == 0 || sorted[s] != sorted[s - 1]) ? 1 : 0;
}

__global__ void k_bias_keys(int64_t n, const int32_t* __restrict__ in, int32_t* __restrict__ out) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n;
       j += (int64_t)gridDim.x * blockDim.x)
    out[j] = (int32_t)((uint32_t)in[j] ^ 0x80000000u);  // signed order as unsigned digits
}

__global__ void k_scatter_rank(int64_t n, const int32_t* __restrict__ perm,
                               const int32_t* __restrict__ rank, const int32_t* __restrict__ flag,
                               int32_t* __restrict__ out) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n;
       s += (int64_t)gridDim.x * blockDim.x)
    out[perm[s]] = rank[s] + flag[s];
}

int64_t scan_tiles(int64_t n) { return (n + kScanTile - 1) / kScanTile; }

// out[0..n] = exclusive scan of in[0..n), out[n] the total; tiles: 2 (scan_tiles(n) + 1) int32
cudaError_t scan_tiled_i32(int64_t n, const int32_t* in, int32_t* out, int32_t* tiles,
                           cudaStream_t st) {
  const int64_t nt = scan_tiles(n);
  int32_t* sum = tiles;
  int32_t* start = tiles + nt + 1;
  k_tile_sum_i32<<<(unsigned)nt, kThreads, 0, st>>>(n, in, sum);
  count_launches(1);
  cudaError_t e = scan_exclusive_i32(sum, nt, start, st);
  if (e != cudaSuccess) return e;
  k_tile_scan_i32<<<(unsigned)nt, kThreads, 0, st>>>(n, in, start, out);
  count_launches(1);
  return cudaGetLastError();
}

// scratch of radix_sort_index, in int32
int64_t radix_work(int64_t n) {
  const int64_t ntiles = (n + kRadixTile - 1) / kRadixTile, nh = kThreads * ntiles;
  return 3 * n + 2 * (nh + 1) + 2 * (scan_tiles(nh) + 1);
}

// Stable LSD radix sort over the low 8 * passes bits of key: vals_out[s] = the element at sorted
// position s; keys_out (optional) the sorted keys.
cudaError_t radix_sort_index(int64_t n, const int32_t* key, int passes, int32_t* work,
                             int32_t* vals_out, int32_t* keys_out, cudaStream_t st) {
  const int64_t ntiles = (n + kRadixTile - 1) / kRadixTile, nh = kThreads * ntiles;
  int32_t* kA = work;
  int32_t* kB = kA + n;
  int32_t* vtmp = kB + n;
  int32_t* hist = vtmp + n;
  int32_t* offs = hist + nh + 1;
  int32_t* tiles = offs + nh + 1;
  const int32_t* kin = key;
  const int32_t* vin = nullptr;
  cudaError_t e = cudaSuccess;
  for (int p = 0; p < passes; p++) {
    const bool last = p == passes - 1;
    int32_t* vout = ((passes - 1 - p) % 2 == 0) ? vals_out : vtmp;  // the last pass: vals_out
    int32_t* kout = last ? keys_out : (p % 2 == 0 ? kA : kB);
    k_radix_hist<<<(unsigned)ntiles, kThreads, 0, st>>>(n, kin, 8 * p, hist, ntiles);
    count_launches(1);
    if ((e = scan_tiled_i32(nh, hist, offs, tiles, st)) != cudaSuccess) return e;
    k_radix_scatter<<<(unsigned)ntiles, kThreads, 0, st>>>(n, kin, vin, 8 * p, offs, ntiles,
                                                           kout, vout);
    count_launches(1);
    kin = kout;
    vin = vout;
  }
  return cudaGetLastError();
}

}  // namespace

int64_t zone_layout_work(int64_t n, int32_t nzones) {
  return n + 2 * ((int64_t)nzones + 1) + radix_work(n) + 4;
}

cudaError_t zone_layout(int64_t n, const int32_t* d_partition, int32_t nzones, int32_t* d_work,
                        int32_t* d_zone_size, int32_t* d_zone_index, int32_t* d_inv_index,
                        int32_t* d_bad, cudaStream_t st) {
  int32_t* key = d_work;
  int32_t* count = key + n;
  int32_t* start = count + nzones + 1;
  int32_t* rwork = start + nzones + 1;
  k_zone_keys<<<grid_for(n), kThreads, 0, st>>>(n, d_partition, key);
  cudaError_t e = cudaMemsetAsync(count, 0, ((size_t)nzones + 1) * sizeof(int32_t), st);
  if (e != cudaSuccess) return e;
  k_key_count_i32<<<grid_for(n), kThreads, 0, st>>>(n, key, nzones, count, d_bad);
  count_launches(2);
  if ((e = scan_tiled_i32(nzones, count, start, rwork, st)) != cudaSuccess) return e;
  k_zone_sizes<<<grid_for(nzones), kThreads, 0, st>>>(nzones, start, d_zone_size, d_bad);
  count_launches(1);
  int bits = 1;
  while (bits < 31 && ((int64_t)1 << bits) < (int64_t)nzones) bits++;
  if ((e = radix_sort_index(n, key, (bits + 7) / 8, rwork, d_zone_index, nullptr, st)) !=
      cudaSuccess)
    return e;
  if (d_inv_index) {
    k_invert<<<grid_for(n), kThreads, 0, st>>>(n, d_zone_index, d_inv_index);
    count_launches(1);
  }
  return cudaGetLastError();
}

int64_t partition_compact_work(int64_t n) { return 5 * n + 1 + radix_work(n) + 4; }

cudaError_t partition_compact(int64_t n, const int32_t* d_labels, int32_t* d_work,
                              int32_t* d_out, cudaStream_t st) {
  int32_t* key = d_work;
  int32_t* perm = key + n;
  int32_t* sorted = perm + n;
  int32_t* flag = sorted + n;
  int32_t* rank = flag + n;  // n + 1, rank[n] = number of distinct labels
  int32_t* rwork = rank + n + 1;
  k_bias_keys<<<grid_for(n), kThreads, 0, st>>>(n, d_labels, key);
  count_launches(1);
  cudaError_t e = radix_sort_index(n, key, 4, rwork, perm, sorted, st);
  if (e != cudaSuccess) return e;
  k_flag_new<<<grid_for(n), kThreads, 0, st>>>(n, sorted, flag);
  count_launches(1);
  if ((e = scan_tiled_i32(n, flag, rank, rwork, st)) != cudaSuccess) return e;
  k_scatter_rank<<<grid_for(n), kThreads, 0, st>>>(n, perm, rank, flag, d_out);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t permute_rows(int64_t n, int ncols, const int32_t* d_index, const double* X,
                         int64_t ldX, double* Y, int64_t ldY, int32_t* d_bad, cudaStream_t st) {
  k_permute_rows<<<grid_for(n * ncols), kThreads, 0, st>>>(n, ncols, d_index, X, ldX, Y, ldY,
                                                          d_bad);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t remap_index(int64_t count, int64_t* d_index, const int32_t* d_inv, int64_t n,
                        int32_t* d_bad, cudaStream_t st) {
  k_remap_index<<<grid_for(count), kThreads, 0, st>>>(count, d_index, d_inv, n, d_bad);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t sea_index(int64_t npts, const uint8_t* d_mask, int32_t* d_tiles, int64_t* d_sea,
                      cudaStream_t st) {
  // d_tiles: 2 (ntiles + 1) int32 (tile counts, then their exclusive scan)
  const int64_t ntiles = (npts + kScanTile - 1) / kScanTile;
  if (ntiles > INT32_MAX / 2) return cudaErrorInvalidValue;
  int32_t* count = d_tiles;
  int32_t* start = d_tiles + (ntiles + 1);
  k_sea_tile_count<<<(unsigned)ntiles, kThreads, 0, st>>>(npts, d_mask, count);
  count_launches(1);
  cudaError_t e = scan_exclusive_i32(count, ntiles, start, st);
  if (e != cudaSuccess) return e;
  k_sea_tile_write<<<(unsigned)ntiles, kThreads, 0, st>>>(npts, d_mask, start, d_sea);
  count_launches(1);
  return cudaGetLastError();
}

int64_t sea_index_tiles(int64_t npts) { return (npts + kScanTile - 1) / kScanTile; }

cudaError_t rectilinear_oper(int ndim, const int32_t* shape, const double* d_coords,
                             const int64_t* d_sea, const double* d_simplex, int nsimplex,
                             int64_t m, const double* d_pos, int64_t offset, int64_t* d_index,
                             double* d_weight, cudaStream_t st) {
  RectGrid gr{};
  int64_t co = 0, io = 1;
  for (int k = 0; k < ndim; k++) {
    gr.shape[k] = shape[k];
    gr.coff[k] = co;
    gr.ioffset[k] = io;
    co += shape[k];
    io *= shape[k];
  }
  const unsigned g = grid_for(m);
  switch (ndim) {
    case 1: k_rect_oper<1><<<g, kThreads, 0, st>>>(gr, d_coords, d_sea, d_simplex, nsimplex, m,
                                                  d_pos, offset, d_index, d_weight); break;
    case 2: k_rect_oper<2><<<g, kThreads, 0, st>>>(gr, d_coords, d_sea, d_simplex, nsimplex, m,
                                                  d_pos, offset, d_index, d_weight); break;
    case 3: k_rect_oper<3><<<g, kThreads, 0, st>>>(gr, d_coords, d_sea, d_simplex, nsimplex, m,
                                                  d_pos, offset, d_index, d_weight); break;
    case 4: k_rect_oper<4><<<g, kThreads, 0, st>>>(gr, d_coords, d_sea, d_simplex, nsimplex, m,
                                                  d_pos, offset, d_index, d_weight); break;
    default: return cudaErrorInvalidValue;
  }
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace oakg
