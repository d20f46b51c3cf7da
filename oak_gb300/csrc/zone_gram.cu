// K1 + K2 -- per-zone observation selection and the Gram / innovation products. Selection is
// always FP64 (the same decisions as a CPU evaluation of the reference); the products are
// accumulated in R: double for the plain form, float for the mixed-precision form (with
// compensated (Kahan) sums for the innovation projection).
//
// For zone z (one CTA at a time, zones handed out by an atomic work counter):
//   selection  (assimilation.F90:3683-3771): d = distance(obs, zone) for loctype 1 (metric
//              0/1/2, assimilation.F90:3635-3672), |dz| (loctype 2) or |dt| (loctype 3);
//              relevant = d <= maxLength;  w = exp(-(d/L)^2)            (Gaussian, :3767)
//              or w = locfun(d/L), relevant also needs w /= 0        (Gaspari-Cohn,
//              covariance.F90:645-667, the rule of test/test_rrsqrt.F90:268-269)
//   R^-1_eff   DCDCovar with D = w over DiagCovar R (rrsqrt.F90:395, covariance.F90:612-619,
//              :425-432): c_q = w_q (w_q / r_q)
//   Gram       G = HS_sel^T diag(c) HS_sel      (rrsqrt.F90:135, N x N, lower triangle
//              accumulated, both triangles stored)
//   innovation g = HS_sel^T diag(c) (yo - Hxf)_sel   (the inner product of :142)
//
// Non-diagonal R of the SMWCovar kind (R = diag(C) + B B^T, covariance.F90:464-570): the rows
// are augmented, [HS_q | B_q] (N + k columns, nx = N weighted ones), staged as
// sh = s_j h, st = s_j h / C_q with s_j = w_q for j < nx and 1 beyond, and the innovation as
// w_q d_q / C_q; the products are then the blocks X^T X, X^T Y, Y^T Y, X^T z, Y^T z of
// X = C^-1/2 W HS, Y = C^-1/2 B, z = C^-1/2 W d that the Woodbury reduction (zone_smw.cu)
// turns into the zone's Gram matrix and innovation projection.
//
// Only the cells of the observation grid that can contain observations within maxLength are
// visited (cell rows are contiguous ranges of the cell-sorted arrays); with
// OAKG_FLAG_BRUTE_SEARCH or localise_obs = false every observation is visited, which is the
// reference's own loop. Work per zone: 2 p N^2/2 + 2 p N FP64 flops; the FP64 pipe bounds it.
#include <cuda_runtime.h>
#include <math.h>

#include "oakg_internal.cuh"
#include "selection.cuh"

namespace oakg {

namespace {

constexpr int kThreads = 256;
constexpr int kListCap = 512;   // selected-observation staging list (flushed at >= 256)
constexpr int kFlushAt = 256;
struct ZoneShared {
  int32_t list_q[kListCap];
  double list_c[kListCap];  // c = w (w / r), or w itself for augmented (SMW) rows
  int32_t warp_cnt[kThreads / 32];
  int32_t list_len;
  int32_t nrel;
  int32_t zone;
};

// Accumulate the staged observations list[0..len) into the per-thread Gram entries.
template <int MAXE, typename R>
__device__ __forceinline__ void flush_list(ZoneShared& zs, int len, const SortedObs& so, int N,
                                           int CH, R* sh, R* st, R* sinn,
                                           const int32_t (&ea)[MAXE], const int32_t (&eb)[MAXE],
                                           R (&acc)[MAXE], R (&cmp)[MAXE], int E, int nent,
                                           int nx) {
  for (int c0 = 0; c0 < len; c0 += CH) {
    int rows = min(CH, len - c0);
    __syncthreads();  // previous chunk fully consumed
    if (nx >= N) {
      for (int idx = threadIdx.x; idx < rows * N; idx += kThreads) {
        int i = idx / N, k = idx - i * N;
        int32_t q = zs.list_q[c0 + i];
        double h = so.HSt[(int64_t)q * N + k];
        sh[i * N + k] = (R)h;
        st[i * N + k] = (R)(zs.list_c[c0 + i] * h);
      }
      for (int i = threadIdx.x; i < rows; i += kThreads) {
        int32_t q = zs.list_q[c0 + i];
        sinn[i] = (R)(zs.list_c[c0 + i] * so.innov[q]);
      }
    } else {  // augmented rows [HS_q | B_q]: list_c holds w_q
      for (int idx = threadIdx.x; idx < rows * N; idx += kThreads) {
        int i = idx / N, k = idx - i * N;
        int32_t q = zs.list_q[c0 + i];
        const double h = so.HSt[(int64_t)q * N + k] * ((k < nx) ? zs.list_c[c0 + i] : 1.0);
        sh[i * N + k] = (R)h;
        st[i * N + k] = (R)(h / so.r[q]);
      }
      for (int i = threadIdx.x; i < rows; i += kThreads) {
        int32_t q = zs.list_q[c0 + i];
        sinn[i] = (R)(zs.list_c[c0 + i] * so.innov[q] / so.r[q]);
      }
    }
    __syncthreads();
#pragma unroll
    for (int s = 0; s < MAXE; s++) {
      int e = threadIdx.x + s * kThreads;
      if (e < nent) {
        R a = acc[s];
        const int ia = ea[s], ib = eb[s];
        if (e < E) {
          for (int i = 0; i < rows; i++) a = fma(sh[i * N + ia], st[i * N + ib], a);
        } else if (sizeof(R) == sizeof(double)) {
          for (int i = 0; i < rows; i++) a = fma(sh[i * N + ia], sinn[i], a);
        } else {
          // compensated (Kahan) sum of the innovation projection in FP32
          R c = cmp[s];
          for (int i = 0; i < rows; i++) {
            const R y = sh[i * N + ia] * sinn[i] - c;
            const R t = a + y;
            c = (t - a) - y;
            a = t;
          }
          cmp[s] = c;
        }
        acc[s] = a;
      }
    }
  }
}

template <int MAXE, typename R>
__global__ void __launch_bounds__(kThreads)
    k_zone_gram(CellGrid g, SortedObs so, int N, LocParams lp, int32_t z0, int32_t nzc,
                const double* __restrict__ zone_xyzt, const double* __restrict__ corr_len,
                const double* __restrict__ max_len, R* __restrict__ G, R* __restrict__ gv,
                int32_t* __restrict__ nobs, int brute, int CH, int32_t* __restrict__ work,
                const int32_t* __restrict__ zlist, const int32_t* __restrict__ order, int nx) {
  extern __shared__ __align__(16) unsigned char dyn_raw[];
  R* dyn = reinterpret_cast<R*>(dyn_raw);
  R* sh = dyn;            // [CH][N]
  R* st = sh + CH * N;    // [CH][N]
  R* sinn = st + CH * N;  // [CH]
  __shared__ ZoneShared zs;

  const int E = N * (N + 1) / 2;
  const int nent = E + N;
  int32_t ea[MAXE], eb[MAXE];
#pragma unroll
  for (int s = 0; s < MAXE; s++) {
    int e = threadIdx.x + s * kThreads;
    if (e < E) {
      int a = (int)((__fsqrt_rn((float)(8 * e + 1)) - 1.0f) * 0.5f);
      while ((a + 1) * (a + 2) / 2 <= e) a++;
      while (a * (a + 1) / 2 > e) a--;
      ea[s] = a;
      eb[s] = e - a * (a + 1) / 2;
    } else {
      ea[s] = (e < nent) ? e - E : 0;
      eb[s] = 0;
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t ncells = (int64_t)g.nu * g.nv;
  const int full_scan = brute || !lp.localise;

  for (;;) {
    if (threadIdx.x == 0) zs.zone = atomicAdd(work, 1);
    __syncthreads();
    const int32_t w = zs.zone;  // pick number; zone order[z0 + w] when a pick order is given
    if (w >= nzc) break;
    const int32_t zl = order ? order[z0 + w] : w;
    const int32_t z = zlist ? zlist[zl] : z0 + zl;
    const double zx = zone_xyzt[4 * (int64_t)z + 0], zy = zone_xyzt[4 * (int64_t)z + 1];
    const double zzc = zone_xyzt[4 * (int64_t)z + 2], ztc = zone_xyzt[4 * (int64_t)z + 3];
    const double zu = (lp.loctype == 1) ? zx : (lp.loctype == 2 ? zzc : ztc);
    const double zv = (lp.loctype == 1) ? zy : 0.0;
    const double L = corr_len[z], Rmax = max_len[z];
    if (threadIdx.x == 0) {
      zs.list_len = 0;
      zs.nrel = 0;
    }
    R acc[MAXE], cmp[MAXE];
#pragma unroll
    for (int s = 0; s < MAXE; s++) acc[s] = cmp[s] = R(0);

    sel::ScanRange sr;
    if (full_scan) {
      sr.cu0 = 0;
      sr.cu1 = g.nu - 1;
      sr.cv0 = 0;
      sr.cv1 = g.nv - 1;
      sr.all_u = 1;
    } else {
      sr = sel::zone_scan_range(g, lp.metric, lp.loctype, zu, zv, Rmax);
    }
    __syncthreads();
    int nrel_local = 0;
    // Segments: one per cell row (two when a periodic range wraps).
    for (int cv = sr.cv0; cv <= sr.cv1; cv++) {
      for (int part = 0; part < 2; part++) {
        int cu_a, cu_b;
        if (sr.all_u) {
          if (part) break;
          cu_a = 0;
          cu_b = g.nu - 1;
        } else if (!g.periodic_u) {
          if (part) break;
          cu_a = sr.cu0;
          cu_b = sr.cu1;
        } else {
          // periodic: [cu0, cu1] may extend below 0 or above nu-1
          int a0 = sr.cu0, b0 = sr.cu1;
          if (a0 < 0) {
            if (part == 0) { cu_a = a0 + g.nu; cu_b = g.nu - 1; }
            else { cu_a = 0; cu_b = b0; }
          } else if (b0 >= g.nu) {
            if (part == 0) { cu_a = a0; cu_b = g.nu - 1; }
            else { cu_a = 0; cu_b = b0 - g.nu; }
          } else {
            if (part) break;
            cu_a = a0;
            cu_b = b0;
          }
        }
        const int64_t c_lo = (int64_t)cu_a + (int64_t)g.nu * cv;
        const int64_t c_hi = (int64_t)cu_b + (int64_t)g.nu * cv;
        if (c_lo > c_hi || c_lo < 0 || c_hi >= ncells) continue;
        const int32_t q_lo = so.cell_start[c_lo], q_hi = so.cell_start[c_hi + 1];
        for (int32_t qb = q_lo; qb < q_hi; qb += kThreads) {
          const int32_t q = qb + threadIdx.x;
          int sel = 0, rel = 0;
          double c = 0.0;
          if (q < q_hi) {
            double d;
            if (lp.loctype == 1)
              d = sel::distance(so.u[q], so.v[q], zu, zv, lp.metric);
            else
              d = fabs(__dsub_rn(so.u[q], zu));
            double w;
            if (lp.weight == OAKG_WEIGHT_GAUSS_CUTOFF) {
              rel = (d <= Rmax);
              double t = d / L;
              w = (rel || !lp.localise) ? exp(-(t * t)) : 0.0;
            } else {
              w = sel::locfun(d / L);
              rel = (d <= Rmax) && (w != 0.0);
            }
            sel = rel || !lp.localise;
            if (sel) c = (nx >= N) ? w * (w / so.r[q]) : w;
          }
          nrel_local += rel;
          unsigned ball = __ballot_sync(0xffffffffu, sel);
          if (lane == 0) zs.warp_cnt[warp] = __popc(ball);
          __syncthreads();
          int base = zs.list_len, before = 0, total = 0;
          for (int w2 = 0; w2 < kThreads / 32; w2++) {
            int cnt = zs.warp_cnt[w2];
            before += (w2 < warp) ? cnt : 0;
            total += cnt;
          }
          if (sel) {
            int slot = base + before + __popc(ball & ((1u << lane) - 1u));
            zs.list_q[slot] = q;
            zs.list_c[slot] = c;
          }
          __syncthreads();
          if (threadIdx.x == 0) zs.list_len = base + total;
          __syncthreads();
          if (zs.list_len >= kFlushAt) {
            int len = zs.list_len;
            flush_list<MAXE, R>(zs, len, so, N, CH, sh, st, sinn, ea, eb, acc, cmp, E, nent, nx);
            __syncthreads();
            if (threadIdx.x == 0) zs.list_len = 0;
            __syncthreads();
          }
        }
      }
    }
    if (zs.list_len > 0) {
      int len = zs.list_len;
      flush_list<MAXE, R>(zs, len, so, N, CH, sh, st, sinn, ea, eb, acc, cmp, E, nent, nx);
    }
    // relevant-observation count of the zone
    for (int o = 16; o > 0; o >>= 1) nrel_local += __shfl_xor_sync(0xffffffffu, nrel_local, o);
    if (lane == 0) atomicAdd(&zs.nrel, nrel_local);
    __syncthreads();
    const int nrel = zs.nrel;
    if (threadIdx.x == 0) nobs[z] = nrel;
    if (nrel > 0) {
      R* Gz = G + (int64_t)zl * N * N;
#pragma unroll
      for (int s = 0; s < MAXE; s++) {
        int e = threadIdx.x + s * kThreads;
        if (e < E) {
          Gz[ea[s] * N + eb[s]] = acc[s];
          Gz[eb[s] * N + ea[s]] = acc[s];
        } else if (e < nent) {
          gv[(int64_t)zl * N + ea[s]] = acc[s];
        }
      }
    }
    __syncthreads();
  }
}

// Global analysis (rrsqrt.F90:196-208): every observation, D = 1 (DiagCovar): c_j = 1/r_j.
// Observations in chunks of CH; partial sums per CTA added atomically into G (zeroed).
template <int MAXE>
__global__ void __launch_bounds__(kThreads)
    k_global_gram_fp64(int64_t m, int N, const double* __restrict__ HSf, int64_t ldH,
                       const double* __restrict__ yo, const double* __restrict__ Hxf,
                       const double* __restrict__ r, double* __restrict__ G,
                       double* __restrict__ gv, int CH) {
  extern __shared__ double dyn[];
  double* sh = dyn;
  double* st = sh + CH * N;
  double* sinn = st + CH * N;
  const int E = N * (N + 1) / 2;
  const int nent = E + N;
  int32_t ea[MAXE], eb[MAXE];
  double acc[MAXE];
#pragma unroll
  for (int s = 0; s < MAXE; s++) {
    int e = threadIdx.x + s * kThreads;
    acc[s] = 0.0;
    if (e < E) {
      int a = (int)((__fsqrt_rn((float)(8 * e + 1)) - 1.0f) * 0.5f);
      while ((a + 1) * (a + 2) / 2 <= e) a++;
      while (a * (a + 1) / 2 > e) a--;
      ea[s] = a;
      eb[s] = e - a * (a + 1) / 2;
    } else {
      ea[s] = (e < nent) ? e - E : 0;
      eb[s] = 0;
    }
  }
  for (int64_t j0 = (int64_t)blockIdx.x * CH; j0 < m; j0 += (int64_t)gridDim.x * CH) {
    int rows = (int)((m - j0 < CH) ? (m - j0) : CH);
    __syncthreads();
    for (int idx = threadIdx.x; idx < rows * N; idx += kThreads) {
      int k = idx / rows, i = idx - k * rows;  // coalesced along observations
      double h = HSf[j0 + i + (int64_t)k * ldH];
      double c = 1.0 / r[j0 + i];
      sh[i * N + k] = h;
      st[i * N + k] = c * h;
    }
    for (int i = threadIdx.x; i < rows; i += kThreads)
      sinn[i] = (1.0 / r[j0 + i]) * (yo[j0 + i] - Hxf[j0 + i]);
    __syncthreads();
#pragma unroll
    for (int s = 0; s < MAXE; s++) {
      int e = threadIdx.x + s * kThreads;
      if (e < nent) {
        double a = acc[s];
        const int ia = ea[s], ib = eb[s];
        if (e < E) {
          for (int i = 0; i < rows; i++) a = fma(sh[i * N + ia], st[i * N + ib], a);
        } else {
          for (int i = 0; i < rows; i++) a = fma(sh[i * N + ia], sinn[i], a);
        }
        acc[s] = a;
      }
    }
  }
#pragma unroll
  for (int s = 0; s < MAXE; s++) {
    int e = threadIdx.x + s * kThreads;
    if (e < E) {
      atomicAdd(&G[ea[s] * N + eb[s]], acc[s]);
      if (ea[s] != eb[s]) atomicAdd(&G[eb[s] * N + ea[s]], acc[s]);
    } else if (e < nent) {
      atomicAdd(&gv[ea[s]], acc[s]);
    }
  }
}

inline int chunk_rows(int N) {
  int ch = 4096 / N;
  if (ch > 128) ch = 128;
  if (ch < 8) ch = 8;
  return ch;
}

template <int MAXE, typename R>
cudaError_t launch_zone(const CellGrid& g, const SortedObs& so, int N, LocParams lp, int32_t z0,
                        int32_t nzc, const double* zone_xyzt, const double* corr_len,
                        const double* max_len, R* d_G, R* d_g, int32_t* d_nobs,
                        int brute, int32_t* d_work, cudaStream_t st,
                        const int32_t* zlist = nullptr, const int32_t* order = nullptr,
                        int nx = -1) {
  int CH = chunk_rows(N);
  size_t smem = (size_t)(2 * CH * N + CH) * sizeof(R);
  cudaError_t e = cudaFuncSetAttribute(k_zone_gram<MAXE, R>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int blocks_per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k_zone_gram<MAXE, R>,
                                                    kThreads, smem);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int grid = sms * (blocks_per_sm > 0 ? blocks_per_sm : 1);
  if (grid > nzc) grid = nzc > 0 ? nzc : 1;
  e = cudaMemsetAsync(d_work, 0, sizeof(int32_t), st);
  if (e != cudaSuccess) return e;
  k_zone_gram<MAXE, R><<<grid, kThreads, smem, st>>>(g, so, N, lp, z0, nzc, zone_xyzt, corr_len,
                                                      max_len, d_G, d_g, d_nobs, brute, CH,
                                                      d_work, zlist, order, nx < 0 ? N : nx);
  count_launches(1);
  return cudaGetLastError();
}

template <int MAXE>
cudaError_t launch_global(int64_t m, int N, const double* HSf, int64_t ldH, const double* yo,
                          const double* Hxf, const double* r, double* d_G, double* d_g,
                          cudaStream_t st) {
  int CH = chunk_rows(N);
  size_t smem = (size_t)(2 * CH * N + CH) * sizeof(double);
  cudaError_t e = cudaFuncSetAttribute(k_global_gram_fp64<MAXE>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int64_t chunks = (m + CH - 1) / CH;
  int grid = (int)(chunks < 152 * 2 ? (chunks < 1 ? 1 : chunks) : 152 * 2);
  e = cudaMemsetAsync(d_G, 0, sizeof(double) * N * N, st);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(d_g, 0, sizeof(double) * N, st);
  if (e != cudaSuccess) return e;
  k_global_gram_fp64<MAXE><<<grid, kThreads, smem, st>>>(m, N, HSf, ldH, yo, Hxf, r, d_G, d_g,
                                                          CH);
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace

int max_fp64_ensemble() { return 128; }
int max_ensemble() { return 128; }

// Per-thread entry count classes: ceil((N(N+1)/2 + N) / 256).
#define OAKG_GRAM_DISPATCH(FN, ...)                                         \
  do {                                                                      \
    int ent_ = N * (N + 1) / 2 + N;                                         \
    int per_ = (ent_ + kThreads - 1) / kThreads;                            \
    if (per_ <= 3) return FN<3>(__VA_ARGS__);                               \
    if (per_ <= 9) return FN<9>(__VA_ARGS__);                               \
    if (per_ <= 19) return FN<19>(__VA_ARGS__);                             \
    if (per_ <= 26) return FN<26>(__VA_ARGS__);                             \
    if (per_ <= 33) return FN<33>(__VA_ARGS__);                             \
    return cudaErrorInvalidValue;                                           \
  } while (0)
#define OAKG_GRAM_DISPATCH_T(FN, R, ...)                                    \
  do {                                                                      \
    int ent_ = N * (N + 1) / 2 + N;                                         \
    int per_ = (ent_ + kThreads - 1) / kThreads;                            \
    if (per_ <= 3) return FN<3, R>(__VA_ARGS__);                            \
    if (per_ <= 9) return FN<9, R>(__VA_ARGS__);                            \
    if (per_ <= 19) return FN<19, R>(__VA_ARGS__);                          \
    if (per_ <= 26) return FN<26, R>(__VA_ARGS__);                          \
    if (per_ <= 33) return FN<33, R>(__VA_ARGS__);                          \
    return cudaErrorInvalidValue;                                           \
  } while (0)

cudaError_t zone_gram_fp64(const CellGrid& g, const SortedObs& so, int N, LocParams lp,
                           int32_t z0, int32_t nzc, const double* zone_xyzt,
                           const double* corr_len, const double* max_len, double* d_G,
                           double* d_g, int32_t* d_nobs, int brute, int32_t* d_work,
                           cudaStream_t st, const int32_t* order) {
  OAKG_GRAM_DISPATCH_T(launch_zone, double, g, so, N, lp, z0, nzc, zone_xyzt, corr_len, max_len,
                       d_G, d_g, d_nobs, brute, d_work, st, nullptr, order);
}

cudaError_t zone_gram_fp32(const CellGrid& g, const SortedObs& so, int N, LocParams lp,
                           int32_t z0, int32_t nzc, const double* zone_xyzt,
                           const double* corr_len, const double* max_len, float* d_G,
                           float* d_g, int32_t* d_nobs, int brute, int32_t* d_work,
                           cudaStream_t st, const int32_t* order) {
  OAKG_GRAM_DISPATCH_T(launch_zone, float, g, so, N, lp, z0, nzc, zone_xyzt, corr_len, max_len,
                       d_G, d_g, d_nobs, brute, d_work, st, nullptr, order);
}

cudaError_t zone_gram_fp64_aug(const CellGrid& g, const SortedObs& so, int N, int nx,
                               LocParams lp, int32_t z0, int32_t nzc, const double* zone_xyzt,
                               const double* corr_len, const double* max_len, double* d_G,
                               double* d_g, int32_t* d_nobs, int brute, int32_t* d_work,
                               cudaStream_t st) {
  OAKG_GRAM_DISPATCH_T(launch_zone, double, g, so, N, lp, z0, nzc, zone_xyzt, corr_len, max_len,
                       d_G, d_g, d_nobs, brute, d_work, st, nullptr, nullptr, nx);
}

cudaError_t zone_gram_fp64_list(const CellGrid& g, const SortedObs& so, int N, LocParams lp,
                                const int32_t* zlist, int32_t nzc, const double* zone_xyzt,
                                const double* corr_len, const double* max_len, double* d_G,
                                double* d_g, int32_t* d_nobs, int brute, int32_t* d_work,
                                cudaStream_t st) {
  OAKG_GRAM_DISPATCH_T(launch_zone, double, g, so, N, lp, 0, nzc, zone_xyzt, corr_len, max_len,
                       d_G, d_g, d_nobs, brute, d_work, st, zlist);
}

cudaError_t global_gram_fp64(int64_t m, int N, const double* HSf, int64_t ldH,
                             const double* yo, const double* Hxf, const double* r, double* d_G,
                             double* d_g, cudaStream_t st) {
  OAKG_GRAM_DISPATCH(launch_global, m, N, HSf, ldH, yo, Hxf, r, d_G, d_g, st);
}

}  // namespace oakg
