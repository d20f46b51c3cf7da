// K6 (FP64) -- adjoint of the analysis mean of locAnalysis.
//
// No counterpart in the reference, which has no derivative code. The forward mean of a zone
// is (rrsqrt.F90:142,151; the rotation and the lambda clamp leave the mean unchanged up to
// rounding):
//   xa_z = xf_z + s Sf_z A^-1 g',   A = I + s^2 G,   g' = s g,
//   G = sum_q c_q h_q h_q^T,  g = sum_q c_q d_q h_q,  c_q = w_q^2 / r_q,  d_q = yo_q - Hxf_q,
// with s the prior anomaly scaling (inflation of Sf and HSf before the analysis) and h_q the
// row of HSf of a selected observation. Given a = dJ/dxa_z (the seed) the zone contributes
//   b = s Sf_z^T a,  y = A^-1 b,  ampl = A^-1 g',  t1 = s h_q^T y,  t2 = s h_q^T ampl
//   dJ/dyo_q += c_q t1                        dJ/dc_q = t1 (d_q - t2)
//   dJ/dr_q  += dJ/dc_q (-c_q / r_q)          dJ/dkappa += dJ/dc_q (2 w_q / r_q) dw_q/dkappa
//   dJ/ds    += (b^T ampl + sum_q c_q t1 (d_q - 2 t2)) / s
// where kappa multiplies every zone's correlation and maximum length (derivative at 1):
// Gaussian w = exp(-t^2): dw/dkappa = 2 t^2 exp(-t^2); Gaspari-Cohn w = locfun(t):
// dw/dkappa = -t locfun'(t), t = d/L. The selected set is held fixed; with Gaspari-Cohn the
// weight and its slope vanish at the cut-off, so nothing is lost there.
//
// A is factorised per zone (Cholesky, in shared memory) from G recomputed by the forward
// selection + Gram kernel for the seeded zones only; no eigensystem is stored.
#include <cuda_runtime.h>
#include <math.h>

#include "oakg_internal.cuh"
#include "selection.cuh"

namespace oakg {

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;

__device__ __forceinline__ double warp_sum(double x) {
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// block-wide sum of x; every thread gets the result
__device__ double block_sum(double x, double* red) {
  x = warp_sum(x);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x < 32) {
    t = (threadIdx.x < kWarps) ? red[threadIdx.x] : 0.0;
    t = warp_sum(t);
    if (threadIdx.x == 0) red[kWarps] = t;
  }
  __syncthreads();
  return red[kWarps];
}

__global__ void k_zone_flags(const double* __restrict__ seed,
                             const int64_t* __restrict__ zone_start, int32_t Z,
                             int32_t* __restrict__ flag) {
  for (int32_t z = blockIdx.x * blockDim.x + threadIdx.x; z < Z; z += gridDim.x * blockDim.x) {
    int f = 0;
    for (int64_t i = zone_start[z]; i < zone_start[z + 1] && !f; i++) f = (seed[i] != 0.0);
    flag[z] = f;
  }
}

// one block: exclusive scan of the flags -> positions, then the compacted zone list;
// pos[Z] = number of seeded zones
__global__ void k_zone_compact(const int32_t* __restrict__ flag, int32_t Z,
                               int32_t* __restrict__ pos, int32_t* __restrict__ list) {
  __shared__ int32_t s[1024];
  __shared__ int32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int32_t base = 0; base < Z; base += 1024) {
    const int32_t i = base + threadIdx.x;
    const int32_t x = (i < Z) ? flag[i] : 0;
    s[threadIdx.x] = x;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
      int32_t t = (threadIdx.x >= off) ? s[threadIdx.x - off] : 0;
      __syncthreads();
      s[threadIdx.x] += t;
      __syncthreads();
    }
    const int32_t p = carry + s[threadIdx.x] - x;
    if (i < Z) {
      pos[i] = p;
      if (x) list[p] = i;
    }
    __syncthreads();
    if (threadIdx.x == 1023) carry += s[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0) pos[Z] = carry;
}

__global__ void __launch_bounds__(kThreads)
    k_zone_adjoint(CellGrid g, SortedObs so, int N, LocParams lp,
                   const int32_t* __restrict__ zlist, int32_t nzc,
                   const double* __restrict__ zone_xyzt, const double* __restrict__ corr_len,
                   const double* __restrict__ max_len, const int64_t* __restrict__ zone_start,
                   const double* __restrict__ Sf, int64_t ldS, const double* __restrict__ seed,
                   double s, const double* __restrict__ G, const double* __restrict__ gv,
                   const int32_t* __restrict__ nobs, double* __restrict__ dyo,
                   double* __restrict__ dr, double* __restrict__ dscal, int brute,
                   int32_t* __restrict__ work) {
  extern __shared__ double dyn[];
  const int ld = N + 1;
  double* A = dyn;           // [N][ld] I + s^2 G, then its Cholesky factor L (lower)
  double* am = A + N * ld;   // [N] ampl = A^-1 s g
  double* y = am + N;        // [N] A^-1 b
  __shared__ double red[kWarps + 1];
  __shared__ int32_t s_zone;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t ncells = (int64_t)g.nu * g.nv;
  const int full_scan = brute || !lp.localise;
  for (;;) {
    if (tid == 0) s_zone = atomicAdd(work, 1);
    __syncthreads();
    const int32_t zl = s_zone;
    if (zl >= nzc) break;
    const int32_t z = zlist[zl];
    if (nobs[z] == 0) {  // zone untouched by the analysis: no dependence on yo, r, lengths
      __syncthreads();
      continue;
    }
    const double* Gz = G + (int64_t)zl * N * N;
    for (int idx = tid; idx < N * N; idx += kThreads) {
      int i = idx / N, j = idx - i * N;
      A[i * ld + j] = s * s * Gz[idx] + ((i == j) ? 1.0 : 0.0);
    }
    const int64_t i1 = zone_start[z], i2 = zone_start[z + 1];
    // am <- s g, y <- b = s Sf_z^T a
    for (int k = tid; k < N; k += kThreads) {
      am[k] = s * gv[(int64_t)zl * N + k];
      double acc = 0.0;
      for (int64_t i = i1; i < i2; i++) acc = fma(Sf[i + (int64_t)k * ldS], seed[i], acc);
      y[k] = s * acc;
    }
    __syncthreads();
    // Cholesky A = L L^T (right-looking, lower triangle)
    for (int k = 0; k < N; k++) {
      if (tid == 0) A[k * ld + k] = sqrt(A[k * ld + k]);
      __syncthreads();
      const double inv = 1.0 / A[k * ld + k];
      for (int i = k + 1 + tid; i < N; i += kThreads) A[i * ld + k] *= inv;
      __syncthreads();
      const int L = N - k - 1;
      for (int idx = tid; idx < L * L; idx += kThreads) {
        int i = idx / L, j = idx - i * L;
        if (j <= i) {
          double* a = A + (k + 1 + i) * ld + (k + 1 + j);
          *a = fma(-A[(k + 1 + i) * ld + k], A[(k + 1 + j) * ld + k], *a);
        }
      }
      __syncthreads();
    }
    // two right-hand sides: L L^T am = s g, L L^T y = b (warp 0 per system, lanes over k)
    if (warp < 2) {
      double* x = (warp == 0) ? am : y;
      for (int i = 0; i < N; i++) {  // forward: L z = rhs
        double t = 0.0;
        for (int k = lane; k < i; k += 32) t = fma(A[i * ld + k], x[k], t);
        t = warp_sum(t);
        if (lane == 0) x[i] = (x[i] - t) / A[i * ld + i];
        __syncwarp();
      }
      for (int i = N - 1; i >= 0; i--) {  // backward: L^T x = z
        double t = 0.0;
        for (int k = i + 1 + lane; k < N; k += 32) t = fma(A[k * ld + i], x[k], t);
        t = warp_sum(t);
        if (lane == 0) x[i] = (x[i] - t) / A[i * ld + i];
        __syncwarp();
      }
    }
    __syncthreads();
    // b^T ampl = s a^T Sf ampl (the direct part of dJ/ds): recompute b per k
    double part = 0.0;
    for (int k = tid; k < N; k += kThreads) {
      double acc = 0.0;
      for (int64_t i = i1; i < i2; i++) acc = fma(Sf[i + (int64_t)k * ldS], seed[i], acc);
      part = fma(s * acc, am[k], part);
    }
    // re-run the zone's selection; every relevant observation adds its terms
    const double zx = zone_xyzt[4 * (int64_t)z + 0], zy = zone_xyzt[4 * (int64_t)z + 1];
    const double zzc = zone_xyzt[4 * (int64_t)z + 2], ztc = zone_xyzt[4 * (int64_t)z + 3];
    const double zu = (lp.loctype == 1) ? zx : (lp.loctype == 2 ? zzc : ztc);
    const double zv = (lp.loctype == 1) ? zy : 0.0;
    const double L = corr_len[z], Rmax = max_len[z];
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
    double dk_loc = 0.0, ds_loc = 0.0;
    for (int cv = sr.cv0; cv <= sr.cv1; cv++) {
      for (int part2 = 0; part2 < 2; part2++) {
        int cu_a, cu_b;
        if (sr.all_u || !g.periodic_u) {
          if (part2) break;
          cu_a = sr.cu0;
          cu_b = sr.cu1;
        } else {
          const int a0 = sr.cu0, b0 = sr.cu1;
          if (a0 < 0) {
            if (part2 == 0) { cu_a = a0 + g.nu; cu_b = g.nu - 1; }
            else { cu_a = 0; cu_b = b0; }
          } else if (b0 >= g.nu) {
            if (part2 == 0) { cu_a = a0; cu_b = g.nu - 1; }
            else { cu_a = 0; cu_b = b0 - g.nu; }
          } else {
            if (part2) break;
            cu_a = a0;
            cu_b = b0;
          }
        }
        const int64_t c_lo = (int64_t)cu_a + (int64_t)g.nu * cv;
        const int64_t c_hi = (int64_t)cu_b + (int64_t)g.nu * cv;
        if (c_lo > c_hi || c_lo < 0 || c_hi >= ncells) continue;
        const int32_t q_lo = so.cell_start[c_lo], q_hi = so.cell_start[c_hi + 1];
        for (int32_t q = q_lo + tid; q < q_hi; q += kThreads) {
          double d;
          if (lp.loctype == 1)
            d = sel::distance(so.u[q], so.v[q], zu, zv, lp.metric);
          else
            d = fabs(__dsub_rn(so.u[q], zu));
          const double t = d / L;
          double w, dw;
          int rel;
          if (lp.weight == OAKG_WEIGHT_GAUSS_CUTOFF) {
            rel = (d <= Rmax);
            w = exp(-(t * t));
            dw = 2.0 * t * t * w;
          } else {
            w = sel::locfun(t);
            rel = (d <= Rmax) && (w != 0.0);
            dw = -t * sel::locfun_deriv(t);
          }
          if (!(rel || !lp.localise)) continue;
          const double rq = so.r[q];
          const double c = w * (w / rq);
          const double* h = so.HSt + (int64_t)q * N;
          double t1 = 0.0, t2 = 0.0;
          for (int k = 0; k < N; k++) {
            t1 = fma(h[k], y[k], t1);
            t2 = fma(h[k], am[k], t2);
          }
          t1 *= s;
          t2 *= s;
          const double dq = so.innov[q];
          const double gc = t1 * (dq - t2);  // dJ/dc_q
          const int32_t j = so.perm[q];
          atomicAdd(&dyo[j], c * t1);
          atomicAdd(&dr[j], -gc * c / rq);
          dk_loc = fma(gc * (2.0 * w / rq), dw, dk_loc);
          ds_loc = fma(c * t1, dq - 2.0 * t2, ds_loc);
        }
      }
    }
    const double dk = block_sum(dk_loc, red);
    const double dsum = block_sum(ds_loc + part, red);
    if (tid == 0) {
      atomicAdd(&dscal[0], dk);
      atomicAdd(&dscal[1], dsum / s);
    }
    __syncthreads();
  }
  (void)warp;
}

}  // namespace

cudaError_t zone_active_list(const double* seed, const int64_t* zone_start, int32_t Z,
                             int32_t* d_flag, int32_t* d_pos, int32_t* d_list,
                             cudaStream_t st) {
  int grid = (Z + 255) / 256;
  if (grid > 152 * 8) grid = 152 * 8;
  if (grid < 1) grid = 1;
  k_zone_flags<<<grid, 256, 0, st>>>(seed, zone_start, Z, d_flag);
  k_zone_compact<<<1, 1024, 0, st>>>(d_flag, Z, d_pos, d_list);
  count_launches(2);
  return cudaGetLastError();
}

cudaError_t zone_adjoint_fp64(const CellGrid& g, const SortedObs& so, int N, LocParams lp,
                              const int32_t* zlist, int32_t nzc, const double* zone_xyzt,
                              const double* corr_len, const double* max_len,
                              const int64_t* zone_start, const double* Sf, int64_t ldS,
                              const double* seed, double infl, const double* d_G,
                              const double* d_g, const int32_t* d_nobs, double* dyo, double* dr,
                              double* dscal, int brute, int32_t* d_work, cudaStream_t st) {
  size_t smem = (size_t)(N * (N + 1) + 2 * N) * sizeof(double);
  cudaError_t e = cudaFuncSetAttribute(k_zone_adjoint,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int bps = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_zone_adjoint, kThreads, smem);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int grid = sms * (bps > 0 ? bps : 1);
  if (grid > nzc) grid = nzc > 0 ? nzc : 1;
  e = cudaMemsetAsync(d_work, 0, sizeof(int32_t), st);
  if (e != cudaSuccess) return e;
  k_zone_adjoint<<<grid, kThreads, smem, st>>>(g, so, N, lp, zlist, nzc, zone_xyzt, corr_len,
                                                max_len, zone_start, Sf, ldS, seed, infl, d_G,
                                                d_g, d_nobs, dyo, dr, dscal, brute, d_work);
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace oakg
