// K5 -- ensemble update per zone (T and the amplitudes in R: double for the plain form, float
// for the mixed-precision form; Sf, Sa, xf, xa in S: the storage type at the boundary, double
// or float):
//   xa(i1:i2) = xf(i1:i2) + Sf(i1:i2,:) ampl          (rrsqrt.F90:151 and :462-464)
//   Sa(i1:i2,:) = Sf(i1:i2,:) T                       (rrsqrt.F90:165-185 with T from K4)
// Zones without relevant observations keep xa = xf and Sa = Sf (rrsqrt.F90:322-326, :371).
//
// Sf/Sa are the reference's column-major (n, N) arrays (leading dimension ldS). In the generic
// kernel a task is a
// tile of up to kRows consecutive rows of one zone; the tile of Sf is staged column by column
// into shared memory (coalesced along rows), T (N x N) next to it, and Sa is written column by
// column. Reads and writes are in place safe (Sa may alias Sf, xa may alias xf).
// Work per zone: 2 nz N^2 FP64 flops, 2 nz N 8-byte reads/writes + N^2 8-byte T read.
#include <cuda_runtime.h>

#include "oakg_internal.cuh"

namespace oakg {

namespace {

constexpr int kThreads = 256;
constexpr int kRows = 64;

template <typename R, typename S>
__global__ void __launch_bounds__(kThreads)
    k_zone_update(int N, int32_t z0, int32_t nzc, const int64_t* __restrict__ zone_start,
                  int tiles_per_zone, const S* __restrict__ xf, const S* __restrict__ Sf,
                  int64_t ldS, const R* __restrict__ T, const R* __restrict__ ampl,
                  const int32_t* __restrict__ nobs, S* __restrict__ xa, S* __restrict__ Sa) {
  extern __shared__ __align__(16) unsigned char dyn_raw[];
  R* dyn = reinterpret_cast<R*>(dyn_raw);
  R* Ts = dyn;                // [N][N]
  R* Ss = Ts + N * N;         // [N][kRows]  (column k of the tile at Ss + k*kRows)
  R* as = Ss + N * kRows;     // [N]
  const int64_t ntasks = (int64_t)nzc * tiles_per_zone;
  for (int64_t task = blockIdx.x; task < ntasks; task += gridDim.x) {
    const int32_t zl = (int32_t)(task / tiles_per_zone);
    const int tile = (int)(task - (int64_t)zl * tiles_per_zone);
    const int32_t z = z0 + zl;
    const int64_t i1 = zone_start[z], i2 = zone_start[z + 1];
    const int64_t r0 = i1 + (int64_t)tile * kRows;
    if (r0 >= i2) continue;  // uniform across the block
    const int R_ = (int)((i2 - r0) < kRows ? (i2 - r0) : kRows);
    if (nobs[zl] == 0) {
      for (int idx = threadIdx.x; idx < R_; idx += kThreads) xa[r0 + idx] = xf[r0 + idx];
      if (Sa && Sa != Sf) {
        for (int idx = threadIdx.x; idx < R_ * N; idx += kThreads) {
          int k = idx / R_, r = idx - k * R_;
          Sa[r0 + r + (int64_t)k * ldS] = Sf[r0 + r + (int64_t)k * ldS];
        }
      }
      continue;
    }
    __syncthreads();  // previous task's shared data consumed
    const R* Tz = T + (int64_t)zl * N * N;
    if (Sa) {
      for (int idx = threadIdx.x; idx < N * N; idx += kThreads) Ts[idx] = Tz[idx];
    }
    for (int idx = threadIdx.x; idx < N; idx += kThreads) as[idx] = ampl[(int64_t)zl * N + idx];
    for (int idx = threadIdx.x; idx < R_ * N; idx += kThreads) {
      int k = idx / R_, r = idx - k * R_;
      Ss[k * kRows + r] = (R)Sf[r0 + r + (int64_t)k * ldS];
    }
    __syncthreads();
    // xa = xf + Sf ampl
    for (int r = threadIdx.x; r < R_; r += kThreads) {
      R s = 0;
      for (int k = 0; k < N; k++) s = fma(Ss[k * kRows + r], as[k], s);
      xa[r0 + r] = (S)((double)xf[r0 + r] + (double)s);
    }
    if (Sa) {
      // Sa(r, c) = sum_k Sf(r, k) T(k, c); consecutive threads -> consecutive rows
      for (int idx = threadIdx.x; idx < R_ * N; idx += kThreads) {
        int c = idx / R_, r = idx - c * R_;
        R s = 0;
        for (int k = 0; k < N; k++) s = fma(Ss[k * kRows + r], Ts[k * N + c], s);
        Sa[r0 + r + (int64_t)c * ldS] = (S)s;
      }
    }
  }
}

// Mixed form (any N). A block takes whole zones (grid-stride over zones), so T and the
// amplitudes are staged in shared memory once per zone: T with its rows padded to NP columns (N
// rounded up to a multiple of 8, zero padding). The zone's rows then go through in tiles of
// kRows, each tile of Sf converted to FP32 and staged column by column (coalesced along rows).
// A work item is one row x 8 columns of Sa; the items of a warp share their 8 columns
// (consecutive threads take consecutive rows), so each k costs the warp one broadcast 128-bit
// T load pair and one Sf load for 8 FMAs per thread; padding columns are not written. The FMA
// order over k is that of k_zone_update<float>.
constexpr int kColBlk = 8;

template <typename S>
__global__ void __launch_bounds__(kThreads)
    k_zone_update_f32(int N, int NP, int32_t z0, int32_t nzc,
                      const int64_t* __restrict__ zone_start, const S* __restrict__ xf,
                      const S* __restrict__ Sf, int64_t ldS, const float* __restrict__ T,
                      const float* __restrict__ ampl, const int32_t* __restrict__ nobs,
                      S* __restrict__ xa, S* __restrict__ Sa) {
  extern __shared__ __align__(16) unsigned char dyn_raw[];
  float* Ts = reinterpret_cast<float*>(dyn_raw);  // [N][NP]
  float* Ss = Ts + N * NP;                         // [N][kRows]
  float* as = Ss + N * kRows;                      // [N]
  const int ncb = NP / kColBlk;
  for (int32_t zl = blockIdx.x; zl < nzc; zl += gridDim.x) {
    const int32_t z = z0 + zl;
    const int64_t i1 = zone_start[z], i2 = zone_start[z + 1];
    if (nobs[zl] == 0) {
      for (int64_t i = i1 + threadIdx.x; i < i2; i += kThreads) xa[i] = xf[i];
      if (Sa && Sa != Sf) {
        const int nr = (int)(i2 - i1);
        for (int idx = threadIdx.x; idx < nr * N; idx += kThreads) {
          const int k = idx / nr, r = idx - k * nr;
          Sa[i1 + r + (int64_t)k * ldS] = Sf[i1 + r + (int64_t)k * ldS];
        }
      }
      continue;
    }
    __syncthreads();  // previous zone's shared data consumed
    const float* Tz = T + (int64_t)zl * N * N;
    if (Sa) {
      if ((N & 3) == 0) {  // rows of T start on 16-byte boundaries: 128-bit loads
        const int nq = NP >> 2;
        const float4* Tz4 = reinterpret_cast<const float4*>(Tz);
        float4* Ts4 = reinterpret_cast<float4*>(Ts);
        for (int idx = threadIdx.x; idx < N * nq; idx += kThreads) {
          const int k = idx / nq, c4 = idx - k * nq;
          Ts4[idx] = (4 * c4 < N) ? Tz4[(k * N >> 2) + c4] : make_float4(0.f, 0.f, 0.f, 0.f);
        }
      } else {
        for (int idx = threadIdx.x; idx < N * NP; idx += kThreads) {
          const int k = idx / NP, c = idx - k * NP;
          Ts[idx] = (c < N) ? Tz[k * N + c] : 0.f;
        }
      }
    }
    for (int idx = threadIdx.x; idx < N; idx += kThreads) as[idx] = ampl[(int64_t)zl * N + idx];
    for (int64_t r0 = i1; r0 < i2; r0 += kRows) {
      const int R_ = (int)((i2 - r0) < kRows ? (i2 - r0) : kRows);
      if (r0 > i1) __syncthreads();  // previous tile consumed
      for (int idx = threadIdx.x; idx < R_ * N; idx += kThreads) {
        const int k = idx / R_, r = idx - k * R_;
        Ss[k * kRows + r] = (float)Sf[r0 + r + (int64_t)k * ldS];
      }
      __syncthreads();
      for (int r = threadIdx.x; r < R_; r += kThreads) {  // xa = xf + Sf ampl
        float sx = 0.f;
        for (int k = 0; k < N; k++) sx = fmaf(Ss[k * kRows + r], as[k], sx);
        xa[r0 + r] = (S)((double)xf[r0 + r] + (double)sx);
      }
      if (Sa) {
        for (int it = threadIdx.x; it < R_ * ncb; it += kThreads) {
          const int cb = it / R_, r = it - cb * R_;
          const int c0 = kColBlk * cb;
          float acc[kColBlk];
#pragma unroll
          for (int t = 0; t < kColBlk; t++) acc[t] = 0.f;
#pragma unroll 4
          for (int k = 0; k < N; k++) {
            const float sk = Ss[k * kRows + r];
            const float4 ta = *reinterpret_cast<const float4*>(Ts + k * NP + c0);
            const float4 tb = *reinterpret_cast<const float4*>(Ts + k * NP + c0 + 4);
            acc[0] = fmaf(sk, ta.x, acc[0]);
            acc[1] = fmaf(sk, ta.y, acc[1]);
            acc[2] = fmaf(sk, ta.z, acc[2]);
            acc[3] = fmaf(sk, ta.w, acc[3]);
            acc[4] = fmaf(sk, tb.x, acc[4]);
            acc[5] = fmaf(sk, tb.y, acc[5]);
            acc[6] = fmaf(sk, tb.z, acc[6]);
            acc[7] = fmaf(sk, tb.w, acc[7]);
          }
#pragma unroll
          for (int t = 0; t < kColBlk; t++)
            if (c0 + t < N) Sa[r0 + r + (int64_t)(c0 + t) * ldS] = (S)acc[t];
        }
      }
    }
  }
}

template <typename R, typename S>
__global__ void k_write_amplitudes(int N, int32_t z0, int32_t nzc, const R* __restrict__ za,
                                   const int32_t* __restrict__ nobs, int all_zones,
                                   S* __restrict__ out) {
  const int64_t total = (int64_t)nzc * N;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int32_t zl = (int32_t)(idx / N);
    double v = (all_zones && nobs[zl] > 0) ? (double)za[idx] : 0.0;
    out[(int64_t)z0 * N + idx] = (S)v;
  }
}

}  // namespace

template <typename R, typename S>
cudaError_t zone_update_impl(int N, int32_t z0, int32_t nzc, const int64_t* d_zone_start,
                             int32_t zone_max, const S* xf, const S* Sf, int64_t ldS,
                             const R* d_T, const R* d_ampl, const int32_t* d_nobs, S* xa, S* Sa,
                             cudaStream_t st) {
  size_t smem = (size_t)(N * N + N * kRows + N) * sizeof(R);
  cudaError_t e = cudaFuncSetAttribute(k_zone_update<R, S>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int tiles = (zone_max + kRows - 1) / kRows;
  if (tiles < 1) tiles = 1;
  int64_t ntasks = (int64_t)nzc * tiles;
  int grid = (int)(ntasks < 152 * 16 ? (ntasks < 1 ? 1 : ntasks) : 152 * 16);
  k_zone_update<R, S><<<grid, kThreads, smem, st>>>(N, z0, nzc, d_zone_start, tiles, xf, Sf,
                                                    ldS, d_T, d_ampl, d_nobs, xa, Sa);
  count_launches(1);
  return cudaGetLastError();
}

template <typename R, typename S>
cudaError_t write_amplitudes_impl(int N, int32_t z0, int32_t nzc, const R* d_ampl,
                                  const int32_t* d_nobs, int all_zones, S* ampl_out,
                                  cudaStream_t st) {
  int64_t total = (int64_t)nzc * N;
  int grid = (int)((total + 255) / 256 < 152 * 8 ? (total + 255) / 256 : 152 * 8);
  if (grid < 1) grid = 1;
  k_write_amplitudes<R, S><<<grid, 256, 0, st>>>(N, z0, nzc, d_ampl, d_nobs, all_zones,
                                                 ampl_out);
  count_launches(1);
  return cudaGetLastError();
}

template <typename S>
cudaError_t zone_update_mixed_impl(int N, int32_t z0, int32_t nzc, const int64_t* d_zone_start,
                                   int32_t zone_max, const S* xf, const S* Sf, int64_t ldS,
                                   const float* d_T, const float* d_ampl, const int32_t* d_nobs,
                                   S* xa, S* Sa, cudaStream_t st) {
  const int NP = (N + kColBlk - 1) / kColBlk * kColBlk;
  const size_t smem = (size_t)(N * NP + N * kRows + N) * sizeof(float);
  if (smem <= 200 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k_zone_update_f32<S>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int bps = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_zone_update_f32<S>, kThreads, smem);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t cap = (int64_t)sms * (bps > 0 ? bps : 1) * 4;
    const int grid = (int)(nzc < cap ? (nzc < 1 ? 1 : nzc) : cap);
    k_zone_update_f32<S><<<grid, kThreads, smem, st>>>(N, NP, z0, nzc, d_zone_start, xf, Sf,
                                                       ldS, d_T, d_ampl, d_nobs, xa, Sa);
    count_launches(1);
    return cudaGetLastError();
  }
  return zone_update_impl<float, S>(N, z0, nzc, d_zone_start, zone_max, xf, Sf, ldS, d_T,
                                    d_ampl, d_nobs, xa, Sa, st);
}

cudaError_t zone_update_fp64(int N, int32_t z0, int32_t nzc, const int64_t* d_zone_start,
                             int32_t zone_max, const double* xf, const double* Sf,
                             int64_t ldS, const double* d_T, const double* d_ampl,
                             const int32_t* d_nobs, double* xa, double* Sa, cudaStream_t st) {
  return zone_update_impl<double, double>(N, z0, nzc, d_zone_start, zone_max, xf, Sf, ldS, d_T,
                                          d_ampl, d_nobs, xa, Sa, st);
}

cudaError_t zone_update_fp64(int N, int32_t z0, int32_t nzc, const int64_t* d_zone_start,
                             int32_t zone_max, const float* xf, const float* Sf, int64_t ldS,
                             const double* d_T, const double* d_ampl, const int32_t* d_nobs,
                             float* xa, float* Sa, cudaStream_t st) {
  return zone_update_impl<double, float>(N, z0, nzc, d_zone_start, zone_max, xf, Sf, ldS, d_T,
                                         d_ampl, d_nobs, xa, Sa, st);
}

cudaError_t zone_update_fp32(int N, int32_t z0, int32_t nzc, const int64_t* d_zone_start,
                             int32_t zone_max, const double* xf, const double* Sf,
                             int64_t ldS, const float* d_T, const float* d_ampl,
                             const int32_t* d_nobs, double* xa, double* Sa, cudaStream_t st) {
  return zone_update_mixed_impl<double>(N, z0, nzc, d_zone_start, zone_max, xf, Sf, ldS, d_T,
                                        d_ampl, d_nobs, xa, Sa, st);
}

cudaError_t zone_update_fp32(int N, int32_t z0, int32_t nzc, const int64_t* d_zone_start,
                             int32_t zone_max, const float* xf, const float* Sf, int64_t ldS,
                             const float* d_T, const float* d_ampl, const int32_t* d_nobs,
                             float* xa, float* Sa, cudaStream_t st) {
  return zone_update_mixed_impl<float>(N, z0, nzc, d_zone_start, zone_max, xf, Sf, ldS, d_T,
                                       d_ampl, d_nobs, xa, Sa, st);
}

cudaError_t write_amplitudes(int N, int32_t z0, int32_t nzc, const double* d_ampl,
                             const int32_t* d_nobs, int all_zones, double* ampl_out,
                             cudaStream_t st) {
  return write_amplitudes_impl<double, double>(N, z0, nzc, d_ampl, d_nobs, all_zones, ampl_out,
                                               st);
}

cudaError_t write_amplitudes(int N, int32_t z0, int32_t nzc, const double* d_ampl,
                             const int32_t* d_nobs, int all_zones, float* ampl_out,
                             cudaStream_t st) {
  return write_amplitudes_impl<double, float>(N, z0, nzc, d_ampl, d_nobs, all_zones, ampl_out,
                                              st);
}

cudaError_t write_amplitudes_fp32(int N, int32_t z0, int32_t nzc, const float* d_ampl,
                                  const int32_t* d_nobs, int all_zones, double* ampl_out,
                                  cudaStream_t st) {
  return write_amplitudes_impl<float, double>(N, z0, nzc, d_ampl, d_nobs, all_zones, ampl_out,
                                              st);
}

cudaError_t write_amplitudes_fp32(int N, int32_t z0, int32_t nzc, const float* d_ampl,
                                  const int32_t* d_nobs, int all_zones, float* ampl_out,
                                  cudaStream_t st) {
  return write_amplitudes_impl<float, float>(N, z0, nzc, d_ampl, d_nobs, all_zones, ampl_out,
                                             st);
}

}  // namespace oakg
