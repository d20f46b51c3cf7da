// FP64-accurate refinement of the mixed form's FP32 eigenpairs (zone_eig32.cu), after
// T. Ogita and K. Aishima, "Iterative refinement for symmetric eigenvalue decomposition",
// Japan J. Indust. Appl. Math. 35 (2018) 1007-1035, Algorithm 1. For the zone matrix A = G
// (symmetric, N x N, FP32) and its approximate eigenvectors X (columns x_j, FP32):
//   R = I - X^T X,   S = X^T A X,   lambda_i = s_ii / (1 - r_ii),
//   delta = 2 (||S - diag(lambda)|| + ||A|| ||R||)      (Frobenius norms bound the 2-norms),
//   e_ij = (s_ij + lambda_j r_ij) / (lambda_j - lambda_i)   if |lambda_i - lambda_j| > delta,
//          r_ij / 2                                         otherwise,
//   X' = X + X E.
// One step takes eigenpairs accurate to FP32 (errors ~eps_32 ||A|| / gap) to errors of
// order eps_32^2 ||A|| / gap, i.e. FP64 accuracy, provided R and S are accurate to that level:
// they are formed with exact products and compensated sums of FP32 values (double-float
// arithmetic: TwoProduct by FMA and TwoSum, Ogita-Rump-Oishi), on the FP32 pipe, which on
// GB300 runs ~50x the FP64 rate. The entries of R and of S off the diagonal are of order
// eps_32 and are kept as FP32 numbers after the exact evaluation (absolute error eps_32^2);
// W = A X is kept as double-float (hi + lo) for S = X^T W. The corrections X E are of order
// eps_32 and are formed in FP32. The refined vectors and eigenvalues are rounded to FP32 and
// handed to the transform stage (k_eig_transform32 / 128 in mode 2), which forms T and the
// amplitudes with the FP64 scalings (1 + lambda)^-1/2 and (1 + lambda)^-1.
//
// One CTA of 256 threads per zone (persistent grid), the matrices in shared memory; every
// product is a set of 64 x 64 output blocks, a 4 x 4 tile per thread.
#include <cuda_runtime.h>

#include "oakg_internal.cuh"

namespace oakg {

namespace {

constexpr int kThreads = 256;

// per-zone auxiliary layout of the FP32 eigensolve (zone_eig.cu aux_stride): lambda at 3 N
__host__ __device__ inline int aux_stride_r(int N) { return 5 * N + 2; }

// exact product a b = p + e and compensated accumulation into (hi, lo)
__device__ __forceinline__ void df_mac(float& hi, float& lo, float a, float b) {
  const float p = __fmul_rn(a, b);
  const float e = __fmaf_rn(a, b, -p);
  const float t = __fadd_rn(hi, p);
  const float z = __fsub_rn(t, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(t, z)), __fsub_rn(p, z));
  hi = t;
  lo = __fadd_rn(lo, __fadd_rn(err, e));
}

// C[a][b] (a in [a0, a0 + 4), b in [b0, b0 + 4)) = sum_{l < K} P[l][a] Q[l][b] with exact
// products and compensated sums; P, Q row-major with leading dimensions ldp, ldq (floats),
// rows 16-byte aligned. With Qlo, the terms P[l][a] Qlo[l][b] are added in FP32 (Q = Q + Qlo
// as a double-float operand).
__device__ __forceinline__ void df_tile(const float* P, int ldp, const float* Q, int ldq,
                                        const float* Qlo, int K, int a0, int b0,
                                        float (&hi)[4][4], float (&lo)[4][4]) {
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) hi[i][j] = lo[i][j] = 0.f;
  for (int l = 0; l < K; l++) {
    const float4 p4 = *reinterpret_cast<const float4*>(P + l * ldp + a0);
    const float4 q4 = *reinterpret_cast<const float4*>(Q + l * ldq + b0);
    const float pa[4] = {p4.x, p4.y, p4.z, p4.w}, qb[4] = {q4.x, q4.y, q4.z, q4.w};
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int j = 0; j < 4; j++) df_mac(hi[i][j], lo[i][j], pa[i], qb[j]);
    if (Qlo) {
      const float4 r4 = *reinterpret_cast<const float4*>(Qlo + l * ldq + b0);
      const float rb[4] = {r4.x, r4.y, r4.z, r4.w};
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) lo[i][j] = __fmaf_rn(pa[i], rb[j], lo[i][j]);
    }
  }
}

__device__ __forceinline__ float block_sum(float v, float* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  float s = 0.f;
#pragma unroll
  for (int w = 0; w < kThreads / 32; w++) s += red[w];
  return s;
}

// Shared memory (NP = N padded to 64 or 128): two NP x NP FP32 regions and one of
// 2 NP x 64 floats (NP x NP for NP = 128):
//   X   [k][j] = x_j[k]                      (all phases but the last)
//   M1  A [k][r], then R [i][j], then U [j][k] (vector-major)
//   M2  W block (hi [NP][64], lo [NP][64]), then E [i][j]
template <int NP>
constexpr size_t refine_smem_floats() { return (size_t)2 * NP * NP + (size_t)2 * NP * 64; }

template <int NP>
__global__ void __launch_bounds__(kThreads, NP == 64 ? 3 : 1)
    k_eig_refine(int N, int32_t nzc, const float* __restrict__ G0, float* __restrict__ Zg,
                 float* __restrict__ aux, const int32_t* __restrict__ nobs,
                 float* __restrict__ Sg) {
  extern __shared__ __align__(16) float smem[];
  __shared__ float red[kThreads / 32];
  __shared__ double lam_d[NP];
  __shared__ float lam_hi[NP], lam_lo[NP];
  float* X = smem;
  float* M1 = X + NP * NP;
  float* M2 = M1 + NP * NP;
  const int tid = threadIdx.x;
  const int ty = tid >> 4, tx = tid & 15;  // 4 x 4 tile (4 ty, 4 tx) of a 64 x 64 block
  constexpr int NB = NP / 64;
  for (int32_t zl = blockIdx.x; zl < nzc; zl += gridDim.x) {
    if (nobs[zl] == 0) continue;  // block-uniform
    const float* Az = G0 + (int64_t)zl * N * N;
    float* Uz = Zg + (int64_t)zl * N * N;
    float* ax = aux + (int64_t)zl * aux_stride_r(N);
    float* Sz = Sg + (int64_t)zl * 2 * NP * NP;  // S as (hi, lo) [i][j]
    __syncthreads();  // previous zone's shared data consumed
    for (int idx = tid; idx < NP * NP; idx += kThreads) {
      const int a = idx / NP, b = idx - a * NP;
      // X[k = b][j = a] = U[a][b]; A[a][b]
      X[b * NP + a] = (a < N && b < N) ? Uz[(int64_t)a * N + b] : 0.f;
      M1[idx] = (a < N && b < N) ? Az[(int64_t)a * N + b] : 0.f;
    }
    __syncthreads();
    // ||A||_F
    float an = 0.f;
    for (int idx = tid; idx < NP * NP; idx += kThreads) an = fmaf(M1[idx], M1[idx], an);
    const float normA = sqrtf(block_sum(an, red));
    // W = A X and S = X^T W, a block of 64 columns of W at a time
    float* Wh = M2;
    float* Wl = M2 + NP * 64;
    for (int jb = 0; jb < NB; jb++) {
      for (int bi = 0; bi < NB; bi++) {
        // W[k][j] = sum_l A[l][k] X[l][j]  (A symmetric), j in block jb
        float hi[4][4], lo[4][4];
        const int k0 = 64 * bi + 4 * ty, j0 = 64 * jb + 4 * tx;
        df_tile(M1, NP, X, NP, nullptr, NP, k0, j0, hi, lo);
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
          for (int j = 0; j < 4; j++) {
            // renormalise the pair so that lo holds what hi cannot
            const float s = __fadd_rn(hi[i][j], lo[i][j]);
            Wh[(k0 + i) * 64 + 4 * tx + j] = s;
            Wl[(k0 + i) * 64 + 4 * tx + j] = __fadd_rn(lo[i][j], __fsub_rn(hi[i][j], s));
          }
      }
      __syncthreads();
      for (int bi = 0; bi < NB; bi++) {
        // S[i][j] = sum_k X[k][i] (Wh + Wl)[k][j]
        float hi[4][4], lo[4][4];
        const int i0 = 64 * bi + 4 * ty;
        df_tile(X, NP, Wh, 64, Wl, NP, i0, 4 * tx, hi, lo);
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
          for (int j = 0; j < 4; j++) {
            const int64_t e = (int64_t)(i0 + i) * NP + 64 * jb + 4 * tx + j;
            const float s = __fadd_rn(hi[i][j], lo[i][j]);
            Sz[2 * e] = s;
            Sz[2 * e + 1] = __fadd_rn(lo[i][j], __fsub_rn(hi[i][j], s));
          }
      }
      __syncthreads();  // the W block is consumed
    }
    // R = I - X^T X (FP32 entries, exact evaluation) into M1 (A no longer needed)
    float rn = 0.f;
    for (int bi = 0; bi < NB; bi++)
      for (int bj = 0; bj < NB; bj++) {
        float hi[4][4], lo[4][4];
        const int i0 = 64 * bi + 4 * ty, j0 = 64 * bj + 4 * tx;
        df_tile(X, NP, X, NP, nullptr, NP, i0, j0, hi, lo);  // reads X only
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
          for (int j = 0; j < 4; j++) {
            const int ii = i0 + i, jj = j0 + j;
            float r;
            if (ii == jj) {
              r = (ii < N) ? __fsub_rn(__fsub_rn(1.f, hi[i][j]), lo[i][j]) : 0.f;
            } else {
              r = -__fadd_rn(hi[i][j], lo[i][j]);
            }
            M1[ii * NP + jj] = r;
            rn = fmaf(r, r, rn);
          }
      }
    const float normR = sqrtf(block_sum(rn, red));  // also publishes R
    // refined eigenvalues lambda_i = s_ii / (1 - r_ii) (FP64 for these N scalars)
    if (tid < NP) {
      double l = 0.0;
      if (tid < N) {
        const int64_t e = (int64_t)tid * NP + tid;
        const double sii = (double)Sz[2 * e] + (double)Sz[2 * e + 1];
        l = sii / (1.0 - (double)M1[tid * NP + tid]);
      }
      lam_d[tid] = l;
      const float h = (float)l;
      lam_hi[tid] = h;
      lam_lo[tid] = (float)(l - (double)h);
    }
    __syncthreads();
    // ||S - diag(lambda)||_F
    float sn = 0.f;
    for (int idx = tid; idx < N * N; idx += kThreads) {
      const int i = idx / N, j = idx - i * N;
      const int64_t e = (int64_t)i * NP + j;
      float v = __fadd_rn(Sz[2 * e], Sz[2 * e + 1]);
      if (i == j) v = (float)((double)Sz[2 * e] + (double)Sz[2 * e + 1] - lam_d[i]);
      sn = fmaf(v, v, sn);
    }
    const float delta = 2.f * (sqrtf(block_sum(sn, red)) + normA * normR);
    // E[i][j] into M2 (the W blocks are done)
    float* E = M2;
    for (int idx = tid; idx < NP * NP; idx += kThreads) {
      const int i = idx / NP, j = idx - i * NP;
      float ev = 0.f;
      if (i < N && j < N) {
        const float r = M1[i * NP + j];
        const float dl = __fadd_rn(__fsub_rn(lam_hi[j], lam_hi[i]),
                                   __fsub_rn(lam_lo[j], lam_lo[i]));
        if (fabsf(dl) > delta) {
          // s_ij + lambda_j r_ij with the cancellation resolved: (S_hi + p) by TwoSum, then
          // the small terms
          const int64_t e = (int64_t)i * NP + j;
          const float sh = Sz[2 * e], sl = Sz[2 * e + 1];
          const float p = __fmul_rn(lam_hi[j], r);
          const float pe = __fmaf_rn(lam_hi[j], r, -p);
          const float t = __fadd_rn(sh, p);
          const float z = __fsub_rn(t, sh);
          const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, z)), __fsub_rn(p, z));
          const float num =
              __fadd_rn(t, __fadd_rn(__fadd_rn(err, sl), __fmaf_rn(lam_lo[j], r, pe)));
          ev = __fdiv_rn(num, dl);
        } else {
          ev = 0.5f * r;
        }
      }
      E[idx] = ev;
    }
    __syncthreads();
    // U (vector-major) into M1 (R is consumed), then U'[j][k] = U[j][k] + sum_i E[i][j] U[i][k]
    for (int idx = tid; idx < NP * NP; idx += kThreads) {
      const int a = idx / NP, b = idx - a * NP;
      M1[idx] = (a < N && b < N) ? Uz[(int64_t)a * N + b] : 0.f;
    }
    __syncthreads();
    for (int bi = 0; bi < NB; bi++)
      for (int bj = 0; bj < NB; bj++) {
        const int j0 = 64 * bi + 4 * ty, k0 = 64 * bj + 4 * tx;
        float c[4][4];
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
          for (int j = 0; j < 4; j++) c[i][j] = 0.f;
        for (int i = 0; i < NP; i++) {
          const float4 e4 = *reinterpret_cast<const float4*>(E + i * NP + j0);
          const float4 u4 = *reinterpret_cast<const float4*>(M1 + i * NP + k0);
          const float ea[4] = {e4.x, e4.y, e4.z, e4.w}, ub[4] = {u4.x, u4.y, u4.z, u4.w};
#pragma unroll
          for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 4; b++) c[a][b] = fmaf(ea[a], ub[b], c[a][b]);
        }
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
          for (int b = 0; b < 4; b++) {
            const int jj = j0 + a, kk = k0 + b;
            if (jj < N && kk < N) Uz[(int64_t)jj * N + kk] = M1[jj * NP + kk] + c[a][b];
          }
      }
    if (tid < N) ax[3 * N + tid] = (float)lam_d[tid];
  }
}

template <int NP>
cudaError_t launch_refine(int N, int32_t nzc, const float* d_G0, float* d_Z, float* d_aux,
                          const int32_t* d_nobs, float* d_S, cudaStream_t st) {
  const size_t smem = refine_smem_floats<NP>() * sizeof(float);
  cudaError_t e = cudaFuncSetAttribute(k_eig_refine<NP>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0, bps = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_eig_refine<NP>, kThreads, smem);
  int grid = sms * (bps > 0 ? bps : 1);
  if (grid > nzc) grid = nzc > 0 ? nzc : 1;
  k_eig_refine<NP><<<grid, kThreads, smem, st>>>(N, nzc, d_G0, d_Z, d_aux, d_nobs, d_S);
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace

size_t zone_refine_scratch(int N) { return (size_t)2 * (N <= 64 ? 64 : 128) * (N <= 64 ? 64 : 128); }

cudaError_t zone_eig_refine(int N, int32_t nzc, const float* d_G0, float* d_Z, float* d_aux,
                            const int32_t* d_nobs, float* d_S, cudaStream_t st) {
  if (N < 2 || N > 128) return cudaErrorInvalidValue;
  if (N <= 64) return launch_refine<64>(N, nzc, d_G0, d_Z, d_aux, d_nobs, d_S, st);
  return launch_refine<128>(N, nzc, d_G0, d_Z, d_aux, d_nobs, d_S, st);
}

}  // namespace oakg
