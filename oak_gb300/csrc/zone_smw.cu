// Non-diagonal observation error covariance of the SMWCovar kind, R = diag(C) + B B^T
// (covariance.F90:464-570), in the local analysis (FP64).
//
// The reference solves with R by Sherman-Morrison-Woodbury: R^-1 x = C^-1 x - C^-1 B D B^T C^-1 x,
// D = (B^T C^-1 B + I)^-1 (SMWCovar_init :475-483, SMWCovar_mldivide_vec :525-535), with B and C
// packed to each zone's relevant observations (SMWCovar_pack :540-570) and the localisation
// weights applied outside (DCDCovar(w, R), rrsqrt.F90:395: R_loc^-1 = W R^-1 W). With
// X = C^-1/2 W HS_sel, Y = C^-1/2 B_sel and z = C^-1/2 W (yo - Hxf)_sel:
//   G = HS^T R_loc^-1 HS = X^T X - (X^T Y) D (Y^T X),   D = (Y^T Y + I)^-1
//   g = HS^T R_loc^-1 d  = X^T z - (X^T Y) D (Y^T z).
// The zone Gram kernel computes every block at once from augmented rows [HS_q | B_q] (zone_gram.cu);
// k_smw_reduce applies the reduction per zone: Cholesky of M = Y^T Y + I (k x k, SPD), two
// triangular solves for the N + 1 right-hand sides [Y^T X | Y^T z], then the rank-k update.
#include <cuda_runtime.h>
#include <math.h>

#include "oakg_internal.cuh"

namespace oakg {

namespace {

constexpr int kThreads = 256;

// HStA(s, j) = HSt(s, j) for j < N, B(perm(s), j - N) beyond
__global__ void k_smw_rows(int64_t m, int N, int k, const double* __restrict__ HSt,
                           const int32_t* __restrict__ perm, const double* __restrict__ B,
                           int64_t ldB, double* __restrict__ HStA) {
  const int NA = N + k;
  const int64_t total = m * NA;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = t / NA;
    const int j = (int)(t - s * NA);
    HStA[t] = (j < N) ? HSt[s * N + j] : B[(int64_t)perm[s] + (int64_t)(j - N) * ldB];
  }
}

// one block per zone; shared: A [NA][NA] (the augmented products), Y [k][N + 1]
__global__ void __launch_bounds__(kThreads)
    k_smw_reduce(int N, int k, int32_t nzc, const double* __restrict__ Ga,
                 const double* __restrict__ ga, const int32_t* __restrict__ nobs,
                 double* __restrict__ G, double* __restrict__ gv) {
  extern __shared__ __align__(16) double sm[];
  const int NA = N + k, R1 = N + 1;
  double* A = sm;           // [NA][NA]
  double* Y = A + NA * NA;  // [k][N + 1]
  const int tid = threadIdx.x;
  const int32_t zl = blockIdx.x;
  if (zl >= nzc || nobs[zl] == 0) return;  // block-uniform
  const double* Gz = Ga + (int64_t)zl * NA * NA;
  const double* gz = ga + (int64_t)zl * NA;
  for (int idx = tid; idx < NA * NA; idx += kThreads) A[idx] = Gz[idx];
  for (int idx = tid; idx < k * R1; idx += kThreads) {
    const int l = idx / R1, c = idx - l * R1;  // right-hand sides: Y^T X (c < N), Y^T z (c = N)
    Y[idx] = (c < N) ? Gz[(int64_t)(N + l) * NA + c] : gz[N + l];
  }
  __syncthreads();
  // Cholesky of M = Y^T Y + I in place (lower triangle of A's trailing block), right-looking
  double* M = A + N * NA + N;  // M(i, j) = M[i * NA + j]
  if (tid < k) M[tid * NA + tid] += 1.0;
  __syncthreads();
  for (int j = 0; j < k; j++) {
    if (tid == 0) M[j * NA + j] = sqrt(M[j * NA + j]);
    __syncthreads();
    const double djj = M[j * NA + j];
    for (int i = j + 1 + tid; i < k; i += kThreads) M[i * NA + j] /= djj;
    __syncthreads();
    const int rem = k - j - 1;
    for (int idx = tid; idx < rem * rem; idx += kThreads) {
      const int i = j + 1 + idx / rem, l = j + 1 + idx % rem;
      if (l <= i) M[i * NA + l] = fma(-M[i * NA + j], M[l * NA + j], M[i * NA + l]);
    }
    __syncthreads();
  }
  // Y <- M^-1 Y: L L^T y = b, one right-hand side per thread
  for (int c = tid; c < R1; c += kThreads) {
    for (int l = 0; l < k; l++) {
      double s = Y[l * R1 + c];
      for (int t = 0; t < l; t++) s = fma(-M[l * NA + t], Y[t * R1 + c], s);
      Y[l * R1 + c] = s / M[l * NA + l];
    }
    for (int l = k - 1; l >= 0; l--) {
      double s = Y[l * R1 + c];
      for (int t = l + 1; t < k; t++) s = fma(-M[t * NA + l], Y[t * R1 + c], s);
      Y[l * R1 + c] = s / M[l * NA + l];
    }
  }
  __syncthreads();
  // G = X^T X - (X^T Y) (M^-1 Y^T X), g = X^T z - (X^T Y) (M^-1 Y^T z)
  double* Gout = G + (int64_t)zl * N * N;
  for (int idx = tid; idx < N * N; idx += kThreads) {
    const int i = idx / N, j = idx - i * N;
    double s = A[i * NA + j];
    for (int l = 0; l < k; l++) s = fma(-A[i * NA + N + l], Y[l * R1 + j], s);
    Gout[idx] = s;
  }
  for (int i = tid; i < N; i += kThreads) {
    double s = gz[i];
    for (int l = 0; l < k; l++) s = fma(-A[i * NA + N + l], Y[l * R1 + N], s);
    gv[(int64_t)zl * N + i] = s;
  }
}

}  // namespace

cudaError_t smw_rows(int64_t m, int N, int k, const double* HSt, const int32_t* perm,
                     const double* B, int64_t ldB, double* HStA, cudaStream_t st) {
  const int64_t total = m * (N + k);
  int64_t blocks = (total + kThreads - 1) / kThreads;
  if (blocks > 152 * 32) blocks = 152 * 32;
  k_smw_rows<<<(unsigned)(blocks < 1 ? 1 : blocks), kThreads, 0, st>>>(m, N, k, HSt, perm, B, ldB,
                                                                      HStA);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t smw_reduce(int N, int k, int32_t nzc, const double* Ga, const double* ga,
                       const int32_t* nobs, double* G, double* gv, cudaStream_t st) {
  const int NA = N + k;
  const size_t smem = ((size_t)NA * NA + (size_t)k * (N + 1)) * sizeof(double);
  cudaError_t e = cudaFuncSetAttribute(k_smw_reduce, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  k_smw_reduce<<<nzc > 0 ? nzc : 1, kThreads, smem, st>>>(N, k, nzc, Ga, ga, nobs, G, gv);
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace oakg
