// Ensemble prologue and epilogue of the analysis (Assim, assimilation.F90), FP64:
//   prologue  HE_f(:,k) = obsoper(H, E_f(:,k)) + Hshift        (assimilation.F90:3110-3114)
//             x_f = mean_k E_f(:,k),  Hx_f = mean_k HE_f(:,k)  (:3127-3128)
//             S_f = (E_f - x_f) / scaling,  HS_f = (HE_f - Hx_f) / scaling,
//             scaling = sqrt(N - 1)                            (:3130-3134, ASSIM_SCALING = 1)
//   epilogue  S_a = mult S_a                                   (inflation, :3299-3304)
//             x_a clipped to x_f +- maxCorrection              (:3305-3312)
//             E_a(:,k) = x_a + scaling S_a(:,k)                 (:3558-3565)
// The observation operator is the reference's sparse interpolation matrix H (m x n, a few
// non-zeros per row: nearest cell, n-linear), stored row-wise as K (index, weight) pairs per
// observation; a negative index marks an unused pair.
//
// Ensembles are the reference's column-major (rows, N) arrays. The mean/anomaly kernel runs one
// thread per state row (members at stride ld: coalesced across the warp for each member); the
// operator gathers K rows per observation and member (one thread per observation and member,
// consecutive threads on consecutive observations); all are HBM- or gather-bound.
#include <cuda_runtime.h>
#include <math.h>

#include "oakg_internal.cuh"

namespace oakg {

namespace {

constexpr int kThreads = 256;

inline unsigned grid_for(int64_t n) {
  int64_t b = (n + kThreads - 1) / kThreads;
  if (b > 152 * 64) b = 152 * 64;
  return (unsigned)(b < 1 ? 1 : b);
}

// mean and scaled anomalies of the rows of E (rows x N, leading dimension ldE)
__global__ void k_mean_anomalies(int64_t rows, int N, const double* __restrict__ E, int64_t ldE,
                                 double scaling, double* __restrict__ mean,
                                 double* __restrict__ S, int64_t ldS) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < rows;
       i += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int k = 0; k < N; k++) s += E[i + (int64_t)k * ldE];
    const double mu = s / N;
    mean[i] = mu;
    for (int k = 0; k < N; k++) S[i + (int64_t)k * ldS] = (E[i + (int64_t)k * ldE] - mu) / scaling;
  }
}

// HE(j, k) = sum_t w(j, t) E(idx(j, t), k) + shift(j)
__global__ void k_obsoper(int64_t m, int N, int K, const int64_t* __restrict__ idx,
                          const double* __restrict__ w, const double* __restrict__ shift,
                          const double* __restrict__ E, int64_t ldE, double* __restrict__ HE,
                          int64_t ldH) {
  const int64_t total = m * (int64_t)N;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(t / m);
    const int64_t j = t - (int64_t)k * m;
    double s = 0.0;
    for (int q = 0; q < K; q++) {
      const int64_t r = idx[j * K + q];
      if (r >= 0) s += w[j * K + q] * E[r + (int64_t)k * ldE];
    }
    if (shift) s += shift[j];
    HE[j + (int64_t)k * ldH] = s;
  }
}

__global__ void k_epilogue(int64_t n, int N, const double* __restrict__ xf,
                           const double* __restrict__ xa, const double* __restrict__ Sa,
                           int64_t ldS, double mult, double scaling,
                           const double* __restrict__ maxcorr,
                           double* __restrict__ Ea, int64_t ldE) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double x = xa[i];
    if (maxcorr) {
      const double mc = maxcorr[i], f = xf[i];
      if (x - mc > f) x = f + mc;  // the reference's two where() in this order
      if (x < f - mc) x = f - mc;
    }
    for (int k = 0; k < N; k++)
      Ea[i + (int64_t)k * ldE] = x + scaling * (mult * Sa[i + (int64_t)k * ldS]);
  }
}

}  // namespace

cudaError_t ensemble_prologue(int64_t n, int N, const double* Ef, int64_t ldE, int64_t m, int K,
                              const int64_t* idx, const double* w, const double* shift,
                              double* xf, double* Sf, int64_t ldS, double* Hxf, double* HSf,
                              int64_t ldH, double* HEf_scratch, cudaStream_t st) {
  const double scaling = sqrt((double)N - 1.0);
  k_mean_anomalies<<<grid_for(n), kThreads, 0, st>>>(n, N, Ef, ldE, scaling, xf, Sf, ldS);
  count_launches(1);
  if (m > 0) {
    k_obsoper<<<grid_for(m * (int64_t)N), kThreads, 0, st>>>(m, N, K, idx, w, shift, Ef, ldE,
                                                             HEf_scratch, m);
    k_mean_anomalies<<<grid_for(m), kThreads, 0, st>>>(m, N, HEf_scratch, m, scaling, Hxf, HSf,
                                                       ldH);
    count_launches(2);
  }
  return cudaGetLastError();
}

cudaError_t ensemble_epilogue(int64_t n, int N, const double* xf, const double* xa,
                              const double* Sa, int64_t ldS, double inflation,
                              const double* maxcorr, double* Ea, int64_t ldE, cudaStream_t st) {
  k_epilogue<<<grid_for(n), kThreads, 0, st>>>(n, N, xf, xa, Sa, ldS, inflation,
                                               sqrt((double)N - 1.0), maxcorr, Ea, ldE);
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace oakg
