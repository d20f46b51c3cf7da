// Ensemble prologue and epilogue of the analysis (Assim, assimilation.F90), FP64:
//   prologue  HE_f(:,k) = obsoper(H, E_f(:,k)) + Hshift        (assimilation.F90:3110-3114)
//             x_f = mean_k E_f(:,k),  Hx_f = mean_k HE_f(:,k)  (:3127-3128)
//             S_f = (E_f - x_f) / scaling,  HS_f = (HE_f - Hx_f) / scaling,
//             scaling = sqrt(N - 1)                            (:3130-3134, ASSIM_SCALING = 1)
//   epilogue  S_a = mult S_a                                   (inflation, :3299-3304)
//             x_a clipped to x_f +- maxCorrection              (:3305-3312)
//             E_a(:,k) = x_a + scaling S_a(:,k)                 (:3558-3565)
// and the ensemble conversions of rrsqrt.F90 (ens2sqrt, sqrt2ens: N <-> N - 1 columns) and the
// elementwise steps of the bias-aware analysis (biasedLocAnalysis).
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

// mean and scaled anomalies of the rows of E (rows x N, leading dimension ldE). A thread takes
// a row: the sum over the members, then (E - mean) / scaling as one FMA, E (1/scaling) -
// mean (1/scaling): its error is within an ulp of mean / scaling, the resolution E itself has
// at the mean's magnitude. The FP64 pipe is what bounds this kernel (the row's E is read twice,
// the second time from L2): two FP64 operations an element instead of three (subtract,
// multiply) is what lets it approach the HBM rate.
__global__ void __launch_bounds__(kThreads)
    k_mean_anomalies(int64_t rows, int N, const double* __restrict__ E, int64_t ldE,
                     double scaling, double* __restrict__ mean, double* __restrict__ S,
                     int64_t ldS) {
  const double isc = 1.0 / scaling;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < rows;
       i += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
#pragma unroll 8
    for (int k = 0; k < N; k++) s += E[i + (int64_t)k * ldE];
    const double mu = s / N;
    mean[i] = mu;
    const double off = -mu * isc;
#pragma unroll 8
    for (int k = 0; k < N; k++) S[i + (int64_t)k * ldS] = fma(E[i + (int64_t)k * ldE], isc, off);
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
    const double f = scaling * mult;  // one FMA an element: the FP64 pipe bounds this loop
    for (int k = 0; k < N; k++) Ea[i + (int64_t)k * ldE] = fma(f, Sa[i + (int64_t)k * ldS], x);
  }
}

// Pham's reduction of an ensemble to N - 1 anomaly columns (ens2sqrt, rrsqrt.F90:786-806):
//   alpha = (sqrt(N) - 1) / (N - 1), shift = (1 - alpha) mean + alpha E(:, N),
//   S(:, i) = (E(:, i) - shift) / sqrt(N - 1), i < N
__global__ void k_ens2sqrt(int64_t rows, int N, const double* __restrict__ E, int64_t ldE,
                           double* __restrict__ mean, double* __restrict__ S, int64_t ldS) {
  const double alpha = (-1.0 + sqrt((double)N)) / (N - 1.0);
  const double isc = 1.0 / sqrt(N - 1.0);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < rows;
       i += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int k = 0; k < N; k++) s += E[i + (int64_t)k * ldE];
    const double mu = s / N;
    mean[i] = mu;
    const double shift = (1.0 - alpha) * mu + alpha * E[i + (int64_t)(N - 1) * ldE];
    const double off = -shift * isc;  // (E - shift) / sqrt(N - 1) as one FMA (as the prologue)
    for (int k = 0; k < N - 1; k++) S[i + (int64_t)k * ldS] = fma(E[i + (int64_t)k * ldE], isc, off);
  }
}

// sqrt2ens (rrsqrt.F90:815-839): E(i, j) = mean(i) + sum_k S(i, k) Om(j, k), Om (N x N-1,
// row-major, staged in shared memory); a block takes tiles of kRowsE rows, the S tile staged
// column by column (coalesced along rows), one thread per (row, member) item
constexpr int kRowsE = 64;
__global__ void __launch_bounds__(kThreads)
    k_sqrt2ens(int64_t rows, int N, const double* __restrict__ mean, const double* __restrict__ S,
               int64_t ldS, const double* __restrict__ Om, double* __restrict__ E, int64_t ldE) {
  extern __shared__ __align__(16) unsigned char dyn_raw[];
  double* so = reinterpret_cast<double*>(dyn_raw);  // [N][N-1]
  double* st = so + N * (N - 1);                    // [N-1][kRowsE]
  const int K = N - 1;
  for (int idx = threadIdx.x; idx < N * K; idx += kThreads) so[idx] = Om[idx];
  const int64_t ntiles = (rows + kRowsE - 1) / kRowsE;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int64_t r0 = t * kRowsE;
    const int R_ = (int)((rows - r0) < kRowsE ? (rows - r0) : kRowsE);
    __syncthreads();  // Om staged / previous tile consumed
    for (int idx = threadIdx.x; idx < R_ * K; idx += kThreads) {
      const int k = idx / R_, r = idx - k * R_;
      st[k * kRowsE + r] = S[r0 + r + (int64_t)k * ldS];
    }
    __syncthreads();
    for (int it = threadIdx.x; it < R_ * N; it += kThreads) {
      const int j = it / R_, r = it - j * R_;
      const double* oj = so + j * K;
      double acc = 0.0;
      for (int k = 0; k < K; k++) acc = fma(st[k * kRowsE + r], oj[k], acc);
      E[r0 + r + (int64_t)j * ldE] = mean[r0 + r] + acc;
    }
  }
}

// sqrt2ens with Theta = I: Om = sqrt(N-1) perpSpace(w) has rows sqrt(N-1) (e_i + a w^2 1) for
// i < N-1 and sqrt(N-1) a (w + 1) w 1 for the last (a = -1 / (w + 1), w = 1/sqrt(N)), so
//   E(:, i) = mean + sqrt(N-1) (S(:, i) + a w^2 rs),  E(:, N-1) = mean + sqrt(N-1) a (w+1) w rs,
// rs the row sums of S: no N x N-1 product. A thread takes a row in two passes over S (the
// second from L2) with few registers, and one FMA an element: the FP64 pipe bounds the loop.
__global__ void __launch_bounds__(kThreads)
    k_sqrt2ens_identity(int64_t rows, int N, const double* __restrict__ mean,
                        const double* __restrict__ S, int64_t ldS, double* __restrict__ E,
                        int64_t ldE) {
  const int K = N - 1;
  const double w = 1.0 / sqrt((double)N), a = -1.0 / (w + 1.0), sc = sqrt((double)N - 1.0);
  const double cw = a * w * w, cl = sc * a * (w + 1.0) * w;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < rows;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double mu = mean[i];
    double rs = 0.0;
#pragma unroll 8
    for (int k = 0; k < K; k++) rs += S[i + (int64_t)k * ldS];
    const double base = fma(sc * cw, rs, mu);
#pragma unroll 8
    for (int k = 0; k < K; k++) E[i + (int64_t)k * ldE] = fma(sc, S[i + (int64_t)k * ldS], base);
    E[i + (int64_t)K * ldE] = fma(cl, rs, mu);
  }
}

// E(:, j) = mean (the ensemble mean under the S Om^T product added by the library GEMM)
__global__ void k_fill_columns(int64_t rows, int N, const double* __restrict__ mean,
                               double* __restrict__ E, int64_t ldE) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < rows;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double mu = mean[i];
    for (int k = 0; k < N; k++) E[i + (int64_t)k * ldE] = mu;
  }
}

// the elementwise steps of the bias-aware analysis (rrsqrt.F90:520-540):
//   ba = bf - gamma inc, ux = xf - ba
__global__ void k_bias_update(int64_t n, double gamma, const double* __restrict__ bf,
                              const double* __restrict__ inc, const double* __restrict__ xf,
                              double* __restrict__ ba, double* __restrict__ ux) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double b = bf[i] - gamma * inc[i];
    ba[i] = b;
    ux[i] = xf[i] - b;
  }
}

// y = a x + b z (any of b, z may be absent: y = a x)
__global__ void k_axpby(int64_t n, double a, const double* __restrict__ x, double b,
                        const double* __restrict__ z, double* __restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = z ? fma(b, z[i], a * x[i]) : a * x[i];
}

}  // namespace

cudaError_t ensemble_ens2sqrt(int64_t n, int N, const double* E, int64_t ldE, double* mean,
                              double* S, int64_t ldS, cudaStream_t st) {
  k_ens2sqrt<<<grid_for(n), kThreads, 0, st>>>(n, N, E, ldE, mean, S, ldS);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t ensemble_sqrt2ens(int64_t n, int N, const double* mean, const double* S, int64_t ldS,
                              const double* Om, double* E, int64_t ldE, cudaStream_t st) {
  const size_t smem = ((size_t)N * (N - 1) + (size_t)(N - 1) * kRowsE) * sizeof(double);
  cudaError_t e = cudaFuncSetAttribute(k_sqrt2ens, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  int64_t tiles = (n + kRowsE - 1) / kRowsE;
  const int grid = (int)(tiles < 152 * 4 ? (tiles < 1 ? 1 : tiles) : 152 * 4);
  k_sqrt2ens<<<grid, kThreads, smem, st>>>(n, N, mean, S, ldS, Om, E, ldE);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t ensemble_sqrt2ens_identity(int64_t n, int N, const double* mean, const double* S,
                                       int64_t ldS, double* E, int64_t ldE, cudaStream_t st) {
  k_sqrt2ens_identity<<<grid_for(n), kThreads, 0, st>>>(n, N, mean, S, ldS, E, ldE);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t ensemble_fill_columns(int64_t n, int N, const double* mean, double* E, int64_t ldE,
                                  cudaStream_t st) {
  k_fill_columns<<<grid_for(n), kThreads, 0, st>>>(n, N, mean, E, ldE);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t obsoper_apply(int64_t m, int K, const int64_t* idx, const double* w,
                          const double* shift, const double* x, int64_t ldx, double* y,
                          cudaStream_t st) {
  k_obsoper<<<grid_for(m), kThreads, 0, st>>>(m, 1, K, idx, w, shift, x, ldx, y, m);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t bias_update(int64_t n, double gamma, const double* bf, const double* inc,
                        const double* xf, double* ba, double* ux, cudaStream_t st) {
  k_bias_update<<<grid_for(n), kThreads, 0, st>>>(n, gamma, bf, inc, xf, ba, ux);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t axpby(int64_t n, double a, const double* x, double b, const double* z, double* y,
                  cudaStream_t st) {
  k_axpby<<<grid_for(n), kThreads, 0, st>>>(n, a, x, b, z, y);
  count_launches(1);
  return cudaGetLastError();
}

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
