// K3 + K4 (FP64) -- per-zone symmetric eigensolve and the square-root transform.
//
// For each zone with relevant observations (G = HS^T R^-1_eff HS and g = HS^T R^-1_eff d
// from K2), this computes what rrsqrt.F90:136-185 computes:
//   symeig(G) -> U, lambda        (dsyev('V','L'), matoper_inc.F90:986-1005)
//   lambda <- 1 / (1 + max(lambda, 0))                                    (:137-140)
//   ampl = U (lambda .* (U^T g))                                          (:142)
//   NaN check on ampl                                                     (:145-149)
//   T = U diag(sqrt(lambda)) U^T Omega,  Omega = RotateVector(w, v)       (:162-185)
//       w = 1/sqrt(N),  v = normate(U (colsum(U) / sqrt(lambda)))
// T (N x N, row-major, T[k][c]) overwrites G's slot; Sa = Sf T is formed by K5.
//
// Algorithm (one CTA per zone, matrix in shared memory, all FP64):
//  1. Householder tridiagonalisation A = Q_h Tri Q_h^T (Golub & Van Loan, Matrix
//     Computations 4th ed., 8.3.1), reflector vectors kept below the sub-diagonal.
//  2. Q_h formed explicitly by backward accumulation (GvL 5.1.6).
//  3. Implicit symmetric QR sweeps with Wilkinson shift (GvL 8.3.3-8.3.5) on (d, e): one warp
//     runs the bulge chase and records the Givens rotations of a sweep, then the CTA applies
//     them to the rows of Q.
//  4. With Q = U: ampl, v, T_sym = U diag(sqrt(lambda)) U^T (lower triangle + mirror), then
//     T = T_sym Omega applied in O(N^2): with P_x = I - u_x u_x^T / (1 + |x_N|),
//     u_x = x + sign(x_N) e_N (the reflector whose first N-1 columns are perpSpace(x),
//     matoper.F90:509-535), Omega = P_v P_w + (1 - s_v s_w) v w^T.
#include <cuda_runtime.h>
#include <math.h>

#include "oakg_internal.cuh"

namespace oakg {

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kMaxSweepsPerN = 30;

__device__ __forceinline__ double warp_sum(double x) {
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// Block-wide sum; red must hold kWarps doubles. All threads receive the result.
__device__ __forceinline__ double block_sum(double x, double* red) {
  x = warp_sum(x);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = x;
  __syncthreads();
  double t = 0.0;
#pragma unroll
  for (int w = 0; w < kWarps; w++) t += red[w];
  return t;
}

struct EigShared {
  double red[kWarps];
  double beta_k;
  double scal[8];
  int32_t ctl[4];
};

__global__ void __launch_bounds__(kThreads)
    k_zone_eig_fp64(int N, int32_t nzc, double* __restrict__ GT, const double* __restrict__ gv,
                    const int32_t* __restrict__ nobs, int rotate, double* __restrict__ ampl_out,
                    int32_t* __restrict__ status, int32_t* __restrict__ work) {
  extern __shared__ double dyn[];
  const int ld = N + 1;
  double* A = dyn;            // [N][ld]  matrix, then T_sym
  double* Q = A + N * ld;     // [N][ld]  Q_h, then U
  double* d = Q + N * ld;     // [N] diagonal / eigenvalues
  double* e = d + N;          // [N] off-diagonal
  double* beta = e + N;       // [N] Householder scalars
  double* vec0 = beta + N;    // [N] work vectors
  double* vec1 = vec0 + N;    // [N]
  double* vec2 = vec1 + N;    // [N]
  double* rc = vec2 + N;      // [N] rotation cosines of one sweep
  double* rs = rc + N;        // [N] rotation sines
  __shared__ EigShared es;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  for (;;) {
    if (tid == 0) es.ctl[0] = atomicAdd(work, 1);
    __syncthreads();
    const int32_t zl = es.ctl[0];
    if (zl >= nzc) break;
    if (nobs[zl] == 0) {
      __syncthreads();
      continue;
    }
    double* Gz = GT + (int64_t)zl * N * N;
    for (int idx = tid; idx < N * N; idx += kThreads) {
      int i = idx / N, j = idx - i * N;
      A[i * ld + j] = Gz[idx];
    }
    for (int i = tid; i < N; i += kThreads) vec2[i] = gv[(int64_t)zl * N + i];  // g
    __syncthreads();
    // ||A||_max for the deflation threshold
    double amax = 0.0;
    for (int idx = tid; idx < N * N; idx += kThreads) {
      int i = idx / N, j = idx - i * N;
      amax = fmax(amax, fabs(A[i * ld + j]));
    }
    for (int o = 16; o > 0; o >>= 1) amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    if (lane == 0) es.red[warp] = amax;
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int w = 0; w < kWarps; w++) t = fmax(t, es.red[w]);
      es.scal[7] = t;
    }
    __syncthreads();
    const double anorm = es.scal[7] * N;

    // ---- 1. tridiagonalisation
    for (int k = 0; k < N - 2; k++) {
      const int L = N - k - 1;
      double* col = A + (k + 1) * ld + k;  // x_i = A[k+1+i][k] = col[i*ld]
      double sig = 0.0;
      for (int i = 1 + tid; i < L; i += kThreads) sig += col[i * ld] * col[i * ld];
      sig = block_sum(sig, es.red);
      if (tid == 0) {
        double x0 = col[0];
        if (sig == 0.0) {
          e[k] = x0;
          beta[k] = 0.0;
        } else {
          double mu = sqrt(x0 * x0 + sig);
          double v0 = (x0 <= 0.0) ? x0 - mu : x0 + mu;  // v0 = x0 + sign(x0) mu
          e[k] = (x0 <= 0.0) ? mu : -mu;               // alpha = -sign(x0) ||x||
          beta[k] = 2.0 / (v0 * v0 + sig);
          col[0] = v0;
        }
        d[k] = A[k * ld + k];
        es.beta_k = beta[k];
      }
      __syncthreads();
      const double bk = es.beta_k;
      if (bk == 0.0) continue;
      // v (length L) is col[i*ld]; copy to vec0 for contiguous access
      for (int i = tid; i < L; i += kThreads) vec0[i] = col[i * ld];
      __syncthreads();
      // p = beta A22 v   (A22 = A[k+1.., k+1..], full symmetric storage)
      for (int i = warp; i < L; i += kWarps) {
        const double* row = A + (k + 1 + i) * ld + (k + 1);
        double s = 0.0;
        for (int j = lane; j < L; j += 32) s = fma(row[j], vec0[j], s);
        s = warp_sum(s);
        if (lane == 0) vec1[i] = bk * s;
      }
      __syncthreads();
      double pv = 0.0;
      for (int i = tid; i < L; i += kThreads) pv = fma(vec1[i], vec0[i], pv);
      pv = block_sum(pv, es.red);
      const double Kc = 0.5 * bk * pv;
      for (int i = tid; i < L; i += kThreads) vec1[i] = vec1[i] - Kc * vec0[i];  // w
      __syncthreads();
      // A22 -= v w^T + w v^T
      for (int idx = tid; idx < L * L; idx += kThreads) {
        int i = idx / L, j = idx - i * L;
        double* a = A + (k + 1 + i) * ld + (k + 1 + j);
        *a = *a - vec0[i] * vec1[j] - vec1[i] * vec0[j];
      }
      __syncthreads();
    }
    if (tid == 0) {
      if (N >= 2) {
        d[N - 2] = A[(N - 2) * ld + (N - 2)];
        e[N - 2] = A[(N - 1) * ld + (N - 2)];
      }
      d[N - 1] = A[(N - 1) * ld + (N - 1)];
      e[N - 1] = 0.0;
    }
    // ---- 2. Q_h = H_0 ... H_{N-3} (backward accumulation)
    for (int idx = tid; idx < N * N; idx += kThreads) {
      int i = idx / N, j = idx - i * N;
      Q[i * ld + j] = (i == j) ? 1.0 : 0.0;
    }
    __syncthreads();
    for (int k = N - 3; k >= 0; k--) {
      const double bk = beta[k];
      if (bk == 0.0) continue;
      const int L = N - k - 1;
      const double* col = A + (k + 1) * ld + k;
      // y_j = sum_i v_i Q[k+1+i][k+1+j]
      for (int j = tid; j < L; j += kThreads) {
        double s = 0.0;
        for (int i = 0; i < L; i++) s = fma(col[i * ld], Q[(k + 1 + i) * ld + (k + 1 + j)], s);
        vec1[j] = bk * s;
      }
      __syncthreads();
      for (int idx = tid; idx < L * L; idx += kThreads) {
        int i = idx / L, j = idx - i * L;
        double* q = Q + (k + 1 + i) * ld + (k + 1 + j);
        *q = fma(-col[i * ld], vec1[j], *q);
      }
      __syncthreads();
    }
    // ---- 3. implicit QR sweeps on (d, e) with rotations applied to Q's columns
    const double eps = 1.1102230246251565e-16;
    int hi = N - 1, sweeps = 0, failed = 0;
    const int max_sweeps = kMaxSweepsPerN * N;
    while (hi > 0) {
      // deflation scan (warp 0 decides, everyone follows)
      if (tid == 0) {
        int h = hi;
        while (h > 0) {
          double t = fabs(e[h - 1]);
          if (t <= eps * (fabs(d[h - 1]) + fabs(d[h])) || t <= eps * anorm * 1e-3) {
            e[h - 1] = 0.0;
            h--;
          } else {
            break;
          }
        }
        int lo = h;
        if (h > 0) {
          lo = h - 1;
          while (lo > 0) {
            double t = fabs(e[lo - 1]);
            if (t <= eps * (fabs(d[lo - 1]) + fabs(d[lo])) || t <= eps * anorm * 1e-3) {
              e[lo - 1] = 0.0;
              break;
            }
            lo--;
          }
        }
        es.ctl[1] = h;
        es.ctl[2] = lo;
      }
      __syncthreads();
      hi = es.ctl[1];
      const int lo = es.ctl[2];
      if (hi <= 0) break;
      if (++sweeps > max_sweeps) {
        failed = 1;
        break;
      }
      // one implicit QR step on [lo, hi], computed by warp 0 (all lanes redundantly)
      if (warp == 0) {
        double a = d[hi - 1], b = d[hi], f = e[hi - 1];
        double del = 0.5 * (a - b);
        double den = del + copysign(sqrt(del * del + f * f), del == 0.0 ? 1.0 : del);
        double mu = (den == 0.0) ? b : b - f * f / den;
        double x = d[lo] - mu, z = e[lo], bulge = 0.0;
        for (int k = lo; k < hi; k++) {
          // every lane reads its operands before lane 0 writes this step's results
          if (k > lo) {
            x = e[k - 1];
            z = bulge;
          }
          const double dk = d[k], dk1 = d[k + 1], ek = e[k];
          const double ek1 = (k + 1 < hi) ? e[k + 1] : 0.0;
          __syncwarp();
          double r = hypot(x, z);
          double c = 1.0, s = 0.0;
          if (r != 0.0) {
            c = x / r;
            s = z / r;
          }
          double cc = c * c, ss = s * s, cs = c * s;
          double nd0 = cc * dk + 2.0 * cs * ek + ss * dk1;
          double nd1 = ss * dk - 2.0 * cs * ek + cc * dk1;
          double ne = cs * (dk1 - dk) + (cc - ss) * ek;
          if (lane == 0) {
            if (k > lo) e[k - 1] = r;
            d[k] = nd0;
            d[k + 1] = nd1;
            e[k] = ne;
            if (k + 1 < hi) e[k + 1] = c * ek1;
            rc[k] = c;
            rs[k] = s;
          }
          bulge = s * ek1;
          __syncwarp();
        }
      }
      __syncthreads();
      // Q <- Q P_k^T for k = lo..hi-1: new col_k = c col_k + s col_{k+1},
      // new col_{k+1} = -s col_k + c col_{k+1}
      for (int row = tid; row < N; row += kThreads) {
        double* qr = Q + row * ld;
        double qa = qr[lo];
        for (int k = lo; k < hi; k++) {
          const double c = rc[k], s = rs[k];
          const double qb = qr[k + 1];
          qr[k] = c * qa + s * qb;
          qa = -s * qa + c * qb;
        }
        qr[hi] = qa;
      }
      __syncthreads();
    }
    // ---- 4. amplitudes, rotation vector, transform
    // d = eigenvalues; lambda <- 1/(1+max(d,0)), vec0 = lambda, vec1 = sqrt(lambda)
    for (int i = tid; i < N; i += kThreads) {
      double l = d[i];
      if (l < 0.0) l = 0.0;
      double lam = 1.0 / (1.0 + l);
      vec0[i] = lam;
      vec1[i] = sqrt(lam);
    }
    __syncthreads();
    // y = lambda .* (U^T g) -> beta[] (free now)
    for (int i = tid; i < N; i += kThreads) {
      double s = 0.0;
      for (int j = 0; j < N; j++) s = fma(Q[j * ld + i], vec2[j], s);
      beta[i] = vec0[i] * s;
    }
    __syncthreads();
    int nan_flag = 0;
    for (int j = tid; j < N; j += kThreads) {
      double s = 0.0;
      for (int i = 0; i < N; i++) s = fma(Q[j * ld + i], beta[i], s);
      ampl_out[(int64_t)zl * N + j] = s;
      if (!(s == s) || isinf(s)) nan_flag = 1;
    }
    nan_flag = __syncthreads_or(nan_flag);
    if (rotate) {
      // t_i = colsum(U)_i / sqrt(lambda_i) -> rc[]
      for (int i = tid; i < N; i += kThreads) {
        double s = 0.0;
        for (int j = 0; j < N; j++) s += Q[j * ld + i];
        rc[i] = s / vec1[i];
      }
      __syncthreads();
      double nrm = 0.0;
      for (int j = tid; j < N; j += kThreads) {
        double s = 0.0;
        for (int i = 0; i < N; i++) s = fma(Q[j * ld + i], rc[i], s);
        rs[j] = s;  // v (unnormalised)
        nrm = fma(s, s, nrm);
      }
      nrm = block_sum(nrm, es.red);
      const double inv = 1.0 / sqrt(nrm);
      for (int j = tid; j < N; j += kThreads) rs[j] = rs[j] * inv;  // v = normate(v)
      __syncthreads();
    }
    // T_sym = U diag(sqrt(lambda)) U^T: scale U's columns by lambda^(1/4), then U U^T
    for (int idx = tid; idx < N * N; idx += kThreads) {
      int i = idx / N, k = idx - i * N;
      Q[i * ld + k] *= sqrt(vec1[k]);
    }
    __syncthreads();
    const int E = N * (N + 1) / 2;
    for (int e2 = tid; e2 < E; e2 += kThreads) {
      int a = (int)((sqrt(8.0 * e2 + 1.0) - 1.0) * 0.5);
      while ((a + 1) * (a + 2) / 2 <= e2) a++;
      while (a * (a + 1) / 2 > e2) a--;
      int b = e2 - a * (a + 1) / 2;
      const double* qa = Q + a * ld;
      const double* qb = Q + b * ld;
      double s = 0.0;
      for (int k = 0; k < N; k++) s = fma(qa[k], qb[k], s);
      A[a * ld + b] = s;
      A[b * ld + a] = s;
    }
    __syncthreads();
    if (rotate) {
      // v in rs[], w = 1/sqrt(N). u_v = v + s_v e_N, c_v = 1 + |v_N|; same for w.
      const double vN = rs[N - 1];
      const double sv = signbit(vN) ? -1.0 : 1.0;
      const double cv = 1.0 + fabs(vN);
      const double wv = 1.0 / sqrt((double)N);
      const double cw = 1.0 + wv;
      // a = T_sym u_v -> vec0 ; tv = T_sym v -> vec2 (g is no longer needed)
      for (int i = tid; i < N; i += kThreads) {
        const double* ti = A + i * ld;
        double sa = 0.0, sb = 0.0;
        for (int j = 0; j < N; j++) {
          double uj = rs[j] + ((j == N - 1) ? sv : 0.0);
          sa = fma(ti[j], uj, sa);
          sb = fma(ti[j], rs[j], sb);
        }
        vec0[i] = sa;
        vec2[i] = sb;
      }
      __syncthreads();
      // T1 = T_sym - a u_v^T / c_v
      for (int idx = tid; idx < N * N; idx += kThreads) {
        int i = idx / N, j = idx - i * N;
        double uj = rs[j] + ((j == N - 1) ? sv : 0.0);
        A[i * ld + j] -= vec0[i] * uj / cv;
      }
      __syncthreads();
      // b = T1 u_w -> vec1
      for (int i = tid; i < N; i += kThreads) {
        const double* ti = A + i * ld;
        double s = 0.0;
        for (int j = 0; j < N; j++) s = fma(ti[j], wv + ((j == N - 1) ? 1.0 : 0.0), s);
        vec1[i] = s;
      }
      __syncthreads();
      // T = T1 - b u_w^T / c_w + (1 - s_v s_w) (T_sym v) w^T   (s_w = +1)
      const double extra = 1.0 - sv;
      for (int idx = tid; idx < N * N; idx += kThreads) {
        int i = idx / N, j = idx - i * N;
        double uj = wv + ((j == N - 1) ? 1.0 : 0.0);
        double t = A[i * ld + j] - vec1[i] * uj / cw;
        if (extra != 0.0) t = fma(extra * vec2[i], wv, t);
        Gz[idx] = t;
      }
    } else {
      for (int idx = tid; idx < N * N; idx += kThreads) {
        int i = idx / N, j = idx - i * N;
        Gz[idx] = A[i * ld + j];
      }
    }
    if (tid == 0) status[zl] = (failed ? ZST_EIG : 0) | (nan_flag ? ZST_NAN : 0);
    __syncthreads();
  }
}

}  // namespace

size_t zone_eig_fp64_smem(int N) { return (size_t)(2 * N * (N + 1) + 8 * N) * sizeof(double); }

cudaError_t zone_eig_fp64(int N, int32_t nzc, double* d_GT, const double* d_g,
                          const int32_t* d_nobs, int rotate, double* d_ampl, int32_t* d_status,
                          int32_t* d_work, cudaStream_t st) {
  size_t smem = zone_eig_fp64_smem(N);
  cudaError_t e = cudaFuncSetAttribute(k_zone_eig_fp64,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int bps = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_zone_eig_fp64, kThreads, smem);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int grid = sms * (bps > 0 ? bps : 1);
  if (grid > nzc) grid = nzc > 0 ? nzc : 1;
  e = cudaMemsetAsync(d_work, 0, sizeof(int32_t), st);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(d_status, 0, sizeof(int32_t) * (nzc > 0 ? nzc : 1), st);
  if (e != cudaSuccess) return e;
  k_zone_eig_fp64<<<grid, kThreads, smem, st>>>(N, nzc, d_GT, d_g, d_nobs, rotate, d_ampl,
                                                 d_status, d_work);
  return cudaGetLastError();
}

}  // namespace oakg
