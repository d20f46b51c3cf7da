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
// GB300 executes one FP64 warp instruction per ~16 SM cycles whatever its active-lane mask,
// so the work is split into kernels whose FP64 instructions keep all 32 lanes busy:
//  E1  (one CTA per zone): Householder tridiagonalisation A = Q_h Tri Q_h^T (Golub & Van
//      Loan, Matrix Computations 4th ed., 8.3.1) in shared memory on the lower triangle; the
//      reflector vectors stay below the diagonal of G's slot.
//  E2a (one thread per zone): eigenvalues of Tri by implicit symmetric QR sweeps with
//      Wilkinson shift (GvL 8.3.3-8.3.5), sorted; shifts for inverse iteration separated
//      as LAPACK dstein does (lambda_j >= lambda_{j-1} + 10 eps |lambda_j|).
//  E2b (one thread per eigenpair): eigenvector of Tri by inverse iteration, two solves with
//      the partial-pivoting LU of Tri - shift I.
//  E3  (one CTA per zone): eigenvectors re-orthogonalised inside clusters
//      |lambda_j - lambda_{j-1}| <= 1e-3 ||Tri||_1 (the dstein convention) by two classical
//      Gram-Schmidt passes; U = Q_h Z; ampl, v, T_sym = U diag(sqrt(lambda)) U^T and
//      T = T_sym Omega, Omega applied in O(N^2) through its reflector form: with
//      P_x = I - u_x u_x^T / (1 + |x_N|), u_x = x + sign(x_N) e_N (the reflector whose first
//      N-1 columns are perpSpace(x), matoper.F90:509-535), Omega = P_v P_w + (1 - s_v s_w) v w^T.
#include <cuda_runtime.h>
#include <math.h>

#include "oakg_internal.cuh"

namespace oakg {

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kNMax = 112;               // largest N (matches max_fp64_ensemble)
constexpr int kMaxSweepsPerN = 30;
constexpr double kEps = 1.1102230246251565e-16;

// per-zone auxiliary layout (doubles):
//   d[N] e[N] beta[N] lambda[N] shift[N] | anorm onenrm
__host__ __device__ inline int aux_stride(int N) { return 5 * N + 2; }

__device__ __forceinline__ double warp_sum(double x) {
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// (row, col) of the e2-th lower-triangle entry. The estimate uses an FP32 square root (the
// FP64 pipe is the bottleneck of every kernel here) and integer fix-ups make it exact.
__device__ __forceinline__ void lower_index(int e2, int& a, int& b) {
  a = (int)((__fsqrt_rn((float)(8 * e2 + 1)) - 1.0f) * 0.5f);
  while ((a + 1) * (a + 2) / 2 <= e2) a++;
  while (a * (a + 1) / 2 > e2) a--;
  b = e2 - a * (a + 1) / 2;
}

// ------------------------------------------------------------------------------------ E1
__global__ void __launch_bounds__(kThreads)
    k_eig_tridiag(int N, int32_t nzc, double* __restrict__ GT, double* __restrict__ aux,
                  const int32_t* __restrict__ nobs, int32_t* __restrict__ work) {
  extern __shared__ double dyn[];
  const int ld = N + 1;
  double* A = dyn;          // [N][ld], lower triangle valid
  double* v = A + N * ld;   // [N]
  double* w = v + N;        // [N]
  __shared__ double red[kWarps];
  __shared__ double s_beta, s_kc;
  __shared__ int32_t s_zone;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (;;) {
    if (tid == 0) s_zone = atomicAdd(work, 1);
    __syncthreads();
    const int32_t zl = s_zone;
    if (zl >= nzc) break;
    if (nobs[zl] == 0) {
      __syncthreads();
      continue;
    }
    double* Gz = GT + (int64_t)zl * N * N;
    double* ax = aux + (int64_t)zl * aux_stride(N);
    double amax = 0.0;
    for (int idx = tid; idx < N * N; idx += kThreads) {
      int i = idx / N, j = idx - i * N;
      double g = Gz[idx];
      if (j <= i) A[i * ld + j] = g;
      amax = fmax(amax, fabs(g));
    }
    for (int o = 16; o > 0; o >>= 1) amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    if (lane == 0) red[warp] = amax;
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int k = 0; k < kWarps; k++) t = fmax(t, red[k]);
      ax[5 * N] = t * N;  // bound on ||G||, deflation floor
    }
    double* d = ax;
    double* e = ax + N;
    double* beta = ax + 2 * N;
    for (int k = 0; k < N - 2; k++) {
      const int L = N - k - 1;
      if (warp == 0) {
        // column k below the diagonal: x_i = A[k+1+i][k]
        double sig = 0.0;
        for (int i = 1 + lane; i < L; i += 32) {
          double x = A[(k + 1 + i) * ld + k];
          sig = fma(x, x, sig);
        }
        sig = warp_sum(sig);
        if (lane == 0) {
          double x0 = A[(k + 1) * ld + k];
          double bk = 0.0;
          if (sig == 0.0) {
            e[k] = x0;
          } else {
            double mu = sqrt(x0 * x0 + sig);
            double v0 = (x0 <= 0.0) ? x0 - mu : x0 + mu;  // v0 = x0 + sign(x0) mu
            e[k] = (x0 <= 0.0) ? mu : -mu;               // alpha = -sign(x0) ||x||
            bk = 2.0 / (v0 * v0 + sig);
            A[(k + 1) * ld + k] = v0;
          }
          d[k] = A[k * ld + k];
          beta[k] = bk;
          s_beta = bk;
        }
      }
      __syncthreads();
      const double bk = s_beta;
      if (bk == 0.0) continue;  // uniform across the block
      for (int i = tid; i < L; i += kThreads) v[i] = A[(k + 1 + i) * ld + k];
      __syncthreads();
      // p = beta A22 v, one thread per row, A22 symmetric with its lower triangle stored
      for (int i = tid; i < L; i += kThreads) {
        const double* row = A + (k + 1 + i) * ld + (k + 1);
        const double* col = A + (k + 1) * ld + (k + 1 + i);
        double s = 0.0;
        for (int j = 0; j < L; j++) s = fma((j <= i) ? row[j] : col[j * ld], v[j], s);
        w[i] = bk * s;
      }
      __syncthreads();
      if (warp == 0) {
        double pv = 0.0;
        for (int i = lane; i < L; i += 32) pv = fma(w[i], v[i], pv);
        pv = warp_sum(pv);
        if (lane == 0) s_kc = 0.5 * bk * pv;
      }
      __syncthreads();
      const double Kc = s_kc;
      for (int i = tid; i < L; i += kThreads) w[i] = fma(-Kc, v[i], w[i]);
      __syncthreads();
      // A22 -= v w^T + w v^T on the lower triangle
      const int E = L * (L + 1) / 2;
      for (int e2 = tid; e2 < E; e2 += kThreads) {
        int i, j;
        lower_index(e2, i, j);
        double* a = A + (k + 1 + i) * ld + (k + 1 + j);
        *a = fma(-v[i], w[j], fma(-w[i], v[j], *a));
      }
      __syncthreads();
    }
    if (tid == 0) {
      if (N >= 2) {
        d[N - 2] = A[(N - 2) * ld + (N - 2)];
        e[N - 2] = A[(N - 1) * ld + (N - 2)];
        beta[N - 2] = 0.0;
      }
      d[N - 1] = A[(N - 1) * ld + (N - 1)];
      e[N - 1] = 0.0;
      beta[N - 1] = 0.0;
    }
    // reflector vectors (strictly below the diagonal of each column) back to G's slot
    for (int idx = tid; idx < N * N; idx += kThreads) {
      int i = idx / N, j = idx - i * N;
      if (i > j) Gz[idx] = A[i * ld + j];
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------------------------ E2a
// One thread per zone: eigenvalues of Tri (sorted) and the inverse-iteration shifts.
__global__ void __launch_bounds__(128)
    k_eig_tridiag_values(int N, int32_t nzc, double* __restrict__ aux,
                         const int32_t* __restrict__ nobs, int32_t* __restrict__ status) {
  const int32_t zl = blockIdx.x * blockDim.x + threadIdx.x;
  if (zl >= nzc || nobs[zl] == 0) return;
  double* ax = aux + (int64_t)zl * aux_stride(N);
  double d[kNMax], e[kNMax];
  double onenrm = 0.0;
  for (int i = 0; i < N; i++) {
    d[i] = ax[i];
    e[i] = (i < N - 1) ? ax[N + i] : 0.0;
  }
  for (int i = 0; i < N; i++) {
    double s = fabs(d[i]) + fabs(e[i]) + (i > 0 ? fabs(e[i - 1]) : 0.0);
    onenrm = fmax(onenrm, s);
  }
  const double anorm = ax[5 * N];
  int st = 0;
  int hi = N - 1, sweeps = 0;
  const int max_sweeps = kMaxSweepsPerN * N;
  const double abs_tol = kEps * anorm * 1e-3;
  while (hi > 0) {
    while (hi > 0) {
      double t = fabs(e[hi - 1]);
      if (t <= kEps * (fabs(d[hi - 1]) + fabs(d[hi])) || t <= abs_tol) {
        e[hi - 1] = 0.0;
        hi--;
      } else {
        break;
      }
    }
    if (hi == 0) break;
    int lo = hi - 1;
    while (lo > 0) {
      double t = fabs(e[lo - 1]);
      if (t <= kEps * (fabs(d[lo - 1]) + fabs(d[lo])) || t <= abs_tol) {
        e[lo - 1] = 0.0;
        break;
      }
      lo--;
    }
    if (++sweeps > max_sweeps) {
      st |= ZST_EIG;
      break;
    }
    const double a = d[hi - 1], b = d[hi], f = e[hi - 1];
    const double del = 0.5 * (a - b);
    const double den = del + copysign(sqrt(del * del + f * f), del == 0.0 ? 1.0 : del);
    const double mu = (den == 0.0) ? b : b - f * f / den;
    double x = d[lo] - mu, z = e[lo], bulge = 0.0;
    for (int k = lo; k < hi; k++) {
      if (k > lo) {
        x = e[k - 1];
        z = bulge;
      }
      const double r2 = x * x + z * z;
      double c = 1.0, s = 0.0, r = 0.0;
      if (r2 > 0.0) {
        const double ri = rsqrt(r2);
        c = x * ri;
        s = z * ri;
        r = r2 * ri;
      }
      if (k > lo) e[k - 1] = r;
      const double dk = d[k], dk1 = d[k + 1], ek = e[k];
      const double ek1 = (k + 1 < hi) ? e[k + 1] : 0.0;
      const double cc = c * c, ss = s * s, cs = c * s;
      d[k] = cc * dk + 2.0 * cs * ek + ss * dk1;
      d[k + 1] = ss * dk - 2.0 * cs * ek + cc * dk1;
      e[k] = cs * (dk1 - dk) + (cc - ss) * ek;
      if (k + 1 < hi) e[k + 1] = c * ek1;
      bulge = s * ek1;
    }
  }
  // ascending order (insertion sort)
  for (int i = 1; i < N; i++) {
    double t = d[i];
    int k = i - 1;
    while (k >= 0 && d[k] > t) {
      d[k + 1] = d[k];
      k--;
    }
    d[k + 1] = t;
  }
  double prev = 0.0;
  for (int j = 0; j < N; j++) {
    ax[3 * N + j] = d[j];
    double s = d[j];
    if (j > 0) {
      const double pert = 10.0 * kEps * fabs(s);
      if (s - prev < pert) s = prev + pert;
    }
    ax[4 * N + j] = s;
    prev = s;
  }
  ax[5 * N + 1] = onenrm;
  if (st) status[zl] |= st;
}

// ------------------------------------------------------------------------------------ E2b
// One thread per eigenpair (zone zl, eigenvalue j): inverse iteration on Tri.
__global__ void __launch_bounds__(128)
    k_eig_tridiag_vectors(int N, int32_t nzc, const double* __restrict__ aux,
                          double* __restrict__ Zg, const int32_t* __restrict__ nobs) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int32_t zl = (int32_t)(t / N);
  const int j = (int)(t - (int64_t)zl * N);
  if (zl >= nzc || nobs[zl] == 0) return;
  const double* ax = aux + (int64_t)zl * aux_stride(N);
  const double* td = ax;
  const double* te = ax + N;
  const double l = ax[4 * N + j];
  const double onenrm = ax[5 * N + 1];
  double* zj = Zg + (int64_t)zl * N * N + (int64_t)j * N;
  if (!(onenrm > 1e-290)) {  // Tri = 0: every vector is an eigenvector
    for (int i = 0; i < N; i++) zj[i] = (i == j) ? 1.0 : 0.0;
    return;
  }
  const double tiny = kEps * onenrm;
  double u1[kNMax], u2[kNMax], lm[kNMax], uinv[kNMax], x[kNMax];
  unsigned char piv[kNMax];
  // LU with partial pivoting of Tri - l I (U: diagonal + two super-diagonals), branch-free
  double cd = td[0] - l, csup = (N > 1) ? te[0] : 0.0;
  for (int i = 0; i < N - 1; i++) {
    const double sub = te[i], dg = td[i + 1] - l, sp = (i + 1 < N - 1) ? te[i + 1] : 0.0;
    const bool swap = fabs(cd) < fabs(sub);
    double pivot = swap ? sub : cd;
    if (!swap && fabs(pivot) < tiny) pivot = copysign(tiny, pivot);
    const double ui = 1.0 / pivot;
    const double li = (swap ? cd : sub) * ui;
    u1[i] = swap ? dg : csup;
    u2[i] = swap ? sp : 0.0;
    piv[i] = swap ? 1 : 0;
    lm[i] = li;
    uinv[i] = ui;
    const double a = swap ? csup : dg, b = swap ? dg : csup;
    cd = fma(-li, b, a);
    const double nls = -li * sp;
    csup = swap ? nls : sp;
  }
  {
    double pivot = cd;
    if (fabs(pivot) < tiny) pivot = copysign(tiny, pivot);
    uinv[N - 1] = 1.0 / pivot;
  }
  // deterministic pseudo-random start vector
  for (int i = 0; i < N; i++) {
    unsigned h = (unsigned)i * 2654435761u ^ ((unsigned)j * 40503u + 0x9e3779b9u);
    h ^= h >> 15;
    h *= 2246822519u;
    h ^= h >> 13;
    x[i] = (double)(h & 0xffffff) * (1.0 / 16777216.0) - 0.5;
  }
  for (int it = 0; it < 2; it++) {
    for (int i = 0; i < N - 1; i++) {
      const double a = x[i], b = x[i + 1];
      const double xi = piv[i] ? b : a, xn = piv[i] ? a : b;
      x[i] = xi;
      x[i + 1] = fma(-lm[i], xi, xn);
    }
    x[N - 1] *= uinv[N - 1];
    if (N > 1) x[N - 2] = (x[N - 2] - u1[N - 2] * x[N - 1]) * uinv[N - 2];
    for (int i = N - 3; i >= 0; i--)
      x[i] = fma(-u2[i], x[i + 2], fma(-u1[i], x[i + 1], x[i])) * uinv[i];
    // scale by the largest entry first, so the sum of squares cannot overflow
    double mx = 0.0;
    for (int i = 0; i < N; i++) mx = fmax(mx, fabs(x[i]));
    const double im = 1.0 / mx;
    double nrm = 0.0;
    for (int i = 0; i < N; i++) {
      x[i] *= im;
      nrm = fma(x[i], x[i], nrm);
    }
    const double sc = rsqrt(nrm);
    for (int i = 0; i < N; i++) x[i] *= sc;
  }
  for (int i = 0; i < N; i++) zj[i] = x[i];
}

// ------------------------------------------------------------------------------------ E3
__global__ void __launch_bounds__(kThreads)
    k_eig_transform(int N, int32_t nzc, double* __restrict__ GT, const double* __restrict__ aux,
                    const double* __restrict__ Zg, const double* __restrict__ gv,
                    const int32_t* __restrict__ nobs, int rotate, double* __restrict__ ampl_out,
                    int32_t* __restrict__ status, int32_t* __restrict__ work) {
  extern __shared__ double dyn[];
  const int ld = N + 1;
  double* A = dyn;           // [N][ld] reflectors, then T_sym
  double* U = A + N * ld;    // [N][ld] Z, then U
  double* lam = U + N * ld;  // [N] 1/(1+lambda)
  double* sq = lam + N;      // [N] sqrt(1/(1+lambda))
  double* g = sq + N;        // [N]
  double* beta = g + N;      // [N]
  double* t0 = beta + N;     // [N]
  double* t1 = t0 + N;       // [N]
  double* vv = t1 + N;       // [N]
  double* qs = vv + N;       // [N] lambda^(1/4)
  int* cst = reinterpret_cast<int*>(qs + N);  // [N] cluster start of each eigenvector
  __shared__ double red[kWarps];
  __shared__ int32_t s_zone;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (;;) {
    if (tid == 0) s_zone = atomicAdd(work, 1);
    __syncthreads();
    const int32_t zl = s_zone;
    if (zl >= nzc) break;
    if (nobs[zl] == 0) {
      __syncthreads();
      continue;
    }
    double* Gz = GT + (int64_t)zl * N * N;
    const double* ax = aux + (int64_t)zl * aux_stride(N);
    const double* Z = Zg + (int64_t)zl * N * N;
    for (int idx = tid; idx < N * N; idx += kThreads) {
      int i = idx / N, j = idx - i * N;
      A[i * ld + j] = (i > j) ? Gz[idx] : 0.0;
      U[j * ld + i] = Z[idx];  // Z[i*N + j] = component j of eigenvector i -> U[j][i]
    }
    for (int i = tid; i < N; i += kThreads) {
      double l = ax[3 * N + i];
      if (l < 0.0) l = 0.0;
      const double li = 1.0 / (1.0 + l);
      lam[i] = li;
      sq[i] = sqrt(li);
      qs[i] = sqrt(sq[i]);
      g[i] = gv[(int64_t)zl * N + i];
      beta[i] = ax[2 * N + i];
    }
    if (tid == 0) {
      const double ortol = 1e-3 * ax[5 * N + 1];
      int c0 = 0;
      cst[0] = 0;
      for (int j = 1; j < N; j++) {
        if (ax[3 * N + j] - ax[3 * N + j - 1] > ortol) c0 = j;
        cst[j] = c0;
      }
    }
    __syncthreads();
    // clusters: two classical Gram-Schmidt passes of column j against columns [cst[j], j)
    for (int j = 1; j < N; j++) {
      const int k0 = cst[j], nk = j - k0;
      if (nk == 0) continue;  // uniform
      for (int pass = 0; pass < 2; pass++) {
        // one thread per dot product (no cross-lane reductions on the FP64 pipe)
        for (int kk = tid; kk < nk; kk += kThreads) {
          double s = 0.0;
          for (int i = 0; i < N; i++) s = fma(U[i * ld + k0 + kk], U[i * ld + j], s);
          t0[kk] = s;
        }
        __syncthreads();
        for (int i = tid; i < N; i += kThreads) {
          double s = U[i * ld + j];
          for (int kk = 0; kk < nk; kk++) s = fma(-t0[kk], U[i * ld + k0 + kk], s);
          U[i * ld + j] = s;
        }
        __syncthreads();
      }
      if (warp == 0) {
        double s = 0.0;
        for (int i = lane; i < N; i += 32) s = fma(U[i * ld + j], U[i * ld + j], s);
        s = warp_sum(s);
        if (lane == 0) red[0] = rsqrt(s);
      }
      __syncthreads();
      const double sc = red[0];
      for (int i = tid; i < N; i += kThreads) U[i * ld + j] *= sc;
      __syncthreads();
    }
    // U = Q_h Z = H_0 H_1 ... H_{N-3} Z: apply H_k for k = N-3 .. 0
    for (int k = N - 3; k >= 0; k--) {
      const double bk = beta[k];
      if (bk == 0.0) continue;  // uniform across the block
      const int L = N - k - 1;
      for (int j = tid; j < N; j += kThreads) {
        double s = 0.0;
        for (int i = 0; i < L; i++) s = fma(A[(k + 1 + i) * ld + k], U[(k + 1 + i) * ld + j], s);
        t0[j] = bk * s;
      }
      __syncthreads();
      for (int idx = tid; idx < L * N; idx += kThreads) {
        int i = idx / N, j = idx - i * N;
        double* u = U + (k + 1 + i) * ld + j;
        *u = fma(-A[(k + 1 + i) * ld + k], t0[j], *u);
      }
      __syncthreads();
    }
    // ampl = U (lambda .* (U^T g))
    for (int i = tid; i < N; i += kThreads) {
      double s = 0.0;
      for (int r = 0; r < N; r++) s = fma(U[r * ld + i], g[r], s);
      t0[i] = lam[i] * s;
    }
    __syncthreads();
    int nan_flag = 0;
    for (int r = tid; r < N; r += kThreads) {
      double s = 0.0;
      for (int i = 0; i < N; i++) s = fma(U[r * ld + i], t0[i], s);
      ampl_out[(int64_t)zl * N + r] = s;
      if (!(s == s) || isinf(s)) nan_flag = 1;
    }
    nan_flag = __syncthreads_or(nan_flag);
    if (rotate) {
      // v = normate(U (colsum(U) / sqrt(lambda)))
      for (int i = tid; i < N; i += kThreads) {
        double s = 0.0;
        for (int r = 0; r < N; r++) s += U[r * ld + i];
        t1[i] = s / sq[i];
      }
      __syncthreads();
      for (int r = tid; r < N; r += kThreads) {
        double s = 0.0;
        for (int i = 0; i < N; i++) s = fma(U[r * ld + i], t1[i], s);
        vv[r] = s;
      }
      __syncthreads();
      if (warp == 0) {
        double s = 0.0;
        for (int r = lane; r < N; r += 32) s = fma(vv[r], vv[r], s);
        s = warp_sum(s);
        if (lane == 0) red[0] = 1.0 / sqrt(s);
      }
      __syncthreads();
      const double inv = red[0];
      for (int r = tid; r < N; r += kThreads) vv[r] *= inv;
    }
    // T_sym = U diag(sqrt(lambda)) U^T: U's columns scaled by lambda^(1/4), then U U^T
    for (int idx = tid; idx < N * N; idx += kThreads) {
      int r = idx / N, i = idx - r * N;
      U[r * ld + i] *= qs[i];
    }
    __syncthreads();
    const int E = N * (N + 1) / 2;
    for (int e2 = tid; e2 < E; e2 += kThreads) {
      int a, b;
      lower_index(e2, a, b);
      const double* qa = U + a * ld;
      const double* qb = U + b * ld;
      double s = 0.0;
      for (int k = 0; k < N; k++) s = fma(qa[k], qb[k], s);
      A[a * ld + b] = s;
      A[b * ld + a] = s;
    }
    __syncthreads();
    if (rotate) {
      const double vN = vv[N - 1];
      const double sv = signbit(vN) ? -1.0 : 1.0;
      const double cv = 1.0 + fabs(vN);
      const double wv = 1.0 / sqrt((double)N);
      const double cw = 1.0 + wv;
      // t0 = T_sym u_v, t1 = T_sym v
      for (int i = tid; i < N; i += kThreads) {
        const double* ti = A + i * ld;
        double sa = 0.0, sb = 0.0;
        for (int j = 0; j < N; j++) {
          sa = fma(ti[j], vv[j] + ((j == N - 1) ? sv : 0.0), sa);
          sb = fma(ti[j], vv[j], sb);
        }
        t0[i] = sa;
        t1[i] = sb;
      }
      __syncthreads();
      // T1 = T_sym - t0 u_v^T / c_v
      const double icv = 1.0 / cv, icw = 1.0 / cw;
      for (int idx = tid; idx < N * N; idx += kThreads) {
        int i = idx / N, j = idx - i * N;
        double uj = vv[j] + ((j == N - 1) ? sv : 0.0);
        A[i * ld + j] = fma(-t0[i] * icv, uj, A[i * ld + j]);
      }
      __syncthreads();
      // g <- T1 u_w (g is no longer needed)
      for (int i = tid; i < N; i += kThreads) {
        const double* ti = A + i * ld;
        double s = 0.0;
        for (int j = 0; j < N; j++) s = fma(ti[j], wv + ((j == N - 1) ? 1.0 : 0.0), s);
        g[i] = s * icw;
      }
      __syncthreads();
      // T = T1 - (T1 u_w) u_w^T / c_w + (1 - s_v s_w) (T_sym v) w^T   (s_w = +1)
      const double extra = 1.0 - sv;
      for (int idx = tid; idx < N * N; idx += kThreads) {
        int i = idx / N, j = idx - i * N;
        double uj = wv + ((j == N - 1) ? 1.0 : 0.0);
        double t = fma(-g[i], uj, A[i * ld + j]);
        if (extra != 0.0) t = fma(extra * t1[i], wv, t);
        Gz[idx] = t;
      }
    } else {
      for (int idx = tid; idx < N * N; idx += kThreads) {
        int i = idx / N, j = idx - i * N;
        Gz[idx] = A[i * ld + j];
      }
    }
    if (tid == 0 && nan_flag) status[zl] |= ZST_NAN;
    __syncthreads();
  }
}

int grid_for_smem(const void* fn, size_t smem, int32_t nzc) {
  int bps = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, fn, kThreads, smem);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int grid = sms * (bps > 0 ? bps : 1);
  if (grid > nzc) grid = nzc > 0 ? nzc : 1;
  return grid;
}

}  // namespace

size_t zone_eig_fp64_aux(int N) { return (size_t)aux_stride(N); }

cudaError_t zone_eig_fp64(int N, int32_t nzc, double* d_GT, const double* d_g,
                          const int32_t* d_nobs, int rotate, double* d_ampl, int32_t* d_status,
                          double* d_aux, double* d_Z, int32_t* d_work, cudaStream_t st) {
  if (N < 2 || N > kNMax) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(d_status, 0, sizeof(int32_t) * (nzc > 0 ? nzc : 1), st);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(d_work, 0, 2 * sizeof(int32_t), st);
  if (e != cudaSuccess) return e;
  // E1
  size_t smem1 = (size_t)(N * (N + 1) + 2 * N) * sizeof(double);
  e = cudaFuncSetAttribute(k_eig_tridiag, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem1);
  if (e != cudaSuccess) return e;
  k_eig_tridiag<<<grid_for_smem((const void*)k_eig_tridiag, smem1, nzc), kThreads, smem1, st>>>(
      N, nzc, d_GT, d_aux, d_nobs, d_work);
  // E2a, E2b
  k_eig_tridiag_values<<<(nzc + 127) / 128, 128, 0, st>>>(N, nzc, d_aux, d_nobs, d_status);
  const int64_t pairs = (int64_t)nzc * N;
  k_eig_tridiag_vectors<<<(unsigned)((pairs + 127) / 128), 128, 0, st>>>(N, nzc, d_aux, d_Z,
                                                                          d_nobs);
  // E3
  size_t smem3 = (size_t)(2 * N * (N + 1) + 9 * N) * sizeof(double);
  e = cudaFuncSetAttribute(k_eig_transform, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem3);
  if (e != cudaSuccess) return e;
  k_eig_transform<<<grid_for_smem((const void*)k_eig_transform, smem3, nzc), kThreads, smem3,
                    st>>>(N, nzc, d_GT, d_aux, d_Z, d_g, d_nobs, rotate, d_ampl, d_status,
                          d_work + 1);
  count_launches(4);
  return cudaGetLastError();
}

}  // namespace oakg
