// K3 + K4 -- per-zone symmetric eigensolve and the square-root transform, templated on the
// arithmetic type R: double for the plain form, float for the mixed-precision form (where the
// (1 + lambda)^-1/2 and (1 + lambda)^-1 scalings are still evaluated in FP64).
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
// so the work is split into kernels whose arithmetic keeps all 32 lanes busy:
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
constexpr int kNMax = 128;               // largest N of the eigensolve stages
constexpr int kT64 = 32;    // threads a block of the FP64 E2a / E2b kernels for N <= kNV64
constexpr int kNV64 = 64;
constexpr int kMaxSweepsPerN = 30;
constexpr int32_t kFewZones = 152;  // below this zone count E2a runs one block per zone

template <typename R>
struct Prec;
template <>
struct Prec<double> {
  static __device__ __forceinline__ double eps() { return 1.1102230246251565e-16; }
  static __device__ __forceinline__ double tiny() { return 1e-300; }
  static __device__ __forceinline__ double sqrt_(double x) { return sqrt(x); }
  static __device__ __forceinline__ double rsqrt_(double x) { return rsqrt(x); }
};
template <>
struct Prec<float> {
  static __device__ __forceinline__ float eps() { return 5.9604645e-8f; }
  static __device__ __forceinline__ float tiny() { return 1e-36f; }
  static __device__ __forceinline__ float sqrt_(float x) { return sqrtf(x); }
  static __device__ __forceinline__ float rsqrt_(float x) { return rsqrtf(x); }
};

// per-zone auxiliary layout (elements of R). The eigensolve works on G / scale with
// scale = max|G_ij| (LAPACK-style scaling: keeps FP32 squares away from underflow):
//   d[N] e[N] beta[N]      tridiagonal of G/scale and the Householder scalars
//   lambda[N]              eigenvalues of G (unscaled, ascending)
//   shift[N]               inverse-iteration shifts (scaled units)
//   scale ||Tri||_1        (||Tri||_1 in scaled units)
__host__ __device__ inline int aux_stride(int N) { return 5 * N + 2; }

template <typename R>
__device__ __forceinline__ R warp_sum(R x) {
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// (row, col) of the e2-th lower-triangle entry. The estimate uses an FP32 square root (the
// FP64 pipe is the bottleneck of the FP64 kernels) and integer fix-ups make it exact.
__device__ __forceinline__ void lower_index(int e2, int& a, int& b) {
  a = (int)((__fsqrt_rn((float)(8 * e2 + 1)) - 1.0f) * 0.5f);
  while ((a + 1) * (a + 2) / 2 <= e2) a++;
  while (a * (a + 1) / 2 > e2) a--;
  b = e2 - a * (a + 1) / 2;
}

// ------------------------------------------------------------------------------------ E1
template <typename R>
__global__ void __launch_bounds__(kThreads)
    k_eig_tridiag(int N, int32_t nzc, R* __restrict__ GT, R* __restrict__ aux,
                  const int32_t* __restrict__ nobs, int32_t* __restrict__ work) {
  extern __shared__ __align__(16) unsigned char dyn_raw[];
  R* dyn = reinterpret_cast<R*>(dyn_raw);
  const int ld = N + 1;
  R* A = dyn;          // [N][ld], lower triangle valid
  R* v = A + N * ld;   // [N]
  R* w = v + N;        // [N]
  __shared__ R red[kWarps];
  __shared__ R s_beta, s_kc;
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
    R* Gz = GT + (int64_t)zl * N * N;
    R* ax = aux + (int64_t)zl * aux_stride(N);
    R amax = 0;  // G is symmetric: its lower triangle (the half read below) holds the maximum
    for (int idx = tid; idx < N * N; idx += kThreads) {
      const int i = idx / N, j = idx - i * N;
      if (j <= i) amax = fmax(amax, fabs(Gz[idx]));
    }
    for (int o = 16; o > 0; o >>= 1) amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    if (lane == 0) red[warp] = amax;
    __syncthreads();
    R scale = 0;
    for (int k = 0; k < kWarps; k++) scale = fmax(scale, red[k]);
    if (!(scale > R(0)) || isinf(scale)) scale = R(1);
    const R iscale = R(1) / scale;
    for (int idx = tid; idx < N * N; idx += kThreads) {
      int i = idx / N, j = idx - i * N;
      if (j <= i) A[i * ld + j] = Gz[idx] * iscale;
    }
    if (tid == 0) ax[5 * N] = scale;
    __syncthreads();
    R* d = ax;
    R* e = ax + N;
    R* beta = ax + 2 * N;
    for (int k = 0; k < N - 2; k++) {
      const int L = N - k - 1;
      if (warp == 0) {
        // column k below the diagonal: x_i = A[k+1+i][k]
        R sig = 0;
        for (int i = 1 + lane; i < L; i += 32) {
          R x = A[(k + 1 + i) * ld + k];
          sig = fma(x, x, sig);
        }
        sig = warp_sum(sig);
        if (lane == 0) {
          R x0 = A[(k + 1) * ld + k];
          R bk = 0;
          const R mu = Prec<R>::sqrt_(x0 * x0 + sig);
          const R v0 = (x0 <= R(0)) ? x0 - mu : x0 + mu;  // v0 = x0 + sign(x0) mu
          const R vv = v0 * v0 + sig;
          if (sig == R(0) || !(vv > R(0)) || isinf(vv)) {  // nothing to annihilate
            e[k] = x0;
          } else {
            e[k] = (x0 <= R(0)) ? mu : -mu;               // alpha = -sign(x0) ||x||
            bk = R(2) / vv;
            A[(k + 1) * ld + k] = v0;
          }
          d[k] = A[k * ld + k];
          beta[k] = bk;
          s_beta = bk;
        }
      }
      __syncthreads();
      const R bk = s_beta;
      if (bk == R(0)) continue;  // uniform across the block
      for (int i = tid; i < L; i += kThreads) v[i] = A[(k + 1 + i) * ld + k];
      __syncthreads();
      // p = beta A22 v, one thread per row, A22 symmetric with its lower triangle stored
      for (int i = tid; i < L; i += kThreads) {
        const R* row = A + (k + 1 + i) * ld + (k + 1);
        const R* col = A + (k + 1) * ld + (k + 1 + i);
        R s = 0;
        for (int j = 0; j < L; j++) s = fma((j <= i) ? row[j] : col[j * ld], v[j], s);
        w[i] = bk * s;
      }
      __syncthreads();
      if (warp == 0) {
        R pv = 0;
        for (int i = lane; i < L; i += 32) pv = fma(w[i], v[i], pv);
        pv = warp_sum(pv);
        if (lane == 0) s_kc = R(0.5) * bk * pv;
      }
      __syncthreads();
      const R Kc = s_kc;
      for (int i = tid; i < L; i += kThreads) w[i] = fma(-Kc, v[i], w[i]);
      __syncthreads();
      // A22 -= v w^T + w v^T on the lower triangle
      const int E = L * (L + 1) / 2;
      for (int e2 = tid; e2 < E; e2 += kThreads) {
        int i, j;
        lower_index(e2, i, j);
        R* a = A + (k + 1 + i) * ld + (k + 1 + j);
        *a = fma(-v[i], w[j], fma(-w[i], v[j], *a));
      }
      __syncthreads();
    }
    if (tid == 0) {
      if (N >= 2) {
        d[N - 2] = A[(N - 2) * ld + (N - 2)];
        e[N - 2] = A[(N - 1) * ld + (N - 2)];
        beta[N - 2] = 0;
      }
      d[N - 1] = A[(N - 1) * ld + (N - 1)];
      e[N - 1] = 0;
      beta[N - 1] = 0;
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
template <typename R>
__global__ void __launch_bounds__(128)
    k_eig_tridiag_values(int N, int32_t nzc, R* __restrict__ aux,
                         const int32_t* __restrict__ nobs, int32_t* __restrict__ status) {
  const int32_t zl = blockIdx.x * blockDim.x + threadIdx.x;
  if (zl >= nzc || nobs[zl] == 0) return;
  const R eps = Prec<R>::eps();
  R* ax = aux + (int64_t)zl * aux_stride(N);
  R d[kNMax], e[kNMax];
  R onenrm = 0;
  for (int i = 0; i < N; i++) {
    d[i] = ax[i];
    e[i] = (i < N - 1) ? ax[N + i] : R(0);
  }
  for (int i = 0; i < N; i++) {
    R s = fabs(d[i]) + fabs(e[i]) + (i > 0 ? fabs(e[i - 1]) : R(0));
    onenrm = fmax(onenrm, s);
  }
  const R scale = ax[5 * N];
  int st = 0;
  int hi = N - 1, sweeps = 0;
  const int max_sweeps = kMaxSweepsPerN * N;
  const R abs_tol = eps * onenrm;  // deflation floor: the rounding level of Tri
  while (hi > 0) {
    while (hi > 0) {
      R t = fabs(e[hi - 1]);
      if (t <= eps * (fabs(d[hi - 1]) + fabs(d[hi])) || t <= abs_tol) {
        e[hi - 1] = 0;
        hi--;
      } else {
        break;
      }
    }
    if (hi == 0) break;
    int lo = hi - 1;
    while (lo > 0) {
      R t = fabs(e[lo - 1]);
      if (t <= eps * (fabs(d[lo - 1]) + fabs(d[lo])) || t <= abs_tol) {
        e[lo - 1] = 0;
        break;
      }
      lo--;
    }
    if (++sweeps > max_sweeps) {
      st |= ZST_EIG;
      break;
    }
    const R a = d[hi - 1], b = d[hi], f = e[hi - 1];
    const R del = R(0.5) * (a - b);
    const R den = del + copysign(Prec<R>::sqrt_(del * del + f * f), del == R(0) ? R(1) : del);
    const R mu = (den == R(0)) ? b : b - f * f / den;
    R x = d[lo] - mu, z = e[lo], bulge = 0;
    for (int k = lo; k < hi; k++) {
      if (k > lo) {
        x = e[k - 1];
        z = bulge;
      }
      const R r2 = x * x + z * z;
      R c = 1, s = 0, r = 0;
      if (r2 > R(0)) {
        const R ri = Prec<R>::rsqrt_(r2);
        c = x * ri;
        s = z * ri;
        r = r2 * ri;
      }
      if (k > lo) e[k - 1] = r;
      const R dk = d[k], dk1 = d[k + 1], ek = e[k];
      const R ek1 = (k + 1 < hi) ? e[k + 1] : R(0);
      const R cc = c * c, ss = s * s, cs = c * s;
      d[k] = cc * dk + R(2) * cs * ek + ss * dk1;
      d[k + 1] = ss * dk - R(2) * cs * ek + cc * dk1;
      e[k] = cs * (dk1 - dk) + (cc - ss) * ek;
      if (k + 1 < hi) e[k + 1] = c * ek1;
      bulge = s * ek1;
    }
  }
  // ascending order (insertion sort)
  for (int i = 1; i < N; i++) {
    R t = d[i];
    int k = i - 1;
    while (k >= 0 && d[k] > t) {
      d[k + 1] = d[k];
      k--;
    }
    d[k + 1] = t;
  }
  R prev = 0;
  for (int j = 0; j < N; j++) {
    ax[3 * N + j] = d[j] * scale;
    R s = d[j];
    if (j > 0) {
      const R pert = R(10) * eps * fabs(s);
      if (s - prev < pert) s = prev + pert;
    }
    ax[4 * N + j] = s;
    prev = s;
  }
  ax[5 * N + 1] = onenrm;
  if (st) status[zl] |= st;
}

// E2a for few zones (fewer than the GPU has SMs, e.g. the one-zone global analysis), where the
// thread-per-zone QR above leaves the GPU idle and its latency is the whole stage: one warp per
// eigenvalue (grid N x zones), so that the zone's eigenvalues spread over the SMs. Eigenvalue
// k is the point where the Sturm count of Tri - x I passes k: the number of sign changes along
// the leading principal minors p_i = det(Tri_{1:i} - x I), from
// p_i = (d_i - x) p_{i-1} - e_{i-1}^2 p_{i-2} (bisection after Givens; a zero minor takes the
// sign opposite to its predecessor, as the pivot -pivmin of the ratio form does), rescaled by
// powers of two to stay in range, with no division. Each step evaluates the count at the 32
// lanes' interior points of the current interval and keeps the sub-interval where it passes k
// (multisection, a 33-fold narrowing per step), until the interval is at the rounding level of
// Tri. k_eig_shifts then writes the outputs of the QR kernel.
template <typename R>
__device__ __forceinline__ int sturm_count(const R* __restrict__ d, const R* __restrict__ e2,
                                           int N, R x) {
  R p0 = R(1), p1 = d[0] - x;
  bool s1 = !(p1 > R(0));  // a zero takes the sign opposite to p0 > 0
  int c = s1;
  for (int i = 1; i < N; i++) {
    const R p2 = fma(d[i] - x, p1, -e2[i - 1] * p0);
    const bool s2 = (p2 == R(0)) ? !s1 : (p2 < R(0));
    c += s2 != s1;
    s1 = s2;
    p0 = p1;
    p1 = p2;
    if ((i & 7) == 0) {
      const R mx = fmax(fabs(p0), fabs(p1));
      if (mx > R(1e150) || (mx < R(1e-150) && mx > R(0))) {
        int ex;
        frexp(mx, &ex);
        p0 = ldexp(p0, -ex);
        p1 = ldexp(p1, -ex);
      }
    }
  }
  return c;
}

template <typename R>
__global__ void __launch_bounds__(32)
    k_eig_values_multisect(int N, int32_t nzc, R* __restrict__ aux,
                           const int32_t* __restrict__ nobs) {
  __shared__ R sd[kNMax], se2[kNMax];
  const int k = blockIdx.x;
  const int32_t zl = blockIdx.y;
  if (zl >= nzc || nobs[zl] == 0) return;  // uniform across the block
  const R eps = Prec<R>::eps();
  R* ax = aux + (int64_t)zl * aux_stride(N);
  const int lane = threadIdx.x;
  R onenrm = 0, gl = 0, gu = 0;
  bool first = true;
  for (int i0 = 0; i0 < N; i0 += 32) {
    const int i = i0 + lane;
    R di = 0, r = 0;
    if (i < N) {
      di = ax[i];
      const R ei = (i < N - 1) ? ax[N + i] : R(0), em = (i > 0) ? ax[N + i - 1] : R(0);
      sd[i] = di;
      se2[i] = ei * ei;
      r = fabs(ei) + fabs(em);
    }
    R nrm = (i < N) ? fabs(di) + r : R(0);
    R lo = (i < N) ? di - r : R(INFINITY), hi = (i < N) ? di + r : R(-INFINITY);
    for (int o = 16; o > 0; o >>= 1) {
      nrm = fmax(nrm, __shfl_xor_sync(0xffffffffu, nrm, o));
      lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
      hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    onenrm = fmax(onenrm, nrm);
    gl = first ? lo : fmin(gl, lo);
    gu = first ? hi : fmax(gu, hi);
    first = false;
  }
  __syncwarp();
  const R pad = R(2) * eps * onenrm + Prec<R>::tiny();
  R a = gl - pad, b = gu + pad;
  for (int it = 0; it < 64; it++) {
    const R x = a + (b - a) * R(lane + 1) / R(33);
    const unsigned past = __ballot_sync(0xffffffffu, sturm_count(sd, se2, N, x) > k);
    const int ss = past ? __ffs(past) - 1 : 32;  // first point past eigenvalue k
    const R xl = (ss == 0) ? a : a + (b - a) * R(ss) / R(33);
    const R xu = (ss == 32) ? b : a + (b - a) * R(ss + 1) / R(33);
    a = xl;
    b = xu;
    if (b - a <= R(2) * eps * fmax(fabs(a), fabs(b)) + eps * onenrm) break;  // uniform
  }
  if (lane == 0) {
    ax[3 * N + k] = R(0.5) * (a + b);  // unscaled until k_eig_shifts
    if (k == 0) ax[5 * N + 1] = onenrm;
  }
}

// the QR kernel's outputs from the multisection eigenvalues: scaled eigenvalues and the
// inverse-iteration shifts separated as LAPACK dstein does (one thread per zone)
template <typename R>
__global__ void k_eig_shifts(int N, int32_t nzc, R* __restrict__ aux,
                             const int32_t* __restrict__ nobs) {
  const int32_t zl = blockIdx.x * blockDim.x + threadIdx.x;
  if (zl >= nzc || nobs[zl] == 0) return;
  const R eps = Prec<R>::eps();
  R* ax = aux + (int64_t)zl * aux_stride(N);
  const R scale = ax[5 * N];
  R prev = 0;
  for (int j = 0; j < N; j++) {
    const R lam = ax[3 * N + j];
    ax[3 * N + j] = lam * scale;
    R sh = lam;
    if (j > 0) {
      const R pert = R(10) * eps * fabs(sh);
      if (sh - prev < pert) sh = prev + pert;
    }
    ax[4 * N + j] = sh;
    prev = sh;
  }
}

// ------------------------------------------------------------------------------------ E2b
// One thread per eigenpair (zone zl, eigenvalue j): inverse iteration on Tri.
template <typename R>
__global__ void __launch_bounds__(128)
    k_eig_tridiag_vectors(int N, int32_t nzc, const R* __restrict__ aux, R* __restrict__ Zg,
                          const int32_t* __restrict__ nobs) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int32_t zl = (int32_t)(t / N);
  const int j = (int)(t - (int64_t)zl * N);
  if (zl >= nzc || nobs[zl] == 0) return;
  const R* ax = aux + (int64_t)zl * aux_stride(N);
  const R* td = ax;
  const R* te = ax + N;
  const R l = ax[4 * N + j];
  const R onenrm = ax[5 * N + 1];
  R* zj = Zg + (int64_t)zl * N * N + (int64_t)j * N;
  if (!(onenrm > R(1e4) * Prec<R>::tiny())) {  // Tri = 0: every vector is an eigenvector
    for (int i = 0; i < N; i++) zj[i] = (i == j) ? R(1) : R(0);
    return;
  }
  const R tiny = Prec<R>::eps() * onenrm;
  R u1[kNMax], u2[kNMax], lm[kNMax], uinv[kNMax], x[kNMax];
  unsigned char piv[kNMax];
  // LU with partial pivoting of Tri - l I (U: diagonal + two super-diagonals), branch-free
  R cd = td[0] - l, csup = (N > 1) ? te[0] : R(0);
  for (int i = 0; i < N - 1; i++) {
    const R sub = te[i], dg = td[i + 1] - l, sp = (i + 1 < N - 1) ? te[i + 1] : R(0);
    const bool swap = fabs(cd) < fabs(sub);
    R pivot = swap ? sub : cd;
    if (!swap && fabs(pivot) < tiny) pivot = copysign(tiny, pivot);
    const R ui = R(1) / pivot;
    const R li = (swap ? cd : sub) * ui;
    u1[i] = swap ? dg : csup;
    u2[i] = swap ? sp : R(0);
    piv[i] = swap ? 1 : 0;
    lm[i] = li;
    uinv[i] = ui;
    const R a = swap ? csup : dg, b = swap ? dg : csup;
    cd = fma(-li, b, a);
    const R nls = -li * sp;
    csup = swap ? nls : sp;
  }
  {
    R pivot = cd;
    if (fabs(pivot) < tiny) pivot = copysign(tiny, pivot);
    uinv[N - 1] = R(1) / pivot;
  }
  // deterministic pseudo-random start vector
  for (int i = 0; i < N; i++) {
    unsigned h = (unsigned)i * 2654435761u ^ ((unsigned)j * 40503u + 0x9e3779b9u);
    h ^= h >> 15;
    h *= 2246822519u;
    h ^= h >> 13;
    x[i] = (R)((double)(h & 0xffffff) * (1.0 / 16777216.0) - 0.5);
  }
  for (int it = 0; it < 2; it++) {
    for (int i = 0; i < N - 1; i++) {
      const R a = x[i], b = x[i + 1];
      const R xi = piv[i] ? b : a, xn = piv[i] ? a : b;
      x[i] = xi;
      x[i + 1] = fma(-lm[i], xi, xn);
    }
    x[N - 1] *= uinv[N - 1];
    if (N > 1) x[N - 2] = (x[N - 2] - u1[N - 2] * x[N - 1]) * uinv[N - 2];
    for (int i = N - 3; i >= 0; i--)
      x[i] = fma(-u2[i], x[i + 2], fma(-u1[i], x[i + 1], x[i])) * uinv[i];
    // scale by the largest entry first, so the sum of squares cannot overflow
    R mx = 0;
    for (int i = 0; i < N; i++) mx = fmax(mx, fabs(x[i]));
    const R im = R(1) / mx;
    R nrm = 0;
    for (int i = 0; i < N; i++) {
      x[i] *= im;
      nrm = fma(x[i], x[i], nrm);
    }
    const R sc = Prec<R>::rsqrt_(nrm);
    for (int i = 0; i < N; i++) x[i] *= sc;
  }
  for (int i = 0; i < N; i++) zj[i] = x[i];
}

// E2b for N <= 64 in FP64: blocks of kT64 = 32 threads (one warp), two per zone, thread j =
// eigenpair j, with the arithmetic of k_eig_tridiag_vectors<double> (same LU, start vector
// and two solves; reciprocals by Newton steps and a power-of-two prescaling before the
// normalisation, so the vectors agree to rounding). The per-thread factor arrays of the generic
// kernel live in local memory, and with thousands of threads per SM they go to DRAM (most of
// the eigensolve's traffic); here the partial-pivoting LU is recomputed in each forward sweep
// (fused with the elimination), the iterate is kept in registers (loops unrolled to 64), the
// factor's first superdiagonal, pivot reciprocals and multipliers in shared memory ([i][j]
// layout: consecutive threads, consecutive words) and its second superdiagonal as one bit per
// row (it is the tridiagonal's next off-diagonal entry where rows were swapped, else 0); the
// second solve applies the stored factors instead of refactoring. 48 KB a block.

// 1/p by two Newton steps from the FP32 reciprocal (relative error below 2^-52, not always
// correctly rounded). The IEEE FP64 division is a called routine whose call keeps the live
// register array x in local memory; this is inline. Valid for |p| inside FP32's normal range:
// the tridiagonal is of G / max|G_ij|, so ||Tri||_F >= 1, ||Tri||_1 >= 1/sqrt(N) and every
// pivot lies in [eps ||Tri||_1, 3 N].
__device__ __forceinline__ double rcp_newton(double p) {
  double r = (double)__frcp_rn((float)p);
  double e = fma(-p, r, 1.0);
  r = fma(r, e, r);
  e = fma(-p, r, 1.0);
  return fma(r, e, r);
}

// 1/sqrt(a) by Newton steps from the FP32 estimate, for a in [1, 4 N] (a normalised sum of
// squares); inline for the same reason as rcp_newton.
__device__ __forceinline__ double rsqrt_newton(double a) {
  double y = (double)rsqrtf((float)a);
#pragma unroll
  for (int k = 0; k < 3; k++) y = y * fma(-0.5 * a * y, y, 1.5);
  return y;
}

// 2^-e for the binary exponent e of x > 0 (normal), by its bits
__device__ __forceinline__ double pow2_inv_exponent(double x) {
  const long long e = ((__double_as_longlong(x) >> 52) & 0x7ff) - 1023;
  return __longlong_as_double((1023 - e) << 52);
}

__global__ void __launch_bounds__(kT64)
    k_eig_vectors_fp64(int N, int32_t nzc, const double* __restrict__ aux,
                       double* __restrict__ Zg, const int32_t* __restrict__ nobs) {
  constexpr int NV = kNV64;
  extern __shared__ __align__(16) double sfac64[];  // u1, 1/pivot, multiplier: [i][jl] each
  __shared__ double sd[NV], se[NV + 1];
  double* su1 = sfac64;
  double* sui = sfac64 + NV * kT64;
  double* sli = sfac64 + 2 * NV * kT64;
  const int jl = threadIdx.x, j = kT64 * blockIdx.y + jl;  // eigenpair j
  const int32_t zl = blockIdx.x;
  if (zl >= nzc || nobs[zl] == 0) return;  // block-uniform
  const double* ax = aux + (int64_t)zl * aux_stride(N);
  for (int i = jl; i <= NV; i += kT64) {
    if (i < NV) sd[i] = (i < N) ? ax[i] : 0.0;
    se[i] = (i < N - 1) ? ax[N + i] : 0.0;
  }
  __syncthreads();
  const double onenrm = ax[5 * N + 1];
  double* Zz = Zg + (int64_t)zl * N * N;
  double x[NV];
#pragma unroll
  for (int i = 0; i < NV; i++) x[i] = 0.0;
  if (!(onenrm > 1e4 * Prec<double>::tiny())) {  // Tri = 0: every vector is an eigenvector
#pragma unroll
    for (int i = 0; i < NV; i++) x[i] = (i == j) ? 1.0 : 0.0;
  } else if (j < N) {
    const double l = ax[4 * N + j];
    const double tiny = Prec<double>::eps() * onenrm;
#pragma unroll
    for (int i = 0; i < NV; i++) {
      unsigned h = (unsigned)i * 2654435761u ^ ((unsigned)j * 40503u + 0x9e3779b9u);
      h ^= h >> 15;
      h *= 2246822519u;
      h ^= h >> 13;
      x[i] = (i < N) ? (double)(h & 0xffffff) * (1.0 / 16777216.0) - 0.5 : 0.0;
    }
    unsigned long long piv = 0ull;  // bit i: rows i and i + 1 swapped in step i
#pragma unroll 1
    for (int it = 0; it < 2; it++) {
      double cd = sd[0] - l, csup = (N > 1) ? se[0] : 0.0;
      if (it == 0) {
        // the factorisation, fused with the elimination of the first right-hand side
#pragma unroll
        for (int i = 0; i < NV - 1; i++) {
          if (i < N - 1) {
            const double sub = se[i], dg = sd[i + 1] - l, sp = se[i + 1];  // 0 past N - 2
            const bool swap = fabs(cd) < fabs(sub);
            double pivot = swap ? sub : cd;
            if (!swap && fabs(pivot) < tiny) pivot = copysign(tiny, pivot);
            const double ui = rcp_newton(pivot);
            const double li = (swap ? cd : sub) * ui;
            su1[i * kT64 + jl] = swap ? dg : csup;
            sui[i * kT64 + jl] = ui;
            sli[i * kT64 + jl] = li;
            if (swap) piv |= 1ull << i;
            const double aa = swap ? csup : dg, bb = swap ? dg : csup;
            cd = fma(-li, bb, aa);
            const double nls = -li * sp;
            csup = swap ? nls : sp;
            const double xi = swap ? x[i + 1] : x[i], xn = swap ? x[i] : x[i + 1];
            x[i] = xi;
            x[i + 1] = fma(-li, xi, xn);
          }
        }
      } else {
        // the second solve has the same factors (same Tri, same shift): apply the stored
        // interchanges and multipliers only (the same values the factorisation produced, so
        // the result is the one a recomputation would give, bit for bit)
#pragma unroll
        for (int i = 0; i < NV - 1; i++) {
          if (i < N - 1) {
            const bool swap = (piv >> i) & 1ull;
            const double li = sli[i * kT64 + jl];
            const double xi = swap ? x[i + 1] : x[i], xn = swap ? x[i] : x[i + 1];
            x[i] = xi;
            x[i + 1] = fma(-li, xi, xn);
          }
        }
      }
      if (it == 0) {
        double pivot = cd;
        if (fabs(pivot) < tiny) pivot = copysign(tiny, pivot);
        sui[(N - 1) * kT64 + jl] = rcp_newton(pivot);
        // the factor has no entries right of the last column: zeros make one formula serve
        // every row (x beyond N is 0)
        su1[(N - 1) * kT64 + jl] = 0.0;
      }
      // back substitution x[i] = (x[i] - u1 x[i+1] - u2 x[i+2]) / p; every index is a
      // compile-time constant after unrolling (guards compare with N, never select by it), so
      // x stays in registers
#pragma unroll
      for (int i = NV - 1; i >= 0; i--) {
        if (i < N) {
          double v = x[i];
          if (i + 1 < NV) v = fma(-su1[i * kT64 + jl], x[i + 1], v);
          if (i + 2 < NV) {
            const double u2 = ((piv >> i) & 1ull) ? se[i + 1] : 0.0;
            v = fma(-u2, x[i + 2], v);
          }
          x[i] = v * sui[i * kT64 + jl];
        }
      }
      // scale by a power of two near 1/max|x| (the sum of squares cannot overflow), then
      // normalise
      double mx = 0.0;
#pragma unroll
      for (int i = 0; i < NV; i++)
        if (i < N) mx = fmax(mx, fabs(x[i]));
      const double im = pow2_inv_exponent(mx);
      double nrm = 0.0;
#pragma unroll
      for (int i = 0; i < NV; i++) {
        if (i < N) {
          x[i] *= im;
          nrm = fma(x[i], x[i], nrm);
        }
      }
      const double sc = rsqrt_newton(nrm);
#pragma unroll
      for (int i = 0; i < NV; i++) x[i] *= sc;
    }
  }
  __syncthreads();  // factors no longer read: reuse them as the transpose buffer
  double* tr = sfac64;  // [i][kT64 + 1]
#pragma unroll
  for (int i = 0; i < NV; i++) tr[i * (kT64 + 1) + jl] = x[i];
  __syncthreads();
  // this block's vectors kT64 blockIdx.y + jj (rows of Z), coalesced along the rows
  const int j0 = kT64 * blockIdx.y;
  const int nv = (N - j0 < kT64) ? N - j0 : kT64;
  for (int idx = jl; idx < nv * N; idx += kT64) {
    const int jj = idx / N, i = idx - jj * N;
    Zz[(int64_t)(j0 + jj) * N + i] = tr[i * (kT64 + 1) + jj];
  }
}

// ------------------------------------------------------------------------------------ E3
template <typename R>
__global__ void __launch_bounds__(kThreads)
    k_eig_transform(int N, int32_t nzc, R* __restrict__ GT, R* __restrict__ aux,
                    R* __restrict__ Zg, const R* __restrict__ gv,
                    const int32_t* __restrict__ nobs, int rotate, R* __restrict__ ampl_out,
                    int32_t* __restrict__ status, int32_t* __restrict__ work, int a_global,
                    int tc_out) {
  extern __shared__ __align__(16) unsigned char dyn_raw[];
  R* dyn = reinterpret_cast<R*>(dyn_raw);
  const int ld = N + 1;
  // A: [N][ld] reflectors, then T_sym. When two N x N matrices do not fit in shared memory
  // (a_global), A is the zone's own slot of GT ([N][N]: the reflectors E1 left there, then
  // T_sym), read and written only between block barriers
  R* A = dyn;
  R* U = a_global ? dyn : A + N * ld;  // [N][ld] Z, then U
  R* lam = U + N * ld;  // [N] 1/(1+lambda)         (evaluated in FP64)
  R* sq = lam + N;      // [N] sqrt(1/(1+lambda))   (evaluated in FP64)
  R* g = sq + N;        // [N]
  R* beta = g + N;      // [N]
  R* t0 = beta + N;     // [N]
  R* t1 = t0 + N;       // [N]
  R* vv = t1 + N;       // [N]
  R* qs = vv + N;       // [N] lambda^(1/4)        (evaluated in FP64)
  R* cf = qs + N;       // [4][N] back-transform coefficients of four reflectors
  R* pc = cf + 4 * N;   // [3][N] reflector couplings p_s[k] = v_k . v_(k-s), s = 1, 2, 3
  int* cst = reinterpret_cast<int*>(pc + 3 * N);  // [N] cluster start of each eigenvector
  __shared__ R red[kWarps];
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
    R* Gz = GT + (int64_t)zl * N * N;
    R* ax = aux + (int64_t)zl * aux_stride(N);
    R* Z = Zg + (int64_t)zl * N * N;
    R* Aw = a_global ? Gz : A;
    const int la = a_global ? N : ld;
    for (int idx = tid; idx < N * N; idx += kThreads) {
      int i = idx / N, j = idx - i * N;
      if (!a_global) A[i * ld + j] = (i > j) ? Gz[idx] : R(0);
      U[j * ld + i] = Z[idx];  // Z[i*N + j] = component j of eigenvector i -> U[j][i]
    }
    for (int i = tid; i < N; i += kThreads) {
      double l = (double)ax[3 * N + i];
      if (l < 0.0) l = 0.0;
      const double li = 1.0 / (1.0 + l);
      const double s = sqrt(li);
      lam[i] = (R)li;
      sq[i] = (R)s;
      qs[i] = (R)sqrt(s);
      g[i] = gv[(int64_t)zl * N + i];
      beta[i] = ax[2 * N + i];
    }
    if (tid == 0) {
      const R ortol = R(1e-3) * ax[5 * N + 1] * ax[5 * N];
      int c0 = 0;
      cst[0] = 0;
      for (int j = 1; j < N; j++) {
        if (ax[3 * N + j] - ax[3 * N + j - 1] > ortol) c0 = j;
        cst[j] = c0;
      }
    }
    __syncthreads();
    // FP64: classical Gram-Schmidt of column j against its cluster [cst[j], j). FP32 (larger
    // relative rounding, gaps between clusters less reliable): every column against all columns
    // of larger eigenvalue, largest first. Column j is a unit vector and the earlier columns
    // are orthonormal: if one pass leaves it at least half its squared norm, it is orthogonal to
    // them to working precision ("twice is enough", Kahan-Parlett; Parlett, The Symmetric
    // Eigenvalue Problem, 6-9) and accepted after that pass. A vector that keeps less is
    // collapsed (replaced below); it still gets the second pass, since later columns of the
    // cluster are projected against its (normalised) residual, which must then be orthogonal
    // to the earlier columns.
    const bool full = sizeof(R) < sizeof(double);
    for (int jj = 1; jj < N; jj++) {
      const int j = full ? N - 1 - jj : jj;
      const int k0 = full ? j + 1 : cst[j], nk = full ? N - 1 - j : j - k0;
      if (nk == 0) continue;  // uniform
      for (int pass = 0; pass < 2; pass++) {
        // one thread per dot product (no cross-lane reductions)
        for (int kk = tid; kk < nk; kk += kThreads) {
          R s = 0;
          for (int i = 0; i < N; i++) s = fma(U[i * ld + k0 + kk], U[i * ld + j], s);
          t0[kk] = s;
        }
        __syncthreads();
        for (int i = tid; i < N; i += kThreads) {
          R s = U[i * ld + j];
          for (int kk = 0; kk < nk; kk++) s = fma(-t0[kk], U[i * ld + k0 + kk], s);
          U[i * ld + j] = s;
        }
        __syncthreads();
        if (warp == 0) {
          R s = 0;
          for (int i = lane; i < N; i += 32) s = fma(U[i * ld + j], U[i * ld + j], s);
          s = warp_sum(s);
          // a unit vector that kept less than half its norm lay (almost) in the span of the
          // cluster's earlier vectors: mark it for the complement fill below
          if (lane == 0) {
            red[0] = (s > R(0)) ? Prec<R>::rsqrt_(s) : R(0);
            red[1] = (s < R(0.5)) ? R(1) : R(0);
            if (pass == 1 && s < R(0.5)) cst[j] = -1;
          }
        }
        __syncthreads();
        if (red[1] == R(0)) break;  // uniform: accepted after this pass
      }
      const R sc = red[0];
      for (int i = tid; i < N; i += kThreads) U[i * ld + j] *= sc;
      __syncthreads();
    }
    // complement fill: a collapsed vector is replaced by a pseudo-random vector made
    // orthogonal (two classical Gram-Schmidt passes) to every accepted eigenvector. When the
    // accepted vectors are accurate, the complement is the missing part of the degenerate
    // cluster's invariant subspace, so any unit vector in it is an eigenvector.
    for (int j = 0; j < N; j++) {
      if (cst[j] >= 0) continue;  // uniform
      for (int i = tid; i < N; i += kThreads) {
        unsigned h = (unsigned)i * 2246822519u ^ ((unsigned)j * 3266489917u + 0x27d4eb2fu);
        h ^= h >> 15;
        h *= 2654435761u;
        h ^= h >> 13;
        U[i * ld + j] = (R)((double)(h & 0xffffff) * (1.0 / 16777216.0) - 0.5);
      }
      __syncthreads();
      for (int pass = 0; pass < 2; pass++) {
        for (int k = tid; k < N; k += kThreads) {
          R s = 0;
          if (k != j && cst[k] >= 0)
            for (int i = 0; i < N; i++) s = fma(U[i * ld + k], U[i * ld + j], s);
          t0[k] = s;
        }
        __syncthreads();
        for (int i = tid; i < N; i += kThreads) {
          R s = U[i * ld + j];
          for (int k = 0; k < N; k++) s = fma(-t0[k], U[i * ld + k], s);
          U[i * ld + j] = s;
        }
        __syncthreads();
      }
      if (warp == 0) {
        R s = 0;
        for (int i = lane; i < N; i += 32) s = fma(U[i * ld + j], U[i * ld + j], s);
        s = warp_sum(s);
        if (lane == 0) {
          red[0] = (s > R(0)) ? Prec<R>::rsqrt_(s) : R(0);
          cst[j] = j;  // accepted
        }
      }
      __syncthreads();
      const R sc = red[0];
      for (int i = tid; i < N; i += kThreads) U[i * ld + j] *= sc;
      __syncthreads();
    }
    // U = Q_h Z = H_0 H_1 ... H_{N-3} Z, H_k = I - b_k v_k v_k^T (v_k below the diagonal of
    // column k of A): four reflectors at a time, k, k-1, k-2, k-3 in that order. The four dots
    // d_r = v_(k-r) . u_j of the unchanged column u_j are independent (one thread each, all
    // 4 x N of them at once); the coefficients follow from c_r = b_(k-r) (d_r - sum_(r'<r) c_r'
    // v_(k-r) . v_(k-r')), and one pass subtracts sum_r c_r v_(k-r): three barriers per four
    // reflectors instead of eight, the same products as one reflector at a time.
    for (int kk = tid; kk < N - 2; kk += kThreads) {
#pragma unroll
      for (int sft = 1; sft <= 3; sft++) {
        R sp = 0;
        if (kk >= sft)  // v_kk and v_(kk-s) overlap on rows kk + 1 .. N - 1
          for (int i = kk + 1; i < N; i++) sp = fma(Aw[i * la + kk], Aw[i * la + kk - sft], sp);
        pc[(sft - 1) * N + kk] = sp;
      }
    }
    __syncthreads();
    int kb = N - 3;
    for (; kb >= 3; kb -= 4) {
      for (int it = tid; it < 4 * N; it += kThreads) {
        const int r = it / N, j = it - r * N, kr = kb - r;
        R sd = 0;
        for (int i = kr + 1; i < N; i++) sd = fma(Aw[i * la + kr], U[i * ld + j], sd);
        cf[r * N + j] = sd;
      }
      __syncthreads();
      for (int j = tid; j < N; j += kThreads) {
        const R d0 = cf[j], d1 = cf[N + j], d2 = cf[2 * N + j], d3 = cf[3 * N + j];
        const R c0 = beta[kb] * d0;
        const R c1 = beta[kb - 1] * fma(-c0, pc[kb], d1);
        const R c2 = beta[kb - 2] * fma(-c1, pc[kb - 1], fma(-c0, pc[N + kb], d2));
        const R c3 = beta[kb - 3] *
                     fma(-c2, pc[kb - 2], fma(-c1, pc[N + kb - 1], fma(-c0, pc[2 * N + kb], d3)));
        cf[j] = c0;
        cf[N + j] = c1;
        cf[2 * N + j] = c2;
        cf[3 * N + j] = c3;
      }
      __syncthreads();
      // rows kb - 2 .. N - 1 (v_(kb-3) starts at row kb - 2; the others vanish there first)
      const int r0 = kb - 2, L = N - r0;
      for (int idx = tid; idx < L * N; idx += kThreads) {
        const int i = r0 + idx / N, j = idx - (idx / N) * N;
        const R v0 = (i > kb) ? Aw[i * la + kb] : R(0);
        const R v1 = (i > kb - 1) ? Aw[i * la + kb - 1] : R(0);
        const R v2 = (i > kb - 2) ? Aw[i * la + kb - 2] : R(0);
        const R v3 = Aw[i * la + kb - 3];
        R* u = U + i * ld + j;
        *u = fma(-cf[3 * N + j], v3,
                 fma(-cf[2 * N + j], v2, fma(-cf[N + j], v1, fma(-cf[j], v0, *u))));
      }
      __syncthreads();
    }
    for (int k = kb; k >= 0; k--) {  // the remaining reflectors one at a time
      const R bk = beta[k];
      if (bk == R(0)) continue;  // uniform across the block
      const int L = N - k - 1;
      for (int j = tid; j < N; j += kThreads) {
        R s = 0;
        for (int i = 0; i < L; i++) s = fma(Aw[(k + 1 + i) * la + k], U[(k + 1 + i) * ld + j], s);
        t0[j] = bk * s;
      }
      __syncthreads();
      for (int idx = tid; idx < L * N; idx += kThreads) {
        int i = idx / N, j = idx - i * N;
        R* u = U + (k + 1 + i) * ld + j;
        *u = fma(-Aw[(k + 1 + i) * la + k], t0[j], *u);
      }
      __syncthreads();
    }
    // ampl = U (lambda .* (U^T g))
    for (int i = tid; i < N; i += kThreads) {
      R s = 0;
      for (int r = 0; r < N; r++) s = fma(U[r * ld + i], g[r], s);
      t0[i] = lam[i] * s;
    }
    __syncthreads();
    int nan_flag = 0;
    for (int r = tid; r < N; r += kThreads) {
      R s = 0;
      for (int i = 0; i < N; i++) s = fma(U[r * ld + i], t0[i], s);
      ampl_out[(int64_t)zl * N + r] = s;
      if (!(s == s) || isinf(s)) nan_flag = 1;
    }
    nan_flag = __syncthreads_or(nan_flag);
    if (rotate) {
      // v = normate(U (colsum(U) / sqrt(lambda)))
      for (int i = tid; i < N; i += kThreads) {
        R s = 0;
        for (int r = 0; r < N; r++) s += U[r * ld + i];
        t1[i] = s / sq[i];
      }
      __syncthreads();
      for (int r = tid; r < N; r += kThreads) {
        R s = 0;
        for (int i = 0; i < N; i++) s = fma(U[r * ld + i], t1[i], s);
        vv[r] = s;
      }
      __syncthreads();
      if (warp == 0) {
        R s = 0;
        for (int r = lane; r < N; r += 32) s = fma(vv[r], vv[r], s);
        s = warp_sum(s);
        if (lane == 0) red[0] = R(1) / Prec<R>::sqrt_(s);
      }
      __syncthreads();
      const R inv = red[0];
      for (int r = tid; r < N; r += kThreads) vv[r] *= inv;
    }
    if (tc_out) {
      // T_sym and T are formed on the tensor cores (zone_tsym_oz): the eigenvectors go to the
      // zone's Z slot vector-major (Z[k N + i] = U_ik; Z was read above), (1 + lambda)^-1/4 to
      // the shift slots and v to the d slots of aux (neither is read after this stage)
      for (int idx = tid; idx < N * N; idx += kThreads) {
        const int k = idx / N, i = idx - k * N;
        Z[idx] = U[i * ld + k];
      }
      for (int i = tid; i < N; i += kThreads) {  // vv[i] was scaled by this thread
        ax[4 * N + i] = qs[i];
        ax[i] = rotate ? vv[i] : R(0);
      }
      if (tid == 0 && nan_flag) status[zl] |= ZST_NAN;
      __syncthreads();
      continue;
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
      const R* qa = U + a * ld;
      const R* qb = U + b * ld;
      R s = 0;
      for (int k = 0; k < N; k++) s = fma(qa[k], qb[k], s);
      Aw[a * la + b] = s;
      Aw[b * la + a] = s;
    }
    __syncthreads();
    if (rotate) {
      const R vN = vv[N - 1];
      const R sv = signbit(vN) ? R(-1) : R(1);
      const R cv = R(1) + fabs(vN);
      const R wv = (R)(1.0 / sqrt((double)N));
      const R cw = R(1) + wv;
      // t0 = T_sym u_v, t1 = T_sym v
      for (int i = tid; i < N; i += kThreads) {
        const R* ti = Aw + i * la;
        R sa = 0, sb = 0;
        for (int j = 0; j < N; j++) {
          sa = fma(ti[j], vv[j] + ((j == N - 1) ? sv : R(0)), sa);
          sb = fma(ti[j], vv[j], sb);
        }
        t0[i] = sa;
        t1[i] = sb;
      }
      __syncthreads();
      // T1 = T_sym - t0 u_v^T / c_v
      const R icv = R(1) / cv, icw = R(1) / cw;
      for (int idx = tid; idx < N * N; idx += kThreads) {
        int i = idx / N, j = idx - i * N;
        R uj = vv[j] + ((j == N - 1) ? sv : R(0));
        Aw[i * la + j] = fma(-t0[i] * icv, uj, Aw[i * la + j]);
      }
      __syncthreads();
      // g <- T1 u_w (g is no longer needed)
      for (int i = tid; i < N; i += kThreads) {
        const R* ti = Aw + i * la;
        R s = 0;
        for (int j = 0; j < N; j++) s = fma(ti[j], wv + ((j == N - 1) ? R(1) : R(0)), s);
        g[i] = s * icw;
      }
      __syncthreads();
      // T = T1 - (T1 u_w) u_w^T / c_w + (1 - s_v s_w) (T_sym v) w^T   (s_w = +1)
      const R extra = R(1) - sv;
      for (int idx = tid; idx < N * N; idx += kThreads) {
        int i = idx / N, j = idx - i * N;
        R uj = wv + ((j == N - 1) ? R(1) : R(0));
        R t = fma(-g[i], uj, Aw[i * la + j]);
        if (extra != R(0)) t = fma(extra * t1[i], wv, t);
        Gz[idx] = t;
      }
    } else {
      for (int idx = tid; idx < N * N; idx += kThreads) {
        int i = idx / N, j = idx - i * N;
        Gz[idx] = Aw[i * la + j];
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

// E1 and E3 of the generic path
template <typename R>
cudaError_t launch_e1(int N, int32_t nzc, R* d_GT, R* d_aux, const int32_t* d_nobs,
                      int32_t* d_work, cudaStream_t st) {
  size_t smem1 = (size_t)(N * (N + 1) + 2 * N) * sizeof(R);
  cudaError_t e = cudaFuncSetAttribute(k_eig_tridiag<R>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem1);
  if (e != cudaSuccess) return e;
  k_eig_tridiag<R><<<grid_for_smem((const void*)k_eig_tridiag<R>, smem1, nzc), kThreads, smem1,
                     st>>>(N, nzc, d_GT, d_aux, d_nobs, d_work);
  return cudaSuccess;
}

template <typename R>
cudaError_t launch_e3(int N, int32_t nzc, R* d_GT, R* d_aux, R* d_Z, const R* d_g,
                      const int32_t* d_nobs, int rotate, R* d_ampl, int32_t* d_status,
                      int32_t* d_work, cudaStream_t st, int tc_out = 0) {
  // two N x N matrices in shared memory when they fit (227 KB a block), else one (A in GT)
  size_t smem3 = (size_t)(2 * N * (N + 1) + 16 * N) * sizeof(R) + (size_t)N * sizeof(int);
  int a_global = 0;
  if (smem3 > (size_t)227 * 1024) {
    smem3 = (size_t)(N * (N + 1) + 16 * N) * sizeof(R) + (size_t)N * sizeof(int);
    a_global = 1;
  }
  cudaError_t e = cudaFuncSetAttribute(k_eig_transform<R>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem3);
  if (e != cudaSuccess) return e;
  k_eig_transform<R><<<grid_for_smem((const void*)k_eig_transform<R>, smem3, nzc), kThreads,
                       smem3, st>>>(N, nzc, d_GT, d_aux, d_Z, d_g, d_nobs, rotate, d_ampl,
                                    d_status, d_work, a_global, tc_out);
  return cudaSuccess;
}

// FP32 with at most 128 members: the register-blocked E1/E3 of zone_eig32.cu (they share the
// aux layout and the inverse-iteration output with E2a/E2b, and store the reflectors
// vector-major, so both are used together): warp-per-zone kernels up to 64 members,
// block-per-zone kernels up to 128
template <>
cudaError_t launch_e1<float>(int N, int32_t nzc, float* d_GT, float* d_aux,
                             const int32_t* d_nobs, int32_t* d_work, cudaStream_t st) {
  if (N <= eig32_max_n()) return eig32_tridiag(N, nzc, d_GT, d_aux, d_nobs, st);
  if (N <= eig128_max_n()) return eig128_tridiag(N, nzc, d_GT, d_aux, d_nobs, st);
  size_t smem1 = (size_t)(N * (N + 1) + 2 * N) * sizeof(float);
  cudaError_t e = cudaFuncSetAttribute(k_eig_tridiag<float>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem1);
  if (e != cudaSuccess) return e;
  k_eig_tridiag<float><<<grid_for_smem((const void*)k_eig_tridiag<float>, smem1, nzc), kThreads,
                         smem1, st>>>(N, nzc, d_GT, d_aux, d_nobs, d_work);
  return cudaSuccess;
}

template <>
cudaError_t launch_e3<float>(int N, int32_t nzc, float* d_GT, float* d_aux, float* d_Z,
                             const float* d_g, const int32_t* d_nobs, int rotate, float* d_ampl,
                             int32_t* d_status, int32_t* d_work, cudaStream_t st,
                             int /*tc_out*/) {
  // mode 0 does not write Z
  if (N <= eig32_max_n())
    return eig32_transform(N, nzc, d_GT, d_aux, d_Z, d_g, d_nobs, rotate, d_ampl, d_status, st);
  if (N <= eig128_max_n())
    return eig128_transform(N, nzc, d_GT, d_aux, d_Z, d_g, d_nobs, rotate, d_ampl, d_status,
                            st);
  size_t smem3 = (size_t)(2 * N * (N + 1) + 16 * N) * sizeof(float) + (size_t)N * sizeof(int);
  cudaError_t e = cudaFuncSetAttribute(k_eig_transform<float>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem3);
  if (e != cudaSuccess) return e;
  k_eig_transform<float><<<grid_for_smem((const void*)k_eig_transform<float>, smem3, nzc),
                           kThreads, smem3, st>>>(N, nzc, d_GT, d_aux, d_Z, d_g, d_nobs, rotate,
                                                  d_ampl, d_status, d_work, 0, 0);
  return cudaSuccess;
}

template <typename R>
cudaError_t launch_e2(int N, int32_t nzc, R* d_aux, R* d_Z, const int32_t* d_nobs,
                      int32_t* d_status, cudaStream_t st) {
  if (nzc < kFewZones) {
    k_eig_values_multisect<R><<<dim3((unsigned)N, (unsigned)nzc), 32, 0, st>>>(N, nzc, d_aux,
                                                                               d_nobs);
    k_eig_shifts<R><<<(nzc + 127) / 128, 128, 0, st>>>(N, nzc, d_aux, d_nobs);
  } else {
    k_eig_tridiag_values<R><<<(nzc + 127) / 128, 128, 0, st>>>(N, nzc, d_aux, d_nobs, d_status);
  }
  if (sizeof(R) == sizeof(double) && N <= kNV64) {
    const size_t smem = (size_t)3 * kNV64 * kT64 * sizeof(double);
    cudaError_t e = cudaFuncSetAttribute(k_eig_vectors_fp64,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const unsigned yb = (unsigned)((N + kT64 - 1) / kT64);
    k_eig_vectors_fp64<<<dim3((unsigned)(nzc > 0 ? nzc : 1), yb), kT64, smem, st>>>(
        N, nzc, reinterpret_cast<const double*>(d_aux), reinterpret_cast<double*>(d_Z), d_nobs);
    return cudaSuccess;
  }
  const int64_t pairs = (int64_t)nzc * N;
  k_eig_tridiag_vectors<R><<<(unsigned)((pairs + 127) / 128), 128, 0, st>>>(N, nzc, d_aux, d_Z,
                                                                             d_nobs);
  return cudaSuccess;
}

template <>
cudaError_t launch_e2<float>(int N, int32_t nzc, float* d_aux, float* d_Z, const int32_t* d_nobs,
                             int32_t* d_status, cudaStream_t st) {
  if (N <= eig32_max_n()) {  // shared-memory E2a / E2b of zone_eig32.cu
    cudaError_t e = eig32_values(N, nzc, d_aux, d_nobs, d_status, st);
    if (e != cudaSuccess) return e;
    return eig32_vectors(N, nzc, d_aux, d_Z, d_nobs, st);
  }
  k_eig_tridiag_values<float><<<(nzc + 127) / 128, 128, 0, st>>>(N, nzc, d_aux, d_nobs, d_status);
  const int64_t pairs = (int64_t)nzc * N;
  k_eig_tridiag_vectors<float><<<(unsigned)((pairs + 127) / 128), 128, 0, st>>>(N, nzc, d_aux,
                                                                                 d_Z, d_nobs);
  return cudaSuccess;
}

template <typename R>
cudaError_t zone_eig_impl(int N, int32_t nzc, R* d_GT, const R* d_g, const int32_t* d_nobs,
                          int rotate, R* d_ampl, int32_t* d_status, R* d_aux, R* d_Z,
                          int32_t* d_work, cudaStream_t st, int tc_products = 0) {
  if (N < 2 || N > kNMax) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(d_status, 0, sizeof(int32_t) * (nzc > 0 ? nzc : 1), st);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(d_work, 0, 2 * sizeof(int32_t), st);
  if (e != cudaSuccess) return e;
  e = launch_e1<R>(N, nzc, d_GT, d_aux, d_nobs, d_work, st);
  if (e != cudaSuccess) return e;
  // E2a, E2b
  e = launch_e2<R>(N, nzc, d_aux, d_Z, d_nobs, d_status, st);
  if (e != cudaSuccess) return e;
  // T_sym on the tensor cores (FP64 only): E3 hands over U, (1 + lambda)^-1/4 and v
  const int tc = (sizeof(R) == sizeof(double) && tc_products && N <= gram_oz_max_n()) ? 1 : 0;
  e = launch_e3<R>(N, nzc, d_GT, d_aux, d_Z, d_g, d_nobs, rotate, d_ampl, d_status, d_work + 1,
                   st, tc);
  if (e != cudaSuccess) return e;
  count_launches(4);
  if (tc) {
    e = zone_tsym_oz(N, nzc, reinterpret_cast<double*>(d_GT),
                     reinterpret_cast<const double*>(d_aux), reinterpret_cast<const double*>(d_Z),
                     d_nobs, rotate, d_status, st);
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

}  // namespace

size_t zone_eig_aux(int N) { return (size_t)aux_stride(N); }

cudaError_t zone_eig_fp64(int N, int32_t nzc, double* d_GT, const double* d_g,
                          const int32_t* d_nobs, int rotate, double* d_ampl, int32_t* d_status,
                          double* d_aux, double* d_Z, int32_t* d_work, cudaStream_t st,
                          int tc_products) {
  return zone_eig_impl<double>(N, nzc, d_GT, d_g, d_nobs, rotate, d_ampl, d_status, d_aux, d_Z,
                               d_work, st, tc_products);
}

cudaError_t zone_eig_fp32(int N, int32_t nzc, float* d_GT, const float* d_g,
                          const int32_t* d_nobs, int rotate, float* d_ampl, int32_t* d_status,
                          float* d_aux, float* d_Z, int32_t* d_work, cudaStream_t st) {
  return zone_eig_impl<float>(N, nzc, d_GT, d_g, d_nobs, rotate, d_ampl, d_status, d_aux, d_Z,
                              d_work, st);
}

// The FP32 eigensolve with its eigenpairs refined to FP64 accuracy before the transform: G is
// kept in d_G0 (E1 overwrites it with reflectors), E3 stops after the back-transform and leaves
// the eigenvectors of G in d_Z, zone_eig_refine refines them and the eigenvalues in place (its
// S scratch: zone_refine_scratch(N) floats a zone), and E3 forms T and the amplitudes from
// them.
cudaError_t zone_eig_fp32_refined(int N, int32_t nzc, float* d_GT, const float* d_g,
                                  const int32_t* d_nobs, int rotate, float* d_ampl,
                                  int32_t* d_status, float* d_aux, float* d_Z, int32_t* d_work,
                                  float* d_G0, float* d_S, cudaStream_t st) {
  if (N < 2 || N > eig128_max_n()) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(d_status, 0, sizeof(int32_t) * (nzc > 0 ? nzc : 1), st);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(d_work, 0, 2 * sizeof(int32_t), st);
  if (e != cudaSuccess) return e;
  e = cudaMemcpyAsync(d_G0, d_GT, sizeof(float) * (size_t)nzc * N * N, cudaMemcpyDeviceToDevice,
                      st);
  if (e != cudaSuccess) return e;
  e = launch_e1<float>(N, nzc, d_GT, d_aux, d_nobs, d_work, st);
  if (e != cudaSuccess) return e;
  e = launch_e2<float>(N, nzc, d_aux, d_Z, d_nobs, d_status, st);
  if (e != cudaSuccess) return e;
  e = (N <= eig32_max_n())
          ? eig32_transform(N, nzc, d_GT, d_aux, d_Z, d_g, d_nobs, rotate, d_ampl, d_status, st, 1)
          : eig128_transform(N, nzc, d_GT, d_aux, d_Z, d_g, d_nobs, rotate, d_ampl, d_status, st,
                             1);
  if (e != cudaSuccess) return e;
  e = zone_eig_refine(N, nzc, d_G0, d_Z, d_aux, d_nobs, d_S, st);
  if (e != cudaSuccess) return e;
  e = (N <= eig32_max_n())
          ? eig32_transform(N, nzc, d_GT, d_aux, d_Z, d_g, d_nobs, rotate, d_ampl, d_status, st, 2)
          : eig128_transform(N, nzc, d_GT, d_aux, d_Z, d_g, d_nobs, rotate, d_ampl, d_status, st,
                             2);
  if (e != cudaSuccess) return e;
  count_launches(5);
  return cudaGetLastError();
}

}  // namespace oakg
