// Mixed-precision eigensolve kernels for ensembles of up to 64 members: E1 (Householder
// tridiagonalisation) and E3 (eigenvector orthogonalisation, back-transform, amplitudes and the
// square-root transform) in FP32, built around register blocking instead of the shared-memory
// loops of the generic kernels in zone_eig.cu. E2a/E2b (tridiagonal eigenvalues and inverse
// iteration) are shared with the generic path.
//
// The arithmetic follows rrsqrt.F90:136-185 as the generic kernels do (the comment block at the
// top of zone_eig.cu lists the reference lines); the matrix is padded to 64 x 64 with zeros,
// which adds decoupled zero rows that no output reads.
//
// E1 (one CTA of 256 threads per zone): thread (bi, bj), bi, bj in [0,16), holds the 16
// elements A[bi + 16a][bj + 16b], a, b in [0,4) of the scaled symmetric matrix in registers.
//   Column k lives in one half-warp (bj = k mod 16), so the reflector's norm is a half-warp
//   reduction; p = beta A v is formed as column sums (A is symmetric) reduced over the
//   half-warp; two CTA barriers per step. Reflector k is stored vector-major, zero padded,
//   in row k of the zone's matrix slot: slot[k*N + r] = v_k[r] (v_k[r] = 0 for r <= k).
//
// E3 (one CTA of 256 threads per zone): thread t works on eigenvector j = t/4, components
//   16 (t mod 4) .. +15, held in registers.
//   back-transform U = H_0 ... H_{N-3} Z: per reflector a 4-lane dot and an axpy, no barrier;
//   orthogonalisation: right-looking modified Gram-Schmidt, two sweeps, largest eigenvalue
//     first (a vector is final when every larger-eigenvalue vector has been projected out of
//     it); a vector that keeps less than half its norm is marked collapsed and replaced, after
//     the sweeps, by a pseudo-random vector orthogonalised against every accepted one;
//   T_sym = (U Q)(U Q)^T with Q = diag((1+lambda)^-1/4): 4 x 4 register blocks, 128-bit
//     shared loads; Omega = RotateVector(w, v) applied to the register blocks in its
//     reflector form (rank-one updates, matoper.F90:509-535).
#include <cuda_runtime.h>
#include <math.h>

#include "oakg_internal.cuh"

namespace oakg {

namespace {

constexpr int NB = 64;        // padded ensemble size
constexpr int kT = 256;       // threads per CTA
constexpr int LDV = NB + 4;   // row stride of vector-major shared matrices (16-byte rows,
                              // 8 consecutive rows fall in 8 different 16-byte bank groups)

__host__ __device__ inline int aux_stride32(int N) { return 5 * N + 2; }

__device__ __forceinline__ float hsum16(float x) {  // sum over the 16 lanes of a half-warp
  x += __shfl_xor_sync(0xffffffffu, x, 1);
  x += __shfl_xor_sync(0xffffffffu, x, 2);
  x += __shfl_xor_sync(0xffffffffu, x, 4);
  x += __shfl_xor_sync(0xffffffffu, x, 8);
  return x;
}

// sum over the 4 lanes of one vector; only those 4 lanes need to be converged
__device__ __forceinline__ float qsum4(float x) {
  const unsigned m = 0xFu << (threadIdx.x & 28);
  x += __shfl_xor_sync(m, x, 1);
  x += __shfl_xor_sync(m, x, 2);
  return x;
}

// ------------------------------------------------------------------------------------ E1
template <int KB>
__device__ __forceinline__ void tridiag_step(int k, int N, float (&A)[4][4], float* vbuf,
                                             float* pbuf, float* red, float* s_beta, float* Gz,
                                             float* ax, int tid, int bi, int bj, int warp) {
  const int kk = k & 15;
  // (1) reflector of column k (owned by half-warp bj == kk of warp kk/2)
  if (warp == (kk >> 1)) {
    const bool mine = (bj == kk);
    float sig = 0.f, x0 = 0.f;
    if (mine) {
#pragma unroll
      for (int a = 0; a < 4; a++) {
        const int r = bi + 16 * a;
        const float x = A[a][KB];
        if (r > k + 1) sig = fmaf(x, x, sig);
        if (r == k + 1) x0 = x;
      }
    }
    sig = hsum16(sig);
    x0 = hsum16(x0);
    const float mu = sqrtf(fmaf(x0, x0, sig));
    const float v0 = (x0 <= 0.f) ? x0 - mu : x0 + mu;
    const float vv = fmaf(v0, v0, sig);
    const bool skip = (sig == 0.f) || !(vv > 0.f) || isinf(vv);
    const float bk = skip ? 0.f : 2.f / vv;
    if (mine) {
#pragma unroll
      for (int a = 0; a < 4; a++) {
        const int r = bi + 16 * a;
        const float val = (r > k + 1) ? A[a][KB] : ((r == k + 1) ? (skip ? x0 : v0) : 0.f);
        vbuf[r] = val;
        if (r < N) Gz[(int64_t)k * N + r] = val;
        if (r == k) ax[k] = A[a][KB];  // d_k
      }
      if (bi == 0) {
        ax[N + k] = skip ? x0 : ((x0 <= 0.f) ? mu : -mu);  // e_k
        ax[2 * N + k] = bk;                                 // beta_k
        s_beta[k & 1] = bk;
      }
    }
  }
  __syncthreads();  // S1: v and beta published
  // beta is double-buffered by step parity: after an identity step (no S2) the next step's
  // owner may already write its beta while slower warps still read this one
  const float bk = s_beta[k & 1];
  if (bk == 0.f) return;  // uniform: identity reflector
  float vr[4], vc[4];
#pragma unroll
  for (int a = 0; a < 4; a++) vr[a] = vbuf[bi + 16 * a];
#pragma unroll
  for (int b = 0; b < 4; b++) vc[b] = vbuf[bj + 16 * b];
  // p_c = beta sum_r A[r][c] v_r (column sums; A symmetric), reduced over the half-warp
  float q[4];
#pragma unroll
  for (int b = 0; b < 4; b++) {
    float s = A[0][b] * vr[0];
    s = fmaf(A[1][b], vr[1], s);
    s = fmaf(A[2][b], vr[2], s);
    s = fmaf(A[3][b], vr[3], s);
    q[b] = hsum16(s) * bk;
  }
  float pv = 0.f;
  if (bi == 0) {
#pragma unroll
    for (int b = 0; b < 4; b++) {
      pbuf[bj + 16 * b] = q[b];
      pv = fmaf(q[b], vc[b], pv);
    }
  }
  pv += __shfl_xor_sync(0xffffffffu, pv, 16);
  if ((tid & 31) == 0) red[warp] = pv;
  __syncthreads();  // S2: p and the partial dots published
  float kc = 0.f;
#pragma unroll
  for (int w = 0; w < kT / 32; w++) kc += red[w];
  kc *= 0.5f * bk;
  float wr[4], wc[4];
#pragma unroll
  for (int a = 0; a < 4; a++) wr[a] = fmaf(-kc, vr[a], pbuf[bi + 16 * a]);
#pragma unroll
  for (int b = 0; b < 4; b++) wc[b] = fmaf(-kc, vc[b], pbuf[bj + 16 * b]);
  // A -= v w^T + w v^T
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) A[a][b] = fmaf(-vr[a], wc[b], fmaf(-wr[a], vc[b], A[a][b]));
}

__global__ void __launch_bounds__(kT, 4)
    k_eig_tridiag32(int N, int32_t nzc, float* __restrict__ GT, float* __restrict__ aux,
                    const int32_t* __restrict__ nobs, int32_t* __restrict__ work) {
  __shared__ __align__(16) float vbuf[NB];
  __shared__ __align__(16) float pbuf[NB];
  __shared__ float red[kT / 32];
  __shared__ float s_beta[2];
  __shared__ int32_t s_zone;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int bi = tid & 15, bj = tid >> 4;
  for (;;) {
    if (tid == 0) s_zone = atomicAdd(work, 1);
    __syncthreads();
    const int32_t zl = s_zone;
    if (zl >= nzc) break;
    if (nobs[zl] == 0) {
      __syncthreads();
      continue;
    }
    float* Gz = GT + (int64_t)zl * N * N;
    float* ax = aux + (int64_t)zl * aux_stride32(N);
    float A[4][4];
    float amax = 0.f;
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
      for (int b = 0; b < 4; b++) {
        const int r = bi + 16 * a, c = bj + 16 * b;
        const float gval = (r < N && c < N) ? Gz[r * N + c] : 0.f;
        A[a][b] = gval;
        amax = fmaxf(amax, fabsf(gval));
      }
    for (int o = 16; o > 0; o >>= 1) amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    if ((tid & 31) == 0) red[warp] = amax;
    __syncthreads();
    float scale = 0.f;
#pragma unroll
    for (int w = 0; w < kT / 32; w++) scale = fmaxf(scale, red[w]);
    if (!(scale > 0.f) || isinf(scale)) scale = 1.f;
    const float iscale = 1.f / scale;
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
      for (int b = 0; b < 4; b++) A[a][b] *= iscale;
    if (tid == 0) ax[5 * N] = scale;
    __syncthreads();  // red reused below; the slot is overwritten by reflectors from here on
    const int ksteps = N - 2;
#pragma unroll 1
    for (int k = 0; k < ksteps && k < 16; k++)
      tridiag_step<0>(k, N, A, vbuf, pbuf, red, s_beta, Gz, ax, tid, bi, bj, warp);
#pragma unroll 1
    for (int k = 16; k < ksteps && k < 32; k++)
      tridiag_step<1>(k, N, A, vbuf, pbuf, red, s_beta, Gz, ax, tid, bi, bj, warp);
#pragma unroll 1
    for (int k = 32; k < ksteps && k < 48; k++)
      tridiag_step<2>(k, N, A, vbuf, pbuf, red, s_beta, Gz, ax, tid, bi, bj, warp);
#pragma unroll 1
    for (int k = 48; k < ksteps; k++)
      tridiag_step<3>(k, N, A, vbuf, pbuf, red, s_beta, Gz, ax, tid, bi, bj, warp);
    // trailing 2 x 2 block
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
      for (int b = 0; b < 4; b++) {
        const int r = bi + 16 * a, c = bj + 16 * b;
        if (c == N - 2 && r == N - 2) ax[N - 2] = A[a][b];
        if (c == N - 2 && r == N - 1) ax[N + N - 2] = A[a][b];
        if (c == N - 1 && r == N - 1) ax[N - 1] = A[a][b];
      }
    if (tid == 0) {
      ax[N + N - 1] = 0.f;
      ax[2 * N + N - 2] = 0.f;
      ax[2 * N + N - 1] = 0.f;
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------------------------ E3
__device__ __forceinline__ float dot16(const float (&x)[16], const float* p) {
  const float4* p4 = reinterpret_cast<const float4*>(p);
  float s[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
  for (int m = 0; m < 4; m++) {
    const float4 v = p4[m];
    s[m] = fmaf(x[4 * m + 0], v.x, s[m]);
    s[m] = fmaf(x[4 * m + 1], v.y, s[m]);
    s[m] = fmaf(x[4 * m + 2], v.z, s[m]);
    s[m] = fmaf(x[4 * m + 3], v.w, s[m]);
  }
  return (s[0] + s[1]) + (s[2] + s[3]);
}

__device__ __forceinline__ void axpy16(float (&x)[16], float f, const float* p) {
  const float4* p4 = reinterpret_cast<const float4*>(p);
#pragma unroll
  for (int m = 0; m < 4; m++) {
    const float4 v = p4[m];
    x[4 * m + 0] = fmaf(-f, v.x, x[4 * m + 0]);
    x[4 * m + 1] = fmaf(-f, v.y, x[4 * m + 1]);
    x[4 * m + 2] = fmaf(-f, v.z, x[4 * m + 2]);
    x[4 * m + 3] = fmaf(-f, v.w, x[4 * m + 3]);
  }
}

__device__ __forceinline__ void store16(const float (&x)[16], float* p) {
  float4* p4 = reinterpret_cast<float4*>(p);
#pragma unroll
  for (int m = 0; m < 4; m++)
    p4[m] = make_float4(x[4 * m + 0], x[4 * m + 1], x[4 * m + 2], x[4 * m + 3]);
}

__device__ __forceinline__ void load16(float (&x)[16], const float* p) {
  const float4* p4 = reinterpret_cast<const float4*>(p);
#pragma unroll
  for (int m = 0; m < 4; m++) {
    const float4 v = p4[m];
    x[4 * m + 0] = v.x;
    x[4 * m + 1] = v.y;
    x[4 * m + 2] = v.z;
    x[4 * m + 3] = v.w;
  }
}

constexpr size_t kSmem3 = (size_t)(2 * NB * LDV + 12 * NB) * sizeof(float);

__global__ void __launch_bounds__(kT, 4)
    k_eig_transform32(int N, int32_t nzc, float* __restrict__ GT, const float* __restrict__ aux,
                      const float* __restrict__ Zg, const float* __restrict__ gv,
                      const int32_t* __restrict__ nobs, int rotate, float* __restrict__ ampl_out,
                      int32_t* __restrict__ status, int32_t* __restrict__ work) {
  extern __shared__ __align__(16) float sm[];
  float* Vs = sm;               // [NB][LDV] reflectors, vector-major, zero padded
  float* Us = Vs + NB * LDV;    // [NB][LDV] eigenvectors (vector-major), later Q-scaled
  float* lam = Us + NB * LDV;   // [NB] 1/(1+lambda)            (evaluated in FP64)
  float* sq = lam + NB;         // [NB] (1+lambda)^-1/2         (evaluated in FP64)
  float* qs = sq + NB;          // [NB] (1+lambda)^-1/4         (evaluated in FP64)
  float* gs = qs + NB;          // [NB] g
  float* bet = gs + NB;         // [NB] Householder scalars
  float* tt = bet + NB;         // [NB] lambda' .* (U^T g)
  float* cc = tt + NB;          // [NB] colsum(U) / sqrt(lambda')
  float* vv = cc + NB;          // [NB] v (unnormalised)
  float* t0 = vv + NB;          // [NB] scratch
  int* flag = reinterpret_cast<int*>(t0 + NB);  // [NB] 1 accepted, 0 collapsed
  __shared__ float red[kT / 32];
  __shared__ int32_t s_zone;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int j = tid >> 2, q = tid & 3;  // eigenvector j, components 16q .. 16q + 15
  for (;;) {
    if (tid == 0) s_zone = atomicAdd(work, 1);
    __syncthreads();
    const int32_t zl = s_zone;
    if (zl >= nzc) break;
    if (nobs[zl] == 0) {
      __syncthreads();
      continue;
    }
    float* Gz = GT + (int64_t)zl * N * N;
    const float* ax = aux + (int64_t)zl * aux_stride32(N);
    for (int idx = tid; idx < NB * NB; idx += kT) {
      const int k = idx >> 6, r = idx & (NB - 1);
      Vs[k * LDV + r] = (k < N - 2 && r < N) ? Gz[k * N + r] : 0.f;
    }
    if (tid < NB) {
      const int i = tid;
      double l = (i < N) ? (double)ax[3 * N + i] : 0.0;
      if (l < 0.0) l = 0.0;
      const double li = 1.0 / (1.0 + l);
      const double s = sqrt(li);
      lam[i] = (float)li;
      sq[i] = (float)s;
      qs[i] = (float)sqrt(s);
      gs[i] = (i < N) ? gv[(int64_t)zl * N + i] : 0.f;
      bet[i] = (i < N - 2) ? ax[2 * N + i] : 0.f;
      flag[i] = 1;
    }
    float x[16];
    {
      const float* zj = Zg + (int64_t)zl * N * N + (int64_t)j * N;
#pragma unroll
      for (int i = 0; i < 16; i++) {
        const int r = 16 * q + i;
        x[i] = (j < N) ? ((r < N) ? zj[r] : 0.f) : ((r == j) ? 1.f : 0.f);
      }
    }
    __syncthreads();
    // back-transform: U = H_0 H_1 ... H_{N-3} Z, applied right to left
    for (int k = N - 3; k >= 0; k--) {
      const float bk = bet[k];
      if (bk == 0.f) continue;  // uniform
      const float* vk = Vs + k * LDV + 16 * q;
      const float s = qsum4(dot16(x, vk));
      axpy16(x, bk * s, vk);
    }
    // modified Gram-Schmidt, two sweeps, largest eigenvalue first
    for (int sweep = 0; sweep < 2; sweep++) {
      for (int c = N - 1; c >= 0; c--) {
        if (j == c) {
          float s = 0.f;
#pragma unroll
          for (int i = 0; i < 16; i++) s = fmaf(x[i], x[i], s);
          s = qsum4(s);
          const bool ok = flag[c] && (s >= 0.5f);
          const float sc = ok ? rsqrtf(s) : 0.f;
#pragma unroll
          for (int i = 0; i < 16; i++) x[i] *= sc;
          store16(x, Us + c * LDV + 16 * q);
          if (q == 0 && !ok) flag[c] = 0;
        }
        __syncthreads();
        if (j < c && flag[c]) {
          const float* uc = Us + c * LDV + 16 * q;
          const float d = qsum4(dot16(x, uc));
          axpy16(x, d, uc);
        }
      }
    }
    int ncol = 0;
    for (int i = tid; i < N; i += kT) ncol += (flag[i] == 0);
    ncol = __syncthreads_or(ncol);
    if (ncol) {
      // complement fill (rare): a collapsed vector is replaced by a pseudo-random vector made
      // orthogonal (two classical Gram-Schmidt passes) to every accepted eigenvector
      for (int c = 0; c < N; c++) {
        if (flag[c]) continue;  // uniform
        for (int r = tid; r < NB; r += kT) {
          unsigned h = (unsigned)r * 2246822519u ^ ((unsigned)c * 3266489917u + 0x27d4eb2fu);
          h ^= h >> 15;
          h *= 2654435761u;
          h ^= h >> 13;
          Us[c * LDV + r] = (r < N) ? (float)((double)(h & 0xffffff) * (1.0 / 16777216.0) - 0.5)
                                    : 0.f;
        }
        __syncthreads();
        for (int pass = 0; pass < 2; pass++) {
          for (int k = tid; k < N; k += kT) {
            float s = 0.f;
            if (k != c && flag[k])
              for (int r = 0; r < N; r++) s = fmaf(Us[k * LDV + r], Us[c * LDV + r], s);
            t0[k] = s;
          }
          __syncthreads();
          for (int r = tid; r < N; r += kT) {
            float s = Us[c * LDV + r];
            for (int k = 0; k < N; k++) s = fmaf(-t0[k], Us[k * LDV + r], s);
            Us[c * LDV + r] = s;
          }
          __syncthreads();
        }
        if (warp == 0) {
          float s = 0.f;
          for (int r = lane; r < N; r += 32) s = fmaf(Us[c * LDV + r], Us[c * LDV + r], s);
          for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
          if (lane == 0) {
            red[0] = (s > 0.f) ? rsqrtf(s) : 0.f;
            flag[c] = 1;
          }
        }
        __syncthreads();
        const float sc = red[0];
        for (int r = tid; r < NB; r += kT) Us[c * LDV + r] *= sc;
        __syncthreads();
      }
      if (j < N) load16(x, Us + j * LDV + 16 * q);
    }
    // per-vector scalars: lambda' (u_j . g) and colsum(u_j) / sqrt(lambda')
    {
      float y = dot16(x, gs + 16 * q);
      float cs = 0.f;
#pragma unroll
      for (int i = 0; i < 16; i++) cs += x[i];
      y = qsum4(y);
      cs = qsum4(cs);
      if (q == 0) {
        tt[j] = (j < N) ? lam[j] * y : 0.f;
        cc[j] = (j < N) ? cs / sq[j] : 0.f;
      }
    }
    __syncthreads();
    // ampl = U tt, v = U cc (one thread per component)
    int nan_flag = 0;
    if (tid < NB) {
      const int r = tid;
      float s = 0.f;
      for (int jj = 0; jj < N; jj++) s = fmaf(Us[jj * LDV + r], tt[jj], s);
      if (r < N) {
        ampl_out[(int64_t)zl * N + r] = s;
        if (!(s == s) || isinf(s)) nan_flag = 1;
      }
    } else if (tid < 2 * NB && rotate) {
      const int r = tid - NB;
      float s = 0.f;
      for (int jj = 0; jj < N; jj++) s = fmaf(Us[jj * LDV + r], cc[jj], s);
      vv[r] = (r < N) ? s : 0.f;
    }
    nan_flag = __syncthreads_or(nan_flag);
    // W = U Q into Us (every vector, the padding ones included)
    {
      const float qj = qs[j];
#pragma unroll
      for (int i = 0; i < 16; i++) x[i] *= qj;
      store16(x, Us + j * LDV + 16 * q);
    }
    if (rotate && warp == 0) {
      float s = 0.f;
      for (int r = lane; r < N; r += 32) s = fmaf(vv[r], vv[r], s);
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) red[0] = 1.f / sqrtf(s);
    }
    __syncthreads();
    // T_sym = W W^T, rows 4ab .. 4ab+3, columns 4bb .. 4bb+3 per thread
    const int ab = tid >> 4, bb = tid & 15;
    float T[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int c = 0; c < 4; c++) T[i][c] = 0.f;
#pragma unroll 4
    for (int jj = 0; jj < N; jj++) {
      const float4 wa = *reinterpret_cast<const float4*>(Us + jj * LDV + 4 * ab);
      const float4 wb = *reinterpret_cast<const float4*>(Us + jj * LDV + 4 * bb);
      const float ra[4] = {wa.x, wa.y, wa.z, wa.w};
      const float rb[4] = {wb.x, wb.y, wb.z, wb.w};
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int c = 0; c < 4; c++) T[i][c] = fmaf(ra[i], rb[c], T[i][c]);
    }
    if (rotate) {
      // Omega = P_v P_w + (1 - s_v s_w) v w^T with P_x = I - u_x u_x^T / (1 + |x_N|),
      // u_x = x + sign(x_N) e_N, w = 1/sqrt(N) (s_w = +1)
      const float inv = red[0];
      const float vN = vv[N - 1] * inv;
      const float sv = signbit(vN) ? -1.f : 1.f;
      const float icv = 1.f / (1.f + fabsf(vN));
      const float wv = (float)(1.0 / sqrt((double)N));
      const float icw = 1.f / (1.f + wv);
      float uv[4], vn[4], uw[4];
#pragma unroll
      for (int c = 0; c < 4; c++) {
        const int col = 4 * bb + c;
        const bool in = col < N;
        vn[c] = in ? vv[col] * inv : 0.f;
        uv[c] = vn[c] + ((col == N - 1) ? sv : 0.f);
        uw[c] = in ? wv + ((col == N - 1) ? 1.f : 0.f) : 0.f;
      }
      float pa[4], pb[4], pg[4];
#pragma unroll
      for (int i = 0; i < 4; i++) {
        float sa = 0.f, sb = 0.f;
#pragma unroll
        for (int c = 0; c < 4; c++) {
          sa = fmaf(T[i][c], uv[c], sa);
          sb = fmaf(T[i][c], vn[c], sb);
        }
        pa[i] = hsum16(sa);  // (T_sym u_v)_row
        pb[i] = hsum16(sb);  // (T_sym v)_row
      }
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int c = 0; c < 4; c++) T[i][c] = fmaf(-pa[i] * icv, uv[c], T[i][c]);
#pragma unroll
      for (int i = 0; i < 4; i++) {
        float s = 0.f;
#pragma unroll
        for (int c = 0; c < 4; c++) s = fmaf(T[i][c], uw[c], s);
        pg[i] = hsum16(s) * icw;
      }
      const float extra = 1.f - sv;
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int c = 0; c < 4; c++) {
          float t = fmaf(-pg[i], uw[c], T[i][c]);
          if (extra != 0.f && 4 * bb + c < N) t = fmaf(extra * pb[i], wv, t);
          T[i][c] = t;
        }
    }
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const int row = 4 * ab + i;
      if (row >= N) continue;
      if (N == NB) {
        *reinterpret_cast<float4*>(Gz + row * N + 4 * bb) =
            make_float4(T[i][0], T[i][1], T[i][2], T[i][3]);
      } else {
#pragma unroll
        for (int c = 0; c < 4; c++)
          if (4 * bb + c < N) Gz[row * N + 4 * bb + c] = T[i][c];
      }
    }
    if (tid == 0 && nan_flag) status[zl] |= ZST_NAN;
    __syncthreads();
  }
}

// ------------------------------------------------------------------------------------ E2a
// One thread per zone: eigenvalues of Tri by implicit symmetric QR sweeps with Wilkinson shift
// (the arithmetic of the generic E2a in zone_eig.cu), with d and e in shared memory and the
// chase's running values in registers; ascending sort; inverse-iteration shifts.
constexpr int kT2 = 64;

__global__ void __launch_bounds__(kT2)
    k_eig_values32(int N, int32_t nzc, float* __restrict__ aux, const int32_t* __restrict__ nobs,
                   int32_t* __restrict__ status) {
  __shared__ float sd[NB * kT2], se[NB * kT2];  // element i of thread t at [i * kT2 + t]
  const int t = threadIdx.x;
  const int32_t zl = blockIdx.x * kT2 + t;
  if (zl >= nzc || nobs[zl] == 0) return;  // no barrier below
  const float eps = 5.9604645e-8f;
  float* ax = aux + (int64_t)zl * aux_stride32(N);
  float* d = sd + t;
  float* e = se + t;
  float onenrm = 0.f;
  for (int i = 0; i < N; i++) {
    d[i * kT2] = ax[i];
    e[i * kT2] = (i < N - 1) ? ax[N + i] : 0.f;
  }
  for (int i = 0; i < N; i++) {
    const float sabs = fabsf(d[i * kT2]) + fabsf(e[i * kT2]) + (i > 0 ? fabsf(e[(i - 1) * kT2]) : 0.f);
    onenrm = fmaxf(onenrm, sabs);
  }
  const float scale = ax[5 * N];
  const float abs_tol = eps * onenrm;
  int st = 0, hi = N - 1, sweeps = 0;
  const int max_sweeps = 30 * N;
  while (hi > 0) {
    while (hi > 0) {
      const float tt = fabsf(e[(hi - 1) * kT2]);
      if (tt <= eps * (fabsf(d[(hi - 1) * kT2]) + fabsf(d[hi * kT2])) || tt <= abs_tol) {
        e[(hi - 1) * kT2] = 0.f;
        hi--;
      } else {
        break;
      }
    }
    if (hi == 0) break;
    int lo = hi - 1;
    while (lo > 0) {
      const float tt = fabsf(e[(lo - 1) * kT2]);
      if (tt <= eps * (fabsf(d[(lo - 1) * kT2]) + fabsf(d[lo * kT2])) || tt <= abs_tol) {
        e[(lo - 1) * kT2] = 0.f;
        break;
      }
      lo--;
    }
    if (++sweeps > max_sweeps) {
      st |= ZST_EIG;
      break;
    }
    const float a = d[(hi - 1) * kT2], b = d[hi * kT2], f = e[(hi - 1) * kT2];
    const float del = 0.5f * (a - b);
    const float den = del + copysignf(sqrtf(del * del + f * f), del == 0.f ? 1.f : del);
    const float mu = (den == 0.f) ? b : b - f * f / den;
    float dk = d[lo * kT2], ek = e[lo * kT2], ep = 0.f;  // d[k], e[k], e[k-1] (running)
    float x = dk - mu, z = ek, bulge = 0.f;
    for (int k = lo; k < hi; k++) {
      const float dk1 = d[(k + 1) * kT2];
      const float ek1 = (k + 1 < hi) ? e[(k + 1) * kT2] : 0.f;
      if (k > lo) {
        x = ep;
        z = bulge;
      }
      const float r2 = x * x + z * z;
      float c = 1.f, s = 0.f, r = 0.f;
      if (r2 > 0.f) {
        const float ri = rsqrtf(r2);
        c = x * ri;
        s = z * ri;
        r = r2 * ri;
      }
      if (k > lo) e[(k - 1) * kT2] = r;
      const float cc = c * c, ss = s * s, cs = c * s;
      d[k * kT2] = cc * dk + 2.f * cs * ek + ss * dk1;
      const float nd1 = ss * dk - 2.f * cs * ek + cc * dk1;
      ep = cs * (dk1 - dk) + (cc - ss) * ek;
      dk = nd1;
      ek = c * ek1;
      bulge = s * ek1;
    }
    d[hi * kT2] = dk;
    e[(hi - 1) * kT2] = ep;
  }
  for (int i = 1; i < N; i++) {  // ascending (insertion sort)
    const float v = d[i * kT2];
    int k = i - 1;
    while (k >= 0 && d[k * kT2] > v) {
      d[(k + 1) * kT2] = d[k * kT2];
      k--;
    }
    d[(k + 1) * kT2] = v;
  }
  float prev = 0.f;
  for (int j = 0; j < N; j++) {
    const float v = d[j * kT2];
    ax[3 * N + j] = v * scale;
    float sh = v;
    if (j > 0) {
      const float pert = 10.f * eps * fabsf(sh);
      if (sh - prev < pert) sh = prev + pert;
    }
    ax[4 * N + j] = sh;
    prev = sh;
  }
  ax[5 * N + 1] = onenrm;
  if (st) status[zl] |= st;
}

// ------------------------------------------------------------------------------------ E2b
// One block of 64 threads per zone, thread j = eigenpair j: inverse iteration on Tri - shift_j I
// (two solves from a fixed pseudo-random start, as the generic E2b). The partial-pivoting LU
// is recomputed in each forward sweep (fused with the elimination), its upper factor kept in
// shared memory; the iterate lives in registers (loops unrolled to 64).
__global__ void __launch_bounds__(kT2)
    k_eig_vectors32(int N, int32_t nzc, const float* __restrict__ aux, float* __restrict__ Zg,
                    const int32_t* __restrict__ nobs) {
  __shared__ float sfac[3 * NB * kT2];  // upper factor u1, u2, 1/diag: [i][j] each
  __shared__ float sd[NB], se[NB];
  float* su1 = sfac;
  float* su2 = sfac + NB * kT2;
  float* sui = sfac + 2 * NB * kT2;
  const int j = threadIdx.x;
  const int32_t zl = blockIdx.x;
  if (zl >= nzc || nobs[zl] == 0) return;  // block-uniform
  const float* ax = aux + (int64_t)zl * aux_stride32(N);
  if (j < N) {
    sd[j] = ax[j];
    se[j] = (j < N - 1) ? ax[N + j] : 0.f;
  }
  __syncthreads();
  const float onenrm = ax[5 * N + 1];
  float* Zz = Zg + (int64_t)zl * N * N;
  float* tr = sfac;  // [i][NB + 1] transpose staging, used at the end
  float x[NB];
#pragma unroll
  for (int i = 0; i < NB; i++) x[i] = 0.f;
  if (!(onenrm > 1e4f * 1e-36f)) {  // Tri = 0: every vector is an eigenvector
#pragma unroll
    for (int i = 0; i < NB; i++) x[i] = (i == j) ? 1.f : 0.f;
  } else if (j < N) {
    const float l = ax[4 * N + j];
    const float tiny = 5.9604645e-8f * onenrm;
#pragma unroll
    for (int i = 0; i < NB; i++) {
      unsigned h = (unsigned)i * 2654435761u ^ ((unsigned)j * 40503u + 0x9e3779b9u);
      h ^= h >> 15;
      h *= 2246822519u;
      h ^= h >> 13;
      x[i] = (i < N) ? (float)(h & 0xffffff) * (1.f / 16777216.f) - 0.5f : 0.f;
    }
#pragma unroll 1
    for (int it = 0; it < 2; it++) {
      float cd = sd[0] - l, csup = (N > 1) ? se[0] : 0.f;
#pragma unroll
      for (int i = 0; i < NB - 1; i++) {
        if (i < N - 1) {
          const float sub = se[i], dg = sd[i + 1] - l, sp = (i + 1 < N - 1) ? se[i + 1] : 0.f;
          const bool swap = fabsf(cd) < fabsf(sub);
          float pivot = swap ? sub : cd;
          if (!swap && fabsf(pivot) < tiny) pivot = copysignf(tiny, pivot);
          const float ui = 1.f / pivot;
          const float li = (swap ? cd : sub) * ui;
          if (it == 0) {
            su1[i * kT2 + j] = swap ? dg : csup;
            su2[i * kT2 + j] = swap ? sp : 0.f;
            sui[i * kT2 + j] = ui;
          }
          const float aa = swap ? csup : dg, bb = swap ? dg : csup;
          cd = fmaf(-li, bb, aa);
          csup = swap ? -li * sp : sp;
          const float xi = swap ? x[i + 1] : x[i], xn = swap ? x[i] : x[i + 1];
          x[i] = xi;
          x[i + 1] = fmaf(-li, xi, xn);
        }
      }
      if (it == 0) {
        float pivot = cd;
        if (fabsf(pivot) < tiny) pivot = copysignf(tiny, pivot);
        sui[(N - 1) * kT2 + j] = 1.f / pivot;
        su1[(N - 1) * kT2 + j] = 0.f;
        su2[(N - 1) * kT2 + j] = 0.f;
        if (N >= 2) su2[(N - 2) * kT2 + j] = 0.f;
      }
      // back substitution with the upper factor (diagonal + two super-diagonals)
#pragma unroll
      for (int i = NB - 1; i >= 0; i--) {
        if (i < N) {
          float v = x[i];
          if (i + 1 < NB) v = fmaf(-su1[i * kT2 + j], x[i + 1], v);
          if (i + 2 < NB) v = fmaf(-su2[i * kT2 + j], x[i + 2], v);
          x[i] = v * sui[i * kT2 + j];
        }
      }
      float mx = 0.f;
#pragma unroll
      for (int i = 0; i < NB; i++) mx = fmaxf(mx, fabsf(x[i]));
      const float im = 1.f / mx;
      float nrm = 0.f;
#pragma unroll
      for (int i = 0; i < NB; i++) {
        x[i] *= im;
        nrm = fmaf(x[i], x[i], nrm);
      }
      const float sc = rsqrtf(nrm);
#pragma unroll
      for (int i = 0; i < NB; i++) x[i] *= sc;
    }
  }
  __syncthreads();  // factors no longer read: reuse su1/su2 as the transpose buffer
#pragma unroll
  for (int i = 0; i < NB; i++) tr[i * (NB + 1) + j] = x[i];
  __syncthreads();
  for (int idx = j; idx < N * N; idx += kT2) {
    const int jj = idx / N, i = idx - jj * N;
    Zz[idx] = tr[i * (NB + 1) + jj];
  }
}

int grid32(const void* fn, size_t smem, int32_t nzc) {
  int bps = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, fn, kT, smem);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int grid = sms * (bps > 0 ? bps : 1);
  if (grid > nzc) grid = nzc > 0 ? nzc : 1;
  return grid;
}

}  // namespace

int eig32_max_n() { return NB; }

cudaError_t eig32_values(int N, int32_t nzc, float* d_aux, const int32_t* d_nobs,
                         int32_t* d_status, cudaStream_t st) {
  if (N < 2 || N > NB) return cudaErrorInvalidValue;
  k_eig_values32<<<(nzc + kT2 - 1) / kT2, kT2, 0, st>>>(N, nzc, d_aux, d_nobs, d_status);
  return cudaGetLastError();
}

cudaError_t eig32_vectors(int N, int32_t nzc, const float* d_aux, float* d_Z,
                          const int32_t* d_nobs, cudaStream_t st) {
  if (N < 2 || N > NB) return cudaErrorInvalidValue;
  k_eig_vectors32<<<nzc > 0 ? nzc : 1, kT2, 0, st>>>(N, nzc, d_aux, d_Z, d_nobs);
  return cudaGetLastError();
}

cudaError_t eig32_tridiag(int N, int32_t nzc, float* d_GT, float* d_aux, const int32_t* d_nobs,
                          int32_t* d_work, cudaStream_t st) {
  if (N < 2 || N > NB) return cudaErrorInvalidValue;
  k_eig_tridiag32<<<grid32((const void*)k_eig_tridiag32, 0, nzc), kT, 0, st>>>(N, nzc, d_GT,
                                                                               d_aux, d_nobs,
                                                                               d_work);
  return cudaGetLastError();
}

cudaError_t eig32_transform(int N, int32_t nzc, float* d_GT, const float* d_aux,
                            const float* d_Z, const float* d_g, const int32_t* d_nobs, int rotate,
                            float* d_ampl, int32_t* d_status, int32_t* d_work, cudaStream_t st) {
  if (N < 2 || N > NB) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(k_eig_transform32,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem3);
  if (e != cudaSuccess) return e;
  k_eig_transform32<<<grid32((const void*)k_eig_transform32, kSmem3, nzc), kT, kSmem3, st>>>(
      N, nzc, d_GT, d_aux, d_Z, d_g, d_nobs, rotate, d_ampl, d_status, d_work);
  return cudaGetLastError();
}

}  // namespace oakg
