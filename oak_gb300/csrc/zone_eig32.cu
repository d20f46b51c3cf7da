// Mixed-precision eigensolve kernels for ensembles of up to 64 members, in FP32: E1
// (Householder tridiagonalisation), E2a (tridiagonal eigenvalues), E2b (inverse iteration) and
// E3 (back-transform, orthogonalisation, amplitudes and the square-root transform). They replace
// the generic FP32 kernels of zone_eig.cu for these sizes.
//
// The arithmetic follows rrsqrt.F90:136-185 as the generic kernels do (the comment block at the
// top of zone_eig.cu lists the reference lines); the matrix is padded to 64 x 64 with zeros,
// which adds decoupled zero rows that no output reads.
//
// The stages keep rows (E1: two per lane, one warp per zone) or eigenvectors (E2b, E3: one per
// thread, 64 threads per zone) of 64 elements in registers, so matrix-vector products need no
// cross-thread reductions: the shared operand is broadcast with 128-bit shared loads.
//
// E1: one warp per zone, lane t holding rows t and t + 32 of the scaled symmetric matrix. Row
//   k equals column k, so the lane holding row k forms reflector k; p = beta A v is a register
//   dot per row; w = p - kc v is formed once per row and shared; warp-level synchronisation.
//   Reflector k is stored vector-major, zero padded, in row k of the zone's matrix slot:
//   slot[k*N + r] = v_k[r] (v_k[r] = 0 for r <= k).
// E2a: one thread per zone, implicit QR sweeps (working arrays in shared memory).
// E2b: thread j = eigenpair j, inverse iteration (LU factor in shared memory).
// E3: thread j holds eigenvector j.
//   back-transform U = H_0 ... H_{N-3} Z: per reflector a register dot and axpy, no barrier;
//   orthogonalisation: right-looking modified Gram-Schmidt, largest eigenvalue first (a vector
//     is final when every larger-eigenvalue vector has been projected out of it); a vector that
//     keeps at least half its squared norm is accepted after this one projection (Kahan-Parlett
//     "twice is enough"), one that does not is marked collapsed and replaced by a
//     pseudo-random vector orthogonalised (two passes) against every accepted one;
//   T_sym = (U Q)(U Q)^T with Q = diag((1+lambda)^-1/4): 4 x 16 register blocks, 128-bit
//     shared loads; Omega = RotateVector(w, v) applied to the register blocks in its
//     reflector form (rank-one updates, matoper.F90:509-535).
#include <cuda_runtime.h>
#include <math.h>

#include "oakg_internal.cuh"

namespace oakg {

namespace {

constexpr int NB = 64;        // padded ensemble size
constexpr int LDV = NB + 4;   // row stride of vector-major shared matrices (16-byte rows,
                              // 8 consecutive rows fall in 8 different 16-byte bank groups)

__host__ __device__ inline int aux_stride32(int N) { return 5 * N + 2; }

__device__ __forceinline__ void vload(float (&x)[NB], const float* p) {
#pragma unroll
  for (int c = 0; c < NB; c += 4) {
    const float4 v = *reinterpret_cast<const float4*>(p + c);
    x[c] = v.x;
    x[c + 1] = v.y;
    x[c + 2] = v.z;
    x[c + 3] = v.w;
  }
}

__device__ __forceinline__ void vstore(const float (&x)[NB], float* p) {
#pragma unroll
  for (int c = 0; c < NB; c += 4)
    *reinterpret_cast<float4*>(p + c) = make_float4(x[c], x[c + 1], x[c + 2], x[c + 3]);
}

// ------------------------------------------------------------------------------------ E1
// One warp per zone (kZpb zones per block). Lane t holds rows t and t + 32 of the scaled
// symmetric matrix in registers (a0[c] = A[t][c], a1[c] = A[t+32][c]). Row k equals column k,
// so the lane holding row k forms reflector k; p = beta A v is a register dot per row; every
// synchronisation is warp-level. Columns at or left of k are not read after step k, so
// 16-column groups lying entirely there are skipped, and the first row set is skipped once all
// its rows are final (k >= 31).
constexpr int kZpb = 4;

template <int SLOT>
__device__ __forceinline__ void owner_reflector(const float (&row)[NB], int k, int N, float* vbuf,
                                                float* ax, float* beta_slot) {
  // single entries are read back through shared memory: an equality-selected register
  // element would become a dynamic index and move the row to local memory
  vstore(row, vbuf);
  const float x0 = vbuf[k + 1], dk = vbuf[k];
  float sig = 0.f;
#pragma unroll
  for (int c = 0; c < NB; c++)
    if (c > k + 1) sig = fmaf(row[c], row[c], sig);
  const float mu = sqrtf(fmaf(x0, x0, sig));
  const float v0 = (x0 <= 0.f) ? x0 - mu : x0 + mu;
  const float vv = fmaf(v0, v0, sig);
  const bool skip = (sig == 0.f) || !(vv > 0.f) || isinf(vv);
  const float bk = skip ? 0.f : 2.f / vv;
#pragma unroll
  for (int c = 0; c < NB; c += 4) {
    float4 q4;
    q4.x = (c + 0 > k + 1) ? row[c + 0] : 0.f;
    q4.y = (c + 1 > k + 1) ? row[c + 1] : 0.f;
    q4.z = (c + 2 > k + 1) ? row[c + 2] : 0.f;
    q4.w = (c + 3 > k + 1) ? row[c + 3] : 0.f;
    *reinterpret_cast<float4*>(vbuf + c) = q4;
  }
  vbuf[k + 1] = skip ? x0 : v0;
  ax[k] = dk;                                        // d_k
  ax[N + k] = skip ? x0 : ((x0 <= 0.f) ? mu : -mu);  // e_k
  ax[2 * N + k] = bk;                                // beta_k
  *beta_slot = bk;
}

__global__ void __launch_bounds__(32 * kZpb, 3)
    k_eig_tridiag32(int N, int32_t nzc, float* __restrict__ GT, float* __restrict__ aux,
                    const int32_t* __restrict__ nobs) {
  __shared__ __align__(16) float vbuf_s[kZpb][NB];
  __shared__ __align__(16) float wbuf_s[kZpb][NB];
  __shared__ float beta_s[kZpb];
  const int lane = threadIdx.x & 31, wz = threadIdx.x >> 5;
  const int32_t zl = blockIdx.x * kZpb + wz;
  if (zl >= nzc || nobs[zl] == 0) return;  // warp-uniform; only warp-level synchronisation
  float* vbuf = vbuf_s[wz];
  float* wbuf = wbuf_s[wz];
  float* Gz = GT + (int64_t)zl * N * N;
  float* ax = aux + (int64_t)zl * aux_stride32(N);
  const int r0 = lane, r1 = lane + 32;
  float a0[NB], a1[NB];
#pragma unroll
  for (int c = 0; c < NB; c++) {
    a0[c] = (r0 < N && c < N) ? Gz[r0 * N + c] : 0.f;
    a1[c] = (r1 < N && c < N) ? Gz[r1 * N + c] : 0.f;
  }
  float amax = 0.f;
#pragma unroll
  for (int c = 0; c < NB; c++) amax = fmaxf(amax, fmaxf(fabsf(a0[c]), fabsf(a1[c])));
  for (int o = 16; o > 0; o >>= 1) amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
  float scale = amax;
  if (!(scale > 0.f) || isinf(scale)) scale = 1.f;
  const float iscale = 1.f / scale;
#pragma unroll
  for (int c = 0; c < NB; c++) {
    a0[c] *= iscale;
    a1[c] *= iscale;
  }
  if (lane == 0) ax[5 * N] = scale;
  __syncwarp();  // every row read before reflectors overwrite the slot
  for (int k = 0; k < N - 2; k++) {
    if (lane == (k & 31)) {
      if (k < 32)
        owner_reflector<0>(a0, k, N, vbuf, ax, &beta_s[wz]);
      else
        owner_reflector<1>(a1, k, N, vbuf, ax, &beta_s[wz]);
    }
    __syncwarp();  // v and beta published
    const float bk = beta_s[wz];
    const float v0r = vbuf[r0], v1r = vbuf[r1];
    if (r0 < N) Gz[(int64_t)k * N + r0] = v0r;  // reflector k, vector-major, zero padded
    if (r1 < N) Gz[(int64_t)k * N + r1] = v1r;
    if (bk != 0.f) {  // warp-uniform; beta = 0 is an identity reflector
      const bool act0 = (k < 31);  // rows 0..31 are all final once k >= 31
      float p00 = 0.f, p01 = 0.f, p10 = 0.f, p11 = 0.f;
#pragma unroll
      for (int g = 0; g < 4; g++) {
        if (16 * g + 15 > k) {  // v vanishes on columns <= k
#pragma unroll
          for (int m = 0; m < 4; m++) {
            const int c = 16 * g + 4 * m;
            const float4 v4 = *reinterpret_cast<const float4*>(vbuf + c);
            if (act0) {
              p00 = fmaf(a0[c + 0], v4.x, p00);
              p01 = fmaf(a0[c + 1], v4.y, p01);
              p00 = fmaf(a0[c + 2], v4.z, p00);
              p01 = fmaf(a0[c + 3], v4.w, p01);
            }
            p10 = fmaf(a1[c + 0], v4.x, p10);
            p11 = fmaf(a1[c + 1], v4.y, p11);
            p10 = fmaf(a1[c + 2], v4.z, p10);
            p11 = fmaf(a1[c + 3], v4.w, p11);
          }
        }
      }
      const float p0 = bk * (p00 + p01), p1 = bk * (p10 + p11);
      float pv = fmaf(p0, v0r, p1 * v1r);
      for (int o = 16; o > 0; o >>= 1) pv += __shfl_xor_sync(0xffffffffu, pv, o);
      const float kc = 0.5f * bk * pv;
      const float w0 = fmaf(-kc, v0r, p0), w1 = fmaf(-kc, v1r, p1);  // w = p - kc v
      wbuf[r0] = w0;
      wbuf[r1] = w1;
      __syncwarp();  // w published
      // A -= v w^T + w v^T
#pragma unroll
      for (int g = 0; g < 4; g++) {
        if (16 * g + 15 > k) {
#pragma unroll
          for (int m = 0; m < 4; m++) {
            const int c = 16 * g + 4 * m;
            const float4 v4 = *reinterpret_cast<const float4*>(vbuf + c);
            const float4 w4 = *reinterpret_cast<const float4*>(wbuf + c);
            const float vc[4] = {v4.x, v4.y, v4.z, v4.w};
            const float wc[4] = {w4.x, w4.y, w4.z, w4.w};
#pragma unroll
            for (int t = 0; t < 4; t++) {
              if (act0) a0[c + t] = fmaf(-v0r, wc[t], fmaf(-w0, vc[t], a0[c + t]));
              a1[c + t] = fmaf(-v1r, wc[t], fmaf(-w1, vc[t], a1[c + t]));
            }
          }
        }
      }
    }
    __syncwarp();  // v and w consumed before the next owner writes
  }
  // trailing 2 x 2 block: rows N-2 and N-1, read back through shared memory
  if (N >= 2) {
    if (lane == ((N - 2) & 31)) {
      if (N - 2 < 32) vstore(a0, vbuf); else vstore(a1, vbuf);
    }
    if (lane == ((N - 1) & 31)) {
      if (N - 1 < 32) vstore(a0, wbuf); else vstore(a1, wbuf);
    }
    __syncwarp();
    if (lane == 0) {
      ax[N - 2] = vbuf[N - 2];
      ax[2 * N + N - 2] = 0.f;
      ax[N + N - 2] = wbuf[N - 2];
      ax[N - 1] = wbuf[N - 1];
      ax[N + N - 1] = 0.f;
      ax[2 * N + N - 1] = 0.f;
    }
  }
}

// ------------------------------------------------------------------------------------ E3
// One block of 64 threads per zone; thread j holds eigenvector j (64 components) in
// registers. Shared matrices are vector-major with 16-byte rows.
constexpr int kT3 = 64;
constexpr size_t kSmem3 = (size_t)(2 * NB * LDV + 12 * NB) * sizeof(float);

// u . x over the 16-component groups g >= g0 (the others are zero in u)
__device__ __forceinline__ float vdot(const float (&x)[NB], const float* u, int g0) {
  float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
#pragma unroll
  for (int g = 0; g < 4; g++) {
    if (g >= g0) {
#pragma unroll
      for (int m = 0; m < 4; m++) {
        const int c = 16 * g + 4 * m;
        const float4 v = *reinterpret_cast<const float4*>(u + c);
        s0 = fmaf(x[c], v.x, s0);
        s1 = fmaf(x[c + 1], v.y, s1);
        s2 = fmaf(x[c + 2], v.z, s2);
        s3 = fmaf(x[c + 3], v.w, s3);
      }
    }
  }
  return (s0 + s1) + (s2 + s3);
}

// x -= f u over the groups g >= g0
__device__ __forceinline__ void vaxpy(float (&x)[NB], float f, const float* u, int g0) {
#pragma unroll
  for (int g = 0; g < 4; g++) {
    if (g >= g0) {
#pragma unroll
      for (int m = 0; m < 4; m++) {
        const int c = 16 * g + 4 * m;
        const float4 v = *reinterpret_cast<const float4*>(u + c);
        x[c] = fmaf(-f, v.x, x[c]);
        x[c + 1] = fmaf(-f, v.y, x[c + 1]);
        x[c + 2] = fmaf(-f, v.z, x[c + 2]);
        x[c + 3] = fmaf(-f, v.w, x[c + 3]);
      }
    }
  }
}

__device__ __forceinline__ float qsum4(float x) {  // the 4 lanes of one row of T blocks
  const unsigned m = 0xFu << (threadIdx.x & 28);
  x += __shfl_xor_sync(m, x, 1);
  x += __shfl_xor_sync(m, x, 2);
  return x;
}

__global__ void __launch_bounds__(kT3, 6)
    k_eig_transform32(int N, int32_t nzc, float* __restrict__ GT, const float* __restrict__ aux,
                      const float* __restrict__ Zg, const float* __restrict__ gv,
                      const int32_t* __restrict__ nobs, int rotate, float* __restrict__ ampl_out,
                      int32_t* __restrict__ status) {
  extern __shared__ __align__(16) float sm[];
  float* Vs = sm;               // [NB][LDV] reflectors (vector-major, zero padded)
  float* Us = Vs + NB * LDV;    // [NB][LDV] Z, eigenvectors, then W = U diag(lambda'^1/4)
  float* lam = Us + NB * LDV;   // [NB] 1/(1+lambda)            (evaluated in FP64)
  float* sq = lam + NB;         // [NB] (1+lambda)^-1/2         (evaluated in FP64)
  float* qs = sq + NB;          // [NB] (1+lambda)^-1/4         (evaluated in FP64)
  float* gs = qs + NB;          // [NB] g
  float* bet = gs + NB;         // [NB] Householder scalars
  float* tt = bet + NB;         // [NB] lambda' (u_j . g)
  float* cc = tt + NB;          // [NB] colsum(u_j) / sqrt(lambda')
  float* vv = cc + NB;          // [NB] v (unnormalised)
  float* t0 = vv + NB;          // [NB] scratch
  int* flag = reinterpret_cast<int*>(t0 + NB);  // [NB] 1 accepted, 0 collapsed
  __shared__ float red[2];
  const int j = threadIdx.x, lane = j & 31, warp = j >> 5;
  const int32_t zl = blockIdx.x;
  if (zl >= nzc || nobs[zl] == 0) return;  // block-uniform
  float* Gz = GT + (int64_t)zl * N * N;
  const float* ax = aux + (int64_t)zl * aux_stride32(N);
  const float* Zz = Zg + (int64_t)zl * N * N;
  if (N == NB) {
    // 16 float4 of each matrix per thread, all loads issued before the stores
    float4 vq[16], zq[16];
#pragma unroll
    for (int i = 0; i < 16; i++) {
      const int idx4 = j + kT3 * i;  // float4 index in the 64 x 64 matrix
      const int k = idx4 >> 4;
      vq[i] = (k < N - 2) ? reinterpret_cast<const float4*>(Gz)[idx4] : make_float4(0, 0, 0, 0);
      zq[i] = reinterpret_cast<const float4*>(Zz)[idx4];
    }
#pragma unroll
    for (int i = 0; i < 16; i++) {
      const int idx4 = j + kT3 * i;
      const int k = idx4 >> 4, c = (idx4 & 15) * 4;
      *reinterpret_cast<float4*>(Vs + k * LDV + c) = vq[i];
      *reinterpret_cast<float4*>(Us + k * LDV + c) = zq[i];
    }
  } else {
#pragma unroll 8
    for (int idx = j; idx < NB * NB; idx += kT3) {
      const int k = idx >> 6, c = idx & (NB - 1);
      Vs[k * LDV + c] = (k < N - 2 && c < N) ? Gz[k * N + c] : 0.f;
      Us[k * LDV + c] = (k < N) ? ((c < N) ? Zz[k * N + c] : 0.f) : ((c == k) ? 1.f : 0.f);
    }
  }
  {
    double l = (j < N) ? (double)ax[3 * N + j] : 0.0;
    if (l < 0.0) l = 0.0;
    const double li = 1.0 / (1.0 + l);
    const double s = sqrt(li);
    lam[j] = (float)li;
    sq[j] = (float)s;
    qs[j] = (float)sqrt(s);
    gs[j] = (j < N) ? gv[(int64_t)zl * N + j] : 0.f;
    bet[j] = (j < N - 2) ? ax[2 * N + j] : 0.f;
    flag[j] = 1;
  }
  __syncthreads();
  float x[NB];
  vload(x, Us + j * LDV);
  // back-transform U = H_0 H_1 ... H_{N-3} Z (reflector k vanishes on components <= k)
  for (int k = N - 3; k >= 0; k--) {
    const float bk = bet[k];
    if (bk == 0.f) continue;  // uniform
    const float* vk = Vs + k * LDV;
    const int g0 = (k + 1) >> 4;
    const float s = vdot(x, vk, g0);
    vaxpy(x, bk * s, vk, g0);
  }
  // modified Gram-Schmidt, largest eigenvalue first: vector c is final once every
  // larger-eigenvalue vector has been projected out of it. A vector that keeps at least half its
  // squared norm (a norm drop below sqrt(2)) is orthogonal to working precision after this one
  // projection ("twice is enough", Kahan-Parlett; Parlett, The Symmetric Eigenvalue Problem,
  // 6-9); one that does not is marked collapsed and replaced below.
  {
    for (int c = N - 1; c >= 0; c--) {
      if (j == c) {
        float s0 = 0.f, s1 = 0.f;
#pragma unroll
        for (int i = 0; i < NB; i += 2) {
          s0 = fmaf(x[i], x[i], s0);
          s1 = fmaf(x[i + 1], x[i + 1], s1);
        }
        const float s = s0 + s1;
        const bool ok = flag[c] && (s >= 0.5f);
        const float sc = ok ? rsqrtf(s) : 0.f;
#pragma unroll
        for (int i = 0; i < NB; i++) x[i] *= sc;
        vstore(x, Us + c * LDV);
        if (!ok) flag[c] = 0;
      }
      __syncthreads();
      if (j < c && flag[c]) {
        const float* uc = Us + c * LDV;
        const float d = vdot(x, uc, 0);
        vaxpy(x, d, uc, 0);
      }
    }
  }
  int ncol = 0;
  if (j < N) ncol = (flag[j] == 0);
  ncol = __syncthreads_or(ncol);
  if (ncol) {
    // complement fill (rare): a collapsed vector is replaced by a pseudo-random vector made
    // orthogonal (two classical Gram-Schmidt passes) to every accepted eigenvector
    for (int c = 0; c < N; c++) {
      if (flag[c]) continue;  // uniform
      {
        unsigned h = (unsigned)j * 2246822519u ^ ((unsigned)c * 3266489917u + 0x27d4eb2fu);
        h ^= h >> 15;
        h *= 2654435761u;
        h ^= h >> 13;
        Us[c * LDV + j] =
            (j < N) ? (float)((double)(h & 0xffffff) * (1.0 / 16777216.0) - 0.5) : 0.f;
      }
      __syncthreads();
      for (int pass = 0; pass < 2; pass++) {
        {
          float s = 0.f;
          if (j < N && j != c && flag[j])
            for (int i = 0; i < N; i++) s = fmaf(Us[j * LDV + i], Us[c * LDV + i], s);
          t0[j] = s;
        }
        __syncthreads();
        {
          float s = Us[c * LDV + j];
          for (int k = 0; k < N; k++) s = fmaf(-t0[k], Us[k * LDV + j], s);
          __syncthreads();
          Us[c * LDV + j] = s;
        }
        __syncthreads();
      }
      {
        const float u = Us[c * LDV + j];
        float s = u * u;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) red[warp] = s;
        __syncthreads();
        const float tot = red[0] + red[1];
        Us[c * LDV + j] = u * ((tot > 0.f) ? rsqrtf(tot) : 0.f);
        if (j == 0) flag[c] = 1;
        __syncthreads();
      }
    }
    vload(x, Us + j * LDV);
  }
  // per-vector scalars: lambda' (u_j . g), colsum(u_j) / sqrt(lambda')
  {
    const float y = vdot(x, gs, 0);
    float s0 = 0.f, s1 = 0.f;
#pragma unroll
    for (int i = 0; i < NB; i += 2) {
      s0 += x[i];
      s1 += x[i + 1];
    }
    tt[j] = (j < N) ? lam[j] * y : 0.f;
    cc[j] = (j < N) ? (s0 + s1) / sq[j] : 0.f;
  }
  __syncthreads();
  // ampl = U tt, v = U cc (thread j: component j)
  int nan_flag = 0;
  {
    float sa = 0.f, sv = 0.f;
    for (int jj = 0; jj < N; jj++) {
      const float u = Us[jj * LDV + j];
      sa = fmaf(u, tt[jj], sa);
      sv = fmaf(u, cc[jj], sv);
    }
    if (j < N) {
      ampl_out[(int64_t)zl * N + j] = sa;
      if (!(sa == sa) || isinf(sa)) nan_flag = 1;
    }
    vv[j] = (j < N) ? sv : 0.f;
  }
  nan_flag = __syncthreads_or(nan_flag);
  {
    const float qj = qs[j];
#pragma unroll
    for (int i = 0; i < NB; i++) x[i] *= qj;
    vstore(x, Us + j * LDV);  // W = U diag(qs); padding vectors stay unit vectors
    if (rotate) {
      float s = (j < N) ? vv[j] * vv[j] : 0.f;
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) red[warp] = s;
    }
  }
  __syncthreads();
  // T_sym = W W^T: thread (rb, cb) = (j / 4, j % 4) computes rows 4 rb .. 4 rb + 3 and the
  // columns of 16-byte chunks cb, cb + 4, cb + 8, cb + 12 (interleaved: conflict-free loads)
  const int rb = j >> 2, cb = j & 3;
  float T[4][16];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int c = 0; c < 16; c++) T[i][c] = 0.f;
#pragma unroll 2
  for (int jj = 0; jj < N; jj++) {
    const float* w = Us + jj * LDV;
    const float4 wa = *reinterpret_cast<const float4*>(w + 4 * rb);
    const float ra[4] = {wa.x, wa.y, wa.z, wa.w};
#pragma unroll
    for (int m = 0; m < 4; m++) {
      const float4 wb = *reinterpret_cast<const float4*>(w + 4 * (cb + 4 * m));
      const float rbv[4] = {wb.x, wb.y, wb.z, wb.w};
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int t = 0; t < 4; t++) T[i][4 * m + t] = fmaf(ra[i], rbv[t], T[i][4 * m + t]);
    }
  }
  if (rotate) {
    // Omega = P_v P_w + (1 - s_v s_w) v w^T with P_x = I - u_x u_x^T / (1 + |x_N|),
    // u_x = x + sign(x_N) e_N, w = 1/sqrt(N) (s_w = +1)  (matoper.F90:509-535)
    const float inv = 1.f / sqrtf(red[0] + red[1]);
    const float vN = vv[N - 1] * inv;
    const float sv = signbit(vN) ? -1.f : 1.f;
    const float icv = 1.f / (1.f + fabsf(vN));
    const float wv = (float)(1.0 / sqrt((double)N));
    const float icw = 1.f / (1.f + wv);
    float pa[4], pb[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
      float sa = 0.f, sb = 0.f;
#pragma unroll
      for (int m = 0; m < 4; m++)
#pragma unroll
        for (int t = 0; t < 4; t++) {
          const int col = 4 * (cb + 4 * m) + t;
          const float vn = (col < N) ? vv[col] * inv : 0.f;
          const float uv = vn + ((col == N - 1) ? sv : 0.f);
          sa = fmaf(T[i][4 * m + t], uv, sa);
          sb = fmaf(T[i][4 * m + t], vn, sb);
        }
      pa[i] = qsum4(sa) * icv;  // (T_sym u_v)_row / c_v
      pb[i] = qsum4(sb);        // (T_sym v)_row
    }
    const float extra = 1.f - sv;
#pragma unroll
    for (int i = 0; i < 4; i++) {
      float sg = 0.f;
#pragma unroll
      for (int m = 0; m < 4; m++)
#pragma unroll
        for (int t = 0; t < 4; t++) {
          const int col = 4 * (cb + 4 * m) + t;
          const float vn = (col < N) ? vv[col] * inv : 0.f;
          const float uv = vn + ((col == N - 1) ? sv : 0.f);
          const float uw = (col < N) ? wv + ((col == N - 1) ? 1.f : 0.f) : 0.f;
          const float t1 = fmaf(-pa[i], uv, T[i][4 * m + t]);  // T1 = T_sym - t0 u_v^T / c_v
          T[i][4 * m + t] = t1;
          sg = fmaf(t1, uw, sg);
        }
      const float g = qsum4(sg) * icw;  // (T1 u_w)_row / c_w
#pragma unroll
      for (int m = 0; m < 4; m++)
#pragma unroll
        for (int t = 0; t < 4; t++) {
          const int col = 4 * (cb + 4 * m) + t;
          const float uw = (col < N) ? wv + ((col == N - 1) ? 1.f : 0.f) : 0.f;
          float tv = fmaf(-g, uw, T[i][4 * m + t]);
          if (extra != 0.f && col < N) tv = fmaf(extra * pb[i], wv, tv);
          T[i][4 * m + t] = tv;
        }
    }
  }
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int row = 4 * rb + i;
    if (row >= N) continue;
#pragma unroll
    for (int m = 0; m < 4; m++) {
      const int col = 4 * (cb + 4 * m);
      if (N == NB) {
        *reinterpret_cast<float4*>(Gz + row * N + col) =
            make_float4(T[i][4 * m], T[i][4 * m + 1], T[i][4 * m + 2], T[i][4 * m + 3]);
      } else {
#pragma unroll
        for (int t = 0; t < 4; t++)
          if (col + t < N) Gz[row * N + col + t] = T[i][4 * m + t];
      }
    }
  }
  if (j == 0 && nan_flag) status[zl] |= ZST_NAN;
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
    // d[k+1], e[k+1] are loaded one rotation ahead (they are not written before use)
    float dk1n = d[(lo + 1) * kT2];
    float ek1n = (lo + 1 < hi) ? e[(lo + 1) * kT2] : 0.f;
    for (int k = lo; k < hi; k++) {
      const float dk1 = dk1n;
      const float ek1 = ek1n;
      if (k + 2 <= hi) {
        dk1n = d[(k + 2) * kT2];
        ek1n = (k + 2 < hi) ? e[(k + 2) * kT2] : 0.f;
      }
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
                          cudaStream_t st) {
  if (N < 2 || N > NB) return cudaErrorInvalidValue;
  const int blocks = (nzc + kZpb - 1) / kZpb;
  k_eig_tridiag32<<<blocks > 0 ? blocks : 1, 32 * kZpb, 0, st>>>(N, nzc, d_GT, d_aux, d_nobs);
  return cudaGetLastError();
}

cudaError_t eig32_transform(int N, int32_t nzc, float* d_GT, const float* d_aux,
                            const float* d_Z, const float* d_g, const int32_t* d_nobs, int rotate,
                            float* d_ampl, int32_t* d_status, cudaStream_t st) {
  if (N < 2 || N > NB) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(k_eig_transform32,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem3);
  if (e != cudaSuccess) return e;
  k_eig_transform32<<<nzc > 0 ? nzc : 1, kT3, kSmem3, st>>>(N, nzc, d_GT, d_aux, d_Z, d_g,
                                                            d_nobs, rotate, d_ampl, d_status);
  return cudaGetLastError();
}

}  // namespace oakg
