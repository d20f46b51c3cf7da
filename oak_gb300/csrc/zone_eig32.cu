// Mixed-precision eigensolve kernels for ensembles of up to 64 members, in FP32: E1
// (Householder tridiagonalisation), E2a (tridiagonal eigenvalues), E2b (inverse iteration) and
// E3 (back-transform, orthogonalisation, amplitudes and the square-root transform). They replace
// the generic FP32 kernels of zone_eig.cu for these sizes.
//
// The arithmetic follows rrsqrt.F90:136-185 as the generic kernels do (the comment block at the
// top of zone_eig.cu lists the reference lines); the matrix is padded to 64 x 64 with zeros,
// which adds decoupled zero rows that no output reads.
//
// The stages keep rows (E1: two per lane, one warp per zone) or eigenvectors (E3: two per lane,
// one warp per zone; E2b: one per thread, 64 threads per zone) of 64 elements in registers, so
// matrix-vector products need no cross-thread reductions: the shared operand is broadcast
// with 128-bit shared loads.
//
// E1: one warp per zone, lane t holding rows t and t + 32 of the scaled symmetric matrix. Row
//   k equals column k, so the lane holding row k publishes it and the warp forms reflector k
//   from it (two entries a lane, a warp reduction); p = beta A v is a register
//   dot per row; w = p - kc v is formed once per row and shared; warp-level synchronisation.
//   Reflector k is stored vector-major, zero padded, in row k of the zone's matrix slot:
//   slot[k*N + r] = v_k[r] (v_k[r] = 0 for r <= k).
// E2a: one thread per zone, implicit QR sweeps (working arrays in shared memory).
// E2b: thread j = eigenpair j, inverse iteration (LU factor in shared memory).
// E3: one warp per zone, lane t holding eigenvectors t and t + 32.
//   orthogonalisation of the eigenvectors Z of Tri: right-looking modified Gram-Schmidt,
//     largest eigenvalue first (a vector is final when every larger-eigenvalue vector has been
//     projected out of it); a vector that keeps at least half its squared norm is accepted
//     after this one projection (Kahan-Parlett "twice is enough"), one that does not is marked
//     collapsed and replaced by a pseudo-random vector orthogonalised (two passes) against
//     every accepted one and refined by inverse iteration with its own shift inside that
//     orthogonal complement;
//   back-transform U = H_0 ... H_{N-3} Z: per reflector a register dot and axpy, no barrier;
//   T_sym = (U Q)(U Q)^T with Q = diag((1+lambda)^-1/4): each lane computes two full rows
//     (128-bit broadcast loads of W's rows); Omega = RotateVector(w, v) applied to those rows
//     in its reflector form (rank-one updates, matoper.F90:509-535).
#include <cuda_runtime.h>
#include <math.h>

#include "oakg_internal.cuh"

namespace oakg {

namespace {

constexpr int NB = 64;        // padded ensemble size
constexpr int LDV = NB + 4;   // row stride of vector-major shared matrices (16-byte rows,
                              // 8 consecutive rows fall in 8 different 16-byte bank groups)

__host__ __device__ inline int aux_stride32(int N) { return 5 * N + 2; }

template <int L>
__device__ __forceinline__ void vload(float (&x)[L], const float* p) {
#pragma unroll
  for (int c = 0; c < L; c += 4) {
    const float4 v = *reinterpret_cast<const float4*>(p + c);
    x[c] = v.x;
    x[c + 1] = v.y;
    x[c + 2] = v.z;
    x[c + 3] = v.w;
  }
}

template <int L>
__device__ __forceinline__ void vstore(const float (&x)[L], float* p) {
#pragma unroll
  for (int c = 0; c < L; c += 4)
    *reinterpret_cast<float4*>(p + c) = make_float4(x[c], x[c + 1], x[c + 2], x[c + 3]);
}

// warp-wide sum; the butterfly adds each pair in both orders, so every lane gets the same value
__device__ __forceinline__ float wsum(float x) {
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// ------------------------------------------------------------------------------------ E1
// One warp per zone (kZpb zones per block). Lane t holds rows t and t + 32 of the scaled
// symmetric matrix in registers (a0[c] = A[t][c], a1[c] = A[t+32][c]). Row k equals column k,
// so the lane holding row k publishes it and the warp forms reflector k from it; p = beta A v
// is a register dot per row; every
// synchronisation is warp-level. Columns at or left of k are not read after step k, so
// 16-column groups lying entirely there are skipped, and the first row set is skipped once all
// its rows are final (k >= 31).
constexpr int kZpb = 4;

// Reflector k of E1 from row k of the matrix, published in rowbuf by the lane that holds it:
// every lane takes entries lane and lane + 32 (sum of squares by a warp reduction), so the
// reflector costs a few instructions a lane instead of a row's worth on one lane. v goes to
// vbuf (zero at and left of k, v[k+1] = x0 -/+ mu), d_k, e_k and beta_k to the aux slots; the
// return value, beta_k, is the same in every lane.
__device__ __forceinline__ float warp_reflector(const float* rowbuf, int k, int N, int lane,
                                                float* vbuf, float* ax) {
  const float xa = rowbuf[lane], xb = rowbuf[lane + 32];
  const float x0 = rowbuf[k + 1], dk = rowbuf[k];
  float part = (lane > k + 1) ? xa * xa : 0.f;
  if (lane + 32 > k + 1) part = fmaf(xb, xb, part);
  const float sig = wsum(part);
  const float mu = sqrtf(fmaf(x0, x0, sig));
  const float v0 = (x0 <= 0.f) ? x0 - mu : x0 + mu;
  const float vv = fmaf(v0, v0, sig);
  const bool skip = (sig == 0.f) || !(vv > 0.f) || isinf(vv);
  const float bk = skip ? 0.f : 2.f / vv;
  const float vk1 = skip ? x0 : v0;
  vbuf[lane] = (lane > k + 1) ? xa : ((lane == k + 1) ? vk1 : 0.f);
  vbuf[lane + 32] = (lane + 32 > k + 1) ? xb : ((lane + 32 == k + 1) ? vk1 : 0.f);
  if (lane == 0) {
    ax[k] = dk;                                        // d_k
    ax[N + k] = skip ? x0 : ((x0 <= 0.f) ? mu : -mu);  // e_k
    ax[2 * N + k] = bk;                                // beta_k
  }
  return bk;
}

__global__ void __launch_bounds__(32 * kZpb, 3)
    k_eig_tridiag32(int N, int32_t nzc, float* __restrict__ GT, float* __restrict__ aux,
                    const int32_t* __restrict__ nobs) {
  __shared__ __align__(16) float vbuf_s[kZpb][NB];
  __shared__ __align__(16) float wbuf_s[kZpb][NB];
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
    if (lane == (k & 31)) {  // row k = column k: its holder publishes it
      if (k < 32)
        vstore(a0, wbuf);
      else
        vstore(a1, wbuf);
    }
    __syncwarp();  // row k published (wbuf is free: the previous w was consumed)
    const float bk = warp_reflector(wbuf, k, N, lane, vbuf, ax);
    __syncwarp();  // v published; row k read by every lane before w overwrites it
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
// One warp per zone (kZpb3 zones per block). Lane t holds eigenvectors t and t + 32 (64
// components each) in registers, so every dot product and axpy is lane-local and the 128-bit
// loads of a shared row (a reflector, a final vector) serve both vectors. One shared 64 x 64
// matrix per zone (vector-major, 16-byte rows) holds the reflectors during the
// back-transform, then the eigenvectors, W = U diag(lambda'^1/4) and finally T for the
// coalesced store.
constexpr int kZpb3 = 2;
struct Zone3 {
  float buf[NB * LDV];
  float lam[NB], sq[NB], qs[NB], gs[NB], bet[NB], tt[NB], cc[NB], vv[NB], uv[NB], vn[NB];
  float t0[NB];
  int flag[NB];
};
constexpr size_t kSmem3 = (size_t)kZpb3 * sizeof(Zone3);

// (x0 . u, x1 . u) over the 16-component groups g >= g0 (the others are zero in u)
__device__ __forceinline__ void vdot2(const float (&x0)[NB], const float (&x1)[NB], const float* u,
                                      int g0, bool use0, float& d0, float& d1) {
  float a0 = 0.f, a1 = 0.f, b0 = 0.f, b1 = 0.f;
#pragma unroll
  for (int g = 0; g < 4; g++) {
    if (g >= g0) {
#pragma unroll
      for (int m = 0; m < 4; m++) {
        const int c = 16 * g + 4 * m;
        const float4 v = *reinterpret_cast<const float4*>(u + c);
        if (use0) {
          a0 = fmaf(x0[c], v.x, a0);
          a1 = fmaf(x0[c + 1], v.y, a1);
          a0 = fmaf(x0[c + 2], v.z, a0);
          a1 = fmaf(x0[c + 3], v.w, a1);
        }
        b0 = fmaf(x1[c], v.x, b0);
        b1 = fmaf(x1[c + 1], v.y, b1);
        b0 = fmaf(x1[c + 2], v.z, b0);
        b1 = fmaf(x1[c + 3], v.w, b1);
      }
    }
  }
  d0 = a0 + a1;
  d1 = b0 + b1;
}

// x0 -= f0 u (if use0), x1 -= f1 u (if use1) over the groups g >= g0
__device__ __forceinline__ void vaxpy2(float (&x0)[NB], float (&x1)[NB], float f0, float f1,
                                       const float* u, int g0, bool use0, bool use1) {
#pragma unroll
  for (int g = 0; g < 4; g++) {
    if (g >= g0) {
#pragma unroll
      for (int m = 0; m < 4; m++) {
        const int c = 16 * g + 4 * m;
        const float4 v = *reinterpret_cast<const float4*>(u + c);
        if (use0) {
          x0[c] = fmaf(-f0, v.x, x0[c]);
          x0[c + 1] = fmaf(-f0, v.y, x0[c + 1]);
          x0[c + 2] = fmaf(-f0, v.z, x0[c + 2]);
          x0[c + 3] = fmaf(-f0, v.w, x0[c + 3]);
        }
        if (use1) {
          x1[c] = fmaf(-f1, v.x, x1[c]);
          x1[c + 1] = fmaf(-f1, v.y, x1[c + 1]);
          x1[c + 2] = fmaf(-f1, v.z, x1[c + 2]);
          x1[c + 3] = fmaf(-f1, v.w, x1[c + 3]);
        }
      }
    }
  }
}

constexpr int kFillIters = 2;     // inverse-iteration steps of a pseudo-random complement fill
constexpr float kResidMin = 1e-6f;  // smallest squared residual norm used as a fill

// x <- (Tri - s I)^-1 x in place, Tri = (d, e); partial-pivoting LU with tiny pivots replaced,
// as in the inverse iteration of E2b (u1, u2, ui: scratch of N)
__device__ void tri_solve32(float* x, const float* d, const float* e, int N, float s, float tiny,
                            float* u1, float* u2, float* ui) {
  float cd = d[0] - s, csup = (N > 1) ? e[0] : 0.f;
  for (int i = 0; i < N - 1; i++) {
    const float sub = e[i], dg = d[i + 1] - s, sp = (i + 1 < N - 1) ? e[i + 1] : 0.f;
    const bool swap = fabsf(cd) < fabsf(sub);
    float pivot = swap ? sub : cd;
    if (!swap && fabsf(pivot) < tiny) pivot = copysignf(tiny, pivot);
    const float inv = __fdividef(1.f, pivot);  // |pivot| >= tiny > 0; ~2 ulp suffices here
    const float li = (swap ? cd : sub) * inv;
    u1[i] = swap ? dg : csup;
    u2[i] = swap ? sp : 0.f;
    ui[i] = inv;
    const float aa = swap ? csup : dg, bb = swap ? dg : csup;
    cd = fmaf(-li, bb, aa);
    csup = swap ? -li * sp : sp;
    const float xi = swap ? x[i + 1] : x[i], xn = swap ? x[i] : x[i + 1];
    x[i] = xi;
    x[i + 1] = fmaf(-li, xi, xn);
  }
  float pivot = cd;
  if (fabsf(pivot) < tiny) pivot = copysignf(tiny, pivot);
  ui[N - 1] = __fdividef(1.f, pivot);
  u1[N - 1] = 0.f;
  u2[N - 1] = 0.f;
  if (N >= 2) u2[N - 2] = 0.f;
  for (int i = N - 1; i >= 0; i--) {
    float v = x[i];
    if (i + 1 < N) v = fmaf(-u1[i], x[i + 1], v);
    if (i + 2 < N) v = fmaf(-u2[i], x[i + 2], v);
    x[i] = v * ui[i];
  }
}

// Vector c, published in row c of buf by the lane that holds it, is normalised there by the
// warp (two entries a lane, a warp reduction for the norm) or, when it keeps less than half its
// squared norm, marked collapsed and left as its residual. Returns whether it was accepted (the
// same in every lane). The holder's registers keep the unnormalised vector: the final vectors
// are reloaded from buf after the orthogonalisation.
__device__ __forceinline__ bool mgs_normalise(int c, int lane, Zone3& zs) {
  float* row = zs.buf + c * LDV;
  const float e0 = row[lane], e1 = row[lane + 32];
  const float s = wsum(fmaf(e0, e0, e1 * e1));
  const bool ok = zs.flag[c] && (s >= 0.5f);
  if (ok) {  // each lane rewrites only the entries it read
    const float sc = rsqrtf(s);
    row[lane] = e0 * sc;
    row[lane + 32] = e1 * sc;
  }
  return ok;
}

// mode 0: the whole stage; 1: stop after the back-transform and write the eigenvectors of G
// (vector-major, over Z); 2: start from eigenvectors of G given in Z (refined, with their
// eigenvalues in aux) and form T and the amplitudes.
__global__ void __launch_bounds__(32 * kZpb3, 4)
    k_eig_transform32(int N, int32_t nzc, float* __restrict__ GT, const float* __restrict__ aux,
                      float* __restrict__ Zg, const float* __restrict__ gv,
                      const int32_t* __restrict__ nobs, int rotate, float* __restrict__ ampl_out,
                      int32_t* __restrict__ status, int mode) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  const int lane = threadIdx.x & 31, wz = threadIdx.x >> 5;
  Zone3& zs = reinterpret_cast<Zone3*>(sm_raw)[wz];
  const int32_t zl = blockIdx.x * kZpb3 + wz;
  if (zl >= nzc || nobs[zl] == 0) return;  // warp-uniform; warp-level synchronisation only
  float* Gz = GT + (int64_t)zl * N * N;
  const float* ax = aux + (int64_t)zl * aux_stride32(N);
  float* Zz = Zg + (int64_t)zl * N * N;
  const int j0 = lane, j1 = lane + 32;
  float* buf = zs.buf;
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const int i = lane + 32 * h;
    double l = (i < N) ? (double)ax[3 * N + i] : 0.0;
    if (l < 0.0) l = 0.0;
    const double li = 1.0 / (1.0 + l);
    const double s = sqrt(li);
    zs.lam[i] = (float)li;
    zs.sq[i] = (float)s;
    zs.qs[i] = (float)sqrt(s);
    zs.gs[i] = (i < N) ? gv[(int64_t)zl * N + i] : 0.f;
    zs.bet[i] = (i < N - 2) ? ax[2 * N + i] : 0.f;
    zs.flag[i] = 1;
  }
  float x0[NB], x1[NB];
#pragma unroll
  for (int i = 0; i < NB; i++) {
    x0[i] = (j0 < N) ? ((i < N) ? Zz[(int64_t)j0 * N + i] : 0.f) : ((i == j0) ? 1.f : 0.f);
    x1[i] = (j1 < N) ? ((i < N) ? Zz[(int64_t)j1 * N + i] : 0.f) : ((i == j1) ? 1.f : 0.f);
  }
  __syncwarp();
  if (mode != 2) {  // eigenvectors of Tri: orthogonalisation and back-transform
  // modified Gram-Schmidt on the eigenvectors of Tri (the back-transform below is orthogonal),
  // largest eigenvalue first: vector c is final once every larger-eigenvalue vector has been
  // projected out of it. A vector that keeps at least half its squared norm is orthogonal to
  // working precision after this one projection ("twice is enough", Kahan-Parlett; Parlett,
  // The Symmetric Eigenvalue Problem, 6-9); one that does not is marked collapsed and replaced
  // below.
  for (int c = N - 1; c >= 0; c--) {
    if (lane == (c & 31)) {
      if (c >= 32)
        vstore(x1, buf + c * LDV);
      else
        vstore(x0, buf + c * LDV);
    }
    __syncwarp();  // vector c published
    const bool ok = mgs_normalise(c, lane, zs);
    __syncwarp();  // row c normalised; every lane has read flag[c]
    if (!ok) {
      if (lane == 0) zs.flag[c] = 0;
    } else {
      const float* uc = buf + c * LDV;
      const bool use0 = j0 < c, use1 = j1 < c;
      if (use0 || use1) {
        float d0, d1;
        vdot2(x0, x1, uc, 0, use0, d0, d1);
        vaxpy2(x0, x1, d0, d1, uc, 0, use0, use1);
      }
    }
  }
  __syncwarp();
  int ncol = 0;
  if (j0 < N && !zs.flag[j0]) ncol = 1;
  if (j1 < N && !zs.flag[j1]) ncol = 1;
  if (__any_sync(0xffffffffu, ncol)) {
    // complement fill. Inverse iteration gives nearly parallel vectors for eigenvalues that
    // FP32 does not separate (gaps below eps ||G||), so one of them collapses above, and the
    // span of the accepted vectors misses directions whose eigenvalues can lie anywhere in the
    // collapsed group: a replacement must point at the right one. The collapsed vector's
    // residual (what the larger-eigenvalue vectors left of it) is its inverse iterate with
    // those directions removed, i.e. already filtered toward its shift inside the missing
    // subspace; made orthogonal (two classical Gram-Schmidt passes) to every accepted vector,
    // it is the replacement. A residual too small to carry that information (squared norm
    // below kResidMin, FP32 noise then dominates) is replaced by a pseudo-random vector that
    // kFillIters steps of inverse iteration with the collapsed vector's shift refine inside the
    // orthogonal complement (x <- P (Tri - shift_c)^-1 x, P the projector of the two passes).
    // Filled vectors count as accepted for the later ones.
    const float onenrm = ax[5 * N + 1];
    // the last replacement spans the remaining one-dimensional complement: no choice to refine
    int left = 0;
    for (int c = 0; c < N; c++) left += zs.flag[c] ? 0 : 1;
    float* td = zs.uv;  // Tri (d, e) for the solves; uv and vn are free until the rotation
    float* te = zs.vn;
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int i = lane + 32 * h;
      td[i] = (i < N) ? ax[i] : 0.f;
      te[i] = (i < N - 1) ? ax[N + i] : 0.f;
    }
    __syncwarp();
    for (int c = 0; c < N; c++) {
      if (zs.flag[c]) continue;  // warp-uniform
      const float r0 = buf[c * LDV + lane], r1 = buf[c * LDV + lane + 32];
      const bool resid = wsum(fmaf(r0, r0, r1 * r1)) >= kResidMin;
      --left;
      const bool refine = !resid && left > 0 && onenrm > 1e4f * 1e-36f;
      if (!resid) {
#pragma unroll
        for (int h = 0; h < 2; h++) {
          const int i = lane + 32 * h;
          unsigned hsh = (unsigned)i * 2246822519u ^ ((unsigned)c * 3266489917u + 0x27d4eb2fu);
          hsh ^= hsh >> 15;
          hsh *= 2654435761u;
          hsh ^= hsh >> 13;
          buf[c * LDV + i] =
              (i < N) ? (float)((double)(hsh & 0xffffff) * (1.0 / 16777216.0) - 0.5) : 0.f;
        }
      }
      __syncwarp();
      for (int it = 0;; it++) {
        for (int pass = 0; pass < 2; pass++) {
#pragma unroll
          for (int h = 0; h < 2; h++) {
            const int k = lane + 32 * h;
            float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;  // padding components are zero
            if (k < N && k != c && zs.flag[k]) {
              const float* uk = buf + k * LDV;
              const float* uc = buf + c * LDV;
#pragma unroll 4
              for (int i = 0; i < NB; i += 4) {
                const float4 a = *reinterpret_cast<const float4*>(uk + i);
                const float4 b = *reinterpret_cast<const float4*>(uc + i);
                s0 = fmaf(a.x, b.x, s0);
                s1 = fmaf(a.y, b.y, s1);
                s2 = fmaf(a.z, b.z, s2);
                s3 = fmaf(a.w, b.w, s3);
              }
            }
            zs.t0[k] = (s0 + s1) + (s2 + s3);
          }
          __syncwarp();
          float sv[2];
#pragma unroll
          for (int h = 0; h < 2; h++) {
            const int i = lane + 32 * h;
            float s0 = buf[c * LDV + i], s1 = 0.f;
            for (int k = 0; k < N; k += 2) {
              s0 = fmaf(-zs.t0[k], buf[k * LDV + i], s0);
              if (k + 1 < N) s1 = fmaf(-zs.t0[k + 1], buf[(k + 1) * LDV + i], s1);
            }
            sv[h] = s0 + s1;
          }
          __syncwarp();
          buf[c * LDV + lane] = sv[0];
          buf[c * LDV + lane + 32] = sv[1];
          __syncwarp();
        }
        float u0 = buf[c * LDV + lane], u1 = buf[c * LDV + lane + 32];
        const float tot = wsum(u0 * u0 + u1 * u1);
        const float sc = (tot > 0.f) ? rsqrtf(tot) : 0.f;
        u0 *= sc;
        u1 *= sc;
        if (it == kFillIters || !refine) {
          __syncwarp();
          buf[c * LDV + lane] = u0;
          buf[c * LDV + lane + 32] = u1;
          break;
        }
        __syncwarp();
        buf[c * LDV + lane] = u0;
        buf[c * LDV + lane + 32] = u1;
        __syncwarp();
        if (lane == 0)
          tri_solve32(buf + c * LDV, td, te, N, ax[4 * N + c], 5.9604645e-8f * onenrm, zs.tt,
                      zs.cc, zs.vv);
        __syncwarp();
      }
      if (lane == 0) zs.flag[c] = 1;
      __syncwarp();
    }
  }
  // the final (normalised or replaced) vectors are the rows of buf
  if (j0 < N) vload(x0, buf + j0 * LDV);
  if (j1 < N) vload(x1, buf + j1 * LDV);
  __syncwarp();  // every lane holds its final vectors: buf takes the reflectors
  // reflectors into buf (rows k < N-2, zero padded)
  if (N == NB) {
#pragma unroll 4
    for (int i = 0; i < NB * NB / 4 / 32; i++) {
      const int idx4 = lane + 32 * i;
      const int k = idx4 >> 4, c = (idx4 & 15) * 4;
      *reinterpret_cast<float4*>(buf + k * LDV + c) =
          (k < N - 2) ? reinterpret_cast<const float4*>(Gz)[idx4] : make_float4(0, 0, 0, 0);
    }
  } else {
    for (int idx = lane; idx < NB * NB; idx += 32) {
      const int k = idx >> 6, c = idx & (NB - 1);
      buf[k * LDV + c] = (k < N - 2 && c < N) ? Gz[k * N + c] : 0.f;
    }
  }
  __syncwarp();
  // back-transform U = H_0 H_1 ... H_{N-3} Z (reflector k vanishes on components <= k)
  for (int k = N - 3; k >= 0; k--) {
    const float bk = zs.bet[k];
    if (bk == 0.f) continue;  // warp-uniform
    const float* vk = buf + k * LDV;
    const int g0 = (k + 1) >> 4;
    float d0, d1;
    vdot2(x0, x1, vk, g0, true, d0, d1);
    vaxpy2(x0, x1, bk * d0, bk * d1, vk, g0, true, true);
  }
  if (mode == 1) {  // the eigenvectors of G for the refinement; this lane's rows of Z only
#pragma unroll
    for (int i = 0; i < NB; i++) {
      if (j0 < N && i < N) Zz[(int64_t)j0 * N + i] = x0[i];
      if (j1 < N && i < N) Zz[(int64_t)j1 * N + i] = x1[i];
    }
    return;
  }
  }  // mode != 2
  __syncwarp();  // the reflectors are read: buf holds U from here on
  vstore(x0, buf + j0 * LDV);
  vstore(x1, buf + j1 * LDV);
  __syncwarp();
  // per-vector scalars: lambda' (u_j . g), colsum(u_j) / sqrt(lambda')
  {
    float y0, y1;
    vdot2(x0, x1, zs.gs, 0, true, y0, y1);
    float c0 = 0.f, c1 = 0.f;
#pragma unroll
    for (int i = 0; i < NB; i++) {
      c0 += x0[i];
      c1 += x1[i];
    }
    zs.tt[j0] = (j0 < N) ? zs.lam[j0] * y0 : 0.f;
    zs.tt[j1] = (j1 < N) ? zs.lam[j1] * y1 : 0.f;
    zs.cc[j0] = (j0 < N) ? c0 / zs.sq[j0] : 0.f;
    zs.cc[j1] = (j1 < N) ? c1 / zs.sq[j1] : 0.f;
  }
  __syncwarp();
  // ampl = U tt, v = U cc (lane: components lane and lane + 32)
  int nan_flag = 0;
  float vsq = 0.f;
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const int r = lane + 32 * h;
    float sa = 0.f, sv = 0.f;
    for (int jj = 0; jj < N; jj++) {
      const float u = buf[jj * LDV + r];
      sa = fmaf(u, zs.tt[jj], sa);
      sv = fmaf(u, zs.cc[jj], sv);
    }
    if (r < N) {
      ampl_out[(int64_t)zl * N + r] = sa;
      if (!(sa == sa) || isinf(sa)) nan_flag = 1;
      vsq = fmaf(sv, sv, vsq);
    }
    zs.vv[r] = (r < N) ? sv : 0.f;
  }
  nan_flag = __any_sync(0xffffffffu, nan_flag);
  const float vinv = rotate ? 1.f / sqrtf(wsum(vsq)) : 0.f;
  __syncwarp();  // buf read by every lane before W overwrites it
  {
    const float q0 = zs.qs[j0], q1 = zs.qs[j1];
#pragma unroll
    for (int i = 0; i < NB; i++) {
      x0[i] *= q0;
      x1[i] *= q1;
    }
    vstore(x0, buf + j0 * LDV);  // W = U diag(qs); padding vectors stay unit vectors
    vstore(x1, buf + j1 * LDV);
  }
  float sv_ = 1.f;
  if (rotate) {
    const float vN = zs.vv[N - 1] * vinv;
    sv_ = signbit(vN) ? -1.f : 1.f;
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int col = lane + 32 * h;
      const float vn = (col < N) ? zs.vv[col] * vinv : 0.f;
      zs.vn[col] = vn;
      zs.uv[col] = vn + ((col == N - 1) ? sv_ : 0.f);
    }
  }
  __syncwarp();
  // T_sym = W W^T: lane computes rows lane and lane + 32 (64 columns each, in registers)
  float T0[NB], T1[NB];
#pragma unroll
  for (int b = 0; b < NB; b++) {
    T0[b] = 0.f;
    T1[b] = 0.f;
  }
  for (int jj = 0; jj < N; jj++) {
    const float* w = buf + jj * LDV;
    const float wa0 = w[j0], wa1 = w[j1];
#pragma unroll
    for (int b = 0; b < NB; b += 4) {
      const float4 wb = *reinterpret_cast<const float4*>(w + b);
      T0[b] = fmaf(wa0, wb.x, T0[b]);
      T0[b + 1] = fmaf(wa0, wb.y, T0[b + 1]);
      T0[b + 2] = fmaf(wa0, wb.z, T0[b + 2]);
      T0[b + 3] = fmaf(wa0, wb.w, T0[b + 3]);
      T1[b] = fmaf(wa1, wb.x, T1[b]);
      T1[b + 1] = fmaf(wa1, wb.y, T1[b + 1]);
      T1[b + 2] = fmaf(wa1, wb.z, T1[b + 2]);
      T1[b + 3] = fmaf(wa1, wb.w, T1[b + 3]);
    }
  }
  if (rotate) {
    // Omega = P_v P_w + (1 - s_v s_w) v w^T with P_x = I - u_x u_x^T / (1 + |x_N|),
    // u_x = x + sign(x_N) e_N, w = 1/sqrt(N) (s_w = +1)  (matoper.F90:509-535); the lane owns
    // whole rows, so the row dots need no reduction
    const float icv = 1.f / (1.f + fabsf(zs.vn[N - 1]));
    const float wv = (float)(1.0 / sqrt((double)N));
    const float icw = 1.f / (1.f + wv);
    const float extra = 1.f - sv_;
    float pa0 = 0.f, pb0 = 0.f, pa1 = 0.f, pb1 = 0.f;
#pragma unroll
    for (int b = 0; b < NB; b += 4) {
      const float4 u4 = *reinterpret_cast<const float4*>(zs.uv + b);
      const float4 n4 = *reinterpret_cast<const float4*>(zs.vn + b);
      const float uvb[4] = {u4.x, u4.y, u4.z, u4.w}, vnb[4] = {n4.x, n4.y, n4.z, n4.w};
#pragma unroll
      for (int t = 0; t < 4; t++) {
        pa0 = fmaf(T0[b + t], uvb[t], pa0);
        pb0 = fmaf(T0[b + t], vnb[t], pb0);
        pa1 = fmaf(T1[b + t], uvb[t], pa1);
        pb1 = fmaf(T1[b + t], vnb[t], pb1);
      }
    }
    pa0 *= icv;
    pa1 *= icv;
    float pg0 = 0.f, pg1 = 0.f;
#pragma unroll
    for (int b = 0; b < NB; b += 4) {
      const float4 u4 = *reinterpret_cast<const float4*>(zs.uv + b);
      const float uvb[4] = {u4.x, u4.y, u4.z, u4.w};
#pragma unroll
      for (int t = 0; t < 4; t++) {
        const int col = b + t;
        const float uw = (col < N) ? wv + ((col == N - 1) ? 1.f : 0.f) : 0.f;
        T0[col] = fmaf(-pa0, uvb[t], T0[col]);  // T1 = T_sym - t0 u_v^T / c_v
        T1[col] = fmaf(-pa1, uvb[t], T1[col]);
        pg0 = fmaf(T0[col], uw, pg0);
        pg1 = fmaf(T1[col], uw, pg1);
      }
    }
    pg0 *= icw;
    pg1 *= icw;
#pragma unroll
    for (int col = 0; col < NB; col++) {
      const float uw = (col < N) ? wv + ((col == N - 1) ? 1.f : 0.f) : 0.f;
      float t0v = fmaf(-pg0, uw, T0[col]), t1v = fmaf(-pg1, uw, T1[col]);
      if (extra != 0.f && col < N) {
        t0v = fmaf(extra * pb0, wv, t0v);
        t1v = fmaf(extra * pb1, wv, t1v);
      }
      T0[col] = t0v;
      T1[col] = t1v;
    }
  }
  __syncwarp();  // W read by every lane before T is staged in buf
  vstore(T0, buf + j0 * LDV);
  vstore(T1, buf + j1 * LDV);
  __syncwarp();
  if (N == NB) {
#pragma unroll 4
    for (int i = 0; i < NB * NB / 4 / 32; i++) {
      const int idx4 = lane + 32 * i;
      const int row = idx4 >> 4, c = (idx4 & 15) * 4;
      reinterpret_cast<float4*>(Gz)[idx4] = *reinterpret_cast<const float4*>(buf + row * LDV + c);
    }
  } else {
    for (int idx = lane; idx < N * N; idx += 32) {
      const int row = idx / N, c = idx - row * N;
      Gz[idx] = buf[row * LDV + c];
    }
  }
  if (lane == 0 && nan_flag) status[zl] |= ZST_NAN;
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
// shared memory: the first super-diagonal and the pivot reciprocals, while the second
// super-diagonal, e_{i+1} where rows i and i+1 were swapped and 0 elsewhere, is kept as one bit
// a row in a register mask (32 KB of shared memory a block: 7 blocks an SM); the iterate lives
// in registers (loops unrolled to NV, the padded length).
// Pivots are at least eps ||Tri||_1 in magnitude, so their reciprocals use the fast
// approximate division (a few ulp: inverse iteration only needs the direction).
template <int NV>
__global__ void __launch_bounds__(kT2)
    k_eig_vectors32(int N, int32_t nzc, const float* __restrict__ aux, float* __restrict__ Zg,
                    const int32_t* __restrict__ nobs) {
  extern __shared__ __align__(16) float sfac[];  // upper factor u1, 1/diag: [i][jl] each
  __shared__ float sd[NV], se[NV];
  float* su1 = sfac;
  float* sui = sfac + NV * kT2;
  // bit i (of word i / 64): rows i, i + 1 swapped (u2[i] = e[i+1])
  unsigned long long swapped[(NV + 63) / 64];
#pragma unroll
  for (int w = 0; w < (NV + 63) / 64; w++) swapped[w] = 0ull;
  const int jl = threadIdx.x, j = kT2 * blockIdx.y + jl;  // eigenpair j of this block's kT2
  const int32_t zl = blockIdx.x;
  if (zl >= nzc || nobs[zl] == 0) return;  // block-uniform
  const float* ax = aux + (int64_t)zl * aux_stride32(N);
  for (int i = jl; i < N; i += kT2) {
    sd[i] = ax[i];
    se[i] = (i < N - 1) ? ax[N + i] : 0.f;
  }
  __syncthreads();
  const float onenrm = ax[5 * N + 1];
  float* Zz = Zg + (int64_t)zl * N * N;
  float* tr = sfac;  // [i][kT2 + 1] transpose staging, used at the end
  float x[NV];
#pragma unroll
  for (int i = 0; i < NV; i++) x[i] = 0.f;
  if (!(onenrm > 1e4f * 1e-36f)) {  // Tri = 0: every vector is an eigenvector
#pragma unroll
    for (int i = 0; i < NV; i++) x[i] = (i == j) ? 1.f : 0.f;
  } else if (j < N) {
    const float l = ax[4 * N + j];
    const float tiny = 5.9604645e-8f * onenrm;
#pragma unroll
    for (int i = 0; i < NV; i++) {
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
      for (int i = 0; i < NV - 1; i++) {
        if (i < N - 1) {
          const float sub = se[i], dg = sd[i + 1] - l, sp = (i + 1 < N - 1) ? se[i + 1] : 0.f;
          const bool swap = fabsf(cd) < fabsf(sub);
          float pivot = swap ? sub : cd;
          if (!swap && fabsf(pivot) < tiny) pivot = copysignf(tiny, pivot);
          const float ui = __fdividef(1.f, pivot);  // |pivot| >= tiny > 0
          const float li = (swap ? cd : sub) * ui;
          if (it == 0) {
            su1[i * kT2 + jl] = swap ? dg : csup;
            sui[i * kT2 + jl] = ui;
            if (swap) swapped[i >> 6] |= 1ull << (i & 63);
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
        sui[(N - 1) * kT2 + jl] = __fdividef(1.f, pivot);
        su1[(N - 1) * kT2 + jl] = 0.f;
        // u2[N-2] = u2[N-1] = 0: a swap at row N - 2 brings e[N-1] = 0, row N - 1 has no bit
      }
      // back substitution with the upper factor (diagonal + two super-diagonals)
#pragma unroll
      for (int i = NV - 1; i >= 0; i--) {
        if (i < N) {
          float v = x[i];
          if (i + 1 < NV) v = fmaf(-su1[i * kT2 + jl], x[i + 1], v);
          if (i + 2 < NV && ((swapped[i >> 6] >> (i & 63)) & 1ull))
            v = fmaf(-se[i + 1], x[i + 2], v);
          x[i] = v * sui[i * kT2 + jl];
        }
      }
      float mx = 0.f;
#pragma unroll
      for (int i = 0; i < NV; i++) mx = fmaxf(mx, fabsf(x[i]));
      const float im = 1.f / mx;
      float nr[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int i = 0; i < NV; i++) {
        x[i] *= im;
        nr[i & 3] = fmaf(x[i], x[i], nr[i & 3]);
      }
      const float sc = rsqrtf((nr[0] + nr[1]) + (nr[2] + nr[3]));
#pragma unroll
      for (int i = 0; i < NV; i++) x[i] *= sc;
    }
  }
  __syncthreads();  // factors no longer read: reuse them as the transpose buffer
#pragma unroll
  for (int i = 0; i < NV; i++) tr[i * (kT2 + 1) + jl] = x[i];
  __syncthreads();
  // this block's vectors kT2 * blockIdx.y + jj (rows of Z), coalesced along the rows
  const int j0 = kT2 * blockIdx.y;
  const int nv = (N - j0 < kT2) ? N - j0 : kT2;
  for (int idx = jl; idx < nv * N; idx += kT2) {
    const int jj = idx / N, i = idx - jj * N;
    Zz[(int64_t)(j0 + jj) * N + i] = tr[i * (kT2 + 1) + jj];
  }
}

// ------------------------------------------------------------------------- N <= 128: E1, E3
// Ensembles of 65 to 128 members: one block of NB2 = 128 threads per zone, thread t holding row
// t (E1) or eigenvector t (E3) of up to 128 elements in registers, so products stay
// thread-local as in the warp-per-zone kernels above; rows and vectors are shared through
// shared memory with block barriers. The arithmetic is that of E1 and E3 above.
constexpr int NB2 = 128;
constexpr int LDV2 = NB2 + 4;

// block-wide sum (every thread gets it); red: 4 floats of shared scratch
__device__ __forceinline__ float block_sum128(float x, float* red) {
  x = wsum(x);
  __syncthreads();  // red free (a previous use is complete)
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
  __syncthreads();
  return (red[0] + red[1]) + (red[2] + red[3]);
}

// E1 for N <= 128. Thread t holds row t of the scaled symmetric matrix (a[c] = A[t][c]); the
// holder of row k publishes it, every warp forms reflector k from it (each lane takes four
// entries; the sum of squares is a warp reduction, the same in every warp, so no block
// reduction is needed) and thread t writes v_t; p = beta A v is a register dot per row;
// kc = beta (p . v) / 2 from per-warp partials; the update A -= v w^T + w v^T takes
// w_c = p_c - kc v_c from the published p. The row, v, p and the partials are double-buffered
// by step parity: three barriers a step. Rows <= k are final after step k and columns <= k are
// not read again, so 16-column groups lying there are skipped.
__global__ void __launch_bounds__(NB2, 3)
    k_eig_tridiag128(int N, int32_t nzc, float* __restrict__ GT, float* __restrict__ aux,
                     const int32_t* __restrict__ nobs) {
  __shared__ __align__(16) float vbuf[2][NB2];
  __shared__ __align__(16) float pbuf[2][NB2];
  __shared__ __align__(16) float rbuf[2][NB2];
  __shared__ float red[2][4];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int32_t zl = blockIdx.x;
  if (zl >= nzc || nobs[zl] == 0) return;  // block-uniform
  float* Gz = GT + (int64_t)zl * N * N;
  float* ax = aux + (int64_t)zl * aux_stride32(N);
  float a[NB2];
#pragma unroll
  for (int c = 0; c < NB2; c++) a[c] = (t < N && c < N) ? Gz[t * N + c] : 0.f;
  float amax = 0.f;
#pragma unroll
  for (int c = 0; c < NB2; c++) amax = fmaxf(amax, fabsf(a[c]));
  for (int o = 16; o > 0; o >>= 1) amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
  if (lane == 0) red[0][warp] = amax;
  __syncthreads();  // also: every row read before reflectors overwrite the slot
  float scale = fmaxf(fmaxf(red[0][0], red[0][1]), fmaxf(red[0][2], red[0][3]));
  if (!(scale > 0.f) || isinf(scale)) scale = 1.f;
  const float iscale = 1.f / scale;
#pragma unroll
  for (int c = 0; c < NB2; c++) a[c] *= iscale;
  if (t == 0) ax[5 * N] = scale;
  __syncthreads();  // red[0] read before step 0 reuses it
  for (int k = 0; k < N - 2; k++) {
    const int b = k & 1;
    float* vb = vbuf[b];
    float* pb = pbuf[b];
    float* rb = rbuf[b];
    if (t == k) vstore(a, rb);  // row k = column k
    __syncthreads();            // row k published
    float bk;
    {
      float part = 0.f;
#pragma unroll
      for (int i = 0; i < NB2 / 32; i++) {
        const int c = lane + 32 * i;
        const float x = rb[c];
        if (c > k + 1) part = fmaf(x, x, part);
      }
      const float sig = wsum(part);  // the same sum in every warp
      const float x0 = rb[k + 1];
      const float mu = sqrtf(fmaf(x0, x0, sig));
      const float v0 = (x0 <= 0.f) ? x0 - mu : x0 + mu;
      const float vv = fmaf(v0, v0, sig);
      const bool skip = (sig == 0.f) || !(vv > 0.f) || isinf(vv);
      bk = skip ? 0.f : 2.f / vv;
      const float xt = rb[t];
      vb[t] = (t > k + 1) ? xt : ((t == k + 1) ? (skip ? x0 : v0) : 0.f);
      if (t == 0) {
        ax[k] = rb[k];                                     // d_k
        ax[N + k] = skip ? x0 : ((x0 <= 0.f) ? mu : -mu);  // e_k
        ax[2 * N + k] = bk;                                // beta_k
      }
    }
    __syncthreads();  // v published
    const float vr = vb[t];
    if (t < N) Gz[(int64_t)k * N + t] = vr;  // reflector k, vector-major, zero padded
    if (bk == 0.f) continue;                 // block-uniform; an identity reflector
    const bool act = t > k;
    float p0 = 0.f, p1 = 0.f, p2 = 0.f, p3 = 0.f;
    if (act) {
#pragma unroll
      for (int g = 0; g < NB2 / 16; g++) {
        if (16 * g + 15 > k) {
#pragma unroll
          for (int m = 0; m < 4; m++) {
            const int c = 16 * g + 4 * m;
            const float4 v4 = *reinterpret_cast<const float4*>(vb + c);
            p0 = fmaf(a[c + 0], v4.x, p0);
            p1 = fmaf(a[c + 1], v4.y, p1);
            p2 = fmaf(a[c + 2], v4.z, p2);
            p3 = fmaf(a[c + 3], v4.w, p3);
          }
        }
      }
    }
    const float p = bk * ((p0 + p1) + (p2 + p3));
    pb[t] = p;
    const float pv = wsum(p * vr);
    if (lane == 0) red[b][warp] = pv;
    __syncthreads();  // p and the partials published
    const float kc = 0.5f * bk * ((red[b][0] + red[b][1]) + (red[b][2] + red[b][3]));
    if (act) {
      const float wr = fmaf(-kc, vr, p);
#pragma unroll
      for (int g = 0; g < NB2 / 16; g++) {
        if (16 * g + 15 > k) {
#pragma unroll
          for (int m = 0; m < 4; m++) {
            const int c = 16 * g + 4 * m;
            const float4 v4 = *reinterpret_cast<const float4*>(vb + c);
            const float4 p4 = *reinterpret_cast<const float4*>(pb + c);
            const float vc[4] = {v4.x, v4.y, v4.z, v4.w};
            const float pc[4] = {p4.x, p4.y, p4.z, p4.w};
#pragma unroll
            for (int q = 0; q < 4; q++) {
              const float wc = fmaf(-kc, vc[q], pc[q]);
              a[c + q] = fmaf(-vr, wc, fmaf(-wr, vc[q], a[c + q]));
            }
          }
        }
      }
    }
  }
  // trailing 2 x 2 block: rows N-2 and N-1, read back through shared memory
  __syncthreads();  // the last step's buffers consumed
  if (t == N - 2) vstore(a, vbuf[0]);
  if (t == N - 1) vstore(a, vbuf[1]);
  __syncthreads();
  if (t == 0) {
    ax[N - 2] = vbuf[0][N - 2];
    ax[2 * N + N - 2] = 0.f;
    ax[N + N - 2] = vbuf[1][N - 2];
    ax[N - 1] = vbuf[1][N - 1];
    ax[N + N - 1] = 0.f;
    ax[2 * N + N - 1] = 0.f;
  }
}

// E3 for N <= 128: thread j holds eigenvector j; the steps of k_eig_transform32 with block
// barriers. One shared NB2 x NB2 matrix (vector-major, 16-byte rows) holds the final vectors
// of the Gram-Schmidt sweep, then the reflectors, U, W = U diag(lambda'^1/4) and T.
struct Zone128 {
  float buf[NB2 * LDV2];
  float lam[NB2], sq[NB2], qs[NB2], gs[NB2], bet[NB2], tt[NB2], cc[NB2], vv[NB2], uv[NB2],
      vn[NB2], t0[NB2];
  int flag[NB2];
  float red[4];
};
constexpr size_t kSmem128 = sizeof(Zone128);

// x . u over the 16-component groups g0 <= g < ng
__device__ __forceinline__ float vdot128(const float (&x)[NB2], const float* u, int g0, int ng) {
  float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
#pragma unroll
  for (int g = 0; g < NB2 / 16; g++) {
    if (g >= g0 && g < ng) {
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

// x -= f u over the groups g0 <= g < ng
__device__ __forceinline__ void vaxpy128(float (&x)[NB2], float f, const float* u, int g0,
                                         int ng) {
#pragma unroll
  for (int g = 0; g < NB2 / 16; g++) {
    if (g >= g0 && g < ng) {
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

// mode as for k_eig_transform32
__global__ void __launch_bounds__(NB2, 3)
    k_eig_transform128(int N, int32_t nzc, float* __restrict__ GT, const float* __restrict__ aux,
                       float* __restrict__ Zg, const float* __restrict__ gv,
                       const int32_t* __restrict__ nobs, int rotate,
                       float* __restrict__ ampl_out, int32_t* __restrict__ status, int mode) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  Zone128& zs = *reinterpret_cast<Zone128*>(sm_raw);
  const int t = threadIdx.x;
  const int32_t zl = blockIdx.x;
  if (zl >= nzc || nobs[zl] == 0) return;  // block-uniform
  float* Gz = GT + (int64_t)zl * N * N;
  const float* ax = aux + (int64_t)zl * aux_stride32(N);
  float* Zz = Zg + (int64_t)zl * N * N;
  float* buf = zs.buf;
  const int ng = (N + 15) >> 4;  // 16-component groups holding the N components
  {
    double l = (t < N) ? (double)ax[3 * N + t] : 0.0;
    if (l < 0.0) l = 0.0;
    const double li = 1.0 / (1.0 + l);
    const double s = sqrt(li);
    zs.lam[t] = (float)li;
    zs.sq[t] = (float)s;
    zs.qs[t] = (float)sqrt(s);
    zs.gs[t] = (t < N) ? gv[(int64_t)zl * N + t] : 0.f;
    zs.bet[t] = (t < N - 2) ? ax[2 * N + t] : 0.f;
    zs.flag[t] = 1;
  }
  float x[NB2];
#pragma unroll
  for (int i = 0; i < NB2; i++)
    x[i] = (t < N) ? ((i < N) ? Zz[(int64_t)t * N + i] : 0.f) : ((i == t) ? 1.f : 0.f);
  __syncthreads();
  if (mode != 2) {  // eigenvectors of Tri: orthogonalisation and back-transform (block-uniform)
  // modified Gram-Schmidt on the eigenvectors of Tri, largest eigenvalue first, with the
  // acceptance test and residual-keeping of k_eig_transform32. The holder publishes vector c
  // as it is; every warp takes its squared norm s (four entries a lane, a warp reduction: the
  // same value in every warp) and the later vectors subtract (x . u_c) / s u_c. Row c is
  // normalised in the next step (thread t scales entry t), when no thread reads it.
  float pend_sc = 1.f;  // the scale owed to entry t of the previous row
  for (int c = N - 1; c >= 0; c--) {
    if (t == c) vstore(x, buf + c * LDV2);
    __syncthreads();  // vector c published; the readers of the previous row are done
    if (c + 1 < N) buf[(c + 1) * LDV2 + t] *= pend_sc;
    const float* uc = buf + c * LDV2;
    float part = 0.f;
#pragma unroll
    for (int i = 0; i < NB2 / 32; i++) {
      const float e = uc[(t & 31) + 32 * i];
      part = fmaf(e, e, part);
    }
    const float s = wsum(part);
    // a rejected vector is flagged by thread 0 while the others read the flag: every reader
    // computes ok = false either way
    const bool ok = zs.flag[c] && (s >= 0.5f);
    if (!ok && t == 0) zs.flag[c] = 0;
    pend_sc = ok ? rsqrtf(s) : 1.f;  // a collapsed vector keeps its residual
    if (ok && t < c) vaxpy128(x, vdot128(x, uc, 0, ng) * (pend_sc * pend_sc), uc, 0, ng);
  }
  __syncthreads();  // the readers of row 0 are done
  buf[t] *= pend_sc;
  int ncol = 0;
  if (t < N && !zs.flag[t]) ncol = 1;
  if (__syncthreads_or(ncol)) {
    // complement fill, as in k_eig_transform32
    const float onenrm = ax[5 * N + 1];
    int left = 0;
    for (int c = 0; c < N; c++) left += zs.flag[c] ? 0 : 1;
    float* td = zs.uv;
    float* te = zs.vn;
    td[t] = (t < N) ? ax[t] : 0.f;
    te[t] = (t < N - 1) ? ax[N + t] : 0.f;
    for (int c = 0; c < N; c++) {
      if (zs.flag[c]) continue;  // block-uniform (flags change only between barriers)
      const float r = buf[c * LDV2 + t];
      const bool resid = block_sum128(r * r, zs.red) >= kResidMin;
      --left;
      const bool refine = !resid && left > 0 && onenrm > 1e4f * 1e-36f;
      if (!resid) {
        unsigned hsh = (unsigned)t * 2246822519u ^ ((unsigned)c * 3266489917u + 0x27d4eb2fu);
        hsh ^= hsh >> 15;
        hsh *= 2654435761u;
        hsh ^= hsh >> 13;
        buf[c * LDV2 + t] =
            (t < N) ? (float)((double)(hsh & 0xffffff) * (1.0 / 16777216.0) - 0.5) : 0.f;
      }
      __syncthreads();
      for (int it = 0;; it++) {
        for (int pass = 0; pass < 2; pass++) {
          float s = 0.f;
          if (t < N && t != c && zs.flag[t]) {
            const float* uk = buf + t * LDV2;
            const float* uc = buf + c * LDV2;
            float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
            for (int i = 0; i < 16 * ng; i += 4) {
              const float4 a4 = *reinterpret_cast<const float4*>(uk + i);
              const float4 b4 = *reinterpret_cast<const float4*>(uc + i);
              s0 = fmaf(a4.x, b4.x, s0);
              s1 = fmaf(a4.y, b4.y, s1);
              s2 = fmaf(a4.z, b4.z, s2);
              s3 = fmaf(a4.w, b4.w, s3);
            }
            s = (s0 + s1) + (s2 + s3);
          }
          zs.t0[t] = s;
          __syncthreads();
          float s0 = buf[c * LDV2 + t], s1 = 0.f;
          for (int k = 0; k < N; k += 2) {
            s0 = fmaf(-zs.t0[k], buf[k * LDV2 + t], s0);
            if (k + 1 < N) s1 = fmaf(-zs.t0[k + 1], buf[(k + 1) * LDV2 + t], s1);
          }
          __syncthreads();
          buf[c * LDV2 + t] = s0 + s1;
          __syncthreads();
        }
        const float u = buf[c * LDV2 + t];
        const float tot = block_sum128(u * u, zs.red);
        buf[c * LDV2 + t] = u * ((tot > 0.f) ? rsqrtf(tot) : 0.f);
        __syncthreads();
        if (it == kFillIters || !refine) break;
        if (t == 0)
          tri_solve32(buf + c * LDV2, td, te, N, ax[4 * N + c], 5.9604645e-8f * onenrm, zs.tt,
                      zs.cc, zs.vv);
        __syncthreads();
      }
      if (t == 0) zs.flag[c] = 1;
      __syncthreads();
    }
  }
  // buf row j holds final vector j (stored by its owner, or filled): reload, so that no
  // vector stays live in registers across the fill
#pragma unroll
  for (int i = 0; i < NB2; i++)
    x[i] = (t < N) ? buf[t * LDV2 + i] : ((i == t) ? 1.f : 0.f);
  __syncthreads();  // every thread holds its final vector: buf takes the reflectors
  for (int idx = t; idx < NB2 * NB2; idx += NB2) {
    const int k = idx >> 7, c = idx & (NB2 - 1);
    buf[k * LDV2 + c] = (k < N - 2 && c < N) ? Gz[k * N + c] : 0.f;
  }
  // couplings of each reflector with the next three applied after it: p_s[k] = v_k . v_{k-s}
  // (s = 1, 2, 3), shared by every vector of the zone (tt, cc, vv are free until the
  // amplitudes)
  float* p1 = zs.tt;
  float* p2 = zs.cc;
  float* p3 = zs.vv;
  __syncthreads();
  if (t < N - 2) {
    // v_k vanishes on components <= k; the rows are zero-padded past N
    const float* vk = buf + t * LDV2;
    const float* w1 = buf + (t >= 1 ? t - 1 : t) * LDV2;
    const float* w2 = buf + (t >= 2 ? t - 2 : t) * LDV2;
    const float* w3 = buf + (t >= 3 ? t - 3 : t) * LDV2;
    float s1 = 0.f, s2 = 0.f, s3 = 0.f;
    for (int c = (t + 1) & ~3; c < NB2; c += 4) {
      const float4 a = *reinterpret_cast<const float4*>(vk + c);
      const float4 q1 = *reinterpret_cast<const float4*>(w1 + c);
      const float4 q2 = *reinterpret_cast<const float4*>(w2 + c);
      const float4 q3 = *reinterpret_cast<const float4*>(w3 + c);
      s1 = fmaf(a.x, q1.x, fmaf(a.y, q1.y, fmaf(a.z, q1.z, fmaf(a.w, q1.w, s1))));
      s2 = fmaf(a.x, q2.x, fmaf(a.y, q2.y, fmaf(a.z, q2.z, fmaf(a.w, q2.w, s2))));
      s3 = fmaf(a.x, q3.x, fmaf(a.y, q3.y, fmaf(a.z, q3.z, fmaf(a.w, q3.w, s3))));
    }
    p1[t] = (t >= 1) ? s1 : 0.f;
    p2[t] = (t >= 2) ? s2 : 0.f;
    p3[t] = (t >= 3) ? s3 : 0.f;
  }
  __syncthreads();
  // back-transform U = H_0 H_1 ... H_{N-3} Z (reflector k vanishes on components <= k), four
  // reflectors at a time: with H_k = I - b_k v_k v_k^T applied in the order k, k-1, k-2, k-3,
  // the four dots d_i = v_{k-i} . x of the original x are independent, the coefficients follow
  // from c_i = b_{k-i} (d_i - sum_{j<i} c_j v_{k-i} . v_{k-j}), and one pass subtracts
  // sum_i c_i v_{k-i}: the same products as one reflector at a time, a quarter of the
  // dependent dot / update steps.
  int k = N - 3;
  for (; k >= 3; k -= 4) {
    const float* v0 = buf + k * LDV2;
    const float* v1 = v0 - LDV2;
    const float* v2 = v1 - LDV2;
    const float* v3 = v2 - LDV2;
    const int g0 = (k - 2) >> 4;  // the widest support of the four: v_{k-3}
    float a0 = 0.f, a1 = 0.f, b0 = 0.f, b1 = 0.f, e0 = 0.f, e1 = 0.f, f0 = 0.f, f1 = 0.f;
#pragma unroll
    for (int g = 0; g < NB2 / 16; g++) {
      if (g >= g0 && g < ng) {
#pragma unroll
        for (int m = 0; m < 4; m++) {
          const int c = 16 * g + 4 * m;
          const float4 q0 = *reinterpret_cast<const float4*>(v0 + c);
          const float4 q1 = *reinterpret_cast<const float4*>(v1 + c);
          const float4 q2 = *reinterpret_cast<const float4*>(v2 + c);
          const float4 q3 = *reinterpret_cast<const float4*>(v3 + c);
          a0 = fmaf(x[c], q0.x, fmaf(x[c + 2], q0.z, a0));
          a1 = fmaf(x[c + 1], q0.y, fmaf(x[c + 3], q0.w, a1));
          b0 = fmaf(x[c], q1.x, fmaf(x[c + 2], q1.z, b0));
          b1 = fmaf(x[c + 1], q1.y, fmaf(x[c + 3], q1.w, b1));
          e0 = fmaf(x[c], q2.x, fmaf(x[c + 2], q2.z, e0));
          e1 = fmaf(x[c + 1], q2.y, fmaf(x[c + 3], q2.w, e1));
          f0 = fmaf(x[c], q3.x, fmaf(x[c + 2], q3.z, f0));
          f1 = fmaf(x[c + 1], q3.y, fmaf(x[c + 3], q3.w, f1));
        }
      }
    }
    const float d0 = a0 + a1, d1 = b0 + b1, d2 = e0 + e1, d3 = f0 + f1;
    // v_{k-i} . v_{k-j} (j < i) = p_{i-j}[k - j]
    const float c0 = zs.bet[k] * d0;
    const float c1 = zs.bet[k - 1] * fmaf(-c0, p1[k], d1);
    const float c2 = zs.bet[k - 2] * fmaf(-c1, p1[k - 1], fmaf(-c0, p2[k], d2));
    const float c3 =
        zs.bet[k - 3] * fmaf(-c2, p1[k - 2], fmaf(-c1, p2[k - 1], fmaf(-c0, p3[k], d3)));
#pragma unroll
    for (int g = 0; g < NB2 / 16; g++) {
      if (g >= g0 && g < ng) {
#pragma unroll
        for (int m = 0; m < 4; m++) {
          const int c = 16 * g + 4 * m;
          const float4 q0 = *reinterpret_cast<const float4*>(v0 + c);
          const float4 q1 = *reinterpret_cast<const float4*>(v1 + c);
          const float4 q2 = *reinterpret_cast<const float4*>(v2 + c);
          const float4 q3 = *reinterpret_cast<const float4*>(v3 + c);
          x[c] = fmaf(-c3, q3.x, fmaf(-c2, q2.x, fmaf(-c1, q1.x, fmaf(-c0, q0.x, x[c]))));
          x[c + 1] =
              fmaf(-c3, q3.y, fmaf(-c2, q2.y, fmaf(-c1, q1.y, fmaf(-c0, q0.y, x[c + 1]))));
          x[c + 2] =
              fmaf(-c3, q3.z, fmaf(-c2, q2.z, fmaf(-c1, q1.z, fmaf(-c0, q0.z, x[c + 2]))));
          x[c + 3] =
              fmaf(-c3, q3.w, fmaf(-c2, q2.w, fmaf(-c1, q1.w, fmaf(-c0, q0.w, x[c + 3]))));
        }
      }
    }
  }
  for (; k >= 0; k--) {  // the remaining reflectors one at a time
    const float bk = zs.bet[k];
    if (bk == 0.f) continue;  // block-uniform
    const float* vk = buf + k * LDV2;
    const int g0 = (k + 1) >> 4;
    vaxpy128(x, bk * vdot128(x, vk, g0, ng), vk, g0, ng);
  }
  if (mode == 1) {  // the eigenvectors of G for the refinement; this thread's row of Z only
#pragma unroll
    for (int i = 0; i < NB2; i++)
      if (t < N && i < N) Zz[(int64_t)t * N + i] = x[i];
    return;
  }
  }  // mode != 2
  __syncthreads();  // the reflectors are read: buf holds U from here on
  vstore(x, buf + t * LDV2);
  {
    // per-vector scalars: lambda' (u_t . g), colsum(u_t) / sqrt(lambda')
    const float y = vdot128(x, zs.gs, 0, ng);
    float cs = 0.f;
#pragma unroll
    for (int i = 0; i < NB2; i++) cs += x[i];
    zs.tt[t] = (t < N) ? zs.lam[t] * y : 0.f;
    zs.cc[t] = (t < N) ? cs / zs.sq[t] : 0.f;
  }
  __syncthreads();
  // ampl = U tt, v = U cc (thread: component t)
  int nan_flag = 0;
  float vsq = 0.f;
  {
    float sa = 0.f, sv = 0.f;
    for (int jj = 0; jj < N; jj++) {
      const float u = buf[jj * LDV2 + t];
      sa = fmaf(u, zs.tt[jj], sa);
      sv = fmaf(u, zs.cc[jj], sv);
    }
    if (t < N) {
      ampl_out[(int64_t)zl * N + t] = sa;
      if (!(sa == sa) || isinf(sa)) nan_flag = 1;
      vsq = sv * sv;
    }
    zs.vv[t] = (t < N) ? sv : 0.f;
  }
  nan_flag = __syncthreads_or(nan_flag);
  const float vinv = rotate ? 1.f / sqrtf(block_sum128(vsq, zs.red)) : 0.f;
  __syncthreads();  // buf read by every thread before W overwrites it
  {
    const float q = zs.qs[t];
#pragma unroll
    for (int i = 0; i < NB2; i++) x[i] *= q;
    vstore(x, buf + t * LDV2);  // W = U diag(qs); padding vectors stay unit vectors
  }
  float sv_ = 1.f;
  const float wv = (float)(1.0 / sqrt((double)N));
  if (rotate) {
    const float vN = zs.vv[N - 1] * vinv;
    sv_ = signbit(vN) ? -1.f : 1.f;
    const float vn = (t < N) ? zs.vv[t] * vinv : 0.f;
    zs.vn[t] = vn;
    zs.uv[t] = vn + ((t == N - 1) ? sv_ : 0.f);
    zs.t0[t] = (t < N) ? wv : 0.f;                            // w (padded)
    zs.tt[t] = (t < N) ? wv + ((t == N - 1) ? 1.f : 0.f) : 0.f;  // u_w = w + e_N
  }
  __syncthreads();
  // T_sym = W W^T: thread t computes row t
  float T0[NB2];
#pragma unroll
  for (int b = 0; b < NB2; b++) T0[b] = 0.f;
  for (int jj = 0; jj < N; jj++) {
    const float* w = buf + jj * LDV2;
    const float wa = w[t];
#pragma unroll
    for (int g = 0; g < NB2 / 16; g++) {
      if (g < ng) {
#pragma unroll
        for (int m = 0; m < 4; m++) {
          const int b = 16 * g + 4 * m;
          const float4 wb = *reinterpret_cast<const float4*>(w + b);
          T0[b] = fmaf(wa, wb.x, T0[b]);
          T0[b + 1] = fmaf(wa, wb.y, T0[b + 1]);
          T0[b + 2] = fmaf(wa, wb.z, T0[b + 2]);
          T0[b + 3] = fmaf(wa, wb.w, T0[b + 3]);
        }
      }
    }
  }
  if (rotate) {
    // Omega = P_v P_w + (1 - s_v s_w) v w^T (matoper.F90:509-535), as in k_eig_transform32:
    // T1 = T_sym - (T_sym u_v) u_v^T / c_v, T2 = T1 - (T1 u_w) u_w^T / c_w + (1 - s_v) (T_sym v) w^T.
    // T1 u_w = T_sym u_w - (T_sym u_v / c_v)(u_v . u_w), so one pass gives every row dot and a
    // second applies the three rank-one terms (u_v, u_w, w and v through shared memory: a
    // per-column select would be kept live for all 128 columns between the passes).
    const float icv = 1.f / (1.f + fabsf(zs.vn[N - 1]));
    const float icw = 1.f / (1.f + wv);
    const float extra = 1.f - sv_;
    float pa = 0.f, pb = 0.f, pw = 0.f, suu = 0.f;
#pragma unroll
    for (int b = 0; b < NB2; b += 4) {
      const float4 u4 = *reinterpret_cast<const float4*>(zs.uv + b);
      const float4 n4 = *reinterpret_cast<const float4*>(zs.vn + b);
      const float4 w4 = *reinterpret_cast<const float4*>(zs.tt + b);
      const float uvb[4] = {u4.x, u4.y, u4.z, u4.w}, vnb[4] = {n4.x, n4.y, n4.z, n4.w};
      const float uwb[4] = {w4.x, w4.y, w4.z, w4.w};
#pragma unroll
      for (int q = 0; q < 4; q++) {
        pa = fmaf(T0[b + q], uvb[q], pa);
        pb = fmaf(T0[b + q], vnb[q], pb);
        pw = fmaf(T0[b + q], uwb[q], pw);
        suu = fmaf(uvb[q], uwb[q], suu);
      }
    }
    pa *= icv;
    const float pg = icw * fmaf(-pa, suu, pw);
    const float eb = extra * pb;
    __syncthreads();  // the pass below reads the vectors again (no 128 values kept live)
#pragma unroll
    for (int b = 0; b < NB2; b += 4) {
      const float4 u4 = *reinterpret_cast<const float4*>(zs.uv + b);
      const float4 w4 = *reinterpret_cast<const float4*>(zs.tt + b);
      const float4 m4 = *reinterpret_cast<const float4*>(zs.t0 + b);
      const float uvb[4] = {u4.x, u4.y, u4.z, u4.w}, uwb[4] = {w4.x, w4.y, w4.z, w4.w};
      const float wb[4] = {m4.x, m4.y, m4.z, m4.w};
#pragma unroll
      for (int q = 0; q < 4; q++)
        T0[b + q] = fmaf(eb, wb[q], fmaf(-pg, uwb[q], fmaf(-pa, uvb[q], T0[b + q])));
    }
  }
  __syncthreads();  // W read by every thread before T is staged in buf
  vstore(T0, buf + t * LDV2);
  __syncthreads();
  for (int idx = t; idx < N * N; idx += NB2) {
    const int row = idx / N, c = idx - row * N;
    Gz[idx] = buf[row * LDV2 + c];
  }
  if (t == 0 && nan_flag) status[zl] |= ZST_NAN;
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
  const size_t smem = (size_t)2 * NB * kT2 * sizeof(float);  // >= NB x (kT2 + 1): transpose
  cudaError_t e = cudaFuncSetAttribute(k_eig_vectors32<NB>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_eig_vectors32<NB><<<dim3(nzc > 0 ? nzc : 1, 1), kT2, smem, st>>>(N, nzc, d_aux, d_Z, d_nobs);
  return cudaGetLastError();
}

cudaError_t eig32_tridiag(int N, int32_t nzc, float* d_GT, float* d_aux, const int32_t* d_nobs,
                          cudaStream_t st) {
  if (N < 2 || N > NB) return cudaErrorInvalidValue;
  const int blocks = (nzc + kZpb - 1) / kZpb;
  k_eig_tridiag32<<<blocks > 0 ? blocks : 1, 32 * kZpb, 0, st>>>(N, nzc, d_GT, d_aux, d_nobs);
  return cudaGetLastError();
}

cudaError_t eig32_transform(int N, int32_t nzc, float* d_GT, const float* d_aux, float* d_Z,
                            const float* d_g, const int32_t* d_nobs, int rotate, float* d_ampl,
                            int32_t* d_status, cudaStream_t st, int mode) {
  if (N < 2 || N > NB) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(k_eig_transform32,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem3);
  if (e != cudaSuccess) return e;
  const int blocks = (nzc + kZpb3 - 1) / kZpb3;
  k_eig_transform32<<<blocks > 0 ? blocks : 1, 32 * kZpb3, kSmem3, st>>>(
      N, nzc, d_GT, d_aux, d_Z, d_g, d_nobs, rotate, d_ampl, d_status, mode);
  return cudaGetLastError();
}

int eig128_max_n() { return NB2; }

cudaError_t eig128_tridiag(int N, int32_t nzc, float* d_GT, float* d_aux, const int32_t* d_nobs,
                           cudaStream_t st) {
  if (N < 2 || N > NB2) return cudaErrorInvalidValue;
  k_eig_tridiag128<<<nzc > 0 ? nzc : 1, NB2, 0, st>>>(N, nzc, d_GT, d_aux, d_nobs);
  return cudaGetLastError();
}

cudaError_t eig128_transform(int N, int32_t nzc, float* d_GT, const float* d_aux, float* d_Z,
                             const float* d_g, const int32_t* d_nobs, int rotate, float* d_ampl,
                             int32_t* d_status, cudaStream_t st, int mode) {
  if (N < 2 || N > NB2) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(k_eig_transform128,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kSmem128);
  if (e != cudaSuccess) return e;
  k_eig_transform128<<<nzc > 0 ? nzc : 1, NB2, kSmem128, st>>>(
      N, nzc, d_GT, d_aux, d_Z, d_g, d_nobs, rotate, d_ampl, d_status, mode);
  return cudaGetLastError();
}

}  // namespace oakg
