// K5 on the tensor cores, mixed-precision form: per zone (rrsqrt.F90:151, :162-185)
//   Sa(i1:i2, :) = Sf(i1:i2, :) T        xa(i1:i2) = xf(i1:i2) + Sf(i1:i2, :) ampl
// as one product D = A B^T with A = Sf's rows of the zone (M = 128 rows a tile) and
// B^T = [T | ampl] (N x (N + 1), padded to NO = round_up(N + 1, 16) columns), on
// tcgen05.mma kind::tf32 with FP32 accumulation in tensor memory. The last real column of D is
// the mean increment Sf ampl, so xa comes from the same product.
//
// Precision: both operands are split into TF32 parts, X = X_hi + X_lo with
// X_hi = tf32(X), X_lo = tf32(X - X_hi) (residual ~2^-22 |X|), and three MMAs per K-step
// accumulate A_hi B_hi + A_hi B_lo + A_lo B_hi: FP32-level products (the A_lo B_lo term is
// 2^-22 relative). A single TF32 product leaves Sa ~5e-4 off the FP32 result on real zones
// (T has eigenvalues spread over (0, 1]), above the 1e-4 bar of the mixed form.
//
// Layout and pipeline (one CTA of 256 threads per zone at a time, persistent over zones):
// the K dimension (members) is staged 32 at a time (one 128-byte swizzle row of TF32) into a
// K-major tile of A (128 rows) and of B (NO rows), hi and lo parts each; the thread that issues
// the MMAs commits them to an mbarrier. Each K-block's global loads are issued into registers
// before the wait for the previous K-block's MMAs, so they overlap the tensor core. Sf is read
// column by column (coalesced along the zone's rows), T row by row (coalesced along its
// columns). The accumulator is read with tcgen05.ld (lane = row, 8 columns a load) and Sa is
// written column by column, 32 consecutive rows a warp store. Every mbarrier wait is bounded;
// on expiry the kernel records ZST_TIMEOUT, stops, waits (bounded) for its MMAs and frees its
// tensor memory. Zones without observations copy (xa = xf, Sa = Sf).
#include <cuda_runtime.h>

#include "oakg_internal.cuh"

namespace oakg {

namespace {

constexpr int kThreads = 256;
constexpr int kRowsTile = 128;                   // MMA M
constexpr int kKB = 32;                          // members per staged K-block
constexpr uint32_t kATile = kRowsTile * 128u;    // one A part of a K-block: 16 KB
constexpr int kWaitPolls = 1 << 22;

// Per padded width NB (64: N <= 64, 128: 64 < N <= 128):
//   NOMAX   largest MMA N (round_up(N + 1, 16)): 80 / 144
//   kCols   tensor-memory columns allocated (power of two >= NOMAX)
//   kCtas   CTAs per SM (kCtas x kCols <= 512); the shared-memory size keeps residency there
template <int NB>
struct UpCfg {
  static constexpr int NOMAX = (NB + 1 + 15) / 16 * 16;
  static constexpr uint32_t kCols = NB == 64 ? 128u : 256u;
  static constexpr int kCtas = NB == 64 ? 4 : 2;
  static constexpr uint32_t kBTile = (uint32_t)NOMAX * 128u;  // one B part of a K-block
  static constexpr size_t kStage = 2 * kATile + 2 * (size_t)kBTile;
  // 1 KB alignment slack; padded so that kCtas + 1 CTAs do not fit in 228 KB
  static constexpr size_t kDynSmem =
      (1024 + kStage) * (kCtas + 1) > 233472 ? 1024 + kStage : 233472 / (kCtas + 1) + 64;
  static_assert(kCols * kCtas <= 512, "tensor memory over-subscribed");
  static_assert(kDynSmem * kCtas <= 232448, "CTAs per SM not reachable");
  static_assert(kDynSmem * (kCtas + 1) > 233472, "more CTAs than tensor memory allows");
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint32_t to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 bytes apart
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);  // start address
  d |= (uint64_t)1 << 16;                   // leading byte offset (unused: K-step within a row)
  d |= (uint64_t)(1024u >> 4) << 32;        // stride byte offset
  d |= (uint64_t)1 << 46;                   // descriptor version
  d |= (uint64_t)2 << 61;                   // 128-byte swizzle
  return d;
}

// instruction descriptor: D F32, A and B TF32, both K-major, M = 128, N = no
__device__ __forceinline__ uint32_t idesc_tf32(uint32_t no) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((no >> 3) << 17) | ((128u >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accum) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %3, 0;\n"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %4, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(accum), "r"(idesc));
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
      : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
  for (int i = 0; i < kWaitPolls; i++) {
    uint32_t ok;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

__device__ __forceinline__ void fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// 8 consecutive accumulator columns of this warp's 32 tensor-memory lanes
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 8; i++) v[i] = __uint_as_float(r[i]);
}

// byte offset of the 16-byte chunk `chunk` (4 members) of operand row `row` in a tile
__device__ __forceinline__ uint32_t tile_off(int row, int chunk) {
  return (uint32_t)((row >> 3) * 1024 + (row & 7) * 128 + ((chunk ^ (row & 7)) << 4));
}

// writes the hi and lo TF32 parts of 4 consecutive members of one operand row
__device__ __forceinline__ void put_split(unsigned char* thi, unsigned char* tlo, uint32_t off,
                                          const float (&x)[4]) {
  uint32_t hi[4], lo[4];
#pragma unroll
  for (int i = 0; i < 4; i++) {
    hi[i] = to_tf32(x[i]);
    lo[i] = to_tf32(x[i] - __uint_as_float(hi[i]));
  }
  *reinterpret_cast<uint4*>(thi + off) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
  *reinterpret_cast<uint4*>(tlo + off) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
}

template <int NB, typename S>
__global__ void __launch_bounds__(kThreads, UpCfg<NB>::kCtas)
    k_zone_update_tc(int N, int32_t z0, int32_t nzc, const int64_t* __restrict__ zone_start,
                     const S* __restrict__ xf, const S* __restrict__ Sf, int64_t ldS,
                     const float* __restrict__ T, const float* __restrict__ ampl,
                     const int32_t* __restrict__ nobs, S* __restrict__ xa, S* __restrict__ Sa,
                     int32_t* __restrict__ err) {
  using C = UpCfg<NB>;
  constexpr int kBPer = (C::NOMAX * (kKB / 4) + kThreads - 1) / kThreads;  // B chunks a thread
  extern __shared__ __align__(16) unsigned char dyn_raw[];
  __shared__ __align__(8) unsigned long long mbar;
  __shared__ uint32_t tmem_base;
  __shared__ int32_t flag;
  const uint32_t raw_addr = smem_u32(dyn_raw);
  const uint32_t pad = ((raw_addr + 1023u) & ~1023u) - raw_addr;
  unsigned char* a_hi = dyn_raw + pad;
  unsigned char* a_lo = a_hi + kATile;
  unsigned char* b_hi = a_lo + kATile;
  unsigned char* b_lo = b_hi + C::kBTile;
  const uint32_t a_hi_s = raw_addr + pad, a_lo_s = a_hi_s + kATile;
  const uint32_t b_hi_s = a_lo_s + kATile, b_lo_s = b_hi_s + C::kBTile;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t mb = smem_u32(&mbar);
  const int NO = (N + 1 + 15) / 16 * 16;
  const int nkb = (N + kKB - 1) / kKB;
  const uint32_t idesc = idesc_tf32((uint32_t)NO);

  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    flag = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base)),
                 "r"(C::kCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = tmem_base;
  uint32_t phase = 0;  // parity of the next mbarrier completion
  int pending = 0;     // MMAs committed and not yet waited for (uniform)

  // waits for the committed MMAs (thread 0, bounded); the result is published in `flag`
  auto drain = [&]() {
    if (tid == 0 && !mbar_wait(mb, phase)) flag = 1;
    phase ^= 1u;
    pending = 0;
  };

  // A staging: row ra, member quads qa0 + 2 j; B staging: (column, quad) pairs tid + 256 j
  const int ra = tid & (kRowsTile - 1), qa0 = tid >> 7;
  bool stop = false;
  for (int32_t zl = blockIdx.x; zl < nzc && !stop; zl += gridDim.x) {
    const int32_t z = z0 + zl;
    const int64_t i1 = zone_start[z], i2 = zone_start[z + 1];
    if (nobs[zl] == 0) {
      for (int64_t i = i1 + tid; i < i2; i += kThreads) xa[i] = xf[i];
      if (Sa && Sa != Sf) {
        const int nr = (int)(i2 - i1);
        for (int idx = tid; idx < nr * N; idx += kThreads) {
          const int k = idx / nr, r = idx - k * nr;
          Sa[i1 + r + (int64_t)k * ldS] = Sf[i1 + r + (int64_t)k * ldS];
        }
      }
      continue;
    }
    const float* Tz = T + (int64_t)zl * N * N;
    const float* az = ampl + (int64_t)zl * N;
    for (int64_t r0 = i1; r0 < i2 && !stop; r0 += kRowsTile) {
      const int nr = (int)((i2 - r0) < kRowsTile ? (i2 - r0) : kRowsTile);
      for (int kb = 0; kb < nkb; kb++) {
        // global loads of this K-block, issued before the wait for the previous MMAs
        float av[4][4], bv[kBPer][4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const int kq = qa0 + 2 * j;
#pragma unroll
          for (int i = 0; i < 4; i++) {
            const int k = kb * kKB + 4 * kq + i;
            av[j][i] = (ra < nr && k < N) ? (float)Sf[r0 + ra + (int64_t)k * ldS] : 0.f;
          }
        }
#pragma unroll
        for (int j = 0; j < kBPer; j++) {
          const int idx = tid + kThreads * j;
          const int c = idx % NO, kq = idx / NO;
#pragma unroll
          for (int i = 0; i < 4; i++) {
            const int k = kb * kKB + 4 * kq + i;
            float v = 0.f;
            if (kq < kKB / 4 && k < N) v = (c < N) ? Tz[(int64_t)k * N + c] : (c == N ? az[k] : 0.f);
            bv[j][i] = v;
          }
        }
        if (pending) drain();
        __syncthreads();  // the tile is free (flag published)
        if (flag) {
          stop = true;
          break;
        }
#pragma unroll
        for (int j = 0; j < 4; j++) put_split(a_hi, a_lo, tile_off(ra, qa0 + 2 * j), av[j]);
#pragma unroll
        for (int j = 0; j < kBPer; j++) {
          const int idx = tid + kThreads * j;
          const int c = idx % NO, kq = idx / NO;
          if (kq < kKB / 4) put_split(b_hi, b_lo, tile_off(c, kq), bv[j]);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();  // tile complete
        if (tid == 0) {
          fence_after();
          const int ksteps = (N - kb * kKB) >= kKB ? kKB / 8 : (N - kb * kKB + 7) / 8;
          for (int kk = 0; kk < ksteps; kk++) {
            const uint32_t acc = (kb > 0 || kk > 0) ? 1u : 0u;
            const uint64_t dah = make_desc(a_hi_s + kk * 32), dal = make_desc(a_lo_s + kk * 32);
            const uint64_t dbh = make_desc(b_hi_s + kk * 32), dbl = make_desc(b_lo_s + kk * 32);
            mma_tf32(tmem, dah, dbh, idesc, acc);
            mma_tf32(tmem, dah, dbl, idesc, 1u);
            mma_tf32(tmem, dal, dbh, idesc, 1u);
          }
          mma_commit(mb);
        }
        pending = 1;
      }
      if (stop) break;
      drain();
      __syncthreads();  // MMAs complete (flag published)
      if (flag) {
        stop = true;
        break;
      }
      fence_after();
      // epilogue: warp w reads lanes 32 (w % 4) .. + 31 (rows), columns half w / 4
      {
        const int q = warp & 3, h = warp >> 2;
        const int r = 32 * q + lane;
        const uint32_t ta = tmem + ((uint32_t)(32 * q) << 16);
        const int half = NO / 2;
        for (int c0 = h * half; c0 < (h + 1) * half; c0 += 8) {
          float v[8];
          tmem_ld8(ta + (uint32_t)c0, v);
          if (r < nr) {
#pragma unroll
            for (int t = 0; t < 8; t++) {
              const int c = c0 + t;
              if (c < N) {
                if (Sa) Sa[r0 + r + (int64_t)c * ldS] = (S)v[t];
              } else if (c == N) {
                xa[r0 + r] = (S)((double)xf[r0 + r] + (double)v[t]);
              }
            }
          }
        }
      }
      fence_before();
      __syncthreads();  // accumulator read before the next tile's first MMA overwrites it
    }
  }
  // teardown: no MMA may still write tensor memory when it is freed
  if (pending) drain();
  if (tid == 0 && flag) atomicOr(err, ZST_TIMEOUT);
  fence_before();
  __syncthreads();
  fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(C::kCols));
}

template <int NB, typename S>
cudaError_t launch_update_tc(int N, int32_t z0, int32_t nzc, const int64_t* d_zone_start,
                             const S* xf, const S* Sf, int64_t ldS, const float* d_T,
                             const float* d_ampl, const int32_t* d_nobs, S* xa, S* Sa,
                             int32_t* d_err, cudaStream_t st) {
  using C = UpCfg<NB>;
  cudaError_t e = cudaFuncSetAttribute(k_zone_update_tc<NB, S>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)C::kDynSmem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_zone_update_tc<NB, S>,
                           cudaFuncAttributePreferredSharedMemoryCarveout,
                           (int)cudaSharedmemCarveoutMaxShared);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int grid = sms * C::kCtas;
  if (grid > nzc) grid = nzc > 0 ? nzc : 1;
  k_zone_update_tc<NB, S><<<grid, kThreads, C::kDynSmem, st>>>(
      N, z0, nzc, d_zone_start, xf, Sf, ldS, d_T, d_ampl, d_nobs, xa, Sa, d_err);
  count_launches(1);
  return cudaGetLastError();
}

template <typename S>
cudaError_t update_tc(int N, int32_t z0, int32_t nzc, const int64_t* d_zone_start,
                      const S* xf, const S* Sf, int64_t ldS, const float* d_T,
                      const float* d_ampl, const int32_t* d_nobs, S* xa, S* Sa,
                      int32_t* d_err, cudaStream_t st) {
  if (N < 2 || N > 128 || !d_err) return cudaErrorInvalidValue;
  if (N <= 64)
    return launch_update_tc<64, S>(N, z0, nzc, d_zone_start, xf, Sf, ldS, d_T, d_ampl, d_nobs,
                                   xa, Sa, d_err, st);
  return launch_update_tc<128, S>(N, z0, nzc, d_zone_start, xf, Sf, ldS, d_T, d_ampl, d_nobs,
                                  xa, Sa, d_err, st);
}

}  // namespace

cudaError_t zone_update_tc(int N, int32_t z0, int32_t nzc, const int64_t* d_zone_start,
                           const double* xf, const double* Sf, int64_t ldS, const float* d_T,
                           const float* d_ampl, const int32_t* d_nobs, double* xa, double* Sa,
                           int32_t* d_err, cudaStream_t st) {
  return update_tc<double>(N, z0, nzc, d_zone_start, xf, Sf, ldS, d_T, d_ampl, d_nobs, xa, Sa,
                           d_err, st);
}

cudaError_t zone_update_tc(int N, int32_t z0, int32_t nzc, const int64_t* d_zone_start,
                           const float* xf, const float* Sf, int64_t ldS, const float* d_T,
                           const float* d_ampl, const int32_t* d_nobs, float* xa, float* Sa,
                           int32_t* d_err, cudaStream_t st) {
  return update_tc<float>(N, z0, nzc, d_zone_start, xf, Sf, ldS, d_T, d_ampl, d_nobs, xa, Sa,
                          d_err, st);
}

}  // namespace oakg
