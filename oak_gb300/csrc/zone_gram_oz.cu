// The plain (FP64) form's products on the tensor cores, ensembles of up to 64 members: K1 + K2
// (selection and the Gram, k_zone_gram_oz) and E4 of the eigensolve (the square-root transform
// T = U (I+L)^-1/2 U^T Omega, k_zone_tsym_oz, further below).
//
// Selection and weights are those of zone_gram.cu (assimilation.F90:3683-3771): the relevance
// decisions of the tensor-core mixed kernel (FP32 distances away from the thresholds, the
// reference's FP64 evaluation near them; the selected set is identical to the plain form's),
// and for every selected observation the FP64 weight w of zone_gram.cu (FP64 distance,
// exp(-(d/L)^2) or locfun(d/L)). The Gram matrix G = HS_sel^T diag(c) HS_sel (rrsqrt.F90:135,
// c = w (w / r), DCDCovar of rrsqrt.F90:395) is formed as X^T X with X = diag(|w| / sqrt(r))
// HS_sel, in FP64, as an exact integer product on the BF16 tensor cores (the slice splitting
// of Ozaki et al., "Error-free transformations of matrix multiplication by using fast routines
// of matrix multiplication and its applications", Numer. Algorithms 59 (2012)):
//
//   Column a of X gets a fixed exponent E_a with |X_qa| <= 2^E_a for every observation q (from
//   max_q |HS_qa| / sqrt(r_q), once per call), so F_qa = round(X_qa 2^(54 - E_a)) is
//   an integer below 2^54 in magnitude, taken from the FP64 bit pattern with integer
//   operations. F is written in 7 balanced base-256 digits, F = sum_p d_p 256^(6-p) with
//   d_0 in [-64, 64] and d_1..d_6 in [-128, 127] (the bytes of F + 0x80808080808080 minus 128);
//   every digit is exact in BF16.
//   Then G_ab = 2^(E_a + E_b - 12) sum_L 256^-L level_L(a, b), level_L = sum_{p+q=L} D_p^T D_q
//   (D_p the digit-p matrix of the zone's rows), for levels 0..6. Levels 7..12 are left out:
//   a row adds at most 6 x 2^14 x 256^5 = 1.5 x 2^56 to level 7 against 2^108 = F_a F_b at the
//   column bounds, so they weigh at most ~2^-51.4 of 2^(E_a + E_b) a row when every digit sits
//   at its bound with one sign (far less for data). A K-tile of 64 observations is staged as
//   7 digit slices (64 members x 64 observations of BF16, K-major, 128-byte swizzle) and each
//   K-step of 16 observations issues tcgen05.mma kind::f16 (BF16 x BF16 -> FP32) with
//   A = [D_p ; D_(p+1)] (M = 128; only rows 0-63 are read back) and B = the run of slices whose
//   level block lands in the right accumulator column: levels 0..3 in tensor-memory columns
//   0..255 (4 MMAs a K-step), levels 4..6 in columns 256..447 (7 MMAs a K-step).
//   Exactness: a digit product is at most 2^14 (2^13 with d_0), so the FP32 sums of levels 0..3
//   stay exact integers below 2^24 over 256 observations; the accumulators are read every 4
//   K-tiles and added into 64-bit integer sums (levels 0..3) and an FP32 sum of
//   level_4 + level_5 / 256 + level_6 / 65536 (its FP32 rounding, about an ulp of level 4 per
//   read, weighs ~2^-52 of 2^(E_a + E_b) per 256 observations). At the end of the zone
//   G = 2^(E_a + E_b - 36) (v + V456 / 256) with v = ((L0 256 + L1) 256 + L2) 256 + L3 as a
//   64-bit integer, converted once to FP64. The error of G is therefore the rounding of X to
//   the fixed point (2^-54 of its column scale) and the dropped levels, not the length of the
//   sums: at most ~2^-51 of 2^(E_a + E_b) per term, typically near 2^-53 (the CPU model of
//   these steps, tests/test_slice_products_model.py, checks the bound and the budgets).
//
// The innovation projection g = X^T (sqrt(c) d) (rrsqrt.F90:142) is accumulated in FP64 by the
// staging threads (one FMA per staged element).
//
// Pipeline per CTA (one zone at a time, one CTA of 512 threads per SM: its shared memory and
// the 512 tensor-memory columns admit no second one): candidates are tested 512 at a time
// (a zone's cell-row ranges flattened into one index space);
// selected observations go to a ring, their FP64 weights are computed one thread an entry
// (|w| / sqrt(r) and w^2 / r (yo - Hxf)); every full K-tile is
// staged into one of two shared buffers (7 slices) and handed to the tensor core by one thread
// (44 MMAs and a commit to the buffer's mbarrier), so staging of the next tile overlaps the
// MMAs. Every mbarrier wait is bounded; on expiry the kernel records ZST_TIMEOUT, stops taking
// zones, waits (bounded) for its MMAs and frees its tensor memory.
#include <cuda_runtime.h>
#include <math.h>

#include "oakg_internal.cuh"
#include "selection.cuh"

namespace oakg {

namespace {

constexpr int kThreads = 512;
constexpr int NB = 64;                 // padded ensemble width
constexpr int KT = 64;                 // observations per K-tile (128 bytes of BF16 a row)
constexpr int kDigits = 7;
constexpr int kRing = 1024;            // selected-observation ring (power of two)
constexpr uint32_t kSliceBytes = 64u * 128u;         // one digit slice of a K-tile
constexpr uint32_t kBufBytes = kDigits * kSliceBytes;  // one K-tile buffer
constexpr uint32_t kTmemCols = 512;
constexpr int kWaitPolls = 1 << 22;
constexpr int kFlushTiles = 4;         // K-tiles between accumulator reads (256 observations)
constexpr int kTri = NB * (NB + 1) / 2;
constexpr int kLevelsExact = 4;        // levels held as 64-bit integer sums
constexpr int kStageGroups = kThreads / NB;  // threads a member in the staging (8-obs chunks)
constexpr unsigned long long kDigitBias = 0x80808080808080ull;
// dynamic shared memory: alignment slack, two K-tile buffers, the slice past the second buffer
// (rows 64-127 of the A operand of the last digit: read by the MMA, never read back), the
// integer and FP32 level sums (lower triangle) and the FP64 innovation partials
constexpr size_t kDynSmem = 1024 + 2 * (size_t)kBufBytes + kSliceBytes +
                            (size_t)kLevelsExact * kTri * sizeof(long long) +
                            (size_t)kTri * sizeof(float) + kStageGroups * NB * sizeof(double);

struct OzShared {
  int32_t ring_q[kRing];
  double ring_s[kRing];  // |w| / sqrt(r_q)
  double ring_t[kRing];  // w^2 / r_q (yo - Hxf)_q
  unsigned long long mbar[2];
  int32_t warp_cnt[kThreads / 32];
  int32_t rlo[kThreads];   // first observation of each candidate range of a block of ranges
  int32_t roff[kThreads];  // exclusive prefix of the ranges' lengths
  int32_t wpre[kThreads / 32];
  int32_t rtotal;
  int32_t E[NB];         // column exponents
  uint32_t tmem_base;
  int32_t zone;
  int32_t nrel;
  int32_t flag;
  int32_t bad;
  sel::ZoneCell32 zc;  // the zone's cell-relative FP32 coordinates (read by broadcast)
  sel::ScanRange sr;   // the zone's cell range
  double iL;           // 1 / L
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 bytes apart
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);  // start address
  d |= (uint64_t)1 << 16;                   // leading byte offset (unused: K fits one swizzle row)
  d |= (uint64_t)(1024u >> 4) << 32;        // stride byte offset
  d |= (uint64_t)1 << 46;                   // descriptor version
  d |= (uint64_t)2 << 61;                   // 128-byte swizzle
  return d;
}

// instruction descriptor: D F32, A and B BF16, both K-major, M = 128, N = n
__device__ __forceinline__ uint32_t idesc_bf16(uint32_t n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((128u >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accum) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %3, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %4, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(accum), "r"(idesc));
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   mbar)
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

// byte offset of the 16-byte chunk `chunk` (8 observations) of operand row `row` in a slice
__device__ __forceinline__ uint32_t tile_off(int row, int chunk) {
  return (uint32_t)((row >> 3) * 1024 + (row & 7) * 128 + ((chunk ^ (row & 7)) << 4));
}

// round(s h 2^(54 - E)) for s >= 0 (|s h| <= 2^E), from the FP64 bit patterns with integer
// arithmetic: the product of the two 53-bit significands is exact in 128 bits and rounded once
// (half away from zero) at the fixed-point position; no FP64 operation. *bad is set for a
// non-finite factor or a product above the bound.
__device__ __forceinline__ long long fixed_prod(double s, double h, int E, int& bad) {
  const unsigned long long sb = (unsigned long long)__double_as_longlong(s);
  const unsigned long long hb = (unsigned long long)__double_as_longlong(h);
  const int es = (int)((sb >> 52) & 0x7FFu), eh = (int)((hb >> 52) & 0x7FFu);
  if (es == 0x7FF || eh == 0x7FF) {
    bad = 1;
    return 0;
  }
  if (es == 0 || eh == 0) return 0;  // a zero or subnormal factor (far under the column scale)
  const unsigned long long ms = (sb & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
  const unsigned long long mh = (hb & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
  // s h 2^(54 - E) = ms mh 2^(es + eh - 2150 + 54 - E) = P 2^-r, P = ms mh < 2^106
  const int r = 2096 + E - es - eh;
  if (r >= 107) return 0;  // below half a unit of the fixed point
  if (r < 50) {            // at least 2^54: above the bound
    bad = 1;
    return 0;
  }
  unsigned long long lo = ms * mh, hi = __umul64hi(ms, mh);
  // P + 2^(r-1), then >> r
  if (r - 1 < 64) {
    const unsigned long long add = 1ull << (r - 1);
    const unsigned long long lo2 = lo + add;
    hi += (lo2 < lo) ? 1ull : 0ull;
    lo = lo2;
  } else {
    hi += 1ull << (r - 1 - 64);
  }
  const unsigned long long F = (r < 64) ? ((hi << (64 - r)) | (lo >> r)) : (hi >> (r - 64));
  if (F > (1ull << 54)) {
    bad = 1;
    return 0;
  }
  return (hb >> 63) ? -(long long)F : (long long)F;
}

// BF16 bits of the digit (byte - 128), exact: the FP32 value has at most 8 significant bits
__device__ __forceinline__ uint32_t digit_bits(uint32_t byte) {
  return __float_as_uint(__uint_as_float(0x4B3FFF80u + byte) - 12582912.f);
}

// 64-bit-integer / FP32 lower-triangle index of (row j, column c <= j)
__device__ __forceinline__ int tri(int j) { return j * (j + 1) / 2; }

__global__ void __launch_bounds__(kThreads, 1)
    k_zone_gram_oz(CellGrid g, SortedObs so, int N, LocParams lp, int32_t z0, int32_t nzc,
                   const double* __restrict__ zone_xyzt, const double* __restrict__ corr_len,
                   const double* __restrict__ max_len, const int32_t* __restrict__ col_exp,
                   const double* __restrict__ isr, double* __restrict__ G,
                   double* __restrict__ gv, int32_t* __restrict__ nobs, int brute, int32_t* __restrict__ work, int32_t* __restrict__ err,
                   const int32_t* __restrict__ order) {
  extern __shared__ __align__(16) unsigned char dyn_raw[];
  __shared__ __align__(16) OzShared ts;
  const uint32_t raw_addr = smem_u32(dyn_raw);
  const uint32_t pad = ((raw_addr + 1023u) & ~1023u) - raw_addr;
  unsigned char* tiles = dyn_raw + pad;  // 2 x kBufBytes + one slice, 1024-aligned
  const uint32_t tile_addr = raw_addr + pad;
  long long* acc64 = reinterpret_cast<long long*>(tiles + 2 * kBufBytes + kSliceBytes);
  float* accf = reinterpret_cast<float*>(acc64 + kLevelsExact * kTri);
  double* gpart = reinterpret_cast<double*>(accf + kTri);  // [kStageGroups][NB]

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // staging: member a, 8-observation chunk kq of a K-tile
  const int a = tid & (NB - 1), kq = tid >> 6;
  const uint32_t mbar0 = smem_u32(&ts.mbar[0]);

  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar0));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar0 + 8));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    ts.flag = 0;
  }
  if (tid < NB) ts.E[tid] = (tid < N) ? col_exp[tid] : 0;
  // the slice past the second buffer is only read into accumulator rows that are never read
  // back; it is cleared once so that those rows hold finite values
  for (uint32_t i = tid; i < kSliceBytes / 16; i += kThreads)
    reinterpret_cast<uint4*>(tiles + 2 * kBufBytes)[i] = make_uint4(0, 0, 0, 0);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&ts.tmem_base)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = ts.tmem_base;
  const int Ea = ts.E[a];

  const int64_t ncells = (int64_t)g.nu * g.nv;
  const int full_scan = brute || !lp.localise;
  const bool fast = (lp.loctype != 1) || (lp.metric == OAKG_METRIC_CARTESIAN);
  int pend0 = 0, pend1 = 0;   // buffer has MMAs not yet waited for (uniform)
  uint32_t ph0 = 0, ph1 = 0;  // parity of the buffer's next completion (uniform)
  bool abort = false;

  // wait for buffer b's outstanding MMAs (thread 0, bounded); result published in ts.flag
  auto drain = [&](int b) {
    if (tid == 0) {
      const uint32_t ph = b ? ph1 : ph0;
      if (!mbar_wait(mbar0 + 8 * b, ph)) ts.flag = 1;
    }
    if (b) {
      ph1 ^= 1u;
      pend1 = 0;
    } else {
      ph0 ^= 1u;
      pend0 = 0;
    }
  };

  // add the accumulators into the level sums (all MMAs complete and published by a barrier).
  // Warp w reads lanes 32 (w % 4) .. + 31, i.e. rows j of the lower (D_p) half for w % 4 < 2;
  // warp group h = w / 4 takes levels 2h, 2h + 1 (h < 2) or 4..6 (h = 2); row j keeps columns
  // c <= j.
  auto flush = [&]() {
    fence_after();
    const int q = warp & 3, h = warp >> 2;
    if (q < 2 && h < 3) {
      const int j = 32 * q + lane;
      const uint32_t ta = tmem + ((uint32_t)(32 * q) << 16);
      const int ncol = 32 * (q + 1);  // warp-uniform bound of the row's lower triangle
      const int tj = tri(j);
      if (h < 2) {
#pragma unroll
        for (int L = 2 * h; L < 2 * h + 2; L++) {
          long long* accL = acc64 + L * kTri + tj;
          for (int c0 = 0; c0 < ncol; c0 += 8) {
            float v[8];
            tmem_ld8(ta + 64 * L + c0, v);
#pragma unroll
            for (int t = 0; t < 8; t++)
              if (c0 + t <= j) accL[c0 + t] += (long long)__float2int_rn(v[t]);
          }
        }
      } else {
        float* af = accf + tj;
        for (int c0 = 0; c0 < ncol; c0 += 8) {
          float v4[8], v5[8], v6[8];
          tmem_ld8(ta + 256 + c0, v4);
          tmem_ld8(ta + 320 + c0, v5);
          tmem_ld8(ta + 384 + c0, v6);
#pragma unroll
          for (int t = 0; t < 8; t++)
            if (c0 + t <= j) af[c0 + t] += fmaf(v6[t], 1.f / 65536.f, fmaf(v5[t], 1.f / 256.f, v4[t]));
        }
      }
    }
    fence_before();
    __syncthreads();
  };

  for (;;) {
    if (tid == 0) ts.zone = atomicAdd(work, 1);
    __syncthreads();
    const int32_t w = ts.zone;  // pick number; zone order[z0 + w] when a pick order is given
    if (w >= nzc || ts.flag) break;
    const int32_t zl = order ? order[z0 + w] : w;
    const int32_t z = z0 + zl;
    const double zx = zone_xyzt[4 * (int64_t)z + 0], zy = zone_xyzt[4 * (int64_t)z + 1];
    const double zzc = zone_xyzt[4 * (int64_t)z + 2], ztc = zone_xyzt[4 * (int64_t)z + 3];
    const double zu = (lp.loctype == 1) ? zx : (lp.loctype == 2 ? zzc : ztc);
    const double zv = (lp.loctype == 1) ? zy : 0.0;
    const double L = corr_len[z], Rmax = max_len[z];
    // the FP32 distance (relative error < 1e-6, sel::ZoneCell32) decides outside a 3e-6 band
    const float r_lo = (float)Rmax * (1.f - 3e-6f), r_hi = (float)Rmax * (1.f + 3e-6f);
    // the zone's FP64 set-up (divisions, floors) once, by one thread
    if (tid == 0) {
      ts.nrel = 0;
      ts.bad = 0;
      ts.zc = sel::zone_cell32(g, zu, zv, Rmax);
      ts.iL = 1.0 / L;
      if (full_scan) {
        ts.sr.cu0 = 0;
        ts.sr.cu1 = g.nu - 1;
        ts.sr.cv0 = 0;
        ts.sr.cv1 = g.nv - 1;
        ts.sr.all_u = 1;
      } else {
        ts.sr = sel::zone_scan_range(g, lp.metric, lp.loctype, zu, zv, Rmax);
      }
    }
    __syncthreads();  // ts.zc, ts.sr, ts.iL published (read only in this zone's scan)
    const sel::ZoneCell32 zc = ts.zc;
    const bool fastz = fast && zc.ok && !brute;  // brute force: one cell, no local offsets
    const double iL = ts.iL, iL2 = iL * iL;
    const float iL32 = (float)iL;
    for (int e = tid; e < kLevelsExact * kTri; e += kThreads) acc64[e] = 0;
    for (int e = tid; e < kTri; e += kThreads) accf[e] = 0.f;
    int head = 0, tail = 0, ntile = 0, ctile = 0, nrel_local = 0, bad = 0;
    double gsum = 0.0, gsum1 = 0.0;

    // stage ring entries [head, head + rows) as one K-tile and issue its MMAs
    auto do_tile = [&](int rows) {
      if (ctile == kFlushTiles) {
        if (pend0) drain(0);
        if (pend1) drain(1);
        __syncthreads();  // MMA completion and flag published
        if (ts.flag) {
          abort = true;
          return;
        }
        flush();
        ctile = 0;
      }
      const int b = ntile & 1;
      if (b ? pend1 : pend0) drain(b);
      __syncthreads();  // buffer free (flag published), ring entries visible
      if (ts.flag) {
        abort = true;
        return;
      }
      unsigned char* tb = tiles + b * kBufBytes;
#pragma unroll 1
      for (int pass = 0; pass < KT / 8 / kStageGroups; pass++) {
        const int chunk = kq + kStageGroups * pass;
        uint32_t pk[kDigits][4];
        // the chunk's 8 elements loaded first (independent loads in flight together)
        double hv[8], sv[8];
#pragma unroll
        for (int i = 0; i < 8; i++) {
          const int k = 8 * chunk + i;
          hv[i] = 0.0;
          sv[i] = 0.0;
          if (k < rows && a < N) {
            const int idx = (head + k) & (kRing - 1);
            hv[i] = so.HSt[(int64_t)ts.ring_q[idx] * N + a];
            sv[i] = ts.ring_s[idx];
            // two accumulators (even / odd observations): shorter FMA chains
            if (i & 1)
              gsum1 = fma(hv[i], ts.ring_t[idx], gsum1);
            else
              gsum = fma(hv[i], ts.ring_t[idx], gsum);
          }
        }
#pragma unroll
        for (int i = 0; i < 8; i += 2) {
          uint32_t lo2[2], hi2[2];
#pragma unroll
          for (int u = 0; u < 2; u++) {
            const long long F = fixed_prod(sv[i + u], hv[i + u], Ea, bad);
            const unsigned long long U = (unsigned long long)F + kDigitBias;
            lo2[u] = (uint32_t)U;
            hi2[u] = (uint32_t)(U >> 32);
          }
          const int wd = i >> 1;
          // digit p is byte 6 - p of U: p = 0..2 in the high word, 3..6 in the low word
#pragma unroll
          for (int p = 0; p < kDigits; p++) {
            const int byte = 6 - p;
            const uint32_t b0 = (byte >= 4) ? (hi2[0] >> (8 * (byte - 4))) & 255u
                                            : (lo2[0] >> (8 * byte)) & 255u;
            const uint32_t b1 = (byte >= 4) ? (hi2[1] >> (8 * (byte - 4))) & 255u
                                            : (lo2[1] >> (8 * byte)) & 255u;
            pk[p][wd] = __byte_perm(digit_bits(b0), digit_bits(b1), 0x7632);
          }
        }
#pragma unroll
        for (int p = 0; p < kDigits; p++)
          *reinterpret_cast<uint4*>(tb + p * kSliceBytes + tile_off(a, chunk)) =
              make_uint4(pk[p][0], pk[p][1], pk[p][2], pk[p][3]);
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncthreads();  // tile complete
      if (tid == 0) {
        fence_after();
        const uint32_t base = tile_addr + b * kBufBytes;
#pragma unroll 1
        for (int kk = 0; kk < KT / 16; kk++) {
          const uint32_t ko = kk * 32;
          const uint32_t acc0 = (ctile > 0 || kk > 0) ? 1u : 0u;
          // levels 0..3, columns 64 L: A = [D_p ; D_p+1], B = D_0 .. D_(3-p) into L = p .. 3
#pragma unroll
          for (int p = 0; p < 4; p++)
            mma_bf16(tmem + 64 * p, make_desc(base + p * kSliceBytes + ko), make_desc(base + ko),
                     idesc_bf16(64u * (4 - p)), p == 0 ? acc0 : 1u);
          // levels 4..6, columns 256 + 64 (L - 4): B = D_qlo .. D_qhi, q = L - p
#pragma unroll
          for (int p = 0; p < kDigits; p++) {
            const int qlo = (4 - p > 0) ? 4 - p : 0;
            const int qhi = (6 - p < kDigits - 1) ? 6 - p : kDigits - 1;
            const int off = qlo - (4 - p);
            mma_bf16(tmem + 256 + 64 * off, make_desc(base + p * kSliceBytes + ko),
                     make_desc(base + qlo * kSliceBytes + ko),
                     idesc_bf16(64u * (qhi - qlo + 1)), p == 0 ? acc0 : 1u);
          }
        }
        mma_commit(mbar0 + 8 * b);
      }
      if (b)
        pend1 = 1;
      else
        pend0 = 1;
      ntile++;
      ctile++;
      head += rows;
    };

    const sel::ScanRange sr = ts.sr;
    // The zone's candidates are the observations of cell rows cv0..cv1, each row one or (a
    // periodic u axis wrapping) two contiguous ranges of the cell-sorted order. Range ri is
    // (row cv0 + ri / 2, part ri % 2); blocks of kThreads ranges are flattened into one index
    // space (exclusive prefix of their lengths), so that a pass of kThreads threads takes
    // kThreads candidates across rows in the order of the rows. The order, and so the ring
    // and the selection, are those of a row-by-row scan.
    const int nranges = 2 * (sr.cv1 - sr.cv0 + 1);
    for (int rbase = 0; rbase < nranges && !abort; rbase += kThreads) {
      {
        const int ri = rbase + tid;
        int32_t rq0 = 0, rlen = 0;
        if (ri < nranges) {
          const int cv = sr.cv0 + (ri >> 1), part = ri & 1;
          int cu_a = 0, cu_b = -1;
          if (sr.all_u) {
            if (!part) cu_b = g.nu - 1;
          } else if (!g.periodic_u) {
            if (!part) {
              cu_a = sr.cu0;
              cu_b = sr.cu1;
            }
          } else {
            const int a0 = sr.cu0, b0 = sr.cu1;
            if (a0 < 0) {
              cu_a = part ? 0 : a0 + g.nu;
              cu_b = part ? b0 : g.nu - 1;
            } else if (b0 >= g.nu) {
              cu_a = part ? 0 : a0;
              cu_b = part ? b0 - g.nu : g.nu - 1;
            } else if (!part) {
              cu_a = a0;
              cu_b = b0;
            }
          }
          const int64_t c_lo = (int64_t)cu_a + (int64_t)g.nu * cv;
          const int64_t c_hi = (int64_t)cu_b + (int64_t)g.nu * cv;
          if (c_lo <= c_hi && c_lo >= 0 && c_hi < ncells) {
            rq0 = so.cell_start[c_lo];
            rlen = so.cell_start[c_hi + 1] - rq0;
          }
        }
        int incl = rlen;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int t = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += t;
        }
        if (lane == 31) ts.warp_cnt[warp] = incl;
        __syncthreads();
        if (warp == 0) {
          const int wsum = (lane < kThreads / 32) ? ts.warp_cnt[lane] : 0;
          int winc = wsum;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, winc, o);
            if (lane >= o) winc += t;
          }
          if (lane < kThreads / 32) ts.wpre[lane] = winc - wsum;
          if (lane == 31) ts.rtotal = winc;
        }
        __syncthreads();
        ts.rlo[tid] = rq0;
        ts.roff[tid] = ts.wpre[warp] + incl - rlen;
        __syncthreads();
      }
      const int32_t ncand = ts.rtotal;
      const int nr = min(kThreads, nranges - rbase);
      for (int32_t gb = 0; gb < ncand && !abort; gb += kThreads) {
        const int32_t gi = gb + tid;
        int32_t q = 0;
        int cv = sr.cv0;
        const bool valid = gi < ncand;
        if (valid) {
          // the last range starting at or before gi (empty ranges share the next one's start)
          int lo_i = 0, hi_i = nr - 1;
          while (lo_i < hi_i) {
            const int mid = (lo_i + hi_i + 1) >> 1;
            if (ts.roff[mid] <= gi) lo_i = mid;
            else hi_i = mid - 1;
          }
          q = ts.rlo[lo_i] + (gi - ts.roff[lo_i]);
          cv = sr.cv0 + ((rbase + lo_i) >> 1);
        }
        int sel = 0, rel = 0;
        if (valid) {
          // FP32 decisions away from the thresholds, the reference's FP64 evaluation near them
          bool done = false;
          if (fastz) {
            const float d32 = sel::cell_distance32(zc, so, q, cv, lp.loctype == 1);
            const int inside = (d32 <= r_lo) ? 1 : ((d32 >= r_hi) ? 0 : -1);
            if (inside >= 0) {
              const float r32 = d32 * iL32;
              if (lp.weight == OAKG_WEIGHT_GAUSS_CUTOFF) {
                rel = inside;
                done = true;
              } else if (r32 >= 2.f + 1e-5f) {  // locfun = 0
                rel = 0;
                done = true;
              } else if (r32 <= 2.f - 1e-3f) {  // locfun > 3e-13, far above its FP64 rounding
                rel = inside;
                done = true;
              }
            }
          }
          if (!done) {
            double d;
            if (lp.loctype == 1)
              d = sel::distance(so.u[q], so.v[q], zu, zv, lp.metric);
            else
              d = fabs(__dsub_rn(so.u[q], zu));
            if (lp.weight == OAKG_WEIGHT_GAUSS_CUTOFF) {
              rel = (d <= Rmax);
            } else {
              rel = (d <= Rmax) && (sel::locfun(d / L) != 0.0);
            }
          }
          sel = rel || !lp.localise;
        }
        nrel_local += rel;
        const unsigned ball = __ballot_sync(0xffffffffu, sel);
        if (lane == 0) ts.warp_cnt[warp] = __popc(ball);
        __syncthreads();
        int before = 0, total = 0;
#pragma unroll
        for (int w2 = 0; w2 < kThreads / 32; w2++) {
          const int cnt = ts.warp_cnt[w2];
          before += (w2 < warp) ? cnt : 0;
          total += cnt;
        }
        if (sel) {
          const int slot = (tail + before + __popc(ball & ((1u << lane) - 1u))) & (kRing - 1);
          ts.ring_q[slot] = q;
        }
        __syncthreads();
        // the plain form's FP64 weights of the new entries (zone_gram.cu), one thread an
        // entry, so that the FP64 work runs with full warps: sqrt(c) = |w| / sqrt(r)
        // (c = w (w / r), DCDCovar, covariance.F90:612-619) and c (yo - Hxf). The values
        // (not the decisions, made above with the reference's rounding) are evaluated with
        // fewer FP64 operations for the Cartesian and 1-D distances: exp(-d^2 / L^2) needs
        // no square root or division, locfun(sqrt(d^2) / L) takes 1/L once a zone.
        if (tid < total) {
          const int slot = (tail + tid) & (kRing - 1);
          const int32_t qs = ts.ring_q[slot];
          double w64;
          if (fast) {
            const double du = so.u[qs] - zu;
            double D2 = du * du;
            if (lp.loctype == 1) {
              const double dv = so.v[qs] - zv;
              D2 = fma(dv, dv, D2);
            }
            w64 = (lp.weight == OAKG_WEIGHT_GAUSS_CUTOFF) ? exp(-(D2 * iL2))
                                                          : sel::locfun_value(sqrt(D2) * iL);
          } else {
            double d;
            if (lp.loctype == 1)
              d = sel::distance(so.u[qs], so.v[qs], zu, zv, lp.metric);
            else
              d = fabs(__dsub_rn(so.u[qs], zu));
            if (lp.weight == OAKG_WEIGHT_GAUSS_CUTOFF) {
              const double t = d / L;
              w64 = exp(-(t * t));
            } else {
              w64 = sel::locfun(d / L);
            }
          }
          const double sc = fabs(w64) * isr[qs];
          ts.ring_s[slot] = sc;
          ts.ring_t[slot] = sc * sc * so.innov[qs];
        }
        tail += total;
        while (tail - head >= KT && !abort) do_tile(KT);
      }
      __syncthreads();  // the block's ranges consumed before the next block overwrites them
    }
    if (!abort && tail > head) do_tile(tail - head);
    if (abort) break;
    // relevant-observation count of the zone
    for (int o = 16; o > 0; o >>= 1) nrel_local += __shfl_xor_sync(0xffffffffu, nrel_local, o);
    if (lane == 0) atomicAdd(&ts.nrel, nrel_local);
    if (bad) atomicOr(&ts.bad, 1);
    gpart[kq * NB + a] = gsum + gsum1;
    if (ntile > 0) {
      if (pend0) drain(0);
      if (pend1) drain(1);
    }
    __syncthreads();  // nrel, bad, partials and the MMA completion published
    if (ts.flag) break;
    const int nrel = ts.nrel;
    if (tid == 0) nobs[z] = nrel;
    if (nrel > 0 && ntile > 0) {
      flush();
      double* Gz = G + (int64_t)zl * N * N;
      const bool zbad = ts.bad != 0;
      for (int e = tid; e < kTri; e += kThreads) {
        int j = (int)((__fsqrt_rn((float)(8 * e + 1)) - 1.0f) * 0.5f);
        while ((j + 1) * (j + 2) / 2 <= e) j++;
        while (j * (j + 1) / 2 > e) j--;
        const int c = e - tri(j);
        if (j >= N) continue;
        const long long v =
            ((acc64[e] * 256 + acc64[kTri + e]) * 256 + acc64[2 * kTri + e]) * 256 +
            acc64[3 * kTri + e];
        // 2^(E_j + E_c - 36), a power of two in the normal range for any practical scale
        int ex = ts.E[j] + ts.E[c] - 36 + 1023;
        ex = ex < 1 ? 1 : (ex > 2046 ? 2046 : ex);
        const double scale = __longlong_as_double((long long)ex << 52);
        double val = fma((double)accf[e], 1.0 / 256.0, (double)v) * scale;
        if (zbad) val = __longlong_as_double(0x7FF8000000000000ll);  // NaN: non-finite input
        Gz[j * N + c] = val;
        Gz[c * N + j] = val;
      }
      if (tid < N) {
        double gs = 0.0;
#pragma unroll
        for (int p = 0; p < kStageGroups; p++) gs += gpart[p * NB + tid];
        gv[(int64_t)zl * N + tid] = gs;
      }
    }
    __syncthreads();  // G staging and partials consumed before the next zone's tiles
  }
  // teardown: no MMA may still write tensor memory when it is freed
  if (pend0) drain(0);
  if (pend1) drain(1);
  if (tid == 0 && ts.flag) atomicOr(err, ZST_TIMEOUT);
  fence_before();
  __syncthreads();
  fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTmemCols));
}

// isr_q = r_q^-1/2 and the column exponents: E_a with max_q |HS_qa| isr_q (1 + 2^-20) <= 2^E_a
// (|w| <= 1, so every |X_qa| of every zone is below it). The maxima of non-negative FP64
// values are taken on their bit patterns (ordered like the values). Non-finite values and
// r <= 0 are left out: the zones that select such an observation get a non-finite weight or
// element, which marks their G as NaN (as the CUDA-core products would propagate it); the
// other zones keep the scale of the finite data.
__global__ void k_oz_colmax(int64_t m, int N, const double* __restrict__ HSt,
                            const double* __restrict__ r, unsigned long long* __restrict__ mx,
                            double* __restrict__ isr) {
  __shared__ unsigned long long smax[NB];
  if (threadIdx.x < NB) smax[threadIdx.x] = 0ull;
  __syncthreads();
  const int a = threadIdx.x & (NB - 1);
  unsigned long long loc = 0ull;
  if (a < N) {
    for (int64_t q = blockIdx.x * (int64_t)(blockDim.x / NB) + threadIdx.x / NB; q < m;
         q += (int64_t)gridDim.x * (blockDim.x / NB)) {
      const double rq = r[q];
      const double iq = rsqrt(rq);
      if (a == 0) isr[q] = iq;
      if (!(rq > 0.0) || !(rq < INFINITY)) continue;
      const double v = fabs(HSt[q * N + a]) * iq;
      const unsigned long long vb = (unsigned long long)__double_as_longlong(v);
      if (vb < 0x7FF0000000000000ull) loc = vb > loc ? vb : loc;
    }
    atomicMax(&smax[a], loc);
  }
  __syncthreads();
  if (threadIdx.x < N) atomicMax(&mx[threadIdx.x], smax[threadIdx.x]);
}

__global__ void k_oz_exponents(int N, const unsigned long long* __restrict__ mx,
                               int32_t* __restrict__ E) {
  const int a = threadIdx.x;
  if (a >= N) return;
  const double vmax = __longlong_as_double((long long)mx[a]);
  int e;
  if (vmax == 0.0) {
    e = 0;  // an all-zero column (or no usable observation)
  } else {
    const double v = vmax * (1.0 + 0x1p-20);
    if (!(v < INFINITY)) {
      e = -4000;  // beyond the FP64 range: every nonzero element is out of range (G is NaN)
    } else {
      // v in [2^(k-1), 2^k) with k = biased exponent - 1022 (normal v)
      const int be = (int)(((unsigned long long)__double_as_longlong(v) >> 52) & 0x7FF);
      e = (be == 0) ? -1022 : be - 1022;
    }
  }
  E[a] = e;
}

// ------------------------------------------------------------------ square-root transform
// The plain form's T_sym = U diag((1 + lambda)^-1/2) U^T (rrsqrt.F90:162-169) as the Gram X^T X
// of X_ka = q_k U_ak, q_k = (1 + lambda_k)^-1/4: row k of X is eigenvector k scaled, so a zone
// is one K-tile of 64 rows and the slice products of k_zone_gram_oz apply unchanged. With one
// K-tile every level (at most 7 x 64 x 2^14 < 2^23 in magnitude) is exact in its FP32
// accumulator, and one read of the tensor memory gives T_sym = 2^(E_a + E_b - 36) (v + V456 /
// 256), recombined here as the integer v 2^16 + round(256 V456) (below 2^62) with one
// conversion to FP64. Column exponents come from the exponent fields: a normal x lies below
// 2^(e(x) - 1022) (e the biased exponent), so E_a = max_k (e(q_k) + e(U_ak)) - 2044 bounds
// |X_ka| (at most two bits above the column's maximum) and every product fits the fixed point.
//
// T = T_sym Omega (rrsqrt.F90:171-185) follows in FP64. Omega = P_v P_w + (1 - s_v s_w) v w^T
// with P_x = I - u_x u_x^T / c_x, u_x = x + s_x e_N, c_x = 1 + |x_N| (matoper.F90:509-535;
// w = N^-1/2 1, s_w = 1), so T = T_sym - a u_v^T - g u_w^T + b w^T is a rank-three update
// with a = T_sym u_v / c_v, g = (T_sym u_w - (u_v . u_w) a) / c_w and b = (1 - s_v) T_sym v.
// T_sym v and the row sums (T_sym u_w = w rowsum + T_sym e_N) are accumulated while T_sym is
// formed; the update is then one FMA and one add an element.
// Pipeline per CTA (one of 512 threads per SM, zones strided): while zone i's MMAs run, zone
// i + 1's U and scalings are copied into shared memory (cp.async); after zone i's accumulator
// read, zone i + 1 is split and its MMAs issued, and zone i's rotation and T write run beside
// them. The levels are recombined into FP64 by integer operations (the FP64 pipe carries only
// the rotation's sums and update). The shared-memory request keeps a second CTA (which would
// wait for the tensor memory) off the SM.
constexpr int kTsLd = NB + 1;
constexpr size_t kTsData = 1024 + (size_t)kBufBytes + kSliceBytes +
                           (size_t)NB * kTsLd * sizeof(double) + (size_t)NB * NB * sizeof(double) +
                           18 * NB * sizeof(double);
constexpr size_t kTsDynSmem = (size_t)148 * 1024;
static_assert(kTsData <= kTsDynSmem, "square-root transform shared memory");

struct TsShared {
  unsigned long long mbar;
  uint32_t tmem_base;
  int32_t emax[NB];  // max_k e(q_k) + e(U_ak) of the zone being split
  int32_t E[NB];     // column exponents of the zone in the accumulators
  int32_t flag;
  int32_t bad[2];    // non-finite input, by zone parity
  double uvuw;       // u_v . u_w of the current zone
};

__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;" ::: "memory");
}

// vt 2^e2 rounded to nearest even, by integer operations (the conversion and scaling FP64
// instructions avoided); |vt| < 2^63. Outside FP64's normal range the FP64 operations decide.
__device__ __forceinline__ double scaled_i64(long long vt, int e2) {
  if (vt == 0) return 0.0;
  const unsigned long long sgn = vt < 0 ? (1ull << 63) : 0ull;
  const unsigned long long m = vt < 0 ? (unsigned long long)(-vt) : (unsigned long long)vt;
  const int lz = __clzll((long long)m);
  const int be = 63 - lz + e2 + 1023;
  if (be < 1 || be > 2045) {
    int ex = e2 + 1023;
    ex = ex < 1 ? 1 : (ex > 2046 ? 2046 : ex);
    return (double)vt * __longlong_as_double((long long)ex << 52);
  }
  const unsigned long long mm = m << lz;  // leading one at bit 63
  const unsigned long long mant = (mm >> 11) & 0xFFFFFFFFFFFFFull;
  const unsigned long long rem = mm & 0x7FFull;
  const unsigned long long up = (rem > 0x400ull || (rem == 0x400ull && (mant & 1ull))) ? 1ull : 0ull;
  return __longlong_as_double((long long)(sgn | (((unsigned long long)be << 52) + mant + up)));
}

// the seven levels' 8 columns at c0 of this warp's 32 lanes: seven loads, one wait; the empty
// asm statements tie the registers' uses to the wait
__device__ __forceinline__ void tmem_ld7x8(uint32_t ta, int c0, uint32_t (&r)[56]) {
  const uint32_t cols[7] = {0u, 64u, 128u, 192u, 256u, 320u, 384u};
#pragma unroll
  for (int L = 0; L < 7; L++)
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=r"(r[8 * L]), "=r"(r[8 * L + 1]), "=r"(r[8 * L + 2]), "=r"(r[8 * L + 3]),
          "=r"(r[8 * L + 4]), "=r"(r[8 * L + 5]), "=r"(r[8 * L + 6]), "=r"(r[8 * L + 7])
        : "r"(ta + cols[L] + (uint32_t)c0));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int q = 0; q < 56; q += 14)
    asm volatile(""
                 : "+r"(r[q]), "+r"(r[q + 1]), "+r"(r[q + 2]), "+r"(r[q + 3]), "+r"(r[q + 4]),
                   "+r"(r[q + 5]), "+r"(r[q + 6]), "+r"(r[q + 7]), "+r"(r[q + 8]),
                   "+r"(r[q + 9]), "+r"(r[q + 10]), "+r"(r[q + 11]), "+r"(r[q + 12]),
                   "+r"(r[q + 13])
                 :
                 : "memory");
}

__global__ void __launch_bounds__(kThreads, 1)
    k_zone_tsym_oz(int N, int32_t nzc, double* __restrict__ GT, const double* __restrict__ aux,
                   const double* __restrict__ Zg, const int32_t* __restrict__ nobs, int rotate,
                   int32_t* __restrict__ status) {
  extern __shared__ __align__(16) unsigned char dyn_raw[];
  __shared__ __align__(16) TsShared ts;
  const uint32_t raw_addr = smem_u32(dyn_raw);
  const uint32_t pad = ((raw_addr + 1023u) & ~1023u) - raw_addr;
  unsigned char* tile = dyn_raw + pad;  // the 7 slices and the zero slice past them
  const uint32_t tile_addr = raw_addr + pad;
  double* Ts = reinterpret_cast<double*>(tile + kBufBytes + kSliceBytes);  // [NB][kTsLd]
  double* Upre = Ts + NB * kTsLd;  // next zone's U slot, as stored (U_ak at k N + a)
  double* qpre = Upre + NB * NB;   // next zone's (1 + lambda)^-1/4
  double* vpre = qpre + NB;        // next zone's v
  double* vvb = vpre + NB;         // [2][NB] v by zone parity
  double* uv = vvb + 2 * NB;       // u_v of the current zone
  double* pv = uv + NB;            // [4][NB] partial T_sym v (column groups)
  double* ps = pv + 4 * NB;        // [4][NB] partial row sums
  double* ar = ps + 4 * NB;        // a
  double* cr = ar + NB;            // (b - g) w
  double* gr = cr + NB;            // g
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int a = tid & (NB - 1), kq = tid >> 6;  // member a; rows 8 kq .. 8 kq + 7 of X
  const uint32_t mbar = smem_u32(&ts.mbar);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    ts.flag = 0;
  }
  if (tid < NB) ts.emax[tid] = 0;
  // rows 64-127 of the last digit's A operand: read by the MMA, never read back
  for (uint32_t i = tid; i < kSliceBytes / 16; i += kThreads)
    reinterpret_cast<uint4*>(tile + kBufBytes)[i] = make_uint4(0, 0, 0, 0);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&ts.tmem_base)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = ts.tmem_base;
  const double wv = 1.0 / sqrt((double)N);
  const double cw = 1.0 + wv, icw = 1.0 / cw;
  const int nmine = (nzc - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x;
  uint32_t ph = 0;
  bool pending = false;  // an MMA group whose completion was not observed (timeout)

  // zone number i of this CTA's share into Upre / qpre / vpre (asynchronous copies)
  auto prefetch = [&](int i) {
    const int32_t zn = (int32_t)blockIdx.x + i * (int32_t)gridDim.x;
    const double* src = Zg + (int64_t)zn * N * N;
    for (int idx = tid; idx < N * N; idx += kThreads) cp_async8(Upre + idx, src + idx);
    const double* axn = aux + (int64_t)zn * (5 * N + 2);
    if (tid < N) {
      cp_async8(qpre + tid, axn + 4 * N + tid);
      cp_async8(vpre + tid, axn + tid);
    }
  };
  // split the prefetched zone (parity par) into the slices and issue its MMAs; its copies
  // have landed and are visible (a barrier since this thread's cp_async_wait_all)
  auto stage_issue = [&](int par) {
    double hv[8], sv[8];
    int em = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) {
      const int k = 8 * kq + i;
      hv[i] = (a < N && k < N) ? Upre[k * N + a] : 0.0;
      sv[i] = (k < N) ? qpre[k] : 0.0;
      const int es = (int)(((unsigned long long)__double_as_longlong(sv[i]) >> 52) & 0x7FFu);
      const int eh = (int)(((unsigned long long)__double_as_longlong(hv[i]) >> 52) & 0x7FFu);
      if (es != 0 && eh != 0 && es != 0x7FF && eh != 0x7FF) em = max(em, es + eh);
    }
    if (em > 0) atomicMax(&ts.emax[a], em);
    if (tid == 0) ts.bad[par] = 0;
    if (tid < NB) vvb[par * NB + tid] = (rotate && tid < N) ? vpre[tid] : 0.0;
    __syncthreads();  // maxima complete; the previous zone's exponents no longer read
    const int ema = ts.emax[a];
    const int Ea = (ema > 0) ? ema - 2044 : 0;
    if (tid < NB) ts.E[tid] = Ea;  // a == tid
    int bad = 0;
    uint32_t pk[kDigits][4];
#pragma unroll
    for (int i = 0; i < 8; i += 2) {
      uint32_t lo2[2], hi2[2];
#pragma unroll
      for (int u = 0; u < 2; u++) {
        const long long F = fixed_prod(sv[i + u], hv[i + u], Ea, bad);
        const unsigned long long Ub = (unsigned long long)F + kDigitBias;
        lo2[u] = (uint32_t)Ub;
        hi2[u] = (uint32_t)(Ub >> 32);
      }
      const int wd = i >> 1;
#pragma unroll
      for (int p = 0; p < kDigits; p++) {
        const int byte = 6 - p;
        const uint32_t b0 = (byte >= 4) ? (hi2[0] >> (8 * (byte - 4))) & 255u
                                        : (lo2[0] >> (8 * byte)) & 255u;
        const uint32_t b1 = (byte >= 4) ? (hi2[1] >> (8 * (byte - 4))) & 255u
                                        : (lo2[1] >> (8 * byte)) & 255u;
        pk[p][wd] = __byte_perm(digit_bits(b0), digit_bits(b1), 0x7632);
      }
    }
#pragma unroll
    for (int p = 0; p < kDigits; p++)
      *reinterpret_cast<uint4*>(tile + p * kSliceBytes + tile_off(a, kq)) =
          make_uint4(pk[p][0], pk[p][1], pk[p][2], pk[p][3]);
    if (bad) atomicOr(&ts.bad[par], 1);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();  // slices staged; Upre, qpre, vpre and the maxima read
    if (tid < NB) ts.emax[tid] = 0;
    if (tid == 0) {
      fence_after();
#pragma unroll 1
      for (int kk = 0; kk < KT / 16; kk++) {
        const uint32_t ko = kk * 32;
        const uint32_t acc0 = kk > 0 ? 1u : 0u;
        // levels 0..3 in columns 64 L: A = [D_p ; D_p+1], B = D_0 .. D_(3-p)
#pragma unroll
        for (int p = 0; p < 4; p++)
          mma_bf16(tmem + 64 * p, make_desc(tile_addr + p * kSliceBytes + ko),
                   make_desc(tile_addr + ko), idesc_bf16(64u * (4 - p)), p == 0 ? acc0 : 1u);
        // levels 4..6 in columns 256 + 64 (L - 4): B = D_qlo .. D_qhi, q = L - p
#pragma unroll
        for (int p = 0; p < kDigits; p++) {
          const int qlo = (4 - p > 0) ? 4 - p : 0;
          const int qhi = (6 - p < kDigits - 1) ? 6 - p : kDigits - 1;
          const int off = qlo - (4 - p);
          mma_bf16(tmem + 256 + 64 * off, make_desc(tile_addr + p * kSliceBytes + ko),
                   make_desc(tile_addr + qlo * kSliceBytes + ko),
                   idesc_bf16(64u * (qhi - qlo + 1)), p == 0 ? acc0 : 1u);
        }
      }
      mma_commit(mbar);
    }
  };

  if (nmine > 0) {
    prefetch(0);
    cp_async_wait_all();
    __syncthreads();
    stage_issue(0);
    if (nmine > 1) prefetch(1);
  }
  for (int i = 0; i < nmine; i++) {
    const int par = i & 1;
    const int32_t zl = (int32_t)blockIdx.x + i * (int32_t)gridDim.x;
    if (tid == 0 && !mbar_wait(mbar, ph)) ts.flag = 1;
    ph ^= 1u;
    __syncthreads();  // MMA completion (or the timeout) published
    if (ts.flag) {
      pending = true;
      if (tid == 0) atomicOr(&status[zl], ZST_TIMEOUT);
      break;
    }
    fence_after();
    const double* vv = vvb + par * NB;
    // T_sym from the accumulators: lanes 0-63 (rows j) are read by warps 0, 1, 4, 5, 8, 9,
    // 12, 13; warp group cg takes columns 16 cg .. 16 cg + 15 of all seven levels, and its
    // partial sums of T_sym v and of the row. Warp 2 forms u_v and u_v . u_w meanwhile.
    if ((warp & 3) < 2) {
      const int qd = warp & 3, cg = warp >> 2;
      const int j = 32 * qd + lane;
      const uint32_t ta = tmem + ((uint32_t)(32 * qd) << 16);
      const bool zbad = ts.bad[par] != 0;
      const int Ej = ts.E[j];
      double sv_part = 0.0, sr_part = 0.0;
#pragma unroll 1
      for (int h8 = 0; h8 < 2; h8++) {
        const int c0 = 16 * cg + 8 * h8;
        uint32_t r[56];
        tmem_ld7x8(ta, c0, r);
#pragma unroll
        for (int t = 0; t < 8; t++) {
          const int c = c0 + t;
          const long long v =
              (((long long)__float2int_rn(__uint_as_float(r[t])) * 256 +
                __float2int_rn(__uint_as_float(r[8 + t]))) * 256 +
               __float2int_rn(__uint_as_float(r[16 + t]))) * 256 +
              __float2int_rn(__uint_as_float(r[24 + t]));
          // 256 V456 is below 2^31 in magnitude (level 4 below 5 x 64 x 2^14)
          const float f456 = fmaf(__uint_as_float(r[48 + t]), 1.f / 65536.f,
                                  fmaf(__uint_as_float(r[40 + t]), 1.f / 256.f,
                                       __uint_as_float(r[32 + t])));
          const long long vt = v * 65536 + (long long)__float2int_rn(f456 * 256.f);
          double val = scaled_i64(vt, Ej + ts.E[c] - 52);
          if (zbad) val = __longlong_as_double(0x7FF8000000000000ll);  // NaN: non-finite input
          Ts[j * kTsLd + c] = val;
          if (rotate) {
            sv_part = fma(val, vv[c], sv_part);
            sr_part += (c < N) ? val : 0.0;
          }
        }
      }
      if (rotate) {
        pv[cg * NB + j] = sv_part;
        ps[cg * NB + j] = sr_part;
      }
    } else if (warp == 2 && rotate) {  // u_v and u_v . u_w, u_w = w 1 + e_N
      const double sgv = signbit(vv[N - 1]) ? -1.0 : 1.0;
      double sdot = 0.0;
      for (int jj = lane; jj < NB; jj += 32) {
        const double u = (jj < N) ? vv[jj] + ((jj == N - 1) ? sgv : 0.0) : 0.0;
        uv[jj] = u;
        sdot = fma(u, wv + ((jj == N - 1) ? 1.0 : 0.0), sdot);
      }
      for (int o = 16; o > 0; o >>= 1) sdot += __shfl_xor_sync(0xffffffffu, sdot, o);
      if (lane == 0) ts.uvuw = sdot;
    }
    if (i + 1 < nmine) cp_async_wait_all();  // the next zone's copies (this thread's)
    fence_before();
    __syncthreads();  // T_sym, sums, u_v published; tensor memory read; next zone landed
    if (i + 1 < nmine) {
      stage_issue(par ^ 1);  // the next zone's MMAs run beside this zone's rotation
      if (i + 2 < nmine) prefetch(i + 2);
    }
    if (nobs[zl] == 0) continue;  // block-uniform: no T for a zone without observations
    double* Gz = GT + (int64_t)zl * N * N;
    if (rotate) {
      const double sgv = signbit(vv[N - 1]) ? -1.0 : 1.0;
      if (tid < N) {
        const int r = tid;
        const double tvi = (pv[r] + pv[NB + r]) + (pv[2 * NB + r] + pv[3 * NB + r]);  // T_sym v
        const double rsi = (ps[r] + ps[NB + r]) + (ps[2 * NB + r] + ps[3 * NB + r]);
        const double tlast = Ts[r * kTsLd + N - 1];
        const double ai = fma(sgv, tlast, tvi) / (1.0 + fabs(vv[N - 1]));  // T_sym u_v / c_v
        const double gi = fma(-ts.uvuw, ai, fma(wv, rsi, tlast)) * icw;
        ar[r] = ai;
        gr[r] = gi;
        cr[r] = ((1.0 - sgv) * tvi - gi) * wv;
      }
      __syncthreads();
      for (int idx = tid; idx < N * N; idx += kThreads) {
        const int r = idx / N, c = idx - r * N;
        double t = fma(-ar[r], uv[c], Ts[r * kTsLd + c]) + cr[r];
        if (c == N - 1) t -= gr[r];
        Gz[idx] = t;
      }
    } else {
      for (int idx = tid; idx < N * N; idx += kThreads) {
        const int r = idx / N, c = idx - r * N;
        Gz[idx] = Ts[r * kTsLd + c];
      }
    }
  }
  // teardown: no MMA may still write tensor memory when it is freed, no copy still land
  cp_async_wait_all();
  if (pending && tid == 0) mbar_wait(mbar, ph ^ 1u);
  fence_before();
  __syncthreads();
  fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTmemCols));
}

}  // namespace

int gram_oz_max_n() { return NB; }

size_t gram_oz_scratch_bytes(int64_t m) {
  return NB * sizeof(unsigned long long) + NB * sizeof(int32_t) + (size_t)m * sizeof(double);
}

cudaError_t zone_gram_oz(const CellGrid& g, const SortedObs& so, int64_t m, int N, LocParams lp,
                         int32_t z0, int32_t nzc, const double* zone_xyzt, const double* corr_len,
                         const double* max_len, double* d_G, double* d_g, int32_t* d_nobs,
                         int brute, int32_t* d_work, int32_t* d_err, void* d_scratch,
                         cudaStream_t st, const int32_t* order) {
  if (N < 1 || N > NB || !so.HSt || !so.r || !d_scratch) return cudaErrorInvalidValue;
  unsigned long long* mx = reinterpret_cast<unsigned long long*>(d_scratch);
  int32_t* E = reinterpret_cast<int32_t*>(mx + NB);
  double* isr = reinterpret_cast<double*>(E + NB);  // 8-byte aligned: NB int32 = 256 bytes
  cudaError_t e = cudaMemsetAsync(mx, 0, NB * sizeof(unsigned long long), st);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (m > 0) {
    const int64_t per = kThreads / NB;
    int64_t blocks = (m + per - 1) / per;
    if (blocks > 4 * (int64_t)sms) blocks = 4 * (int64_t)sms;
    k_oz_colmax<<<(unsigned)(blocks > 0 ? blocks : 1), kThreads, 0, st>>>(m, N, so.HSt, so.r, mx, isr);
    count_launches(1);
  }
  k_oz_exponents<<<1, NB, 0, st>>>(N, mx, E);
  count_launches(1);
  e = cudaFuncSetAttribute(k_zone_gram_oz, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)kDynSmem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_zone_gram_oz, cudaFuncAttributePreferredSharedMemoryCarveout,
                           (int)cudaSharedmemCarveoutMaxShared);
  if (e != cudaSuccess) return e;
  // the shared-memory size admits one CTA per SM (it holds all 512 tensor-memory columns)
  int grid = sms;
  if (grid > nzc) grid = nzc > 0 ? nzc : 1;
  e = cudaMemsetAsync(d_work, 0, sizeof(int32_t), st);
  if (e != cudaSuccess) return e;
  k_zone_gram_oz<<<grid, kThreads, kDynSmem, st>>>(g, so, N, lp, z0, nzc, zone_xyzt, corr_len,
                                                   max_len, E, isr, d_G, d_g, d_nobs, brute,
                                                   d_work, d_err, order);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t zone_tsym_oz(int N, int32_t nzc, double* d_GT, const double* d_aux,
                         const double* d_Z, const int32_t* d_nobs, int rotate,
                         int32_t* d_status, cudaStream_t st) {
  if (N < 1 || N > NB) return cudaErrorInvalidValue;
  if (nzc <= 0) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(k_zone_tsym_oz, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kTsDynSmem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_zone_tsym_oz, cudaFuncAttributePreferredSharedMemoryCarveout,
                           (int)cudaSharedmemCarveoutMaxShared);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int grid = sms < nzc ? sms : nzc;
  k_zone_tsym_oz<<<grid, kThreads, kTsDynSmem, st>>>(N, nzc, d_GT, d_aux, d_Z, d_nobs, rotate,
                                                     d_status);
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace oakg
