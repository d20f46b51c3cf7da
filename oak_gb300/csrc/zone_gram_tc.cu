// K1 + K2, mixed-precision form on the tensor cores (ensembles of up to 128 members).
//
// Selection makes the decisions of zone_gram.cu (assimilation.F90:3683-3771): d <= maxLength
// and, for Gaspari-Cohn, locfun(d/L) /= 0. For Cartesian and 1-D distances they are taken from
// an FP32 distance (relative error < 1e-6, from cell-relative FP32 coordinates: no FP64
// operation a candidate) when it is farther than a relative 3e-6 from maxLength and r = d/L is
// below 2 - 1e-3 or above 2 + 1e-5; inside
// those margins the reference's FP64 distance and locfun with IEEE rounding decide, as they do
// for the spherical metrics. The selected set is therefore identical to the plain form's. The
// weights themselves are FP32 (locfun or exp of the FP32 ratio). The Gram matrix
// G = HS_sel^T diag(c) HS_sel (rrsqrt.F90:135, c = w^2 / r from the DCDCovar of
// rrsqrt.F90:395) is written as G = X^T X with X = diag(sqrt(c)) HS_sel and computed by
// tcgen05.mma kind::tf32 with FP32 accumulation in tensor memory:
//
//   X (FP32) is split into two TF32 parts, X = X_hi + X_lo (X_lo = tf32(X - X_hi)), leaving a
//   residual of ~2^-22 |X|. A K-tile of 32 selected observations is staged in shared memory
//   (K-major, 128-byte swizzle).
//   Up to 64 members: one 128-row operand S = [X_hi^T ; X_lo^T] (rows 0-63: hi parts of
//   members 0-63, rows 64-127: lo parts). One M=128, N=128 MMA chain with S as both A and B
//   accumulates D = S S^T, whose four 64 x 64 blocks are X_hi^T X_hi, X_hi^T X_lo, X_lo^T X_hi
//   and X_lo^T X_lo; G is their sum.
//   65 to 128 members: two 128-row operands X_hi^T and X_lo^T; three MMAs per K-step
//   accumulate D = X_hi^T X_hi + X_hi^T X_lo + X_lo^T X_hi = G (the X_lo^T X_lo term, 2^-22
//   relative, below the FP32 accumulation error, is left out).
//   G is symmetrised from its lower triangle.
//
// The tensor-core accumulator is FP32 and its error grows with the length of the chain: zones on
// dense observation tracks select thousands of observations, and one chain over all of them
// leaves G with an error several times 1e-5 relative to its largest entries, which the
// eigendecomposition carries into the small eigenvalues. The chain is therefore cut into chunks
// of kChunkTiles K-tiles (256 observations): after each chunk the accumulator is read and added
// into a lower-triangle FP32 accumulator in shared memory, and the next chunk's first MMA
// overwrites the tensor-memory accumulator. The error of G is then that of a 256-term sum plus
// a few FP32 additions, whatever the number of observations.
//
// The innovation projection g = X^T (sqrt(c) d) (rrsqrt.F90:142) is accumulated on the CUDA
// cores by the staging threads with compensated (Kahan) FP32 sums.
//
// Pipeline per CTA (one zone at a time): candidates are tested 256 at a time; selected
// observations go to a ring of (index, sqrt(c), sqrt(c) d); every full K-tile is staged into
// one of two shared buffers and handed to the tensor core by one thread (4 MMAs of K = 8 and a
// commit to the buffer's mbarrier), so staging of the next tile overlaps the MMAs. At the end
// of every chunk and of the zone the accumulator is read with tcgen05.ld. Every mbarrier wait is bounded; on
// expiry the kernel records ZST_TIMEOUT, stops taking zones, waits (bounded) for its MMAs and
// frees its tensor memory.
#include <cuda_runtime.h>
#include <math.h>

#include "oakg_internal.cuh"
#include "selection.cuh"

namespace oakg {

namespace {

constexpr int kThreads = 256;
constexpr int KT = 32;            // observations per K-tile (128 bytes of TF32 per row)
constexpr int kRing = 512;        // selected-observation ring (power of two)
constexpr uint32_t kOpBytes = 128u * 128u;  // one 128-row operand tile of a K-tile
constexpr uint32_t kTmemCols = 128;
constexpr int kWaitPolls = 1 << 22;
constexpr int kChunkTiles = 8;    // K-tiles accumulated in tensor memory between reads

// Per padded ensemble width NB:
//   NB = 64: one operand tile per K-tile buffer, S = [X_hi^T ; X_lo^T] (rows 0-63 / 64-127);
//            D = S S^T and G is the sum of D's four 64 x 64 blocks; 4 CTAs per SM.
//   NB = 128: two operand tiles, X_hi^T and X_lo^T; D = X_hi^T X_hi + X_hi^T X_lo + X_lo^T X_hi
//            (X_lo^T X_lo, ~2^-22 relative, is left out) is G; 2 CTAs per SM.
// Dynamic shared memory: 1 KB alignment slack, two K-tile buffers, compensated innovation
// partials and the lower-triangle G accumulator (a tail padded, for NB = 64, so that at most 4
// CTAs share an SM: 4 x 128 tensor-memory columns = all 512).
template <int NB>
struct TcCfg {
  static constexpr int kOps = NB / 64;                    // operand tiles per buffer
  static constexpr uint32_t kBufBytes = kOps * kOpBytes;  // one K-tile buffer
  static constexpr int kTri = NB * (NB + 1) / 2;          // lower triangle of G
  static constexpr int kQ = kThreads / NB;                // staging thread groups per member
  static constexpr int kPasses = 8 / kQ;                  // 4-observation quads per thread
  static constexpr int kCtas = (NB == 64) ? 4 : 2;
  static constexpr size_t kTail = (NB == 64) ? 10 * 1024 : (size_t)kTri * sizeof(float);
  static constexpr size_t kDynSmem =
      1024 + 2 * kBufBytes + 2 * kQ * NB * sizeof(float) + kTail;
  static_assert(kTri * sizeof(float) <= kTail, "G accumulator must fit in the tail");
};

struct TcShared {
  int32_t ring_q[kRing];
  float ring_s[kRing];  // sqrt(c_q)
  float ring_y[kRing];  // sqrt(c_q) (yo - Hxf)_q
  unsigned long long mbar[2];
  int32_t warp_cnt[kThreads / 32];
  int32_t rlo[kThreads];   // first observation of each candidate range of a block of ranges
  int32_t roff[kThreads];  // exclusive prefix of the ranges' lengths
  int32_t wpre[kThreads / 32];
  int32_t rtotal;
  uint32_t tmem_base;
  int32_t zone;
  int32_t nrel;
  int32_t flag;
  sel::ZoneCell32 zc;  // the zone's cell-relative FP32 coordinates (read by broadcast)
  sel::ScanRange sr;   // the zone's cell range
  float iL32;          // 1 / L
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
  d |= (uint64_t)1 << 16;                   // leading byte offset (unused: K fits one swizzle row)
  d |= (uint64_t)(1024u >> 4) << 32;        // stride byte offset
  d |= (uint64_t)1 << 46;                   // descriptor version
  d |= (uint64_t)2 << 61;                   // 128-byte swizzle
  return d;
}

// instruction descriptor: D F32, A and B TF32, both K-major, N = 128, M = 128
constexpr uint32_t kIdesc =
    (1u << 4) | (2u << 7) | (2u << 10) | ((128u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                         uint32_t accum) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %3, 0;\n"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %4, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(accum), "r"(kIdesc));
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

// byte offset of the 16-byte chunk `chunk` (4 observations) of operand row `row` in a tile
__device__ __forceinline__ uint32_t tile_off(int row, int chunk) {
  return (uint32_t)((row >> 3) * 1024 + (row & 7) * 128 + ((chunk ^ (row & 7)) << 4));
}

// Gaspari-Cohn weight in FP32 (covariance.F90:645-667); used for weight values only, never for
// the relevance decision
__device__ __forceinline__ float locfun32(float r) {
  if (r <= 1.f) return fmaf(fmaf(fmaf(fmaf(-0.25f, r, 0.5f), r, 0.625f), r, -5.f / 3.f), r * r, 1.f);
  if (r <= 2.f)
    return fmaf(fmaf(fmaf(fmaf(fmaf(r, 1.f / 12.f, -0.5f), r, 0.625f), r, 5.f / 3.f), r, -5.f), r,
                4.f) -
           2.f / (3.f * r);
  return 0.f;
}

__device__ __forceinline__ void kahan_add(float& s, float& c, float term) {
  const float y = term - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}

template <int NB>
__global__ void __launch_bounds__(kThreads, TcCfg<NB>::kCtas)
    k_zone_gram_tc(CellGrid g, SortedObs so, int N, LocParams lp, int32_t z0, int32_t nzc,
                   const double* __restrict__ zone_xyzt, const double* __restrict__ corr_len,
                   const double* __restrict__ max_len, float* __restrict__ G,
                   float* __restrict__ gv, int32_t* __restrict__ nobs, int brute,
                   int32_t* __restrict__ work, int32_t* __restrict__ err,
                   const int32_t* __restrict__ order) {
  using C = TcCfg<NB>;
  extern __shared__ __align__(16) unsigned char dyn_raw[];
  __shared__ __align__(16) TcShared ts;
  const uint32_t raw_addr = smem_u32(dyn_raw);
  const uint32_t pad = ((raw_addr + 1023u) & ~1023u) - raw_addr;
  unsigned char* tiles = dyn_raw + pad;                 // 2 x C::kBufBytes, 1024-aligned
  const uint32_t tile_addr = raw_addr + pad;
  float* gps = reinterpret_cast<float*>(tiles + 2 * C::kBufBytes);  // [kQ][NB] partial sums
  float* gpc = gps + C::kQ * NB;                                     // [kQ][NB] compensations
  float* gacc = gpc + C::kQ * NB;  // G lower triangle, entry (i, j <= i) at i (i + 1) / 2 + j

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // staging: member a, observation quads kq, kq + kQ, ...
  const int a = tid & (NB - 1), kq = tid / NB;
  const uint32_t mbar0 = smem_u32(&ts.mbar[0]);

  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar0));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar0 + 8));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    ts.flag = 0;
  }
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

  const int64_t ncells = (int64_t)g.nu * g.nv;
  const int full_scan = brute || !lp.localise;
  const bool fast = (lp.loctype != 1) || (lp.metric == OAKG_METRIC_CARTESIAN);
  int pend0 = 0, pend1 = 0;     // buffer has MMAs not yet waited for (uniform)
  uint32_t ph0 = 0, ph1 = 0;    // parity of the buffer's next completion (uniform)
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

  // add the tensor-memory accumulator into gacc (all MMAs complete and published by a barrier).
  // Warp w reads lanes 32 (w % 4) .. + 31 (rows of D).
  // NB = 64: column half w / 4 of both column blocks; G(i, j) = (D(i, j) + D(i, j + 64)) +
  //   (D(i + 64, j) + D(i + 64, j + 64)); the rows of the lo parts are added first, then those
  //   of the hi parts, so the sums are deterministic.
  // NB = 128: D is G; warp w adds columns 64 (w / 4) .. + 63 of its rows (lower triangle).
  auto flush = [&]() {
    fence_after();
    const int q = warp & 3, h = warp >> 2;
    const int i = (32 * q + lane) & (NB - 1);
    const uint32_t ta = tmem + ((uint32_t)(32 * q) << 16);
    float* gi = gacc + i * (i + 1) / 2;
    if constexpr (NB == 64) {
#pragma unroll
      for (int phase = 0; phase < 2; phase++) {
        if ((q >> 1) == 1 - phase) {
#pragma unroll
          for (int s = 0; s < 4; s++) {
            const int c0 = 32 * h + 8 * s;
            float v0[8], v1[8];
            tmem_ld8(ta + c0, v0);
            tmem_ld8(ta + 64 + c0, v1);
#pragma unroll
            for (int t = 0; t < 8; t++)
              if (c0 + t <= i) gi[c0 + t] += v0[t] + v1[t];
          }
        }
        fence_before();
        __syncthreads();
      }
    } else {
      if (64 * h <= 32 * q + 31) {  // warp-uniform: the block has lower-triangle entries
#pragma unroll
        for (int s = 0; s < 8; s++) {
          const int c0 = 64 * h + 8 * s;
          float v[8];
          tmem_ld8(ta + c0, v);
#pragma unroll
          for (int t = 0; t < 8; t++)
            if (c0 + t <= i) gi[c0 + t] += v[t];
        }
      }
      fence_before();
      __syncthreads();
    }
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
    // the zone's FP64 set-up (divisions, floors) once, by one thread: evaluated by every thread
    // it kept the FP64 pipe half busy
    if (tid == 0) {
      ts.nrel = 0;
      ts.zc = sel::zone_cell32(g, zu, zv, Rmax);
      ts.iL32 = (float)(1.0 / L);
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
    __syncthreads();  // ts.zc, ts.sr, ts.iL32 published (read only in this zone's scan)
    const bool fastz = fast && ts.zc.ok && !brute;  // brute force: one cell, no local offsets
    for (int e = tid; e < C::kTri; e += kThreads) gacc[e] = 0.f;
    int head = 0, tail = 0, ntile = 0, ctile = 0, nrel_local = 0;
    float gsum = 0.f, gcmp = 0.f;

    // stage ring entries [head, head + rows) as one K-tile and issue its MMAs
    auto do_tile = [&](int rows) {
      if (ctile == kChunkTiles) {
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
      unsigned char* tb = tiles + b * C::kBufBytes;
      // hi parts: rows 0..NB-1 of the first operand tile; lo parts: rows 64..127 of the same
      // tile (NB = 64) or the second tile (NB = 128)
      unsigned char* tlo = (NB == 64) ? tb : tb + kOpBytes;
      const int rlo = (NB == 64) ? a + 64 : a;
#pragma unroll
      for (int pass = 0; pass < C::kPasses; pass++) {
        const int quad = kq + C::kQ * pass;
        uint32_t hi[4], lo[4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
          const int k = 4 * quad + i;
          float X = 0.f, y = 0.f;
          if (k < rows) {
            const int idx = (head + k) & (kRing - 1);
            const int32_t q = ts.ring_q[idx];
            const float h = (a < N) ? so.HSt32[(int64_t)q * N + a] : 0.f;
            X = ts.ring_s[idx] * h;
            y = ts.ring_y[idx];
          }
          hi[i] = to_tf32(X);
          lo[i] = to_tf32(X - __uint_as_float(hi[i]));
          kahan_add(gsum, gcmp, X * y);
        }
        *reinterpret_cast<uint4*>(tb + tile_off(a, quad)) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
        *reinterpret_cast<uint4*>(tlo + tile_off(rlo, quad)) =
            make_uint4(lo[0], lo[1], lo[2], lo[3]);
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncthreads();  // tile complete
      if (tid == 0) {
        fence_after();
        const uint32_t base = tile_addr + b * C::kBufBytes;
#pragma unroll
        for (int kk = 0; kk < KT / 8; kk++) {
          const uint32_t acc = (ctile > 0 || kk > 0) ? 1u : 0u;
          const uint64_t dh = make_desc(base + kk * 32);
          if constexpr (NB == 64) {
            mma_tf32(tmem, dh, dh, acc);
          } else {
            const uint64_t dl = make_desc(base + kOpBytes + kk * 32);
            mma_tf32(tmem, dh, dh, acc);
            mma_tf32(tmem, dh, dl, 1u);
            mma_tf32(tmem, dl, dh, 1u);
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

    const sel::ScanRange& sr = ts.sr;  // read from shared memory (register pressure)
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
        float w32 = 0.f;
        if (valid) {
          // FP32 decisions away from the thresholds, the reference's FP64 evaluation near them
          bool done = false;
          if (fastz) {
            const float d32 = sel::cell_distance32(ts.zc, so, q, cv, lp.loctype == 1);
            const int inside = (d32 <= r_lo) ? 1 : ((d32 >= r_hi) ? 0 : -1);
            if (inside >= 0) {
              const float r32 = d32 * ts.iL32;
              if (lp.weight == OAKG_WEIGHT_GAUSS_CUTOFF) {
                rel = inside;
                w32 = (rel || !lp.localise) ? expf(-(r32 * r32)) : 0.f;
                done = true;
              } else if (r32 >= 2.f + 1e-5f) {  // locfun = 0
                rel = 0;
                done = true;
              } else if (r32 <= 2.f - 1e-3f) {  // locfun > 3e-13, far above its FP64 rounding (1e-15)
                rel = inside;
                w32 = locfun32(r32);
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
            double w;
            if (lp.weight == OAKG_WEIGHT_GAUSS_CUTOFF) {
              rel = (d <= Rmax);
              const double t = d / L;
              w = (rel || !lp.localise) ? exp(-(t * t)) : 0.0;
            } else {
              w = sel::locfun(d / L);
              rel = (d <= Rmax) && (w != 0.0);
            }
            w32 = (float)w;
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
          // c = w (w / r) (DCDCovar, covariance.F90:612-619); sqrt(c) = |w| / sqrt(r)
          const float sc = fabsf(w32) * rsqrtf(so.r32[q]);
          const int slot = (tail + before + __popc(ball & ((1u << lane) - 1u))) & (kRing - 1);
          ts.ring_q[slot] = q;
          ts.ring_s[slot] = sc;
          ts.ring_y[slot] = sc * so.innov32[q];
        }
        __syncthreads();
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
    gps[kq * NB + a] = gsum;
    gpc[kq * NB + a] = gcmp;
    if (ntile > 0) {
      if (pend0) drain(0);
      if (pend1) drain(1);
    }
    __syncthreads();  // nrel, partials and the MMA completion published
    if (ts.flag) break;
    const int nrel = ts.nrel;
    if (tid == 0) nobs[z] = nrel;
    if (nrel > 0 && ntile > 0) {
      flush();
      float* Gz = G + (int64_t)zl * N * N;
      for (int idx = tid; idx < N * N; idx += kThreads) {
        const int i = idx / N, j = idx - i * N;
        Gz[idx] = (j <= i) ? gacc[i * (i + 1) / 2 + j] : gacc[j * (j + 1) / 2 + i];
      }
      if (tid < N) {
        // compensated combination of the four partial sums of member tid
        float s = 0.f, cmp = 0.f;
#pragma unroll
        for (int p = 0; p < C::kQ; p++) {
          kahan_add(s, cmp, gps[p * NB + tid]);
          kahan_add(s, cmp, -gpc[p * NB + tid]);
        }
        gv[(int64_t)zl * N + tid] = s;
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

template <int NB>
cudaError_t launch_gram_tc(const CellGrid& g, const SortedObs& so, int N, LocParams lp,
                           int32_t z0, int32_t nzc, const double* zone_xyzt,
                           const double* corr_len, const double* max_len, float* d_G,
                           float* d_g, int32_t* d_nobs, int brute, int32_t* d_work,
                           int32_t* d_err, cudaStream_t st, const int32_t* order) {
  using C = TcCfg<NB>;
  cudaError_t e = cudaFuncSetAttribute(k_zone_gram_tc<NB>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)C::kDynSmem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_zone_gram_tc<NB>, cudaFuncAttributePreferredSharedMemoryCarveout,
                           (int)cudaSharedmemCarveoutMaxShared);
  if (e != cudaSuccess) return e;
  // the shared-memory size admits at most kCtas CTAs per SM (kCtas x 128 TMEM columns <= 512)
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int grid = sms * C::kCtas;
  if (grid > nzc) grid = nzc > 0 ? nzc : 1;
  e = cudaMemsetAsync(d_work, 0, sizeof(int32_t), st);
  if (e != cudaSuccess) return e;
  k_zone_gram_tc<NB><<<grid, kThreads, C::kDynSmem, st>>>(g, so, N, lp, z0, nzc, zone_xyzt,
                                                          corr_len, max_len, d_G, d_g, d_nobs,
                                                          brute, d_work, d_err, order);
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace

int gram_tc_max_n() { return 128; }

cudaError_t zone_gram_tc(const CellGrid& g, const SortedObs& so, int N, LocParams lp, int32_t z0,
                         int32_t nzc, const double* zone_xyzt, const double* corr_len,
                         const double* max_len, float* d_G, float* d_g, int32_t* d_nobs,
                         int brute, int32_t* d_work, int32_t* d_err, cudaStream_t st,
                         const int32_t* order) {
  if (N < 1 || N > 128 || !so.HSt32 || !so.r32 || !so.innov32) return cudaErrorInvalidValue;
  if (N <= 64)
    return launch_gram_tc<64>(g, so, N, lp, z0, nzc, zone_xyzt, corr_len, max_len, d_G, d_g,
                              d_nobs, brute, d_work, d_err, st, order);
  return launch_gram_tc<128>(g, so, N, lp, z0, nzc, zone_xyzt, corr_len, max_len, d_G, d_g,
                             d_nobs, brute, d_work, d_err, st, order);
}

}  // namespace oakg
