// C ABI of liboakg.so (declared in include/oakg.h): argument checking, the per-device
// context (stream, events, buffers kept between calls), host<->device staging and the
// stage sequence K0 -> (K1+K2) -> (K3+K4) -> K5 over chunks of zones.
#include <cublas_v2.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "oakg_internal.cuh"

namespace oakg {

namespace {

thread_local std::string t_last_error;
int g_last_status = OAKG_OK;
std::mutex g_mutex;
std::atomic<int64_t> g_launches{0};

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  t_last_error = buf;
  g_last_status = code;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  int code = (e == cudaErrorMemoryAllocation) ? OAKG_ERR_NOMEM : OAKG_ERR_CUDA;
  return fail(code, "%s: %s", what, cudaGetErrorString(e));
}

// A device buffer that only grows.
struct Buf {
  void* p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t want = bytes + bytes / 8 + 256;
    cudaError_t e = cudaMalloc(&p, want);
    if (e == cudaSuccess) cap = want;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
  template <typename T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

enum BufId {
  B_ZONE_SIZE, B_XF, B_HXF, B_YO, B_R, B_SF, B_HSF, B_ZXYZT, B_OX, B_OY, B_OZ, B_OT, B_CORR,
  B_MAXL, B_XA, B_SA, B_AMPL, B_NOBS, B_ZSTART, B_SMALL, B_CELL, B_COUNT, B_CSTART, B_POS,
  B_PERM, B_SU, B_SV, B_SINNOV, B_SR, B_HST, B_HST32, B_OBS32, B_E_EF, B_E_HIDX, B_E_HW, B_E_HSH, B_E_HEF, B_E_XF, B_E_SF,
  B_E_HXF, B_E_HSF, B_E_XA, B_E_SA, B_E_MC, B_E_EA, B_G, B_GV, B_ZAMPL, B_STATUS, B_WORK, B_AUX, B_ZVEC,
  B_ORDER, B_C_E, B_C_MEAN, B_C_S, B_C_OM, B_C_EO, B_C_HE, B_C_HXF, B_C_HSF, B_C_XA, B_C_SA,
  B_C_AMPL, B_C_ZERO, B_C_INC, B_C_UX, B_C_UHX, B_C_R2, B_C_BF, B_C_BA, B_SMWB, B_HSTA, B_GAUG,
  B_GVAUG, B_GLOB, B_L_PART, B_L_WORK, B_L_ZS, B_L_ZI, B_L_INV, B_L_X, B_L_Y, B_L_IDX, B_L_MASK,
  B_L_SEA, B_L_COORD, B_L_POS, B_L_OIDX, B_L_OW, B_L_SIMP, B_HXF64, B_YO64, B_R64, B_G0, B_SREF,
  B_OZSCR, B_SCU, B_SRUV, B_COUNT_
};

struct Ctx {
  int device = -1;
  cudaStream_t stream = nullptr;       // the stream launches go to (own or the caller's)
  cudaStream_t own_stream = nullptr;
  cudaEvent_t ev[8] = {};
  Buf buf[B_COUNT_];
  double timings[5] = {0, 0, 0, 0, 0};
  int64_t chunk_override = 0;  // > 0: zones per chunk fixed (plans: no memory query in capture)
  // host-memory calls: Sf rows in and Sa / xa rows out per zone chunk, beside the kernels
  cudaStream_t copy_in = nullptr, copy_out = nullptr;
  // the library GEMM of sqrt2ens with a general Theta (created on first use)
  cublasHandle_t blas = nullptr;
};

Ctx* g_ctx[64] = {};

int get_ctx(Ctx** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= 64) return fail(OAKG_ERR_CUDA, "device index %d out of range", dev);
  if (!g_ctx[dev]) {
    Ctx* c = new Ctx();
    c->device = dev;
    // blocking stream: ordered after work the caller queued on the legacy default stream
    e = cudaStreamCreate(&c->own_stream);
    if (e != cudaSuccess) {
      delete c;
      return cuda_fail(e, "cudaStreamCreate");
    }
    c->stream = c->own_stream;
    for (auto& ev : c->ev) cudaEventCreate(&ev);
    g_ctx[dev] = c;
  }
  *out = g_ctx[dev];
  return OAKG_OK;
}

// Device view of an input: the caller's pointer (device memory) or a staged copy.
template <typename T>
int stage_in(Ctx* c, BufId id, const T* src, size_t count, int mem, const T** out,
             const char* name) {
  if (!src) {
    *out = nullptr;
    return OAKG_OK;
  }
  if (mem == OAKG_MEM_DEVICE) {
    *out = src;
    return OAKG_OK;
  }
  cudaError_t e = c->buf[id].ensure(count * sizeof(T) + 16);
  if (e != cudaSuccess) return cuda_fail(e, name);
  e = cudaMemcpyAsync(c->buf[id].p, src, count * sizeof(T), cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, name);
  *out = c->buf[id].as<T>();
  return OAKG_OK;
}

template <typename T>
int stage_out(Ctx* c, BufId id, T* dst, size_t count, int mem, T** out, const char* name) {
  if (!dst) {
    *out = nullptr;
    return OAKG_OK;
  }
  if (mem == OAKG_MEM_DEVICE) {
    *out = dst;
    return OAKG_OK;
  }
  cudaError_t e = c->buf[id].ensure(count * sizeof(T) + 16);
  if (e != cudaSuccess) return cuda_fail(e, name);
  *out = c->buf[id].as<T>();
  return OAKG_OK;
}

template <typename T>
int scratch(Ctx* c, BufId id, size_t count, T** out, const char* name) {
  cudaError_t e = c->buf[id].ensure(count * sizeof(T) + 16);
  if (e != cudaSuccess) return cuda_fail(e, name);
  *out = c->buf[id].as<T>();
  return OAKG_OK;
}

int check_dims(const oakg_dims* d) {
  if (!d) return fail(OAKG_ERR_ARGS, "dims is NULL");
  if (d->n <= 0) return fail(OAKG_ERR_ARGS, "n must be positive (got %lld)", (long long)d->n);
  if (d->N < 2 || d->N > max_ensemble())
    return fail(OAKG_ERR_ARGS, "ensemble size N=%d outside [2, %d]", d->N, max_ensemble());
  if (d->m < 0) return fail(OAKG_ERR_ARGS, "m must be >= 0");
  if (d->m > INT32_MAX - 1) return fail(OAKG_ERR_ARGS, "m above 2^31-2");
  if (d->ldS < d->n) return fail(OAKG_ERR_ARGS, "ldS < n");
  if (d->ldH < d->m) return fail(OAKG_ERR_ARGS, "ldH < m");
  if (d->mem != OAKG_MEM_HOST && d->mem != OAKG_MEM_DEVICE)
    return fail(OAKG_ERR_ARGS, "mem must be OAKG_MEM_HOST or OAKG_MEM_DEVICE");
  return OAKG_OK;
}

float elapsed(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

__global__ void k_or_status(const int32_t* __restrict__ st, int32_t n, int32_t* __restrict__ out) {
  int32_t acc = 0;
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    acc |= st[i];
  for (int o = 16; o > 0; o >>= 1) acc |= __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0 && acc) atomicOr(out, acc);
}

__global__ void k_set_int(int32_t* p, int32_t v) { *p = v; }

int status_code(int32_t bits) {
  if (bits & ZST_NAN) return fail(OAKG_ERR_NAN, "NaN in analysis amplitudes (rrsqrt.F90:145-149)");
  if (bits & ZST_EIG) return fail(OAKG_ERR_EIG, "symmetric eigensolver did not converge");
  if (bits & ZST_TIMEOUT) return fail(OAKG_ERR_TIMEOUT, "a bounded device wait expired");
  if (bits) return fail(OAKG_ERR_CUDA, "device status 0x%x", bits);
  return OAKG_OK;
}

// Scratch budget for the per-zone G/T matrices of one chunk.
size_t chunk_budget_bytes() {
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return (size_t)4 << 30;
  size_t b = free_b / 4;
  const size_t cap = (size_t)16 << 30;
  return b > cap ? cap : b;
}

}  // namespace

// Per-precision kernel sets (R = double: plain form; R = float: mixed form).
template <typename R>
struct ZoneKernels;
template <>
struct ZoneKernels<double> {
  // exact slice products on the tensor cores for ensembles of up to gram_oz_max_n() members
  // (unless OAKG_FLAG_SIMT_GRAM), else the FP64 CUDA-core kernel
  static cudaError_t gram(const CellGrid& g, const SortedObs& so, int N, LocParams lp, int32_t z0,
                          int32_t nzc, const double* zxyzt, const double* corr, const double* maxl,
                          double* d_G, double* d_g, int32_t* nobs, int brute, int32_t* work,
                          int32_t* err, cudaStream_t st, const int32_t* order, void* scratch) {
    if (N <= gram_oz_max_n() && so.m > 0 && scratch && !(lp.flags & OAKG_FLAG_SIMT_GRAM))
      return zone_gram_oz(g, so, so.m, N, lp, z0, nzc, zxyzt, corr, maxl, d_G, d_g, nobs, brute,
                          work, err, scratch, st, order);
    return zone_gram_fp64(g, so, N, lp, z0, nzc, zxyzt, corr, maxl, d_G, d_g, nobs, brute, work,
                          st, order);
  }
  // T_sym on the tensor cores as the Gram (unless OAKG_FLAG_SIMT_GRAM)
  static cudaError_t eig(int N, int32_t nzc, double* GT, const double* g, const int32_t* nobs,
                         int rotate, double* ampl, int32_t* status, double* aux, double* Z,
                         int32_t* work, cudaStream_t st, int32_t flags) {
    return zone_eig_fp64(N, nzc, GT, g, nobs, rotate, ampl, status, aux, Z, work, st,
                         (flags & OAKG_FLAG_SIMT_GRAM) ? 0 : 1);
  }
  template <typename... A>
  static cudaError_t update(A... a) { return zone_update_fp64(a...); }
  template <typename... A>
  static cudaError_t ampl(A... a) { return write_amplitudes(a...); }
};
template <>
struct ZoneKernels<float> {
  // tensor-core Gram for ensembles of up to gram_tc_max_n() members, else the CUDA-core one
  static cudaError_t gram(const CellGrid& g, const SortedObs& so, int N, LocParams lp, int32_t z0,
                          int32_t nzc, const double* zxyzt, const double* corr, const double* maxl,
                          float* d_G, float* d_g, int32_t* nobs, int brute, int32_t* work,
                          int32_t* err, cudaStream_t st, const int32_t* order,
                          void* /*scratch*/) {
    if (N <= gram_tc_max_n() && so.HSt32 && so.r32)
      return zone_gram_tc(g, so, N, lp, z0, nzc, zxyzt, corr, maxl, d_G, d_g, nobs, brute, work,
                          err, st, order);
    return zone_gram_fp32(g, so, N, lp, z0, nzc, zxyzt, corr, maxl, d_G, d_g, nobs, brute, work,
                          st, order);
  }
  static cudaError_t eig(int N, int32_t nzc, float* GT, const float* g, const int32_t* nobs,
                         int rotate, float* ampl, int32_t* status, float* aux, float* Z,
                         int32_t* work, cudaStream_t st, int32_t /*flags*/) {
    return zone_eig_fp32(N, nzc, GT, g, nobs, rotate, ampl, status, aux, Z, work, st);
  }
  template <typename... A>
  static cudaError_t update(A... a) { return zone_update_fp32(a...); }
  template <typename... A>
  static cudaError_t ampl(A... a) { return write_amplitudes_fp32(a...); }
};

struct ChunkArgs {
  CellGrid g;
  SortedObs so;
  LocParams lp;
  int32_t Z;
  int N;
  int64_t ldS;
  int32_t zone_max;
  int brute, all_ampl;
  const double *zxyzt, *corr, *maxl;
  const int64_t* zstart;
  const double *xf, *Sf;
  double *xa, *Sa, *ampl;
  int32_t* nobs;
  // FP32 storage at the boundary (oakg_locanalysis_f32): these state arrays replace the five
  // above, which are then null
  bool store32 = false;
  // mixed form: refine the FP32 eigenpairs to FP64 accuracy (OAKG_PREC_MIXED_FP64EIG)
  bool refine = false;
  const float *xf32 = nullptr, *Sf32 = nullptr;
  float *xa32 = nullptr, *Sa32 = nullptr, *ampl32 = nullptr;
  // optional pick order of the selection + Gram stage (chunk-local zone indices, Z entries)
  const int32_t* zorder = nullptr;
  // SMWCovar R = diag(r) + B B^T (FP64 form): k columns of B and the augmented cell-sorted
  // rows [HS_q | B_q] (m x (N + k))
  int smw_k = 0;
  const double* hst_aug = nullptr;
  // host-memory pipeline: Sf (host) rows of each chunk copied into a.Sf on a copy stream, the
  // chunk's Sa / xa rows copied back to the host after its update (rows < n only); elements
  // are those of the state (double, or float with store32)
  const void* sf_host = nullptr;
  void* sa_host = nullptr;
  void* xa_host = nullptr;
  const int64_t* zstart_host = nullptr;  // Z + 1 row offsets
};

// host-memory calls: the update of a chunk in this many zone ranges, so that all but the
// last range's output copy overlaps the update
constexpr int32_t kOutPieces = 4;

int copy_streams(Ctx* c) {
  cudaError_t e = cudaSuccess;
  if (!c->copy_in) e = cudaStreamCreateWithFlags(&c->copy_in, cudaStreamNonBlocking);
  if (e == cudaSuccess && !c->copy_out)
    e = cudaStreamCreateWithFlags(&c->copy_out, cudaStreamNonBlocking);
  return e == cudaSuccess ? OAKG_OK : cuda_fail(e, "copy streams");
}

// How run_chunks issues its work: timed (events + a host wait per chunk), captured into a CUDA
// graph (no event, no host wait), or the selection + Gram stage alone (autotuning).
enum class RunMode { kTimed, kCapture, kGramOnly };

// Runs the zone stages over chunks of zones sized to the scratch budget.
template <typename R>
int run_chunks(Ctx* c, const ChunkArgs& a, int32_t** status_all, double* t_gram, double* t_eig,
               double* t_upd, RunMode mode = RunMode::kTimed) {
  const bool timed = (mode != RunMode::kCapture);
  using K = ZoneKernels<R>;
  const int N = a.N;
  cudaStream_t st = c->stream;
  cudaError_t e;
  int rc;
  const int NA = N + a.smw_k;
  const size_t per_zone =
      ((size_t)N * N * 2 + (size_t)N * 2 + zone_eig_aux(N)) * sizeof(R) + 2 * sizeof(int32_t) +
      (a.smw_k > 0 ? ((size_t)NA * NA + NA) * sizeof(double) : 0) +
      (a.refine ? ((size_t)N * N + zone_refine_scratch(N)) * sizeof(float) : 0);
  int64_t chunk = c->chunk_override > 0 ? c->chunk_override
                                        : (int64_t)(chunk_budget_bytes() / per_zone);
  // host-memory calls: the Sf rows of every chunk go in while the selection, Gram and
  // eigensolve stages run (they do not read Sf). The Sa / xa rows of a chunk go out while the
  // next chunk computes, so large calls are split into kPipeChunks chunks (of at least
  // kPipeMinZones zones, which keep every SM busy in the per-zone stages): only the last
  // chunk's output copy is left behind the kernels
  const bool pipe = a.sf_host != nullptr && mode == RunMode::kTimed;
  constexpr int64_t kPipeChunks = 4, kPipeMinZones = 4096;
  if (pipe && c->chunk_override <= 0 && a.Z >= kPipeChunks * kPipeMinZones)
    chunk = std::min<int64_t>(chunk, (a.Z + kPipeChunks - 1) / kPipeChunks);
  if (chunk < 1) chunk = 1;
  if (chunk > a.Z) chunk = a.Z;
  R *d_G, *d_gv, *d_za, *d_aux, *d_zvec;
  int32_t *d_status, *d_work;
  if ((rc = scratch(c, B_G, (size_t)chunk * N * N, &d_G, "zone matrices"))) return rc;
  if ((rc = scratch(c, B_GV, (size_t)chunk * N, &d_gv, "zone vectors"))) return rc;
  if ((rc = scratch(c, B_ZAMPL, (size_t)chunk * N, &d_za, "zone amplitudes"))) return rc;
  if ((rc = scratch(c, B_STATUS, (size_t)chunk + 1, &d_status, "zone status"))) return rc;
  if ((rc = scratch(c, B_WORK, 8, &d_work, "work counters"))) return rc;
  if ((rc = scratch(c, B_AUX, (size_t)chunk * zone_eig_aux(N), &d_aux, "zone aux"))) return rc;
  if ((rc = scratch(c, B_ZVEC, (size_t)chunk * N * N, &d_zvec, "zone eigenvectors"))) return rc;
  float *d_G0 = nullptr, *d_Sref = nullptr;
  if (a.refine && ((rc = scratch(c, B_G0, (size_t)chunk * N * N, &d_G0, "zone Gram copies")) ||
                   (rc = scratch(c, B_SREF, (size_t)chunk * zone_refine_scratch(N), &d_Sref,
                                 "refinement scratch"))))
    return rc;
  double *d_Ga = nullptr, *d_ga = nullptr;
  if (a.smw_k > 0 && ((rc = scratch(c, B_GAUG, (size_t)chunk * NA * NA, &d_Ga, "augmented Gram")) ||
                      (rc = scratch(c, B_GVAUG, (size_t)chunk * NA, &d_ga, "augmented g"))))
    return rc;
  unsigned char* d_oz = nullptr;  // column exponents of the plain form's tensor-core Gram
  if (sizeof(R) == sizeof(double) &&
      (rc = scratch(c, B_OZSCR, gram_oz_scratch_bytes(a.so.m), &d_oz, "Gram exponents")))
    return rc;
  *status_all = d_work + 2;
  k_set_int<<<1, 1, 0, st>>>(*status_all, 0);
  count_launches(1);
  // host-memory pipeline: every chunk's Sf rows queued on the input copy stream up front (the
  // selection + Gram stage needs none of them); the update of chunk q waits for its rows
  const int64_t nchunks = (a.Z + chunk - 1) / chunk;
  std::vector<cudaEvent_t> ev_in, ev_out;
  struct EventsGuard {
    std::vector<cudaEvent_t>* v[2];
    ~EventsGuard() {
      for (auto* p : v)
        for (cudaEvent_t ev : *p) cudaEventDestroy(ev);
    }
  } guard{{&ev_in, &ev_out}};
  const size_t esz = a.store32 ? sizeof(float) : sizeof(double);
  const size_t pitch = (size_t)a.ldS * esz;
  char* dSf = a.store32 ? (char*)const_cast<float*>(a.Sf32) : (char*)const_cast<double*>(a.Sf);
  char* dSa = a.store32 ? (char*)a.Sa32 : (char*)a.Sa;
  char* dxa = a.store32 ? (char*)a.xa32 : (char*)a.xa;
  // the update of zones [zz0, zz0 + nq) (T and amplitudes at the chunk-local slot)
  // (mixed form: on the tensor cores unless OAKG_FLAG_SIMT_UPDATE asks for the CUDA cores or
  // the zones are shorter than kTcUpdateMinRows rows: the MMA tile is 128 rows, so for short
  // zones it would be mostly padding and the CUDA-core kernel, which stages T once per zone
  // for all its rows, is faster)
  constexpr int32_t kTcUpdateMinRows = 48;
  auto update = [&](int32_t zz0, int32_t nq, const R* T, const R* za,
                    const int32_t* nb) -> cudaError_t {
    if constexpr (std::is_same<R, float>::value) {
      if (!(a.lp.flags & OAKG_FLAG_SIMT_UPDATE) && a.zone_max >= kTcUpdateMinRows)
        return a.store32 ? zone_update_tc(N, zz0, nq, a.zstart, a.xf32, a.Sf32, a.ldS, T, za, nb,
                                          a.xa32, a.Sa32, *status_all, st)
                         : zone_update_tc(N, zz0, nq, a.zstart, a.xf, a.Sf, a.ldS, T, za, nb,
                                          a.xa, a.Sa, *status_all, st);
    }
    return a.store32 ? K::update(N, zz0, nq, a.zstart, a.zone_max, a.xf32, a.Sf32, a.ldS, T, za,
                                 nb, a.xa32, a.Sa32, st)
                     : K::update(N, zz0, nq, a.zstart, a.zone_max, a.xf, a.Sf, a.ldS, T, za, nb,
                                 a.xa, a.Sa, st);
  };
  if (pipe) {
    if ((rc = copy_streams(c))) return rc;
    ev_in.resize(nchunks);
    ev_out.resize(nchunks * kOutPieces);
    for (auto& ev : ev_in) cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    for (auto& ev : ev_out) cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    // the staging buffer is free once the stream's earlier work is done
    cudaEventRecord(c->ev[7], st);
    cudaStreamWaitEvent(c->copy_in, c->ev[7], 0);
    for (int64_t q = 0; q < nchunks; q++) {
      const int64_t r0 = a.zstart_host[q * chunk],
                    r1 = a.zstart_host[std::min<int64_t>((q + 1) * chunk, a.Z)];
      if (r1 > r0 &&
          (e = cudaMemcpy2DAsync(dSf + r0 * esz, pitch, (const char*)a.sf_host + r0 * esz, pitch,
                                 (size_t)(r1 - r0) * esz, N, cudaMemcpyHostToDevice,
                                 c->copy_in)) != cudaSuccess)
        return cuda_fail(e, "H2D Sf rows");
      cudaEventRecord(ev_in[q], c->copy_in);
    }
  }
  for (int64_t z0 = 0; z0 < a.Z; z0 += chunk) {
    const int32_t nzc = (int32_t)std::min<int64_t>(chunk, a.Z - z0);
    if (timed) cudaEventRecord(c->ev[2], st);
    if constexpr (sizeof(R) == sizeof(double)) {
      if (a.smw_k > 0) {
        // SMWCovar: products of the augmented rows, then the per-zone Woodbury reduction
        SortedObs soa = a.so;
        soa.HSt = a.hst_aug;
        e = zone_gram_fp64_aug(a.g, soa, NA, N, a.lp, (int32_t)z0, nzc, a.zxyzt, a.corr, a.maxl,
                               d_Ga, d_ga, a.nobs, a.brute, d_work, st);
        if (e == cudaSuccess)
          e = smw_reduce(N, a.smw_k, nzc, d_Ga, d_ga, a.nobs + z0, (double*)d_G, (double*)d_gv,
                         st);
      } else {
        e = K::gram(a.g, a.so, N, a.lp, (int32_t)z0, nzc, a.zxyzt, a.corr, a.maxl, d_G, d_gv,
                    a.nobs, a.brute, d_work, *status_all, st, a.zorder, d_oz);
      }
    } else {
      e = K::gram(a.g, a.so, N, a.lp, (int32_t)z0, nzc, a.zxyzt, a.corr, a.maxl, d_G, d_gv,
                  a.nobs, a.brute, d_work, *status_all, st, a.zorder, nullptr);
    }
    if (e != cudaSuccess) return cuda_fail(e, "selection/Gram kernel");
    if (mode == RunMode::kGramOnly) {
      cudaEventRecord(c->ev[3], st);
      if ((e = cudaEventSynchronize(c->ev[3])) != cudaSuccess) return cuda_fail(e, "kernels");
      *t_gram += elapsed(c->ev[2], c->ev[3]);
      continue;
    }
    if (timed) cudaEventRecord(c->ev[3], st);
    if constexpr (std::is_same<R, float>::value) {
      if (a.refine)
        e = zone_eig_fp32_refined(N, nzc, d_G, (const R*)d_gv, (const int32_t*)(a.nobs + z0),
                                  a.lp.rotate, d_za, d_status, d_aux, d_zvec, d_work + 4, d_G0,
                                  d_Sref, st);
      else
        e = K::eig(N, nzc, d_G, (const R*)d_gv, (const int32_t*)(a.nobs + z0), a.lp.rotate,
                   d_za, d_status, d_aux, d_zvec, d_work + 4, st, a.lp.flags);
    } else {
      e = K::eig(N, nzc, d_G, (const R*)d_gv, (const int32_t*)(a.nobs + z0), a.lp.rotate, d_za,
                 d_status, d_aux, d_zvec, d_work + 4, st, a.lp.flags);
    }
    if (e != cudaSuccess) return cuda_fail(e, "eigensolve kernel");
    if (timed) cudaEventRecord(c->ev[4], st);
    if (!pipe) {
      e = update((int32_t)z0, nzc, (const R*)d_G, (const R*)d_za, (const int32_t*)(a.nobs + z0));
      if (e != cudaSuccess) return cuda_fail(e, "update kernel");
    } else {
      // host memory: the update in kOutPieces zone ranges, each range's Sa / xa rows copied
      // out while the next range updates
      cudaStreamWaitEvent(st, ev_in[z0 / chunk], 0);
      const int32_t per = (nzc + kOutPieces - 1) / kOutPieces;
      for (int32_t q0 = 0; q0 < nzc; q0 += per) {
        const int32_t nq = std::min(per, nzc - q0);
        e = update((int32_t)(z0 + q0), nq, (const R*)d_G + (size_t)q0 * N * N,
                   (const R*)d_za + (size_t)q0 * N, (const int32_t*)(a.nobs + z0 + q0));
        if (e != cudaSuccess) return cuda_fail(e, "update kernel");
        const int64_t r0 = a.zstart_host[z0 + q0], r1 = a.zstart_host[z0 + q0 + nq];
        cudaEvent_t evp = ev_out[(z0 / chunk) * kOutPieces + q0 / per];
        cudaEventRecord(evp, st);
        cudaStreamWaitEvent(c->copy_out, evp, 0);
        if (r1 > r0) {
          if (a.sa_host &&
              (e = cudaMemcpy2DAsync((char*)a.sa_host + r0 * esz, pitch, dSa + r0 * esz, pitch,
                                     (size_t)(r1 - r0) * esz, N, cudaMemcpyDeviceToHost,
                                     c->copy_out)) != cudaSuccess)
            return cuda_fail(e, "D2H Sa rows");
          if ((e = cudaMemcpyAsync((char*)a.xa_host + r0 * esz, dxa + r0 * esz,
                                   (size_t)(r1 - r0) * esz, cudaMemcpyDeviceToHost,
                                   c->copy_out)) != cudaSuccess)
            return cuda_fail(e, "D2H xa rows");
        }
      }
    }
    if (timed) cudaEventRecord(c->ev[5], st);
    if (a.ampl) {
      e = K::ampl(N, (int32_t)z0, nzc, (const R*)d_za, (const int32_t*)(a.nobs + z0), a.all_ampl,
                  a.ampl, st);
      if (e != cudaSuccess) return cuda_fail(e, "amplitudes");
    } else if (a.ampl32) {
      e = K::ampl(N, (int32_t)z0, nzc, (const R*)d_za, (const int32_t*)(a.nobs + z0), a.all_ampl,
                  a.ampl32, st);
      if (e != cudaSuccess) return cuda_fail(e, "amplitudes");
    }
    k_or_status<<<64, 256, 0, st>>>(d_status, nzc, *status_all);
    count_launches(1);
    if (!timed) continue;
    if ((e = cudaEventSynchronize(c->ev[5])) != cudaSuccess) return cuda_fail(e, "kernels");
    *t_gram += elapsed(c->ev[2], c->ev[3]);
    *t_eig += elapsed(c->ev[3], c->ev[4]);
    *t_upd += elapsed(c->ev[4], c->ev[5]);
  }
  if (pipe) {
    // the call's final synchronisation of the stream covers the output copies
    cudaEventRecord(c->ev[7], c->copy_out);
    cudaStreamWaitEvent(st, c->ev[7], 0);
  }
  return OAKG_OK;
}

// Inputs of a local analysis on the device: staged arrays, zone offsets, the observation
// cell grid and the cell-sorted observations.
struct Prep {
  const int32_t* zsize;
  const double *xf, *Hxf, *yo, *r, *Sf, *HSf, *zxyzt, *u, *v, *corr, *maxl;
  // FP32 storage at the boundary: the state and HSf in FP32 (xf, Sf, HSf above are null);
  // Hxf, yo and r are widened to FP64 copies
  const float *xf32, *Sf32, *HSf32;
  int64_t* zstart;
  int32_t zone_max;
  int brute;
  CellGrid g;
  SortedObs so;
};

int check_loc(const oakg_dims* dims, const oakg_loc* loc, int32_t Z) {
  int rc = check_dims(dims);
  if (rc) return rc;
  if (!loc) return fail(OAKG_ERR_ARGS, "loc is NULL");
  if (Z < 1) return fail(OAKG_ERR_ARGS, "nzones must be >= 1");
  if (loc->weight != OAKG_WEIGHT_GAUSS_CUTOFF && loc->weight != OAKG_WEIGHT_GASPARI_COHN)
    return fail(OAKG_ERR_ARGS, "unknown weight kind %d", loc->weight);
  if (loc->metric < 0 || loc->metric > 2)
    return fail(OAKG_ERR_ARGS, "Unsupported metric: %d (assimilation.F90:3664-3668)",
                loc->metric);
  if (loc->loctype < 1 || loc->loctype > 3)
    return fail(OAKG_ERR_ARGS, "loctype must be 1, 2 or 3 (got %d)", loc->loctype);
  if (loc->precision != OAKG_PREC_FP64 && loc->precision != OAKG_PREC_MIXED &&
      loc->precision != OAKG_PREC_MIXED_FP64EIG)
    return fail(OAKG_ERR_ARGS, "unknown precision mode %d", loc->precision);
  if (loc->precision == OAKG_PREC_FP64 && dims->N > max_fp64_ensemble())
    return fail(OAKG_ERR_ARGS, "the FP64 form takes N <= %d (N=%d: use OAKG_PREC_MIXED)",
                max_fp64_ensemble(), dims->N);
  return OAKG_OK;
}

// Bins the observations into P->g (cell-sorted arrays in P->so), plus the FP32 copies of the
// mixed form. Issues device work only (no host wait), so it can be captured in a graph.
int bin_observations(Ctx* c, const oakg_loc* loc, int64_t m, int N, int64_t ldH, Prep* P) {
  cudaStream_t st = c->stream;
  cudaError_t e;
  int rc;
  const CellGrid& g = P->g;
  const int64_t ncells = (int64_t)g.nu * g.nv;
  SortedObs& so = P->so;
  so = SortedObs{};
  if (m > 0) {
    int32_t *d_cell, *d_count, *d_cstart, *d_pos, *d_perm;
    double *d_su, *d_sv, *d_sinnov, *d_sr, *d_hst;
    if ((rc = scratch(c, B_CELL, (size_t)m, &d_cell, "cells"))) return rc;
    if ((rc = scratch(c, B_COUNT, (size_t)ncells + 1, &d_count, "cells"))) return rc;
    if ((rc = scratch(c, B_CSTART, (size_t)ncells + 1, &d_cstart, "cells"))) return rc;
    if ((rc = scratch(c, B_POS, (size_t)m, &d_pos, "obs"))) return rc;
    if ((rc = scratch(c, B_PERM, (size_t)m, &d_perm, "obs"))) return rc;
    if ((rc = scratch(c, B_SU, (size_t)m, &d_su, "obs"))) return rc;
    if ((rc = scratch(c, B_SV, (size_t)m, &d_sv, "obs"))) return rc;
    if ((rc = scratch(c, B_SINNOV, (size_t)m, &d_sinnov, "obs"))) return rc;
    if ((rc = scratch(c, B_SR, (size_t)m, &d_sr, "obs"))) return rc;
    if ((rc = scratch(c, B_HST, (size_t)m * N, &d_hst, "obs rows"))) return rc;
    int32_t* d_scu;
    float* d_sruv;
    if ((rc = scratch(c, B_SCU, (size_t)m, &d_scu, "obs cells")) ||
        (rc = scratch(c, B_SRUV, (size_t)2 * m, &d_sruv, "obs cell offsets")))
      return rc;
    e = obs_bin_and_sort(g, m, N, P->u, P->v, P->yo, P->Hxf, P->r, P->HSf, P->HSf32, ldH,
                         d_cell, d_count, d_cstart, d_pos, d_perm, d_su, d_sv, d_sinnov, d_sr,
                         d_hst, d_scu, d_sruv, d_sruv + m, st);
    if (e != cudaSuccess) return cuda_fail(e, "observation binning");
    so.u = d_su;
    so.v = d_sv;
    so.innov = d_sinnov;
    so.r = d_sr;
    so.HSt = d_hst;
    so.cell_start = d_cstart;
    so.perm = d_perm;
    so.m = m;
    so.cu = d_scu;
    so.ru = d_sruv;
    so.rv = d_sruv + m;
    if (loc->precision != OAKG_PREC_FP64) {
      float* d_hst32;
      if ((rc = scratch(c, B_HST32, (size_t)m * N, &d_hst32, "obs rows (FP32)"))) return rc;
      if ((e = rows_to_fp32(d_hst, d_hst32, m * N, st)) != cudaSuccess)
        return cuda_fail(e, "FP32 observation rows");
      so.HSt32 = d_hst32;
      float* d_obs32;
      if ((rc = scratch(c, B_OBS32, (size_t)2 * m, &d_obs32, "obs (FP32)"))) return rc;
      if ((e = rows_to_fp32(d_sr, d_obs32, m, st)) != cudaSuccess ||
          (e = rows_to_fp32(d_sinnov, d_obs32 + m, m, st)) != cudaSuccess)
        return cuda_fail(e, "FP32 observation values");
      so.r32 = d_obs32;
      so.innov32 = d_obs32 + m;
    }
  } else {
    int32_t* d_cstart;
    if ((rc = scratch(c, B_CSTART, 2, &d_cstart, "cells"))) return rc;
    cudaMemsetAsync(d_cstart, 0, 2 * sizeof(int32_t), st);
    so.cell_start = d_cstart;
  }
  return OAKG_OK;
}

// Stages an m-vector of observation values as FP64 (a widened copy when S = float).
template <typename S>
int stage_obs_vec(Ctx* c, BufId id, BufId id64, const S* src, int64_t m, int mem,
                  const double** out, const char* name) {
  if constexpr (std::is_same<S, double>::value) {
    (void)id64;
    return stage_in(c, id, src, (size_t)m, mem, out, name);
  } else {
    const float* d_src;
    double* d_out;
    int rc;
    if ((rc = stage_in(c, id, src, (size_t)m, mem, &d_src, name))) return rc;
    if ((rc = scratch(c, id64, (size_t)m, &d_out, name))) return rc;
    cudaError_t e = rows_to_fp64(d_src, d_out, m, c->stream);
    if (e != cudaSuccess) return cuda_fail(e, name);
    *out = d_out;
    return OAKG_OK;
  }
}

template <typename S>
int prepare_loc(Ctx* c, const oakg_dims* dims, const oakg_loc* loc, int32_t Z,
                const int32_t* zone_size, const S* xf, const S* Hxf, const S* yo, const S* Sf,
                const S* HSf, const S* r_diag, const double* zone_xyzt, const double* obs_x,
                const double* obs_y, const double* obs_z, const double* obs_t,
                const double* corr_len, const double* max_len, Prep* P,
                bool defer_sf = false) {
  constexpr bool f32 = std::is_same<S, float>::value;
  const int64_t n = dims->n, m = dims->m, ldS = dims->ldS, ldH = dims->ldH;
  const int N = dims->N, mem = dims->mem;
  int rc;
  if (!zone_size || !zone_xyzt || !corr_len || !max_len || !Sf)
    return fail(OAKG_ERR_ARGS, "zone_size, zone_xyzt, corr_len, max_len and Sf are required");
  if (m > 0 && (!Hxf || !yo || !HSf || !r_diag))
    return fail(OAKG_ERR_ARGS, "Hxf, yo, HSf and r_diag are required when m > 0");
  const double* u_src_h = (loc->loctype == 1) ? obs_x : (loc->loctype == 2 ? obs_z : obs_t);
  const double* v_src_h = (loc->loctype == 1) ? obs_y : nullptr;
  if (m > 0 && (!u_src_h || (loc->loctype == 1 && !v_src_h)))
    return fail(OAKG_ERR_ARGS, "observation coordinates required by loctype %d are NULL",
                loc->loctype);
  cudaStream_t st = c->stream;
  cudaError_t e;
  *P = Prep{};
  if ((rc = stage_in(c, B_ZONE_SIZE, zone_size, (size_t)Z, mem, &P->zsize, "zone_size"))) return rc;
  const S *d_xf = nullptr, *d_Sf = nullptr, *d_HSf = nullptr;
  if ((rc = stage_in(c, B_XF, xf, (size_t)n, mem, &d_xf, "xf"))) return rc;
  if (defer_sf && mem == OAKG_MEM_HOST) {
    // host-memory pipeline: the rows are copied per zone chunk by run_chunks
    S* d_sf;
    if ((rc = scratch(c, B_SF, (size_t)ldS * N, &d_sf, "Sf"))) return rc;
    d_Sf = d_sf;
  } else if ((rc = stage_in(c, B_SF, Sf, (size_t)ldS * N, mem, &d_Sf, "Sf"))) {
    return rc;
  }
  if constexpr (f32) {
    P->xf32 = d_xf;
    P->Sf32 = d_Sf;
  } else {
    P->xf = d_xf;
    P->Sf = d_Sf;
  }
  if ((rc = stage_in(c, B_ZXYZT, zone_xyzt, (size_t)4 * Z, mem, &P->zxyzt, "zone_xyzt"))) return rc;
  if ((rc = stage_in(c, B_CORR, corr_len, (size_t)Z, mem, &P->corr, "corr_len"))) return rc;
  if ((rc = stage_in(c, B_MAXL, max_len, (size_t)Z, mem, &P->maxl, "max_len"))) return rc;
  if (m > 0) {
    if ((rc = stage_obs_vec(c, B_HXF, B_HXF64, Hxf, m, mem, &P->Hxf, "Hxf"))) return rc;
    if ((rc = stage_obs_vec(c, B_YO, B_YO64, yo, m, mem, &P->yo, "yo"))) return rc;
    if ((rc = stage_obs_vec(c, B_R, B_R64, r_diag, m, mem, &P->r, "r_diag"))) return rc;
    if ((rc = stage_in(c, B_HSF, HSf, (size_t)ldH * N, mem, &d_HSf, "HSf"))) return rc;
    if constexpr (f32)
      P->HSf32 = d_HSf;
    else
      P->HSf = d_HSf;
    if ((rc = stage_in(c, B_OX, u_src_h, (size_t)m, mem, &P->u, "obs coordinate u"))) return rc;
    if (v_src_h && (rc = stage_in(c, B_OY, v_src_h, (size_t)m, mem, &P->v, "obs coordinate v")))
      return rc;
  }
  // zone offsets and sizes
  double* d_small;
  if ((rc = scratch(c, B_ZSTART, (size_t)Z + 1, &P->zstart, "zone offsets"))) return rc;
  if ((rc = scratch(c, B_SMALL, 16, &d_small, "small"))) return rc;
  int32_t* d_zmax = reinterpret_cast<int32_t*>(d_small + 8);
  if ((e = zone_offsets(P->zsize, Z, P->zstart, d_zmax, st)) != cudaSuccess)
    return cuda_fail(e, "zone offsets");
  P->brute = (loc->flags & OAKG_FLAG_BRUTE_SEARCH) || !loc->localise_obs;
  if (m > 0) {
    if ((e = obs_bounds(P->u, P->v, m, d_small, st)) != cudaSuccess) return cuda_fail(e, "bounds");
    if ((e = obs_bounds(P->maxl, nullptr, Z, d_small + 4, st)) != cudaSuccess)
      return cuda_fail(e, "bounds");
  }
  double hsmall[9] = {0};
  int64_t htotal = 0;
  if ((e = cudaMemcpyAsync(hsmall, d_small, 9 * sizeof(double), cudaMemcpyDeviceToHost, st)) !=
      cudaSuccess)
    return cuda_fail(e, "D2H");
  if ((e = cudaMemcpyAsync(&htotal, P->zstart + Z, sizeof(int64_t), cudaMemcpyDeviceToHost, st)) !=
      cudaSuccess)
    return cuda_fail(e, "D2H");
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_fail(e, "synchronize");
  std::memcpy(&P->zone_max, &hsmall[8], sizeof(int32_t));
  if (htotal != n)
    return fail(OAKG_ERR_ARGS, "sum(zone_size) = %lld differs from n = %lld", (long long)htotal,
                (long long)n);
  // cell grid over the observation coordinates
  CellGrid& g = P->g;
  g = CellGrid{};
  g.nu = g.nv = 1;
  g.csu = g.csv = 1.0;
  const int spherical = (loc->loctype == 1 && loc->metric != OAKG_METRIC_CARTESIAN);
  if (m > 0 && !P->brute) {
    double umin = hsmall[0], umax = hsmall[1], vmin = hsmall[2], vmax = hsmall[3];
    double Rmax = hsmall[5];
    if (!(std::isfinite(umin) && std::isfinite(umax) && std::isfinite(vmin) && std::isfinite(vmax)))
      return fail(OAKG_ERR_ARGS, "non-finite observation coordinates");
    double reach = Rmax;  // maxLength in coordinate units
    if (spherical) reach = Rmax / (3.141592653589793 * 6378137.0 / 180.0);  // metres -> degrees
    double cs = (loc->cell_size > 0) ? loc->cell_size : 0.5 * reach;
    const double max_cells = 4.0e6;
    g.periodic_u = (loc->metric == OAKG_METRIC_SPHERICAL && loc->loctype == 1);
    if (g.periodic_u) {
      umin = 0.0;
      umax = 360.0;
    }
    double spanu = std::max(umax - umin, 0.0), spanv = std::max(vmax - vmin, 0.0);
    if (!(cs > 0) || !std::isfinite(cs)) cs = std::max(std::max(spanu, spanv), 1.0);
    while ((std::floor(spanu / cs) + 1.0) * (std::floor(spanv / cs) + 1.0) > max_cells) cs *= 2.0;
    g.u0 = umin;
    g.v0 = vmin;
    g.csu = cs;
    g.csv = cs;
    g.nu = (int32_t)std::floor(spanu / cs) + 1;
    g.nv = (loc->loctype == 1) ? (int32_t)std::floor(spanv / cs) + 1 : 1;
    if (g.periodic_u) {
      // the periodic axis is cut into exactly nu cells of 360/nu degrees, so that cell
      // index + nu is the same longitude one period later
      g.nu = std::max(1, (int32_t)std::ceil(360.0 / cs));
      g.csu = 360.0 / g.nu;
    }
  }
  return bin_observations(c, loc, m, N, ldH, P);
}

// ------------------------------------------------------------------------------------------
// SMWCovar R = diag(r_diag) + B B^T: k columns of B (m x k, leading dimension ldB)
struct SmwArg {
  int32_t k = 0;
  const double* B = nullptr;
  int64_t ldB = 0;
};

// S: element type of the state and observation arrays at the boundary (double, or float for
// oakg_locanalysis_f32); the geometry is double either way.
template <typename S>
int locanalysis_impl(const oakg_dims* dims, const oakg_loc* loc, int32_t Z,
                     const int32_t* zone_size, const S* xf, const S* Hxf, const S* yo,
                     const S* Sf, const S* HSf, const S* r_diag, const double* zone_xyzt,
                     const double* obs_x, const double* obs_y, const double* obs_z,
                     const double* obs_t, const double* corr_len, const double* max_len, S* xa,
                     S* Sa, S* ampl, int32_t* nobs_out, const SmwArg* smw = nullptr) {
  constexpr bool f32 = std::is_same<S, float>::value;
  int rc = check_loc(dims, loc, Z);
  if (rc) return rc;
  if (f32 && smw) return fail(OAKG_ERR_ARGS, "the SMWCovar form takes FP64 arrays");
  if (!xf || !xa) return fail(OAKG_ERR_ARGS, "xf and xa are required");
  const int smw_k = (smw && dims->m > 0) ? smw->k : 0;
  if (smw) {
    if (smw->k < 0) return fail(OAKG_ERR_ARGS, "k must be >= 0");
    if (smw_k > 0 && loc->precision != OAKG_PREC_FP64)
      return fail(OAKG_ERR_ARGS, "the SMWCovar observation covariance needs OAKG_PREC_FP64");
    if (smw_k > 0 && (!smw->B || smw->ldB < dims->m))
      return fail(OAKG_ERR_ARGS, "B (ldB >= m) is required when k > 0");
    if (dims->N + smw_k > max_fp64_ensemble())
      return fail(OAKG_ERR_ARGS, "N + k must be <= %d", max_fp64_ensemble());
  }
  const int64_t n = dims->n, ldS = dims->ldS;
  const int N = dims->N, mem = dims->mem;
  Ctx* c = nullptr;
  if ((rc = get_ctx(&c))) return rc;
  cudaStream_t st = c->stream;
  cudaError_t e;
  cudaEventRecord(c->ev[0], st);
  // host memory: Sf in and Sa / xa out per zone chunk beside the kernels (rows < n; with
  // ldS > n the whole arrays are staged as before)
  const bool pipe = mem == OAKG_MEM_HOST && Sa && Sf && ldS == n && Z >= 2;
  std::vector<int64_t> zstart_h;
  if (pipe) {
    zstart_h.resize((size_t)Z + 1);
    zstart_h[0] = 0;
    for (int32_t z = 0; z < Z; z++) zstart_h[z + 1] = zstart_h[z] + zone_size[z];
  }
  Prep P;
  if ((rc = prepare_loc(c, dims, loc, Z, zone_size, xf, Hxf, yo, Sf, HSf, r_diag, zone_xyzt,
                        obs_x, obs_y, obs_z, obs_t, corr_len, max_len, &P, pipe)))
    return rc;
  S *d_xa, *d_Sa, *d_ampl;
  int32_t* d_nobs;
  if ((rc = stage_out(c, B_XA, xa, (size_t)n, mem, &d_xa, "xa"))) return rc;
  if ((rc = stage_out(c, B_SA, Sa, (size_t)ldS * N, mem, &d_Sa, "Sa"))) return rc;
  if ((rc = stage_out(c, B_AMPL, ampl, (size_t)N * Z, mem, &d_ampl, "amplitudes"))) return rc;
  if (mem == OAKG_MEM_DEVICE && nobs_out) {
    d_nobs = nobs_out;
  } else if ((rc = scratch(c, B_NOBS, (size_t)Z, &d_nobs, "nobs"))) {
    return rc;
  }
  if (mem == OAKG_MEM_HOST && Sa && !pipe) {
    // rows beyond n (ldS > n) are returned unchanged
    const void* d_Sf = f32 ? (const void*)P.Sf32 : (const void*)P.Sf;
    e = cudaMemcpyAsync(d_Sa, d_Sf, (size_t)ldS * N * sizeof(S), cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "Sa init");
  }
  cudaEventRecord(c->ev[1], st);

  // zone chunks: selection + Gram, eigensolve + transform, update
  LocParams lp{loc->weight, loc->metric, loc->loctype, loc->localise_obs ? 1 : 0,
               loc->rotate ? 1 : 0, loc->flags};
  const int all_ampl = (!loc->localise_obs) || (loc->flags & OAKG_FLAG_AMPL_ALWAYS);
  int32_t* d_status_all = nullptr;
  ChunkArgs ca{P.g, P.so, lp, Z, N, ldS, P.zone_max, P.brute, all_ampl, P.zxyzt, P.corr, P.maxl,
               P.zstart, nullptr, nullptr, nullptr, nullptr, nullptr, d_nobs};
  if constexpr (f32) {
    ca.store32 = true;
    ca.xf32 = P.xf32;
    ca.Sf32 = P.Sf32;
    ca.xa32 = d_xa;
    ca.Sa32 = d_Sa;
    ca.ampl32 = d_ampl;
  } else {
    ca.xf = P.xf;
    ca.Sf = P.Sf;
    ca.xa = d_xa;
    ca.Sa = d_Sa;
    ca.ampl = d_ampl;
  }
  if (pipe) {
    ca.sf_host = Sf;
    ca.sa_host = Sa;
    ca.xa_host = xa;
    ca.zstart_host = zstart_h.data();
  }
  if constexpr (!f32) if (smw_k > 0) {
    // the augmented cell-sorted rows [HS_q | B_q] of the SMWCovar products
    const int64_t m = dims->m;
    const double* dB;
    double* d_hsta;
    if ((rc = stage_in(c, B_SMWB, smw->B, (size_t)smw->ldB * smw_k, mem, &dB, "B")) ||
        (rc = scratch(c, B_HSTA, (size_t)m * (N + smw_k), &d_hsta, "augmented rows")))
      return rc;
    if ((e = smw_rows(m, N, smw_k, P.so.HSt, P.so.perm, dB, smw->ldB, d_hsta, st)) !=
        cudaSuccess)
      return cuda_fail(e, "augmented rows");
    ca.smw_k = smw_k;
    ca.hst_aug = d_hsta;
  }
  double t_gram = 0, t_eig = 0, t_upd = 0;
  ca.refine = (loc->precision == OAKG_PREC_MIXED_FP64EIG);
  rc = (loc->precision != OAKG_PREC_FP64)
           ? run_chunks<float>(c, ca, &d_status_all, &t_gram, &t_eig, &t_upd)
           : run_chunks<double>(c, ca, &d_status_all, &t_gram, &t_eig, &t_upd);
  if (rc) return rc;
  cudaEventRecord(c->ev[6], st);
  int32_t hstatus = 0;
  if ((e = cudaMemcpyAsync(&hstatus, d_status_all, sizeof(int32_t), cudaMemcpyDeviceToHost, st)) !=
      cudaSuccess)
    return cuda_fail(e, "D2H");
  if (mem == OAKG_MEM_HOST) {
    if (!pipe && (e = cudaMemcpyAsync(xa, d_xa, n * sizeof(S), cudaMemcpyDeviceToHost, st)))
      return cuda_fail(e, "D2H xa");
    if (Sa && !pipe &&
        (e = cudaMemcpyAsync(Sa, d_Sa, (size_t)ldS * N * sizeof(S), cudaMemcpyDeviceToHost,
                             st)))
      return cuda_fail(e, "D2H Sa");
    if (ampl && (e = cudaMemcpyAsync(ampl, d_ampl, (size_t)N * Z * sizeof(S),
                                     cudaMemcpyDeviceToHost, st)))
      return cuda_fail(e, "D2H amplitudes");
    if (nobs_out && (e = cudaMemcpyAsync(nobs_out, d_nobs, (size_t)Z * sizeof(int32_t),
                                         cudaMemcpyDeviceToHost, st)))
      return cuda_fail(e, "D2H nobs");
  }
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_fail(e, "synchronize");
  c->timings[0] = elapsed(c->ev[0], c->ev[1]);
  c->timings[1] = t_gram;
  c->timings[2] = t_eig;
  c->timings[3] = t_upd;
  c->timings[4] = elapsed(c->ev[0], c->ev[6]);
  return status_code(hstatus);
}

// Adjoint of the local analysis mean (zone_adjoint.cu): gradients of J(xa) given dJ/dxa.
int adjoint_impl(const oakg_dims* dims, const oakg_loc* loc, int32_t Z, const int32_t* zone_size,
                 const double* Hxf, const double* yo, const double* Sf, const double* HSf,
                 const double* r_diag, const double* zone_xyzt, const double* obs_x,
                 const double* obs_y, const double* obs_z, const double* obs_t,
                 const double* corr_len, const double* max_len, double inflation,
                 const double* dJ_dxa, double* dJ_dyo, double* dJ_dr, double* dJ_dlen,
                 double* dJ_dinfl) {
  int rc = check_loc(dims, loc, Z);
  if (rc) return rc;
  if (dims->N > max_fp64_ensemble())
    return fail(OAKG_ERR_ARGS, "the adjoint (FP64) takes N <= %d", max_fp64_ensemble());
  if (!dJ_dxa) return fail(OAKG_ERR_ARGS, "dJ_dxa is required");
  if (!(inflation > 0.0)) return fail(OAKG_ERR_ARGS, "inflation must be positive");
  const int64_t n = dims->n, m = dims->m, ldS = dims->ldS;
  const int N = dims->N, mem = dims->mem;
  Ctx* c = nullptr;
  if ((rc = get_ctx(&c))) return rc;
  cudaStream_t st = c->stream;
  cudaError_t e;
  cudaEventRecord(c->ev[0], st);
  Prep P;
  if ((rc = prepare_loc<double>(c, dims, loc, Z, zone_size, nullptr, Hxf, yo, Sf, HSf, r_diag,
                               zone_xyzt,
                        obs_x, obs_y, obs_z, obs_t, corr_len, max_len, &P)))
    return rc;
  const double* d_seed;
  if ((rc = stage_in(c, B_XA, dJ_dxa, (size_t)n, mem, &d_seed, "dJ_dxa"))) return rc;
  double *d_dyo, *d_dr, *d_scal;
  const size_t mm = (size_t)(m > 0 ? m : 1);
  if ((rc = stage_out(c, B_AMPL, dJ_dyo, mm, OAKG_MEM_HOST, &d_dyo, "dJ_dyo"))) return rc;
  if (mem == OAKG_MEM_DEVICE && dJ_dyo) d_dyo = dJ_dyo;
  double* d_dr_buf;
  if ((rc = scratch(c, B_SA, mm + 8, &d_dr_buf, "dJ_dr"))) return rc;
  d_dr = (mem == OAKG_MEM_DEVICE && dJ_dr) ? dJ_dr : d_dr_buf;
  d_scal = d_dr_buf + mm;
  if (!d_dyo) {
    if ((rc = scratch(c, B_AMPL, mm, &d_dyo, "dJ_dyo"))) return rc;
  }
  cudaMemsetAsync(d_dyo, 0, mm * sizeof(double), st);
  cudaMemsetAsync(d_dr, 0, mm * sizeof(double), st);
  cudaMemsetAsync(d_scal, 0, 2 * sizeof(double), st);
  // seeded zones
  int32_t *d_flag, *d_pos, *d_list, *d_nobs, *d_work;
  if ((rc = scratch(c, B_CELL, (size_t)Z + 1, &d_flag, "zone flags"))) return rc;
  if ((rc = scratch(c, B_STATUS, (size_t)Z + 1, &d_pos, "zone positions"))) return rc;
  if ((rc = scratch(c, B_POS, (size_t)Z + 1, &d_list, "zone list"))) return rc;
  if ((rc = scratch(c, B_NOBS, (size_t)Z, &d_nobs, "nobs"))) return rc;
  if ((rc = scratch(c, B_WORK, 8, &d_work, "work counters"))) return rc;
  // the obs-prep buffers B_CELL/B_POS are free once binning is done (binning ran above)
  if ((e = zone_active_list(d_seed, P.zstart, Z, d_flag, d_pos, d_list, st)) != cudaSuccess)
    return cuda_fail(e, "seeded zones");
  int32_t nact = 0;
  if ((e = cudaMemcpyAsync(&nact, d_pos + Z, sizeof(int32_t), cudaMemcpyDeviceToHost, st)))
    return cuda_fail(e, "D2H");
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_fail(e, "synchronize");
  LocParams lp{loc->weight, loc->metric, loc->loctype, loc->localise_obs ? 1 : 0,
               loc->rotate ? 1 : 0, loc->flags};
  const size_t per_zone = (size_t)N * N * 8 + (size_t)N * 8;
  int64_t chunk = c->chunk_override > 0 ? c->chunk_override
                                        : (int64_t)(chunk_budget_bytes() / per_zone);
  if (chunk < 1) chunk = 1;
  if (chunk > nact) chunk = nact;
  double *d_G, *d_gv;
  if (nact > 0) {
    if ((rc = scratch(c, B_G, (size_t)chunk * N * N, &d_G, "zone matrices"))) return rc;
    if ((rc = scratch(c, B_GV, (size_t)chunk * N, &d_gv, "zone vectors"))) return rc;
  }
  cudaEventRecord(c->ev[1], st);
  for (int64_t k0 = 0; k0 < nact; k0 += chunk) {
    const int32_t nk = (int32_t)std::min<int64_t>(chunk, nact - k0);
    e = zone_gram_fp64_list(P.g, P.so, N, lp, d_list + k0, nk, P.zxyzt, P.corr, P.maxl, d_G, d_gv,
                            d_nobs, P.brute, d_work, st);
    if (e != cudaSuccess) return cuda_fail(e, "selection/Gram kernel");
    e = zone_adjoint_fp64(P.g, P.so, N, lp, d_list + k0, nk, P.zxyzt, P.corr, P.maxl, P.zstart,
                          P.Sf, ldS, d_seed, inflation, d_G, d_gv, d_nobs, d_dyo, d_dr, d_scal,
                          P.brute, d_work + 1, st);
    if (e != cudaSuccess) return cuda_fail(e, "adjoint kernel");
  }
  cudaEventRecord(c->ev[6], st);
  double hs[2] = {0, 0};
  if ((e = cudaMemcpyAsync(hs, d_scal, 2 * sizeof(double), cudaMemcpyDeviceToHost, st)))
    return cuda_fail(e, "D2H");
  if (mem == OAKG_MEM_HOST && m > 0) {
    if (dJ_dyo && (e = cudaMemcpyAsync(dJ_dyo, d_dyo, m * sizeof(double), cudaMemcpyDeviceToHost,
                                       st)))
      return cuda_fail(e, "D2H dJ_dyo");
    if (dJ_dr &&
        (e = cudaMemcpyAsync(dJ_dr, d_dr, m * sizeof(double), cudaMemcpyDeviceToHost, st)))
      return cuda_fail(e, "D2H dJ_dr");
  }
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_fail(e, "synchronize");
  if (dJ_dlen) *dJ_dlen = hs[0];
  if (dJ_dinfl) *dJ_dinfl = hs[1];
  c->timings[0] = elapsed(c->ev[0], c->ev[1]);
  c->timings[1] = elapsed(c->ev[1], c->ev[6]);
  c->timings[2] = c->timings[3] = 0.0;
  c->timings[4] = elapsed(c->ev[0], c->ev[6]);
  return OAKG_OK;
}

int analysis_impl(const oakg_dims* dims, const double* xf, const double* Hxf,
                  const double* yo, const double* Sf, const double* HSf, const double* r_diag,
                  double* xa, double* Sa, double* ampl) {
  int rc = check_dims(dims);
  if (rc) return rc;
  if (dims->N > max_fp64_ensemble())
    return fail(OAKG_ERR_ARGS, "the global analysis (FP64) takes N <= %d", max_fp64_ensemble());
  const int64_t n = dims->n, m = dims->m, ldS = dims->ldS, ldH = dims->ldH;
  const int N = dims->N, mem = dims->mem;
  if (!xf || !Sf || !xa) return fail(OAKG_ERR_ARGS, "xf, Sf and xa are required");
  if (m > 0 && (!Hxf || !yo || !HSf || !r_diag))
    return fail(OAKG_ERR_ARGS, "Hxf, yo, HSf and r_diag are required when m > 0");
  Ctx* c = nullptr;
  if ((rc = get_ctx(&c))) return rc;
  cudaStream_t st = c->stream;
  cudaError_t e;
  cudaEventRecord(c->ev[0], st);
  const double *d_xf, *d_Hxf = nullptr, *d_yo = nullptr, *d_r = nullptr, *d_Sf, *d_HSf = nullptr;
  if ((rc = stage_in(c, B_XF, xf, (size_t)n, mem, &d_xf, "xf"))) return rc;
  if ((rc = stage_in(c, B_SF, Sf, (size_t)ldS * N, mem, &d_Sf, "Sf"))) return rc;
  if (m > 0) {
    if ((rc = stage_in(c, B_HXF, Hxf, (size_t)m, mem, &d_Hxf, "Hxf"))) return rc;
    if ((rc = stage_in(c, B_YO, yo, (size_t)m, mem, &d_yo, "yo"))) return rc;
    if ((rc = stage_in(c, B_R, r_diag, (size_t)m, mem, &d_r, "r_diag"))) return rc;
    if ((rc = stage_in(c, B_HSF, HSf, (size_t)ldH * N, mem, &d_HSf, "HSf"))) return rc;
  }
  double *d_xa, *d_Sa, *d_ampl;
  if ((rc = stage_out(c, B_XA, xa, (size_t)n, mem, &d_xa, "xa"))) return rc;
  if ((rc = stage_out(c, B_SA, Sa, (size_t)ldS * N, mem, &d_Sa, "Sa"))) return rc;
  if ((rc = stage_out(c, B_AMPL, ampl, (size_t)N, mem, &d_ampl, "amplitudes"))) return rc;
  if (mem == OAKG_MEM_HOST && Sa) {
    e = cudaMemcpyAsync(d_Sa, d_Sf, (size_t)ldS * N * sizeof(double), cudaMemcpyDeviceToDevice,
                        st);
    if (e != cudaSuccess) return cuda_fail(e, "Sa init");
  }
  double *d_G, *d_gv, *d_za;
  int32_t *d_status, *d_work, *d_nobs;
  int64_t* d_zstart;
  if ((rc = scratch(c, B_G, (size_t)N * N, &d_G, "Gram"))) return rc;
  if ((rc = scratch(c, B_GV, (size_t)N, &d_gv, "Gram"))) return rc;
  if ((rc = scratch(c, B_ZAMPL, (size_t)N, &d_za, "amplitudes"))) return rc;
  if ((rc = scratch(c, B_STATUS, 2, &d_status, "status"))) return rc;
  if ((rc = scratch(c, B_WORK, 8, &d_work, "work"))) return rc;
  double *d_aux, *d_zvec;
  if ((rc = scratch(c, B_AUX, zone_eig_aux(N), &d_aux, "zone aux"))) return rc;
  if ((rc = scratch(c, B_ZVEC, (size_t)N * N, &d_zvec, "zone eigenvectors"))) return rc;
  if ((rc = scratch(c, B_NOBS, 2, &d_nobs, "nobs"))) return rc;
  if ((rc = scratch(c, B_ZSTART, 2, &d_zstart, "zone offsets"))) return rc;
  int64_t hz[2] = {0, n};
  e = cudaMemcpyAsync(d_zstart, hz, sizeof(hz), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return cuda_fail(e, "H2D");
  // The reference runs analysisIncrement even without observations; the result is then
  // xa = xf, Sa = Sf (G = 0 -> T = I, v = w -> Omega = I), which the copy path gives.
  k_set_int<<<1, 1, 0, st>>>(d_nobs, m > 0 ? 1 : 0);
  count_launches(1);
  if (m > 0) {
    e = global_gram_fp64(m, N, d_HSf, ldH, d_yo, d_Hxf, d_r, d_G, d_gv, st);
    if (e != cudaSuccess) return cuda_fail(e, "Gram kernel");
  }
  cudaEventRecord(c->ev[2], st);
  e = zone_eig_fp64(N, 1, d_G, d_gv, d_nobs, 1, d_za, d_status, d_aux, d_zvec, d_work + 4, st);
  if (e != cudaSuccess) return cuda_fail(e, "eigensolve kernel");
  cudaEventRecord(c->ev[3], st);
  if (m == 0) cudaMemsetAsync(d_za, 0, N * sizeof(double), st);
  int32_t zone_max = (int32_t)std::min<int64_t>(n, INT32_MAX);
  e = zone_update_fp64(N, 0, 1, d_zstart, zone_max, d_xf, d_Sf, ldS, d_G, d_za, d_nobs, d_xa,
                       d_Sa, st);
  if (e != cudaSuccess) return cuda_fail(e, "update kernel");
  cudaEventRecord(c->ev[4], st);
  if (d_ampl) {
    e = cudaMemcpyAsync(d_ampl, d_za, N * sizeof(double), cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "amplitudes");
  }
  int32_t hstatus = 0;
  e = cudaMemcpyAsync(&hstatus, d_status, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return cuda_fail(e, "D2H");
  if (mem == OAKG_MEM_HOST) {
    if ((e = cudaMemcpyAsync(xa, d_xa, n * sizeof(double), cudaMemcpyDeviceToHost, st)))
      return cuda_fail(e, "D2H xa");
    if (Sa && (e = cudaMemcpyAsync(Sa, d_Sa, (size_t)ldS * N * sizeof(double),
                                   cudaMemcpyDeviceToHost, st)))
      return cuda_fail(e, "D2H Sa");
    if (ampl && (e = cudaMemcpyAsync(ampl, d_ampl, (size_t)N * sizeof(double),
                                     cudaMemcpyDeviceToHost, st)))
      return cuda_fail(e, "D2H amplitudes");
  }
  cudaEventRecord(c->ev[6], st);
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_fail(e, "synchronize");
  c->timings[0] = 0;
  c->timings[1] = elapsed(c->ev[0], c->ev[2]);
  c->timings[2] = elapsed(c->ev[2], c->ev[3]);
  c->timings[3] = elapsed(c->ev[3], c->ev[4]);
  c->timings[4] = elapsed(c->ev[0], c->ev[6]);
  return status_code(hstatus);
}

// ------------------------------------------------------------------------------------------
// Plans: a local analysis over fixed device buffers, prepared once (staging, zone offsets,
// observation cell grid, scratch) and replayed as one CUDA graph. The graph re-bins the
// observations, so new values and positions in the same buffers are honoured; the cell grid's
// geometry is that of the preparation (observations outside it fall in its edge cells, which
// the zone scans always reach, so results stay exact). With tuning, the cell edge is chosen
// among multiples of the localisation reach by timing the selection + Gram stage on the data.
struct Plan {
  Ctx ctx;  // private buffers, events and the capture stream
  oakg_dims dims{};
  oakg_loc loc{};
  int32_t Z = 0;
  Prep P{};
  ChunkArgs ca{};
  int32_t* d_status_all = nullptr;
  int32_t* h_status = nullptr;  // pinned
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  size_t nodes = 0;
  double cell_size = 0.0;
  double tune_ms[8] = {};
  double tune_cell[8] = {};
  int ntune = 0;
  // zone schedule of the selection + Gram stage: descending observation count (1) or index
  // order (0), with the two measured stage times
  int32_t zorder_used = 0;
  double order_ms[2] = {0.0, 0.0};
};

void plan_free(Plan* pl) {
  if (!pl) return;
  if (pl->ctx.stream) cudaStreamSynchronize(pl->ctx.stream);
  if (pl->exec) cudaGraphExecDestroy(pl->exec);
  if (pl->graph) cudaGraphDestroy(pl->graph);
  if (pl->h_status) cudaFreeHost(pl->h_status);
  for (auto& b : pl->ctx.buf) b.release();
  for (auto& ev : pl->ctx.ev)
    if (ev) cudaEventDestroy(ev);
  if (pl->ctx.own_stream) cudaStreamDestroy(pl->ctx.own_stream);
  delete pl;
}

template <typename R>
int plan_run(Plan* pl, RunMode mode, double* t_gram) {
  double tg = 0, te = 0, tu = 0;
  int rc = run_chunks<R>(&pl->ctx, pl->ca, &pl->d_status_all, &tg, &te, &tu, mode);
  if (t_gram) *t_gram = tg;
  return rc;
}

int plan_run_mode(Plan* pl, RunMode mode, double* t_gram = nullptr) {
  return (pl->loc.precision != OAKG_PREC_FP64) ? plan_run<float>(pl, mode, t_gram)
                                                : plan_run<double>(pl, mode, t_gram);
}

int plan_create_impl(Plan** out, const oakg_dims* dims, const oakg_loc* loc, int32_t Z,
                     const int32_t* zone_size, const double* xf, const double* Hxf,
                     const double* yo, const double* Sf, const double* HSf, const double* r_diag,
                     const double* zone_xyzt, const double* obs_x, const double* obs_y,
                     const double* obs_z, const double* obs_t, const double* corr_len,
                     const double* max_len, double* xa, double* Sa, double* ampl,
                     int32_t* nobs_out, int32_t tune) {
  if (!out) return fail(OAKG_ERR_ARGS, "plan is NULL");
  *out = nullptr;
  int rc = check_loc(dims, loc, Z);
  if (rc) return rc;
  if (dims->mem != OAKG_MEM_DEVICE)
    return fail(OAKG_ERR_ARGS, "plans bind device buffers: dims->mem must be OAKG_MEM_DEVICE");
  if (!xf || !xa) return fail(OAKG_ERR_ARGS, "xf and xa are required");
  Plan* pl = new Plan();
  Ctx* c = &pl->ctx;
  cudaError_t e = cudaGetDevice(&c->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    plan_free(pl);
    return cuda_fail(e, "plan stream");
  }
  c->stream = c->own_stream;
  for (auto& ev : c->ev) cudaEventCreate(&ev);
  pl->dims = *dims;
  pl->loc = *loc;
  pl->Z = Z;
  const int N = dims->N;
  const int64_t m = dims->m, ldH = dims->ldH;
  auto setup = [&](const oakg_loc* lc) -> int {
    int r = prepare_loc(c, dims, lc, Z, zone_size, xf, Hxf, yo, Sf, HSf, r_diag, zone_xyzt,
                        obs_x, obs_y, obs_z, obs_t, corr_len, max_len, &pl->P);
    if (r) return r;
    int32_t* d_nobs = nobs_out;
    if (!d_nobs && (r = scratch(c, B_NOBS, (size_t)Z, &d_nobs, "nobs"))) return r;
    LocParams lp{lc->weight, lc->metric, lc->loctype, lc->localise_obs ? 1 : 0,
                 lc->rotate ? 1 : 0, lc->flags};
    const int all_ampl = (!lc->localise_obs) || (lc->flags & OAKG_FLAG_AMPL_ALWAYS);
    pl->ca = ChunkArgs{pl->P.g, pl->P.so, lp, Z, N, dims->ldS, pl->P.zone_max, pl->P.brute,
                       all_ampl, pl->P.zxyzt, pl->P.corr, pl->P.maxl, pl->P.zstart, pl->P.xf,
                       pl->P.Sf, xa, Sa, ampl, d_nobs};
    pl->ca.refine = (lc->precision == OAKG_PREC_MIXED_FP64EIG);
    return OAKG_OK;
  };
  oakg_loc lc = *loc;
  if ((rc = setup(&lc))) {
    plan_free(pl);
    return rc;
  }
  if (tune && lc.cell_size <= 0.0 && m > 0 && !pl->P.brute) {
    // the default edge is half the reach; candidates from a quarter to one reach
    const double reach = 2.0 * pl->P.g.csv;
    const double factors[5] = {0.25, 0.35, 0.5, 0.7, 1.0};
    double best = -1.0, best_ms = 1e300;
    for (double f : factors) {
      lc.cell_size = f * reach;
      double ms = 0.0;
      if ((rc = setup(&lc)) || (rc = plan_run_mode(pl, RunMode::kGramOnly)) ||
          (rc = plan_run_mode(pl, RunMode::kGramOnly, &ms))) {
        plan_free(pl);
        return rc;
      }
      if (pl->ntune < 8) {
        pl->tune_cell[pl->ntune] = lc.cell_size;
        pl->tune_ms[pl->ntune++] = ms;
      }
      if (ms < best_ms) {
        best_ms = ms;
        best = lc.cell_size;
      }
    }
    lc.cell_size = best;
    if ((rc = setup(&lc))) {
      plan_free(pl);
      return rc;
    }
  }
  pl->loc = lc;
  pl->cell_size = pl->P.g.csv;
  // fix the chunk size so that the captured sequence queries nothing, then one ordinary run
  // allocates every buffer at that size and sets the kernel attributes
  {
    const size_t per_zone =
        ((size_t)N * N * 2 + (size_t)N * 2 + zone_eig_aux(N)) *
            (lc.precision != OAKG_PREC_FP64 ? sizeof(float) : sizeof(double)) +
        2 * sizeof(int32_t) +
        (lc.precision == OAKG_PREC_MIXED_FP64EIG
             ? ((size_t)N * N + zone_refine_scratch(N)) * sizeof(float)
             : 0);
    const int64_t chunk = (int64_t)(chunk_budget_bytes() / per_zone);
    c->chunk_override = std::max<int64_t>(1, std::min<int64_t>(chunk, Z));
  }
  // zone schedule: the persistent selection + Gram blocks take zones off a counter, and the
  // observation counts of a zone range from 0 to thousands; taking each chunk's zones in
  // descending count (longest tasks first) shortens the tail. Kept when it measures faster.
  if (tune && m > 0) {
    double ms_nat = 0.0, ms_ord = 0.0;
    if ((rc = plan_run_mode(pl, RunMode::kGramOnly)) ||
        (rc = plan_run_mode(pl, RunMode::kGramOnly, &ms_nat))) {
      plan_free(pl);
      return rc;
    }
    std::vector<int32_t> cnt((size_t)Z), ord((size_t)Z);
    if ((e = cudaMemcpyAsync(cnt.data(), pl->ca.nobs, sizeof(int32_t) * (size_t)Z,
                             cudaMemcpyDeviceToHost, c->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(c->stream)) != cudaSuccess) {
      plan_free(pl);
      return cuda_fail(e, "observation counts");
    }
    const int64_t chunk = c->chunk_override;
    for (int64_t z0 = 0; z0 < Z; z0 += chunk) {
      const int64_t nzc = std::min<int64_t>(chunk, Z - z0);
      int32_t* o = ord.data() + z0;
      for (int64_t i = 0; i < nzc; i++) o[i] = (int32_t)i;
      const int32_t* cz = cnt.data() + z0;
      std::stable_sort(o, o + nzc, [cz](int32_t a, int32_t b) { return cz[a] > cz[b]; });
    }
    int32_t* d_ord;
    if ((rc = scratch(c, B_ORDER, (size_t)Z, &d_ord, "zone order"))) {
      plan_free(pl);
      return rc;
    }
    if ((e = cudaMemcpyAsync(d_ord, ord.data(), sizeof(int32_t) * (size_t)Z,
                             cudaMemcpyHostToDevice, c->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(c->stream)) != cudaSuccess) {
      plan_free(pl);
      return cuda_fail(e, "zone order");
    }
    pl->ca.zorder = d_ord;
    if ((rc = plan_run_mode(pl, RunMode::kGramOnly)) ||
        (rc = plan_run_mode(pl, RunMode::kGramOnly, &ms_ord))) {
      plan_free(pl);
      return rc;
    }
    pl->order_ms[0] = ms_nat;
    pl->order_ms[1] = ms_ord;
    pl->zorder_used = (ms_ord < ms_nat) ? 1 : 0;
    if (!pl->zorder_used) pl->ca.zorder = nullptr;
  }
  if ((rc = plan_run_mode(pl, RunMode::kTimed))) {
    plan_free(pl);
    return rc;
  }
  if ((e = cudaStreamSynchronize(c->stream)) != cudaSuccess) {
    plan_free(pl);
    return cuda_fail(e, "synchronize");
  }
  e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    plan_free(pl);
    return cuda_fail(e, "begin capture");
  }
  int rc_cap = bin_observations(c, &lc, m, N, ldH, &pl->P);
  if (!rc_cap) {
    pl->ca.so = pl->P.so;
    rc_cap = plan_run_mode(pl, RunMode::kCapture);
  }
  cudaGraph_t graph = nullptr;
  e = cudaStreamEndCapture(c->stream, &graph);
  pl->graph = graph;
  if (rc_cap) {
    plan_free(pl);
    return rc_cap;
  }
  if (e != cudaSuccess) {
    plan_free(pl);
    return cuda_fail(e, "end capture");
  }
  if ((e = cudaGraphInstantiate(&pl->exec, pl->graph, 0)) != cudaSuccess) {
    plan_free(pl);
    return cuda_fail(e, "graph instantiate");
  }
  cudaGraphGetNodes(pl->graph, nullptr, &pl->nodes);
  if ((e = cudaMallocHost(&pl->h_status, sizeof(int32_t))) != cudaSuccess) {
    plan_free(pl);
    return cuda_fail(e, "pinned status");
  }
  *out = pl;
  return OAKG_OK;
}

int plan_execute_impl(Plan* pl, void* stream) {
  if (!pl) return fail(OAKG_ERR_ARGS, "plan is NULL");
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : pl->ctx.stream;
  cudaError_t e = cudaGraphLaunch(pl->exec, st);
  if (e != cudaSuccess) return cuda_fail(e, "graph launch");
  count_launches((int)pl->nodes);
  e = cudaMemcpyAsync(pl->h_status, pl->d_status_all, sizeof(int32_t), cudaMemcpyDeviceToHost,
                      st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "plan execution");
  return status_code(*pl->h_status);
}

// ------------------------------------------------------------------------------------------
// Ensemble prologue / epilogue (ensemble.cu) and the whole-ensemble local analysis.
int check_obsoper(const oakg_obsoper* H, int64_t m) {
  if (m == 0) return OAKG_OK;
  if (!H) return fail(OAKG_ERR_ARGS, "observation operator is NULL with m > 0");
  if (H->m != m) return fail(OAKG_ERR_ARGS, "operator has %lld rows, m = %lld",
                             (long long)H->m, (long long)m);
  if (H->K < 1) return fail(OAKG_ERR_ARGS, "operator K must be >= 1");
  if (!H->index || !H->weight) return fail(OAKG_ERR_ARGS, "operator index/weight are NULL");
  return OAKG_OK;
}

struct EnsDev {
  const double *Ef = nullptr, *w = nullptr, *shift = nullptr;
  const int64_t* idx = nullptr;
  double *xf = nullptr, *Sf = nullptr, *Hxf = nullptr, *HSf = nullptr, *HEf = nullptr;
};

// device view of Ef and H, device outputs of the prologue (caller's buffers in device mode)
int prologue_issue(Ctx* c, const oakg_dims* d, const double* Ef, int64_t ldE,
                   const oakg_obsoper* H, double* xf, double* Sf, double* Hxf, double* HSf,
                   EnsDev* E) {
  const int64_t n = d->n, m = d->m;
  const int N = d->N, mem = d->mem;
  int rc;
  if ((rc = stage_in(c, B_E_EF, Ef, (size_t)ldE * N, mem, &E->Ef, "Ef"))) return rc;
  if (m > 0) {
    const size_t mk = (size_t)m * H->K;
    if ((rc = stage_in(c, B_E_HIDX, H->index, mk, mem, &E->idx, "operator index"))) return rc;
    if ((rc = stage_in(c, B_E_HW, H->weight, mk, mem, &E->w, "operator weight"))) return rc;
    if ((rc = stage_in(c, B_E_HSH, H->shift, (size_t)m, mem, &E->shift, "Hshift"))) return rc;
    if ((rc = scratch(c, B_E_HEF, (size_t)m * N, &E->HEf, "HEf"))) return rc;
  }
  if ((rc = stage_out(c, B_E_XF, xf, (size_t)n, mem, &E->xf, "xf"))) return rc;
  if ((rc = stage_out(c, B_E_SF, Sf, (size_t)d->ldS * N, mem, &E->Sf, "Sf"))) return rc;
  if ((rc = stage_out(c, B_E_HXF, Hxf, (size_t)(m > 0 ? m : 1), mem, &E->Hxf, "Hxf"))) return rc;
  if ((rc = stage_out(c, B_E_HSF, HSf, (size_t)(m > 0 ? d->ldH : 1) * N, mem, &E->HSf, "HSf")))
    return rc;
  cudaError_t e = ensemble_prologue(n, N, E->Ef, ldE, m, m > 0 ? H->K : 1, E->idx, E->w, E->shift,
                                    E->xf, E->Sf, d->ldS, E->Hxf, E->HSf, d->ldH, E->HEf,
                                    c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "ensemble prologue");
  return OAKG_OK;
}

int prologue_impl(const oakg_dims* d, const double* Ef, int64_t ldE, const oakg_obsoper* H,
                  double* xf, double* Sf, double* Hxf, double* HSf) {
  int rc = check_dims(d);
  if (rc) return rc;
  if (!Ef || !xf || !Sf) return fail(OAKG_ERR_ARGS, "Ef, xf and Sf are required");
  if (ldE < d->n) return fail(OAKG_ERR_ARGS, "ldE < n");
  if ((rc = check_obsoper(H, d->m))) return rc;
  if (d->m > 0 && (!Hxf || !HSf)) return fail(OAKG_ERR_ARGS, "Hxf and HSf are required");
  Ctx* c = nullptr;
  if ((rc = get_ctx(&c))) return rc;
  EnsDev E;
  if ((rc = prologue_issue(c, d, Ef, ldE, H, xf, Sf, Hxf, HSf, &E))) return rc;
  cudaStream_t st = c->stream;
  cudaError_t e = cudaSuccess;
  if (d->mem == OAKG_MEM_HOST) {
    const int N = d->N;
    e = cudaMemcpyAsync(xf, E.xf, d->n * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(Sf, E.Sf, (size_t)d->ldS * N * sizeof(double), cudaMemcpyDeviceToHost,
                          st);
    if (e == cudaSuccess && d->m > 0)
      e = cudaMemcpyAsync(Hxf, E.Hxf, d->m * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && d->m > 0)
      e = cudaMemcpyAsync(HSf, E.HSf, (size_t)d->ldH * N * sizeof(double),
                          cudaMemcpyDeviceToHost, st);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "prologue results");
  return OAKG_OK;
}

int epilogue_impl(const oakg_dims* d, const double* xf, const double* xa, const double* Sa,
                  double inflation, const double* max_correction, double* Ea, int64_t ldE) {
  int rc = check_dims(d);
  if (rc) return rc;
  if (!xf || !xa || !Sa || !Ea) return fail(OAKG_ERR_ARGS, "xf, xa, Sa and Ea are required");
  if (ldE < d->n) return fail(OAKG_ERR_ARGS, "ldE < n");
  Ctx* c = nullptr;
  if ((rc = get_ctx(&c))) return rc;
  const int64_t n = d->n;
  const int N = d->N, mem = d->mem;
  const double *dxf, *dxa, *dSa, *dmc;
  double* dEa;
  if ((rc = stage_in(c, B_E_XF, xf, (size_t)n, mem, &dxf, "xf"))) return rc;
  if ((rc = stage_in(c, B_E_XA, xa, (size_t)n, mem, &dxa, "xa"))) return rc;
  if ((rc = stage_in(c, B_E_SA, Sa, (size_t)d->ldS * N, mem, &dSa, "Sa"))) return rc;
  if ((rc = stage_in(c, B_E_MC, max_correction, (size_t)n, mem, &dmc, "maxCorrection")))
    return rc;
  if ((rc = stage_out(c, B_E_EA, Ea, (size_t)ldE * N, mem, &dEa, "Ea"))) return rc;
  cudaStream_t st = c->stream;
  cudaError_t e = ensemble_epilogue(n, N, dxf, dxa, dSa, d->ldS, inflation, dmc, dEa, ldE, st);
  if (e == cudaSuccess && mem == OAKG_MEM_HOST)
    e = cudaMemcpyAsync(Ea, dEa, (size_t)ldE * N * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "ensemble epilogue");
  return OAKG_OK;
}

int ens_locanalysis_impl(const oakg_dims* d, const oakg_loc* loc, int32_t Z,
                         const int32_t* zone_size, const double* Ef, int64_t ldE,
                         const oakg_obsoper* H, const double* yo, const double* r_diag,
                         const double* zone_xyzt, const double* obs_x, const double* obs_y,
                         const double* obs_z, const double* obs_t, const double* corr_len,
                         const double* max_len, double inflation,
                         const double* max_correction, double* Ea) {
  int rc = check_loc(d, loc, Z);
  if (rc) return rc;
  if (!Ef || !Ea) return fail(OAKG_ERR_ARGS, "Ef and Ea are required");
  if (ldE < d->n) return fail(OAKG_ERR_ARGS, "ldE < n");
  if ((rc = check_obsoper(H, d->m))) return rc;
  Ctx* c = nullptr;
  if ((rc = get_ctx(&c))) return rc;
  const int64_t n = d->n, m = d->m;
  const int N = d->N, mem = d->mem;
  // device views of every input (the inner analysis runs in device mode)
  const int32_t* dzs;
  const double *dyo = nullptr, *dr = nullptr, *dzp, *dox = nullptr, *doy = nullptr,
               *doz = nullptr, *dot = nullptr, *dcorr, *dmaxl, *dmc;
  if ((rc = stage_in(c, B_ZONE_SIZE, zone_size, (size_t)Z, mem, &dzs, "zone_size"))) return rc;
  if ((rc = stage_in(c, B_ZXYZT, zone_xyzt, (size_t)4 * Z, mem, &dzp, "zone_xyzt"))) return rc;
  if ((rc = stage_in(c, B_CORR, corr_len, (size_t)Z, mem, &dcorr, "corr_len"))) return rc;
  if ((rc = stage_in(c, B_MAXL, max_len, (size_t)Z, mem, &dmaxl, "max_len"))) return rc;
  if ((rc = stage_in(c, B_E_MC, max_correction, (size_t)n, mem, &dmc, "maxCorrection")))
    return rc;
  if (m > 0) {
    if ((rc = stage_in(c, B_YO, yo, (size_t)m, mem, &dyo, "yo"))) return rc;
    if ((rc = stage_in(c, B_R, r_diag, (size_t)m, mem, &dr, "r_diag"))) return rc;
    if ((rc = stage_in(c, B_OX, obs_x, (size_t)m, mem, &dox, "obs_x"))) return rc;
    if ((rc = stage_in(c, B_OY, obs_y, (size_t)m, mem, &doy, "obs_y"))) return rc;
    if ((rc = stage_in(c, B_OZ, obs_z, (size_t)m, mem, &doz, "obs_z"))) return rc;
    if ((rc = stage_in(c, B_OT, obs_t, (size_t)m, mem, &dot, "obs_t"))) return rc;
  }
  oakg_dims dd = *d;
  dd.mem = OAKG_MEM_DEVICE;
  dd.ldS = n;
  dd.ldH = m > 0 ? m : 1;
  EnsDev E;
  {
    // prologue outputs into library buffers (device mode with NULL outputs is not allowed,
    // so the buffers are claimed here and passed as device pointers)
    double *xf, *Sf, *Hxf, *HSf;
    if ((rc = scratch(c, B_E_XF, (size_t)n, &xf, "xf")) ||
        (rc = scratch(c, B_E_SF, (size_t)n * N, &Sf, "Sf")) ||
        (rc = scratch(c, B_E_HXF, (size_t)(m > 0 ? m : 1), &Hxf, "Hxf")) ||
        (rc = scratch(c, B_E_HSF, (size_t)(m > 0 ? m : 1) * N, &HSf, "HSf")))
      return rc;
    oakg_dims pd = dd;
    pd.mem = mem;  // Ef and H are staged from the caller's memory kind
    const double* Ef_view;
    if ((rc = stage_in(c, B_E_EF, Ef, (size_t)ldE * N, mem, &Ef_view, "Ef"))) return rc;
    oakg_obsoper Hd{};
    if (m > 0) {
      Hd = *H;
      const size_t mk = (size_t)m * H->K;
      if ((rc = stage_in(c, B_E_HIDX, H->index, mk, mem, &Hd.index, "operator index")) ||
          (rc = stage_in(c, B_E_HW, H->weight, mk, mem, &Hd.weight, "operator weight")) ||
          (rc = stage_in(c, B_E_HSH, H->shift, (size_t)m, mem, &Hd.shift, "Hshift")))
        return rc;
    }
    pd.mem = OAKG_MEM_DEVICE;
    if ((rc = prologue_issue(c, &pd, Ef_view, ldE, m > 0 ? &Hd : nullptr, xf, Sf, Hxf, HSf, &E)))
      return rc;
  }
  double *xa, *Sa;
  if ((rc = scratch(c, B_E_XA, (size_t)n, &xa, "xa")) ||
      (rc = scratch(c, B_E_SA, (size_t)n * N, &Sa, "Sa")))
    return rc;
  rc = locanalysis_impl<double>(&dd, loc, Z, dzs, E.xf, E.Hxf, dyo, E.Sf, E.HSf, dr, dzp, dox, doy, doz,
                        dot, dcorr, dmaxl, xa, Sa, nullptr, nullptr);
  if (rc) return rc;
  double* dEa;
  if ((rc = stage_out(c, B_E_EA, Ea, (size_t)ldE * N, mem, &dEa, "Ea"))) return rc;
  cudaStream_t st = c->stream;
  cudaError_t e = ensemble_epilogue(n, N, E.xf, xa, Sa, n, inflation, dmc, dEa, ldE, st);
  if (e == cudaSuccess && mem == OAKG_MEM_HOST)
    e = cudaMemcpyAsync(Ea, dEa, (size_t)ldE * N * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "ensemble epilogue");
  return OAKG_OK;
}

// ens2sqrt (rrsqrt.F90:786-806): mean and the N - 1 anomaly columns of Pham's reduction
int ens2sqrt_impl(const oakg_dims* d, const double* E, int64_t ldE, double* mean, double* S) {
  int rc = check_dims(d);
  if (rc) return rc;
  if (!E || !mean || !S) return fail(OAKG_ERR_ARGS, "E, mean and S are required");
  if (ldE < d->n) return fail(OAKG_ERR_ARGS, "ldE < n");
  Ctx* c = nullptr;
  if ((rc = get_ctx(&c))) return rc;
  const int64_t n = d->n;
  const int N = d->N, mem = d->mem;
  const double* dE;
  double *dmean, *dS;
  if ((rc = stage_in(c, B_C_E, E, (size_t)ldE * N, mem, &dE, "E")) ||
      (rc = stage_out(c, B_C_MEAN, mean, (size_t)n, mem, &dmean, "mean")) ||
      (rc = stage_out(c, B_C_S, S, (size_t)d->ldS * (N - 1), mem, &dS, "S")))
    return rc;
  cudaStream_t st = c->stream;
  cudaError_t e = ensemble_ens2sqrt(n, N, dE, ldE, dmean, dS, d->ldS, st);
  if (e == cudaSuccess && mem == OAKG_MEM_HOST) {
    e = cudaMemcpyAsync(mean, dmean, n * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(S, dS, (size_t)d->ldS * (N - 1) * sizeof(double),
                          cudaMemcpyDeviceToHost, st);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "ens2sqrt");
  return OAKG_OK;
}

// sqrt2ens (rrsqrt.F90:815-839): E = mean + S Om^T, Om = sqrt(N-1) perpSpace(w) Theta, w = 1/sqrt(N)
// (perpSpace: matoper.F90:509-535). The reference draws Theta at random (randOrthMatrix);
// here it is the caller's (N-1) x (N-1) orthogonal matrix, or the identity. With the identity
// E has a closed form (one read of S, one write of E); a general Theta takes the n x (N-1) by
// (N-1) x N product, a plain dense GEMM, from cuBLAS over E pre-filled with the mean.
int sqrt2ens_impl(const oakg_dims* d, const double* mean, const double* S, const double* theta,
                  double* E, int64_t ldE) {
  int rc = check_dims(d);
  if (rc) return rc;
  if (!mean || !S || !E) return fail(OAKG_ERR_ARGS, "mean, S and E are required");
  if (ldE < d->n) return fail(OAKG_ERR_ARGS, "ldE < n");
  Ctx* c = nullptr;
  if ((rc = get_ctx(&c))) return rc;
  const int64_t n = d->n;
  const int N = d->N, K = N - 1, mem = d->mem;
  cudaStream_t st = c->stream;
  cudaError_t e = cudaSuccess;
  if (!theta) {
    const double* dmean;
    const double* dS;
    double* dE;
    if ((rc = stage_in(c, B_C_MEAN, mean, (size_t)n, mem, &dmean, "mean")) ||
        (rc = stage_in(c, B_C_S, S, (size_t)d->ldS * K, mem, &dS, "S")) ||
        (rc = stage_out(c, B_C_EO, E, (size_t)ldE * N, mem, &dE, "E")))
      return rc;
    e = ensemble_sqrt2ens_identity(n, N, dmean, dS, d->ldS, dE, ldE, st);
    if (e == cudaSuccess && mem == OAKG_MEM_HOST)
      e = cudaMemcpyAsync(E, dE, (size_t)ldE * N * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "sqrt2ens");
    return OAKG_OK;
  }
  std::vector<double> th((size_t)K * K, 0.0), om((size_t)N * K, 0.0), P((size_t)N * K, 0.0);
  if (theta) {
    e = cudaMemcpy(th.data(), theta, th.size() * sizeof(double),
                   mem == OAKG_MEM_DEVICE ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost);
    if (e != cudaSuccess) return cuda_fail(e, "theta");
  } else {
    for (int i = 0; i < K; i++) th[(size_t)i * K + i] = 1.0;
  }
  const double w = 1.0 / std::sqrt((double)N), alpha = -1.0 / (w + 1.0);
  for (int i = 0; i < N; i++)
    for (int j = 0; j < K; j++)
      P[(size_t)i * K + j] = (i < K) ? alpha * w * w + (i == j ? 1.0 : 0.0) : alpha * (w + 1.0) * w;
  const double sc = std::sqrt((double)N - 1.0);
  for (int i = 0; i < N; i++)
    for (int k = 0; k < K; k++) {
      double acc = 0.0;
      for (int l = 0; l < K; l++) acc += P[(size_t)i * K + l] * th[(size_t)l + (size_t)k * K];
      om[(size_t)i * K + k] = sc * acc;
    }
  double* dOm;
  if ((rc = scratch(c, B_C_OM, om.size(), &dOm, "Omega"))) return rc;
  const double *dmean, *dS;
  double* dE;
  if ((rc = stage_in(c, B_C_MEAN, mean, (size_t)n, mem, &dmean, "mean")) ||
      (rc = stage_in(c, B_C_S, S, (size_t)d->ldS * K, mem, &dS, "S")) ||
      (rc = stage_out(c, B_C_EO, E, (size_t)ldE * N, mem, &dE, "E")))
    return rc;
  if (!c->blas) {
    if (cublasCreate(&c->blas) != CUBLAS_STATUS_SUCCESS) {
      c->blas = nullptr;
      return fail(OAKG_ERR_CUDA, "cublasCreate failed");
    }
  }
  e = cudaMemcpyAsync(dOm, om.data(), om.size() * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = ensemble_fill_columns(n, N, dmean, dE, ldE, st);
  if (e == cudaSuccess) {
    // E += S Om^T: om is Om row-major (N x K), i.e. Om^T column-major with leading dimension K
    const double one = 1.0;
    cublasStatus_t bs = cublasSetStream(c->blas, st);
    if (bs == CUBLAS_STATUS_SUCCESS)
      bs = cublasDgemm_64(c->blas, CUBLAS_OP_N, CUBLAS_OP_N, n, N, K, &one, dS, d->ldS,
                          dOm, K, &one, dE, ldE);
    if (bs != CUBLAS_STATUS_SUCCESS) {
      cudaStreamSynchronize(st);
      return fail(OAKG_ERR_CUDA, "cublasDgemm failed (status %d)", (int)bs);
    }
  }
  if (e == cudaSuccess && mem == OAKG_MEM_HOST)
    e = cudaMemcpyAsync(E, dE, (size_t)ldE * N * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // also keeps om alive for the copy
  if (e != cudaSuccess) return cuda_fail(e, "sqrt2ens");
  return OAKG_OK;
}

// ensAnalysis (rrsqrt.F90:613-671): mean and scaled anomalies of Ef and HEf, the global
// analysis, Ea = xa + sqrt(N-1) Sa
int ens_analysis_impl(const oakg_dims* d, const double* Ef, int64_t ldE, const double* HEf,
                      int64_t ldHE, const double* yo, const double* r_diag, double* Ea,
                      double* xa, double* ampl) {
  int rc = check_dims(d);
  if (rc) return rc;
  if (!Ef || !Ea) return fail(OAKG_ERR_ARGS, "Ef and Ea are required");
  if (ldE < d->n) return fail(OAKG_ERR_ARGS, "ldE < n");
  if (d->m > 0 && (!HEf || !yo || !r_diag || ldHE < d->m))
    return fail(OAKG_ERR_ARGS, "HEf (ldHE >= m), yo and r_diag are required when m > 0");
  Ctx* c = nullptr;
  if ((rc = get_ctx(&c))) return rc;
  const int64_t n = d->n, m = d->m;
  const int N = d->N, mem = d->mem;
  cudaStream_t st = c->stream;
  const double *dEf, *dHE = nullptr, *dyo = nullptr, *dr = nullptr;
  double *xf, *Sf, *Hxf, *HSf, *dxa, *Sa, *dEa, *dampl;
  if ((rc = stage_in(c, B_C_E, Ef, (size_t)ldE * N, mem, &dEf, "Ef")) ||
      (rc = stage_in(c, B_C_HE, HEf, (size_t)(m > 0 ? ldHE : 0) * N, mem, &dHE, "HEf")) ||
      (rc = stage_in(c, B_YO, m > 0 ? yo : nullptr, (size_t)m, mem, &dyo, "yo")) ||
      (rc = stage_in(c, B_R, m > 0 ? r_diag : nullptr, (size_t)m, mem, &dr, "r_diag")) ||
      (rc = scratch(c, B_C_MEAN, (size_t)n, &xf, "xf")) ||
      (rc = scratch(c, B_C_S, (size_t)n * N, &Sf, "Sf")) ||
      (rc = scratch(c, B_C_HXF, (size_t)(m > 0 ? m : 1), &Hxf, "Hxf")) ||
      (rc = scratch(c, B_C_HSF, (size_t)(m > 0 ? m : 1) * N, &HSf, "HSf")) ||
      (rc = scratch(c, B_C_XA, (size_t)n, &dxa, "xa")) ||
      (rc = scratch(c, B_C_SA, (size_t)n * N, &Sa, "Sa")) ||
      (rc = stage_out(c, B_C_EO, Ea, (size_t)ldE * N, mem, &dEa, "Ea")) ||
      (rc = stage_out(c, B_C_AMPL, ampl, (size_t)N, mem, &dampl, "amplitudes")))
    return rc;
  // the prologue's mean/anomaly kernel on Ef and on HEf (no operator: HEf is given)
  cudaError_t e = ensemble_prologue(n, N, dEf, ldE, 0, 1, nullptr, nullptr, nullptr, xf, Sf, n,
                                    nullptr, nullptr, 1, nullptr, st);
  if (e == cudaSuccess && m > 0)
    e = ensemble_prologue(m, N, dHE, ldHE, 0, 1, nullptr, nullptr, nullptr, Hxf, HSf, m,
                          nullptr, nullptr, 1, nullptr, st);
  if (e != cudaSuccess) return cuda_fail(e, "ensemble anomalies");
  oakg_dims dd = *d;
  dd.mem = OAKG_MEM_DEVICE;
  dd.ldS = n;
  dd.ldH = m > 0 ? m : 1;
  if ((rc = analysis_impl(&dd, xf, m > 0 ? Hxf : nullptr, dyo, Sf, m > 0 ? HSf : nullptr, dr,
                          dxa, Sa, dampl)))
    return rc;
  e = ensemble_epilogue(n, N, xf, dxa, Sa, n, 1.0, nullptr, dEa, ldE, st);
  if (e == cudaSuccess && mem == OAKG_MEM_HOST) {
    e = cudaMemcpyAsync(Ea, dEa, (size_t)ldE * N * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && ampl)
      e = cudaMemcpyAsync(ampl, dampl, N * sizeof(double), cudaMemcpyDeviceToHost, st);
  }
  if (e == cudaSuccess && xa)
    e = cudaMemcpyAsync(xa, dxa, n * sizeof(double),
                        mem == OAKG_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice,
                        st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "ensemble analysis");
  return OAKG_OK;
}

// biasedLocAnalysis (rrsqrt.F90:476-546): the bias increment from a first local analysis, the
// bias ba = bf - gamma inc, the state analysed from xf - ba with R scaled by (1 - gamma)
// (DCDCovar with D = 1/sqrt(1 - gamma): R^-1 -> R^-1 / (1 - gamma), covariance.F90:611-618);
// Sa = Sf.
int biased_locanalysis_impl(const oakg_dims* d, const oakg_loc* loc, int32_t Z,
                            const int32_t* zone_size, double gamma, const oakg_obsoper* H,
                            const double* xf, const double* bf, const double* Hxf,
                            const double* yo, const double* Sf, const double* HSf,
                            const double* r_diag, const double* zone_xyzt, const double* obs_x,
                            const double* obs_y, const double* obs_z, const double* obs_t,
                            const double* corr_len, const double* max_len, double* xa,
                            double* ba, double* Sa) {
  int rc = check_loc(d, loc, Z);
  if (rc) return rc;
  if (!xf || !bf || !Sf || !xa || !ba) return fail(OAKG_ERR_ARGS, "xf, bf, Sf, xa, ba are required");
  if (!(gamma >= 0.0 && gamma < 1.0)) return fail(OAKG_ERR_ARGS, "gamma must be in [0, 1)");
  if ((rc = check_obsoper(H, d->m))) return rc;
  Ctx* c = nullptr;
  if ((rc = get_ctx(&c))) return rc;
  const int64_t n = d->n, m = d->m;
  const int N = d->N, mem = d->mem;
  cudaStream_t st = c->stream;
  // device views of the inputs the two analyses share
  const int32_t* dzs;
  const double *dxf, *dbf, *dHxf = nullptr, *dyo = nullptr, *dSf, *dHSf = nullptr, *dr = nullptr,
               *dzp, *dox = nullptr, *doy = nullptr, *doz = nullptr, *dot = nullptr, *dcorr,
               *dmaxl;
  if ((rc = stage_in(c, B_ZONE_SIZE, zone_size, (size_t)Z, mem, &dzs, "zone_size")) ||
      (rc = stage_in(c, B_ZXYZT, zone_xyzt, (size_t)4 * Z, mem, &dzp, "zone_xyzt")) ||
      (rc = stage_in(c, B_CORR, corr_len, (size_t)Z, mem, &dcorr, "corr_len")) ||
      (rc = stage_in(c, B_MAXL, max_len, (size_t)Z, mem, &dmaxl, "max_len")) ||
      (rc = stage_in(c, B_XF, xf, (size_t)n, mem, &dxf, "xf")) ||
      (rc = stage_in(c, B_C_BF, bf, (size_t)n, mem, &dbf, "bf")) ||
      (rc = stage_in(c, B_SF, Sf, (size_t)d->ldS * N, mem, &dSf, "Sf")))
    return rc;
  oakg_obsoper Hd{};
  if (m > 0) {
    if ((rc = stage_in(c, B_HXF, Hxf, (size_t)m, mem, &dHxf, "Hxf")) ||
        (rc = stage_in(c, B_YO, yo, (size_t)m, mem, &dyo, "yo")) ||
        (rc = stage_in(c, B_HSF, HSf, (size_t)d->ldH * N, mem, &dHSf, "HSf")) ||
        (rc = stage_in(c, B_R, r_diag, (size_t)m, mem, &dr, "r_diag")) ||
        (rc = stage_in(c, B_OX, obs_x, (size_t)m, mem, &dox, "obs_x")) ||
        (rc = stage_in(c, B_OY, obs_y, (size_t)m, mem, &doy, "obs_y")) ||
        (rc = stage_in(c, B_OZ, obs_z, (size_t)m, mem, &doz, "obs_z")) ||
        (rc = stage_in(c, B_OT, obs_t, (size_t)m, mem, &dot, "obs_t")))
      return rc;
    Hd = *H;
    const size_t mk = (size_t)m * H->K;
    if ((rc = stage_in(c, B_E_HIDX, H->index, mk, mem, &Hd.index, "operator index")) ||
        (rc = stage_in(c, B_E_HW, H->weight, mk, mem, &Hd.weight, "operator weight")) ||
        (rc = stage_in(c, B_E_HSH, H->shift, (size_t)m, mem, &Hd.shift, "Hshift")))
      return rc;
  }
  double *zero, *inc, *ux, *uHx = nullptr, *r2 = nullptr, *dba, *dxa, *dSa = nullptr;
  if ((rc = scratch(c, B_C_ZERO, (size_t)n, &zero, "zeros")) ||
      (rc = scratch(c, B_C_INC, (size_t)n, &inc, "increment")) ||
      (rc = scratch(c, B_C_UX, (size_t)n, &ux, "unbiased xf")) ||
      (rc = stage_out(c, B_C_BA, ba, (size_t)n, mem, &dba, "ba")) ||
      (rc = stage_out(c, B_C_XA, xa, (size_t)n, mem, &dxa, "xa")) ||
      (rc = stage_out(c, B_C_SA, Sa, (size_t)d->ldS * N, mem, &dSa, "Sa")))
    return rc;
  if (m > 0 && ((rc = scratch(c, B_C_UHX, (size_t)m, &uHx, "unbiased Hxf")) ||
                (rc = scratch(c, B_C_R2, (size_t)m, &r2, "scaled R"))))
    return rc;
  cudaError_t e = cudaMemsetAsync(zero, 0, n * sizeof(double), st);
  if (e != cudaSuccess) return cuda_fail(e, "zeros");
  oakg_dims dd = *d;
  dd.mem = OAKG_MEM_DEVICE;
  // 1. the bias increment: locAnalysisIncrement with the forecast (xf = 0 gives xa = increment)
  if ((rc = locanalysis_impl<double>(&dd, loc, Z, dzs, zero, dHxf, dyo, dSf, dHSf, dr, dzp, dox, doy, doz,
                             dot, dcorr, dmaxl, inc, nullptr, nullptr, nullptr)))
    return rc;
  // 2. ba = bf - gamma inc, ux = xf - ba; H ux + Hshift; R (1 - gamma)
  e = bias_update(n, gamma, dbf, inc, dxf, dba, ux, st);
  if (e == cudaSuccess && m > 0)
    e = obsoper_apply(m, Hd.K, Hd.index, Hd.weight, Hd.shift, ux, n, uHx, st);
  if (e == cudaSuccess && m > 0) e = axpby(m, 1.0 - gamma, dr, 0.0, nullptr, r2, st);
  if (e != cudaSuccess) return cuda_fail(e, "bias update");
  // 3. the state increment from the unbiased forecast, xa = ux + increment
  if ((rc = locanalysis_impl<double>(&dd, loc, Z, dzs, zero, uHx, dyo, dSf, dHSf, r2, dzp, dox, doy, doz,
                             dot, dcorr, dmaxl, inc, nullptr, nullptr, nullptr)))
    return rc;
  e = axpby(n, 1.0, ux, 1.0, inc, dxa, st);
  if (e == cudaSuccess && dSa && dSa != dSf)
    e = cudaMemcpy2DAsync(dSa, d->ldS * sizeof(double), dSf, d->ldS * sizeof(double),
                          n * sizeof(double), N, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess && mem == OAKG_MEM_HOST) {
    e = cudaMemcpyAsync(xa, dxa, n * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(ba, dba, n * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && Sa)
      e = cudaMemcpyAsync(Sa, dSa, (size_t)d->ldS * N * sizeof(double), cudaMemcpyDeviceToHost,
                          st);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "bias-aware analysis");
  return OAKG_OK;
}

// The global analysis with R = diag(r_diag) + B B^T (rrsqrt.F90:196-208 with an SMWCovar R):
// one zone holding the whole state with every observation at weight 1 (zone and observations
// at one point, Gaussian weight exp(-(0/1)^2) = 1, the non-localised branch: R unpacked).
int analysis_smw_impl(const oakg_dims* d, const double* xf, const double* Hxf, const double* yo,
                      const double* Sf, const double* HSf, const double* r_diag, int32_t k,
                      const double* B, int64_t ldB, double* xa, double* Sa, double* ampl) {
  int rc = check_dims(d);
  if (rc) return rc;
  Ctx* c = nullptr;
  if ((rc = get_ctx(&c))) return rc;
  const int64_t m = d->m;
  const int mem = d->mem;
  // zone geometry (host or device like the other arrays): one zone at the origin, every
  // observation there
  const size_t geo = (size_t)4 + 2 + (size_t)(m > 0 ? m : 1);
  std::vector<double> h0(geo, 0.0);
  h0[4] = 1.0;  // corr_len
  h0[5] = 1.0;  // max_len
  const int32_t zsz = (int32_t)d->n;
  const double* g0;
  const int32_t* zs;
  double* dgeo;
  int32_t* dzs;
  if (mem == OAKG_MEM_DEVICE) {
    if ((rc = scratch(c, B_GLOB, geo + 1, &dgeo, "geometry"))) return rc;
    cudaError_t e = cudaMemcpyAsync(dgeo, h0.data(), geo * sizeof(double),
                                    cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(dgeo + geo, &zsz, sizeof(int32_t), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "geometry");
    g0 = dgeo;
    dzs = reinterpret_cast<int32_t*>(dgeo + geo);
    zs = dzs;
  } else {
    g0 = h0.data();
    zs = &zsz;
  }
  oakg_loc loc{};
  loc.weight = OAKG_WEIGHT_GAUSS_CUTOFF;
  loc.metric = OAKG_METRIC_CARTESIAN;
  loc.loctype = 1;
  loc.localise_obs = 0;
  loc.rotate = 1;
  loc.precision = OAKG_PREC_FP64;
  loc.flags = OAKG_FLAG_BRUTE_SEARCH | OAKG_FLAG_AMPL_ALWAYS;
  SmwArg sa;
  sa.k = k;
  sa.B = B;
  sa.ldB = ldB;
  const double* obs = g0 + 6;
  return locanalysis_impl<double>(d, &loc, 1, zs, xf, Hxf, yo, Sf, HSf, r_diag, g0, obs, obs, nullptr,
                          nullptr, g0 + 4, g0 + 5, xa, Sa, ampl, nullptr, &sa);
}

// ---- layout builders: initPartition, the sea packing and genObservationOper / cinterp

// initPartition (assimilation.F90:578-641) on the device: zone sizes, zoneIndex and its inverse
// (0-based here). A zone number outside 1..nzones or an empty zone is OAKG_ERR_ARGS (the
// reference stops on both, :605-617).
int zone_layout_impl(int64_t n, const int32_t* partition, int32_t nzones, int32_t mem,
                     int32_t* zone_size, int32_t* zone_index, int32_t* inv_index) {
  if (n <= 0 || n > INT32_MAX - 1) return fail(OAKG_ERR_ARGS, "n must be in [1, 2^31-2]");
  if (nzones < 1) return fail(OAKG_ERR_ARGS, "nzones must be positive (got %d)", nzones);
  if (nzones > n)
    return fail(OAKG_ERR_ARGS, "every zone 1..%d must hold at least one element (n = %lld)",
                nzones, (long long)n);
  if (!partition || !zone_size || !zone_index)
    return fail(OAKG_ERR_ARGS, "partition, zone_size and zone_index are required");
  if (mem != OAKG_MEM_HOST && mem != OAKG_MEM_DEVICE)
    return fail(OAKG_ERR_ARGS, "mem must be OAKG_MEM_HOST or OAKG_MEM_DEVICE");
  Ctx* c = nullptr;
  int rc = get_ctx(&c);
  if (rc) return rc;
  const int32_t* dpart;
  int32_t *dzs, *dzi, *dinv, *work;
  const int64_t nw = zone_layout_work(n, nzones);
  if ((rc = stage_in(c, B_L_PART, partition, (size_t)n, mem, &dpart, "partition")) ||
      (rc = stage_out(c, B_L_ZS, zone_size, (size_t)nzones, mem, &dzs, "zone_size")) ||
      (rc = stage_out(c, B_L_ZI, zone_index, (size_t)n, mem, &dzi, "zone_index")) ||
      (rc = stage_out(c, B_L_INV, inv_index, (size_t)n, mem, &dinv, "inv_index")) ||
      (rc = scratch(c, B_L_WORK, (size_t)nw + 1, &work, "layout scratch")))
    return rc;
  cudaStream_t st = c->stream;
  int32_t* dbad = work + nw;
  cudaError_t e = cudaMemsetAsync(dbad, 0, sizeof(int32_t), st);
  if (e == cudaSuccess) e = zone_layout(n, dpart, nzones, work, dzs, dzi, dinv, dbad, st);
  int32_t bad = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, dbad, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && mem == OAKG_MEM_HOST) {
    e = cudaMemcpyAsync(zone_size, dzs, (size_t)nzones * sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(zone_index, dzi, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && inv_index)
      e = cudaMemcpyAsync(inv_index, dinv, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost, st);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "zone layout");
  if (bad & 1) return fail(OAKG_ERR_ARGS, "partition values must lie in 1..%d", nzones);
  if (bad & 2)
    return fail(OAKG_ERR_ARGS, "every zone 1..%d must hold at least one element", nzones);
  return OAKG_OK;
}

// The zone numbering of globalInit (assimilation.F90:416-424): partition labels, any int32
// values with gaps, replaced by their rank among the distinct labels (unique(..., ind2 =
// partition), matoper.F90:1821-1882).
int partition_compact_impl(int64_t n, const int32_t* labels, int32_t mem, int32_t* partition,
                           int32_t* nzones) {
  if (n <= 0 || n > INT32_MAX - 1) return fail(OAKG_ERR_ARGS, "n must be in [1, 2^31-2]");
  if (!labels || !partition) return fail(OAKG_ERR_ARGS, "labels and partition are required");
  if (mem != OAKG_MEM_HOST && mem != OAKG_MEM_DEVICE)
    return fail(OAKG_ERR_ARGS, "mem must be OAKG_MEM_HOST or OAKG_MEM_DEVICE");
  Ctx* c = nullptr;
  int rc = get_ctx(&c);
  if (rc) return rc;
  const int32_t* dl;
  int32_t *dp, *work;
  const int64_t nw = partition_compact_work(n);
  if ((rc = stage_in(c, B_L_PART, labels, (size_t)n, mem, &dl, "labels")) ||
      (rc = stage_out(c, B_L_ZI, partition, (size_t)n, mem, &dp, "partition")) ||
      (rc = scratch(c, B_L_WORK, (size_t)nw, &work, "compaction scratch")))
    return rc;
  if (mem == OAKG_MEM_DEVICE && (const void*)labels == (const void*)partition)
    return fail(OAKG_ERR_ARGS, "labels and partition must not alias");
  cudaStream_t st = c->stream;
  cudaError_t e = partition_compact(n, dl, work, dp, st);
  int32_t nz = 0;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&nz, work + 5 * n, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && mem == OAKG_MEM_HOST)
    e = cudaMemcpyAsync(partition, dp, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "partition compaction");
  if (nzones) *nzones = nz;
  return OAKG_OK;
}

// Y(i, :) = X(index(i), :), i < n, for ncols columns
int permute_rows_impl(int64_t n, int32_t ncols, const int32_t* index, const double* X,
                      int64_t ldX, double* Y, int64_t ldY, int32_t mem) {
  if (n <= 0 || ncols <= 0) return fail(OAKG_ERR_ARGS, "n and ncols must be positive");
  if (!index || !X || !Y) return fail(OAKG_ERR_ARGS, "index, X and Y are required");
  if (ldX < n || ldY < n) return fail(OAKG_ERR_ARGS, "ldX and ldY must be >= n");
  if (mem != OAKG_MEM_HOST && mem != OAKG_MEM_DEVICE)
    return fail(OAKG_ERR_ARGS, "mem must be OAKG_MEM_HOST or OAKG_MEM_DEVICE");
  if (mem == OAKG_MEM_DEVICE && X == Y) return fail(OAKG_ERR_ARGS, "X and Y must not alias");
  Ctx* c = nullptr;
  int rc = get_ctx(&c);
  if (rc) return rc;
  const int32_t* didx;
  const double* dX;
  double* dY;
  int32_t* dbad;
  if ((rc = stage_in(c, B_L_IDX, index, (size_t)n, mem, &didx, "index")) ||
      (rc = stage_in(c, B_L_X, X, (size_t)ldX * ncols, mem, &dX, "X")) ||
      (rc = stage_out(c, B_L_Y, Y, (size_t)ldY * ncols, mem, &dY, "Y")) ||
      (rc = scratch(c, B_L_WORK, 1, &dbad, "permute flag")))
    return rc;
  cudaStream_t st = c->stream;
  cudaError_t e = cudaMemsetAsync(dbad, 0, sizeof(int32_t), st);
  if (e == cudaSuccess) e = permute_rows(n, ncols, didx, dX, ldX, dY, ldY, dbad, st);
  int32_t bad = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, dbad, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && mem == OAKG_MEM_HOST)
    e = cudaMemcpyAsync(Y, dY, (size_t)ldY * ncols * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "permute rows");
  if (bad) return fail(OAKG_ERR_ARGS, "index values must lie in [0, %lld)", (long long)n);
  return OAKG_OK;
}

// H%j = invZoneIndex(H%j) (assimilation.F90:2404-2407) on an operator's row-form indices
int obsoper_to_zone_order_impl(int64_t count, int64_t* index, const int32_t* inv_index,
                               int64_t n, int32_t mem) {
  if (count < 0 || n <= 0) return fail(OAKG_ERR_ARGS, "count must be >= 0 and n positive");
  if (count == 0) return OAKG_OK;
  if (!index || !inv_index) return fail(OAKG_ERR_ARGS, "index and inv_index are required");
  if (mem != OAKG_MEM_HOST && mem != OAKG_MEM_DEVICE)
    return fail(OAKG_ERR_ARGS, "mem must be OAKG_MEM_HOST or OAKG_MEM_DEVICE");
  Ctx* c = nullptr;
  int rc = get_ctx(&c);
  if (rc) return rc;
  const int32_t* dinv;
  int64_t* didx;
  int32_t* dbad;
  if ((rc = stage_in(c, B_L_IDX, inv_index, (size_t)n, mem, &dinv, "inv_index")) ||
      (rc = stage_out(c, B_L_OIDX, index, (size_t)count, mem, &didx, "index")) ||
      (rc = scratch(c, B_L_WORK, 1, &dbad, "remap flag")))
    return rc;
  cudaStream_t st = c->stream;
  cudaError_t e = cudaSuccess;
  if (mem == OAKG_MEM_HOST)
    e = cudaMemcpyAsync(didx, index, (size_t)count * sizeof(int64_t), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(dbad, 0, sizeof(int32_t), st);
  if (e == cudaSuccess) e = remap_index(count, didx, dinv, n, dbad, st);
  int32_t bad = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, dbad, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && mem == OAKG_MEM_HOST)
    e = cudaMemcpyAsync(index, didx, (size_t)count * sizeof(int64_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "operator remap");
  if (bad) return fail(OAKG_ERR_ARGS, "operator index >= n = %lld", (long long)n);
  return OAKG_OK;
}

// The sea packing of a masked grid (the reference's StateVectorSizeSea / removeLandPoints):
// sea[i] = number of unmasked points before point i, or -1 where mask[i] != 0.
int sea_index_impl(int64_t npts, const uint8_t* mask, int32_t mem, int64_t* sea, int64_t* nsea) {
  if (npts <= 0 || npts > INT32_MAX - 1) return fail(OAKG_ERR_ARGS, "npts must be in [1, 2^31-2]");
  if (!mask || !sea) return fail(OAKG_ERR_ARGS, "mask and sea are required");
  if (mem != OAKG_MEM_HOST && mem != OAKG_MEM_DEVICE)
    return fail(OAKG_ERR_ARGS, "mem must be OAKG_MEM_HOST or OAKG_MEM_DEVICE");
  Ctx* c = nullptr;
  int rc = get_ctx(&c);
  if (rc) return rc;
  const int64_t nt = sea_index_tiles(npts);
  const uint8_t* dmask;
  int64_t* dsea;
  int32_t* tiles;
  if ((rc = stage_in(c, B_L_MASK, mask, (size_t)npts, mem, &dmask, "mask")) ||
      (rc = stage_out(c, B_L_SEA, sea, (size_t)npts, mem, &dsea, "sea")) ||
      (rc = scratch(c, B_L_WORK, (size_t)(2 * (nt + 1)), &tiles, "sea scratch")))
    return rc;
  cudaStream_t st = c->stream;
  cudaError_t e = sea_index(npts, dmask, tiles, dsea, st);
  int32_t cnt = 0;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&cnt, tiles + (nt + 1) + nt, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && mem == OAKG_MEM_HOST)
    e = cudaMemcpyAsync(sea, dsea, (size_t)npts * sizeof(int64_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "sea index");
  if (nsea) *nsea = cnt;
  return OAKG_OK;
}

// split (ndgrid.F90:357-435): the simplices of the unit n-cube, each vertex a combination of
// the 2^n corners (corner c: bit k set = upper side of axis k). A sub-cube of dimension subn
// (the corners in sel, the axes in fixed held) becomes, for each free axis and each of its two
// faces, the face's own split extended by the centroid of sel as vertex subn; an edge
// (subn = 1) is its two corners in corner order. T[l][v][c], simplex l of the block starting
// at l0.
void split_cube(int n, int subn, unsigned fixed, const std::vector<char>& sel, int l0,
                std::vector<double>& T, int stride) {
  const int K = 1 << n;
  auto at = [&](int l, int v, int c) -> double& { return T[(size_t)l * stride + (size_t)v * K + c]; };
  if (subn == 1) {
    for (int v = 0; v < 2; v++)
      for (int cc = 0; cc < K; cc++) at(l0, v, cc) = 0.0;
    int j = 0;
    for (int cc = 0; cc < K && j < 2; cc++)
      if (sel[cc]) at(l0, j++, cc) = 1.0;
    return;
  }
  int cnt = 0;
  for (int cc = 0; cc < K; cc++) cnt += sel[cc] ? 1 : 0;
  auto fact = [](int k) {
    int f = 1;
    for (int i = 2; i <= k; i++) f *= i;
    return f;
  };
  const int nbth = fact(subn) << (subn - 1), subnbth = fact(subn - 1) << (subn - 2);
  for (int l = l0; l < l0 + nbth; l++)
    for (int cc = 0; cc < K; cc++) at(l, subn, cc) = sel[cc] ? 1.0 / cnt : 0.0;
  int m = l0;
  std::vector<char> sub(K);
  for (int i = 0; i < n; i++) {
    if ((fixed >> i) & 1u) continue;
    for (int j = 0; j < 2; j++) {
      for (int cc = 0; cc < K; cc++) sub[cc] = sel[cc] && (((cc >> i) & 1) == j);
      split_cube(n, subn - 1, fixed | (1u << i), sub, m, T, stride);
      m += subnbth;
    }
  }
}

// genObservationOper (assimilation.F90:2471-2656) for one variable on a rectilinear grid, with
// cinterp (ndgrid.F90:1183-1257) and interp_cube (:636-665) on the cells of the grid.
int obsoper_rectilinear_impl(int32_t ndim, const int32_t* shape, const double* coords,
                             const int64_t* sea, int64_t offset, int64_t m, const double* pos,
                             int32_t mem, int64_t* index, double* weight) {
  if (ndim < 1 || ndim > 4) return fail(OAKG_ERR_ARGS, "ndim must be 1..4 (got %d)", ndim);
  if (!shape || !coords || !index || !weight || (m > 0 && !pos))
    return fail(OAKG_ERR_ARGS, "shape, coords, pos, index and weight are required");
  if (m < 0 || m > INT32_MAX - 1) return fail(OAKG_ERR_ARGS, "m must be in [0, 2^31-2]");
  if (mem != OAKG_MEM_HOST && mem != OAKG_MEM_DEVICE)
    return fail(OAKG_ERR_ARGS, "mem must be OAKG_MEM_HOST or OAKG_MEM_DEVICE");
  int64_t npts = 1, ncoord = 0;
  for (int k = 0; k < ndim; k++) {
    if (shape[k] < 2)
      return fail(OAKG_ERR_ARGS, "every axis needs at least 2 points (axis %d has %d)", k,
                  shape[k]);
    npts *= shape[k];
    ncoord += shape[k];
    if (npts > ((int64_t)1 << 40)) return fail(OAKG_ERR_ARGS, "grid too large");
  }
  if (m == 0) return OAKG_OK;
  Ctx* c = nullptr;
  int rc = get_ctx(&c);
  if (rc) return rc;
  // the axes must be strictly monotone (the cell search is a bisection)
  std::vector<double> hc((size_t)ncoord);
  cudaError_t e = cudaMemcpy(hc.data(), coords, (size_t)ncoord * sizeof(double),
                             mem == OAKG_MEM_DEVICE ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost);
  if (e != cudaSuccess) return cuda_fail(e, "coords");
  for (int k = 0, o = 0; k < ndim; o += shape[k], k++) {
    const double s = hc[o + 1] - hc[o];
    for (int i = 0; i + 1 < shape[k]; i++) {
      const double d = hc[o + i + 1] - hc[o + i];
      if (!(s > 0 ? d > 0 : d < 0))
        return fail(OAKG_ERR_ARGS, "coordinates of axis %d are not strictly monotone", k);
    }
  }
  const int K = 1 << ndim, NV = ndim + 1;
  int nsimplex = 1;
  for (int i = 2; i <= ndim; i++) nsimplex *= i;
  nsimplex <<= (ndim - 1);
  const int stride = NV * K + ndim * NV;
  std::vector<double> T((size_t)nsimplex * stride, 0.0);
  split_cube(ndim, ndim, 0u, std::vector<char>(K, 1), 0, T, stride);
  for (int l = 0; l < nsimplex; l++)
    for (int k = 0; k < ndim; k++)
      for (int v = 0; v < NV; v++) {
        double u = 0.0;
        for (int cc = 0; cc < K; cc++)
          if ((cc >> k) & 1) u += T[(size_t)l * stride + (size_t)v * K + cc];
        T[(size_t)l * stride + NV * K + (size_t)k * NV + v] = u;
      }
  const double *dcoords, *dpos;
  const int64_t* dsea;
  int64_t* didx;
  double *dw, *dsimp;
  if ((rc = stage_in(c, B_L_COORD, coords, (size_t)ncoord, mem, &dcoords, "coords")) ||
      (rc = stage_in(c, B_L_SEA, sea, (size_t)npts, mem, &dsea, "sea")) ||
      (rc = stage_in(c, B_L_POS, pos, (size_t)m * ndim, mem, &dpos, "pos")) ||
      (rc = stage_out(c, B_L_OIDX, index, (size_t)m * K, mem, &didx, "index")) ||
      (rc = stage_out(c, B_L_OW, weight, (size_t)m * K, mem, &dw, "weight")) ||
      (rc = scratch(c, B_L_SIMP, T.size(), &dsimp, "simplex table")))
    return rc;
  cudaStream_t st = c->stream;
  e = cudaMemcpyAsync(dsimp, T.data(), T.size() * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = rectilinear_oper(ndim, shape, dcoords, dsea, dsimp, nsimplex, m, dpos, offset, didx, dw,
                         st);
  if (e == cudaSuccess && mem == OAKG_MEM_HOST) {
    e = cudaMemcpyAsync(index, didx, (size_t)m * K * sizeof(int64_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(weight, dw, (size_t)m * K * sizeof(double), cudaMemcpyDeviceToHost, st);
  }
  // T and hc are host vectors read by async copies: finish before they go out of scope
  cudaError_t e2 = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = e2;
  if (e != cudaSuccess) return cuda_fail(e, "rectilinear observation operator");
  return OAKG_OK;
}

int release_impl() {
  for (auto& cp : g_ctx) {
    if (!cp) continue;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(cp->device);
    cudaStreamSynchronize(cp->stream);
    for (auto& b : cp->buf) b.release();
    for (auto& ev : cp->ev) cudaEventDestroy(ev);
    if (cp->copy_in) cudaStreamDestroy(cp->copy_in);
    if (cp->copy_out) cudaStreamDestroy(cp->copy_out);
    if (cp->blas) cublasDestroy(cp->blas);
    cudaStreamDestroy(cp->own_stream);
    cudaSetDevice(prev);
    delete cp;
    cp = nullptr;
  }
  return OAKG_OK;
}

int context_init_impl() {
  Ctx* c = nullptr;
  return get_ctx(&c);
}

int timings_impl(double* ms, int n) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64 || !g_ctx[dev]) return 0;
  int k = std::min(n, 5);
  for (int i = 0; i < k; i++) ms[i] = g_ctx[dev]->timings[i];
  return k;
}

void count_launches(int k) { g_launches += k; }
int64_t launch_total() { return g_launches.load(); }

cudaStream_t current_stream() {
  Ctx* c = nullptr;
  if (get_ctx(&c) != OAKG_OK) return nullptr;
  return c->stream;
}

int set_stream_impl(void* stream) {
  Ctx* c = nullptr;
  int rc = get_ctx(&c);
  if (rc) return rc;
  cudaStreamSynchronize(c->stream);
  c->stream = stream ? static_cast<cudaStream_t>(stream) : c->own_stream;
  return OAKG_OK;
}

void set_ok() {
  g_last_status = OAKG_OK;
  t_last_error.clear();
}

std::mutex& api_mutex() { return g_mutex; }
int& last_status() { return g_last_status; }
std::string& last_error() { return t_last_error; }
int record_failure(int code, const char* msg) { return fail(code, "%s", msg); }

}  // namespace oakg

// ------------------------------------------------------------------------------------------
extern "C" {

int oakg_analysis(const oakg_dims* dims, const double* xf, const double* Hxf, const double* yo,
                  const double* Sf, const double* HSf, const double* r_diag, double* xa,
                  double* Sa, double* ampl) {
  std::lock_guard<std::mutex> lk(oakg::api_mutex());
  oakg::set_ok();
  int rc = oakg::analysis_impl(dims, xf, Hxf, yo, Sf, HSf, r_diag, xa, Sa, ampl);
  oakg::last_status() = rc;
  return rc;
}

int oakg_locanalysis_adjoint(const oakg_dims* dims, const oakg_loc* loc, int32_t nzones,
                             const int32_t* zone_size, const double* Hxf, const double* yo,
                             const double* Sf, const double* HSf, const double* r_diag,
                             const double* zone_xyzt, const double* obs_x, const double* obs_y,
                             const double* obs_z, const double* obs_t, const double* corr_len,
                             const double* max_len, double inflation, const double* dJ_dxa,
                             double* dJ_dyo, double* dJ_dr, double* dJ_dlen, double* dJ_dinfl) {
  std::lock_guard<std::mutex> lk(oakg::api_mutex());
  oakg::set_ok();
  int rc = oakg::adjoint_impl(dims, loc, nzones, zone_size, Hxf, yo, Sf, HSf, r_diag, zone_xyzt,
                              obs_x, obs_y, obs_z, obs_t, corr_len, max_len, inflation, dJ_dxa,
                              dJ_dyo, dJ_dr, dJ_dlen, dJ_dinfl);
  oakg::last_status() = rc;
  return rc;
}

int oakg_locanalysis(const oakg_dims* dims, const oakg_loc* loc, int32_t nzones,
                     const int32_t* zone_size, const double* xf, const double* Hxf,
                     const double* yo, const double* Sf, const double* HSf,
                     const double* r_diag, const double* zone_xyzt, const double* obs_x,
                     const double* obs_y, const double* obs_z, const double* obs_t,
                     const double* corr_len, const double* max_len, double* xa, double* Sa,
                     double* ampl, int32_t* nobs) {
  std::lock_guard<std::mutex> lk(oakg::api_mutex());
  oakg::set_ok();
  int rc = oakg::locanalysis_impl<double>(dims, loc, nzones, zone_size, xf, Hxf, yo, Sf, HSf,
                                          r_diag, zone_xyzt, obs_x, obs_y, obs_z, obs_t,
                                          corr_len, max_len, xa, Sa, ampl, nobs);
  oakg::last_status() = rc;
  return rc;
}

int oakg_locanalysis_f32(const oakg_dims* dims, const oakg_loc* loc, int32_t nzones,
                         const int32_t* zone_size, const float* xf, const float* Hxf,
                         const float* yo, const float* Sf, const float* HSf, const float* r_diag,
                         const double* zone_xyzt, const double* obs_x, const double* obs_y,
                         const double* obs_z, const double* obs_t, const double* corr_len,
                         const double* max_len, float* xa, float* Sa, float* ampl,
                         int32_t* nobs) {
  std::lock_guard<std::mutex> lk(oakg::api_mutex());
  oakg::set_ok();
  int rc = oakg::locanalysis_impl<float>(dims, loc, nzones, zone_size, xf, Hxf, yo, Sf, HSf,
                                         r_diag, zone_xyzt, obs_x, obs_y, obs_z, obs_t, corr_len,
                                         max_len, xa, Sa, ampl, nobs);
  oakg::last_status() = rc;
  return rc;
}

size_t oakg_last_error(char* buf, size_t len) {
  const std::string& s = oakg::last_error();
  if (buf && len > 0) {
    size_t k = std::min(len - 1, s.size());
    std::memcpy(buf, s.data(), k);
    buf[k] = '\0';
  }
  return s.size();
}

int oakg_last_status(void) { return oakg::last_status(); }

int oakg_release(void) {
  std::lock_guard<std::mutex> lk(oakg::api_mutex());
  return oakg::release_impl();
}

int oakg_set_stream(void* stream) {
  std::lock_guard<std::mutex> lk(oakg::api_mutex());
  return oakg::set_stream_impl(stream);
}

int64_t oakg_launch_count(void) { return oakg::launch_total(); }

int oakg_last_timings(double* ms, int n) {
  std::lock_guard<std::mutex> lk(oakg::api_mutex());
  if (!ms || n <= 0) return 0;
  return oakg::timings_impl(ms, n);
}

struct oakg_plan {
  oakg::Plan* p;
};

int oakg_plan_locanalysis(oakg_plan** plan, const oakg_dims* dims, const oakg_loc* loc,
                          int32_t nzones, const int32_t* zone_size, const double* xf,
                          const double* Hxf, const double* yo, const double* Sf,
                          const double* HSf, const double* r_diag, const double* zone_xyzt,
                          const double* obs_x, const double* obs_y, const double* obs_z,
                          const double* obs_t, const double* corr_len, const double* max_len,
                          double* xa, double* Sa, double* ampl, int32_t* nobs, int32_t tune) {
  std::lock_guard<std::mutex> lk(oakg::api_mutex());
  oakg::set_ok();
  if (!plan) {
    int rc = oakg::record_failure(OAKG_ERR_ARGS, "plan is NULL");
    oakg::last_status() = rc;
    return rc;
  }
  *plan = nullptr;
  oakg::Plan* p = nullptr;
  int rc = oakg::plan_create_impl(&p, dims, loc, nzones, zone_size, xf, Hxf, yo, Sf, HSf, r_diag,
                                  zone_xyzt, obs_x, obs_y, obs_z, obs_t, corr_len, max_len, xa, Sa,
                                  ampl, nobs, tune);
  if (rc == OAKG_OK) *plan = new oakg_plan{p};
  oakg::last_status() = rc;
  return rc;
}

int oakg_plan_execute(oakg_plan* plan, void* stream) {
  std::lock_guard<std::mutex> lk(oakg::api_mutex());
  oakg::set_ok();
  int rc = oakg::plan_execute_impl(plan ? plan->p : nullptr, stream);
  oakg::last_status() = rc;
  return rc;
}

int oakg_plan_info(const oakg_plan* plan, double* cell_size, int64_t* graph_nodes,
                   double* tune_cell, double* tune_ms, int32_t ntune) {
  if (!plan || !plan->p) return 0;
  const oakg::Plan* p = plan->p;
  if (cell_size) *cell_size = p->cell_size;
  if (graph_nodes) *graph_nodes = (int64_t)p->nodes;
  const int k = std::min<int>(p->ntune, ntune > 0 ? ntune : 0);
  for (int i = 0; i < k; i++) {
    if (tune_cell) tune_cell[i] = p->tune_cell[i];
    if (tune_ms) tune_ms[i] = p->tune_ms[i];
  }
  return p->ntune;
}

int oakg_plan_schedule(const oakg_plan* plan, double* index_order_ms, double* count_order_ms) {
  if (!plan || !plan->p) return 0;
  const oakg::Plan* p = plan->p;
  if (index_order_ms) *index_order_ms = p->order_ms[0];
  if (count_order_ms) *count_order_ms = p->order_ms[1];
  return p->zorder_used;
}

void oakg_plan_destroy(oakg_plan* plan) {
  if (!plan) return;
  std::lock_guard<std::mutex> lk(oakg::api_mutex());
  oakg::plan_free(plan->p);
  delete plan;
}

int oakg_ensemble_prologue(const oakg_dims* dims, const double* Ef, int64_t ldE,
                           const oakg_obsoper* H, double* xf, double* Sf, double* Hxf,
                           double* HSf) {
  std::lock_guard<std::mutex> lk(oakg::api_mutex());
  oakg::set_ok();
  int rc = oakg::prologue_impl(dims, Ef, ldE, H, xf, Sf, Hxf, HSf);
  oakg::last_status() = rc;
  return rc;
}

int oakg_ensemble_epilogue(const oakg_dims* dims, const double* xf, const double* xa,
                           const double* Sa, double inflation, const double* max_correction,
                           double* Ea, int64_t ldE) {
  std::lock_guard<std::mutex> lk(oakg::api_mutex());
  oakg::set_ok();
  int rc = oakg::epilogue_impl(dims, xf, xa, Sa, inflation, max_correction, Ea, ldE);
  oakg::last_status() = rc;
  return rc;
}

int oakg_ens_locanalysis(const oakg_dims* dims, const oakg_loc* loc, int32_t nzones,
                         const int32_t* zone_size, const double* Ef, int64_t ldE,
                         const oakg_obsoper* H, const double* yo, const double* r_diag,
                         const double* zone_xyzt, const double* obs_x, const double* obs_y,
                         const double* obs_z, const double* obs_t, const double* corr_len,
                         const double* max_len, double inflation, const double* max_correction,
                         double* Ea) {
  std::lock_guard<std::mutex> lk(oakg::api_mutex());
  oakg::set_ok();
  int rc = oakg::ens_locanalysis_impl(dims, loc, nzones, zone_size, Ef, ldE, H, yo, r_diag,
                                      zone_xyzt, obs_x, obs_y, obs_z, obs_t, corr_len, max_len,
                                      inflation, max_correction, Ea);
  oakg::last_status() = rc;
  return rc;
}

int oakg_locanalysis_smw(const oakg_dims* dims, const oakg_loc* loc, int32_t nzones,
                         const int32_t* zone_size, const double* xf, const double* Hxf,
                         const double* yo, const double* Sf, const double* HSf,
                         const double* r_diag, int32_t k, const double* B, int64_t ldB,
                         const double* zone_xyzt, const double* obs_x, const double* obs_y,
                         const double* obs_z, const double* obs_t, const double* corr_len,
                         const double* max_len, double* xa, double* Sa, double* ampl,
                         int32_t* nobs) {
  std::lock_guard<std::mutex> lk(oakg::api_mutex());
  oakg::set_ok();
  oakg::SmwArg sa;
  sa.k = k;
  sa.B = B;
  sa.ldB = ldB;
  int rc = oakg::locanalysis_impl<double>(dims, loc, nzones, zone_size, xf, Hxf, yo, Sf, HSf, r_diag,
                                  zone_xyzt, obs_x, obs_y, obs_z, obs_t, corr_len, max_len, xa,
                                  Sa, ampl, nobs, &sa);
  oakg::last_status() = rc;
  return rc;
}

int oakg_analysis_smw(const oakg_dims* dims, const double* xf, const double* Hxf,
                      const double* yo, const double* Sf, const double* HSf,
                      const double* r_diag, int32_t k, const double* B, int64_t ldB, double* xa,
                      double* Sa, double* ampl) {
  std::lock_guard<std::mutex> lk(oakg::api_mutex());
  oakg::set_ok();
  int rc = oakg::analysis_smw_impl(dims, xf, Hxf, yo, Sf, HSf, r_diag, k, B, ldB, xa, Sa, ampl);
  oakg::last_status() = rc;
  return rc;
}

int oakg_ens2sqrt(const oakg_dims* dims, const double* E, int64_t ldE, double* mean,
                  double* S) {
  std::lock_guard<std::mutex> lk(oakg::api_mutex());
  oakg::set_ok();
  int rc = oakg::ens2sqrt_impl(dims, E, ldE, mean, S);
  oakg::last_status() = rc;
  return rc;
}

int oakg_sqrt2ens(const oakg_dims* dims, const double* mean, const double* S,
                  const double* theta, double* E, int64_t ldE) {
  std::lock_guard<std::mutex> lk(oakg::api_mutex());
  oakg::set_ok();
  int rc = oakg::sqrt2ens_impl(dims, mean, S, theta, E, ldE);
  oakg::last_status() = rc;
  return rc;
}

int oakg_ens_analysis(const oakg_dims* dims, const double* Ef, int64_t ldE, const double* HEf,
                      int64_t ldHE, const double* yo, const double* r_diag, double* Ea,
                      double* xa, double* ampl) {
  std::lock_guard<std::mutex> lk(oakg::api_mutex());
  oakg::set_ok();
  int rc = oakg::ens_analysis_impl(dims, Ef, ldE, HEf, ldHE, yo, r_diag, Ea, xa, ampl);
  oakg::last_status() = rc;
  return rc;
}

int oakg_biased_locanalysis(const oakg_dims* dims, const oakg_loc* loc, int32_t nzones,
                            const int32_t* zone_size, double gamma, const oakg_obsoper* H,
                            const double* xf, const double* bf, const double* Hxf,
                            const double* yo, const double* Sf, const double* HSf,
                            const double* r_diag, const double* zone_xyzt, const double* obs_x,
                            const double* obs_y, const double* obs_z, const double* obs_t,
                            const double* corr_len, const double* max_len, double* xa,
                            double* ba, double* Sa) {
  std::lock_guard<std::mutex> lk(oakg::api_mutex());
  oakg::set_ok();
  int rc = oakg::biased_locanalysis_impl(dims, loc, nzones, zone_size, gamma, H, xf, bf, Hxf, yo,
                                         Sf, HSf, r_diag, zone_xyzt, obs_x, obs_y, obs_z, obs_t,
                                         corr_len, max_len, xa, ba, Sa);
  oakg::last_status() = rc;
  return rc;
}

int oakg_zone_layout(int64_t n, const int32_t* partition, int32_t nzones, int32_t mem,
                     int32_t* zone_size, int32_t* zone_index, int32_t* inv_index) {
  std::lock_guard<std::mutex> lk(oakg::api_mutex());
  oakg::set_ok();
  int rc = oakg::zone_layout_impl(n, partition, nzones, mem, zone_size, zone_index, inv_index);
  oakg::last_status() = rc;
  return rc;
}

int oakg_partition_compact(int64_t n, const int32_t* labels, int32_t mem, int32_t* partition,
                           int32_t* nzones) {
  std::lock_guard<std::mutex> lk(oakg::api_mutex());
  oakg::set_ok();
  int rc = oakg::partition_compact_impl(n, labels, mem, partition, nzones);
  oakg::last_status() = rc;
  return rc;
}

int oakg_permute_rows(int64_t n, int32_t ncols, const int32_t* index, const double* X,
                      int64_t ldX, double* Y, int64_t ldY, int32_t mem) {
  std::lock_guard<std::mutex> lk(oakg::api_mutex());
  oakg::set_ok();
  int rc = oakg::permute_rows_impl(n, ncols, index, X, ldX, Y, ldY, mem);
  oakg::last_status() = rc;
  return rc;
}

int oakg_obsoper_to_zone_order(int64_t count, int64_t* index, const int32_t* inv_index,
                               int64_t n, int32_t mem) {
  std::lock_guard<std::mutex> lk(oakg::api_mutex());
  oakg::set_ok();
  int rc = oakg::obsoper_to_zone_order_impl(count, index, inv_index, n, mem);
  oakg::last_status() = rc;
  return rc;
}

int oakg_sea_index(int64_t npts, const uint8_t* mask, int32_t mem, int64_t* sea, int64_t* nsea) {
  std::lock_guard<std::mutex> lk(oakg::api_mutex());
  oakg::set_ok();
  int rc = oakg::sea_index_impl(npts, mask, mem, sea, nsea);
  oakg::last_status() = rc;
  return rc;
}

int oakg_obsoper_rectilinear(int32_t ndim, const int32_t* shape, const double* coords,
                             const int64_t* sea, int64_t offset, int64_t m, const double* pos,
                             int32_t mem, int64_t* index, double* weight) {
  std::lock_guard<std::mutex> lk(oakg::api_mutex());
  oakg::set_ok();
  int rc = oakg::obsoper_rectilinear_impl(ndim, shape, coords, sea, offset, m, pos, mem, index,
                                          weight);
  oakg::last_status() = rc;
  return rc;
}

}  // extern "C"
