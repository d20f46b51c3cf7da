// oakg_analysis_noalloc: the global analysis (the same kernels as oakg_analysis) for callers
// that cannot allocate device memory. Some host programs reserve the whole GPU memory for their
// own pool before the assimilation library is loaded (ocean-model couplers typically do), and
// others must not call cudaMalloc/cudaFree inside a forecast-analysis cycle because those calls
// can synchronise the whole device. For them, every temporary of this entry point lives in one
// file-scope __device__ array of fixed size; inputs and outputs are the caller's device arrays.
//
// Limits and behaviour:
//  - N (ensemble size) <= kNoAllocMaxN = 112; larger N is rejected with OAKG_ERR_ARGS.
//  - all pointers must be device pointers (dims->mem == OAKG_MEM_DEVICE).
//  - the array (kScratchBytes, 256 KiB) is held by every GPU that loads the library until the
//    process exits; all calls share it and it keeps the last call's contents, so everything
//    that must start at zero is cleared on the stream by each call. Calls whose work overlaps
//    on the GPU (other threads, other streams) race on the array: serialise them.
//  - the first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (once per device, with that device current); make that first call
//    before any stream capture. The address is kept for the life of the process, which
//    assumes the device's primary context is not reset (cudaDeviceReset) while the library is
//    loaded: a reset reloads the module and leaves the kept address stale.
//  - no cudaMalloc, cudaFree or other allocating routine is called.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "oakg_internal.cuh"

namespace oakg {
std::mutex& api_mutex();
int& last_status();
std::string& last_error();
}  // namespace oakg

namespace {

constexpr int kNoAllocMaxN = 112;
constexpr size_t kScratchBytes = 256 * 1024;

// Layout for ensemble size N (doubles, then integers):
//   G/T [N*N] | Z [N*N] | aux [5N+2] | g [N] | ampl [N] | zone_start[2] (int64) |
//   status [2] (int32) | nobs [2] (int32) | work counters [8] (int32)
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

size_t scratch_doubles(int N) { return 2 * (size_t)N * N + (size_t)7 * N + 2; }
constexpr size_t kIntBytes = 2 * 8 + 2 * 4 + 2 * 4 + 8 * 4;

static_assert(2 * kNoAllocMaxN * kNoAllocMaxN * 8 + 7 * kNoAllocMaxN * 8 + 16 + kIntBytes + 64 <=
                  kScratchBytes,
              "scratch array too small for the largest ensemble size");

__global__ void k_noalloc_init(int64_t* zone_start, int64_t n, int32_t* nobs, int32_t has_obs) {
  zone_start[0] = 0;
  zone_start[1] = n;
  nobs[0] = has_obs;
}

int fail(int code, const std::string& msg) {
  oakg::last_error() = msg;
  oakg::last_status() = code;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(OAKG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace

extern "C" int oakg_analysis_noalloc(const oakg_dims* dims, const double* xf, const double* Hxf,
                                     const double* yo, const double* Sf, const double* HSf,
                                     const double* r_diag, double* xa, double* Sa, double* ampl,
                                     void* stream) {
  std::lock_guard<std::mutex> lk(oakg::api_mutex());
  oakg::last_error().clear();
  oakg::last_status() = OAKG_OK;
  if (!dims) return fail(OAKG_ERR_ARGS, "dims is NULL");
  const int64_t n = dims->n, m = dims->m, ldS = dims->ldS, ldH = dims->ldH;
  const int N = dims->N;
  if (N < 2 || N > kNoAllocMaxN)
    return fail(OAKG_ERR_ARGS, "oakg_analysis_noalloc: ensemble size N=" + std::to_string(N) +
                                   " outside [2, " + std::to_string(kNoAllocMaxN) +
                                   "] (fixed scratch of " + std::to_string(kScratchBytes) +
                                   " bytes)");
  if (dims->mem != OAKG_MEM_DEVICE)
    return fail(OAKG_ERR_ARGS, "oakg_analysis_noalloc: arrays must be device pointers "
                               "(dims->mem = OAKG_MEM_DEVICE)");
  if (n <= 0 || m < 0 || ldS < n || ldH < m)
    return fail(OAKG_ERR_ARGS, "oakg_analysis_noalloc: invalid n, m, ldS or ldH");
  if (!xf || !Sf || !xa) return fail(OAKG_ERR_ARGS, "xf, Sf and xa are required");
  if (m > 0 && (!Hxf || !yo || !HSf || !r_diag))
    return fail(OAKG_ERR_ARGS, "Hxf, yo, HSf and r_diag are required when m > 0");

  cudaError_t e;
  // the scratch's address, looked up on every call (a host call): a cached address would go
  // stale if the context were reset and the module reloaded
  void* scratch_p = nullptr;
  e = cudaGetSymbolAddress(&scratch_p, g_noalloc_scratch);
  if (e != cudaSuccess || !scratch_p) return cuda_fail(e, "cudaGetSymbolAddress(scratch)");
  cudaStream_t st = static_cast<cudaStream_t>(stream);

  double* base = reinterpret_cast<double*>(scratch_p);
  double* d_G = base;
  double* d_Z = d_G + (size_t)N * N;
  double* d_aux = d_Z + (size_t)N * N;
  double* d_gv = d_aux + 5 * N + 2;
  double* d_za = d_gv + N;
  unsigned char* ib = reinterpret_cast<unsigned char*>(base + scratch_doubles(N));
  int64_t* d_zstart = reinterpret_cast<int64_t*>(ib);
  int32_t* d_status = reinterpret_cast<int32_t*>(ib + 16);
  int32_t* d_nobs = d_status + 2;
  int32_t* d_work = d_nobs + 2;

  k_noalloc_init<<<1, 1, 0, st>>>(d_zstart, n, d_nobs, m > 0 ? 1 : 0);
  oakg::count_launches(1);
  if (m > 0) {
    e = oakg::global_gram_fp64(m, N, HSf, ldH, yo, Hxf, r_diag, d_G, d_gv, st);
    if (e != cudaSuccess) return cuda_fail(e, "Gram kernel");
  }
  e = oakg::zone_eig_fp64(N, 1, d_G, d_gv, d_nobs, 1, d_za, d_status, d_aux, d_Z, d_work, st);
  if (e != cudaSuccess) return cuda_fail(e, "eigensolve kernels");
  if (m == 0 && (e = cudaMemsetAsync(d_za, 0, N * sizeof(double), st)) != cudaSuccess)
    return cuda_fail(e, "clear amplitudes");
  const int32_t zone_max = (int32_t)(n < INT32_MAX ? n : INT32_MAX);
  e = oakg::zone_update_fp64(N, 0, 1, d_zstart, zone_max, xf, Sf, ldS, d_G, d_za, d_nobs, xa, Sa,
                             st);
  if (e != cudaSuccess) return cuda_fail(e, "update kernel");
  if (ampl &&
      (e = cudaMemcpyAsync(ampl, d_za, N * sizeof(double), cudaMemcpyDeviceToDevice, st)) !=
          cudaSuccess)
    return cuda_fail(e, "amplitudes");
  int32_t hstatus = 0;
  if ((e = cudaMemcpyAsync(&hstatus, d_status, sizeof(int32_t), cudaMemcpyDeviceToHost, st)) !=
      cudaSuccess)
    return cuda_fail(e, "status read");
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_fail(e, "synchronize");
  if (hstatus & oakg::ZST_NAN) return fail(OAKG_ERR_NAN, "NaN in analysis amplitudes");
  if (hstatus & oakg::ZST_EIG) return fail(OAKG_ERR_EIG, "eigensolver did not converge");
  return OAKG_OK;
}
