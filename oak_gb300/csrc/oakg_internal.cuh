// Internal declarations shared by the CUDA translation units of liboakg.so.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/oakg.h"

namespace oakg {

// Per-zone status bits written by the device (host folds them into one OAKG_ERR_* code).
enum : int32_t {
  ZST_NAN = 1,       // NaN/Inf amplitudes (rrsqrt.F90:145-149)
  ZST_EIG = 2,       // QL iterations did not converge
  ZST_CAPACITY = 4,  // zone larger than the kernel's row tile (cannot happen: tiles split)
  ZST_TIMEOUT = 8,   // a bounded device wait expired (tensor-core pipeline)
};

// Cell grid over observation coordinates (u, v): cells are cs_u x cs_v, nu x nv of them,
// origin (u0, v0). For longitudes on the sphere (metric 1), u is periodic with period 360.
struct CellGrid {
  double u0, v0;     // origin
  double csu, csv;   // cell edge
  int32_t nu, nv;    // cells per axis
  int32_t periodic_u;
  int32_t pad;
};

// Observation arrays in cell-sorted order (index q), produced by obs_prep.
struct SortedObs {
  const double* u;      // coordinate used by the metric (x, z or t)          [m]
  const double* v;      // second horizontal coordinate (y) or 0              [m]
  const double* innov;  // yo - Hxf                                            [m]
  const double* r;      // observation error variance (R diagonal)            [m]
  const double* HSt;    // HSf rows, row-major [m][N]
  const float* HSt32;   // the same rows in FP32 (mixed precision only, else null)
  const float* r32;     // r in FP32 (mixed precision only)
  const float* innov32; // yo - Hxf in FP32 (mixed precision only)
  const int32_t* cell_start;  // [ncells + 1]
  const int32_t* perm;  // sorted position -> original index                [m]
  int64_t m;            // number of observations
  // cell-relative coordinates: u cell index of the observation (its v cell is the row its cell
  // lies in) and the FP32 offsets u - (u0 + cu csu), v - (v0 + cv csv) inside the cell  [m]
  const int32_t* cu;
  const float* ru;
  const float* rv;
};

struct LocParams {
  int32_t weight, metric, loctype, localise, rotate, flags;
};

// ---- obs_prep.cu
// Fills the sorted-observation arrays and the cell offsets; returns a CUDA error code.
// u_src/v_src are the coordinate arrays for the metric (v_src may be null: v = 0).
cudaError_t obs_bounds(const double* u, const double* v, int64_t m, double* d_out4,
                       cudaStream_t st);
cudaError_t obs_bin_and_sort(const CellGrid& g, int64_t m, int N, const double* u_src,
                             const double* v_src, const double* yo, const double* Hxf,
                             const double* r, const double* HSf, const float* HSf32,
                             int64_t ldH, int32_t* d_cell, int32_t* d_count,
                             int32_t* d_cell_start, int32_t* d_pos, int32_t* d_perm,
                             double* d_u, double* d_v, double* d_innov, double* d_r,
                             double* d_HSt, int32_t* d_cu, float* d_ru, float* d_rv,
                             cudaStream_t st);
cudaError_t zone_offsets(const int32_t* zone_size, int32_t Z, int64_t* d_zone_start,
                         int32_t* d_zone_max, cudaStream_t st);

// ---- zone_gram.cu
// Selection + Gram + innovation projection for zones [z0, z0 + nzc); writes G (N x N, both
// triangles, row-major per zone), gvec (N), nobs per zone. The persistent blocks take zones
// in order (chunk-local indices: the w-th zone taken is order[z0 + w]) when `order` is given,
// else in index order; outputs stay at each zone's own slot.
cudaError_t zone_gram_fp64(const CellGrid& g, const SortedObs& so, int N, LocParams lp,
                           int32_t z0, int32_t nzc, const double* zone_xyzt,
                           const double* corr_len, const double* max_len, double* d_G,
                           double* d_g, int32_t* d_nobs, int brute, int32_t* d_work,
                           cudaStream_t st, const int32_t* order = nullptr);
// Mixed precision: same selection, products accumulated in FP32 (G, g in float).
cudaError_t zone_gram_fp32(const CellGrid& g, const SortedObs& so, int N, LocParams lp,
                           int32_t z0, int32_t nzc, const double* zone_xyzt,
                           const double* corr_len, const double* max_len, float* d_G,
                           float* d_g, int32_t* d_nobs, int brute, int32_t* d_work,
                           cudaStream_t st, const int32_t* order = nullptr);
// Mixed precision on the tensor cores (zone_gram_tc.cu), N <= gram_tc_max_n(); needs
// so.HSt32. d_err receives ZST_TIMEOUT (OR) if a bounded device wait expired.
int gram_tc_max_n();
cudaError_t zone_gram_tc(const CellGrid& g, const SortedObs& so, int N, LocParams lp, int32_t z0,
                         int32_t nzc, const double* zone_xyzt, const double* corr_len,
                         const double* max_len, float* d_G, float* d_g, int32_t* d_nobs,
                         int brute, int32_t* d_work, int32_t* d_err, cudaStream_t st,
                         const int32_t* order = nullptr);
// Plain form on the tensor cores (zone_gram_oz.cu), N <= gram_oz_max_n(): G as an exact
// product of 8-bit slices of X = diag(|w| / sqrt(r)) HS_sel on BF16 tensor cores, combined in
// 64-bit integers and FP64; the same selection, weights and outputs as zone_gram_fp64. d_scratch:
// gram_oz_scratch_bytes(m) of device memory (column exponents, r^-1/2). d_err receives
// ZST_TIMEOUT (OR) if a bounded device wait expired.
int gram_oz_max_n();
size_t gram_oz_scratch_bytes(int64_t m);
// The FP64 square-root transform of zones [0, nzc) on the tensor cores, N <= gram_oz_max_n():
// T_sym = X^T X with X_ka = q_k U_ak (q_k = (1 + lambda_k)^-1/4) as exact 8-bit slice products,
// then T = T_sym Omega (rotate) in FP64, written to d_GT (N x N a zone). Inputs left by the
// eigensolve's transform stage: the eigenvectors vector-major in d_Z (d_Z[k N + a] = U_ak),
// q_k at d_aux[4N + k] and v at d_aux[k] of each zone (zone_eig_aux(N) elements a zone).
// A bounded wait that expires sets ZST_TIMEOUT in the zone's d_status.
cudaError_t zone_tsym_oz(int N, int32_t nzc, double* d_GT, const double* d_aux,
                         const double* d_Z, const int32_t* d_nobs, int rotate,
                         int32_t* d_status, cudaStream_t st);
cudaError_t zone_gram_oz(const CellGrid& g, const SortedObs& so, int64_t m, int N, LocParams lp,
                         int32_t z0, int32_t nzc, const double* zone_xyzt, const double* corr_len,
                         const double* max_len, double* d_G, double* d_g, int32_t* d_nobs,
                         int brute, int32_t* d_work, int32_t* d_err, void* d_scratch,
                         cudaStream_t st, const int32_t* order = nullptr);
// FP32 copy of count doubles (HS rows for the mixed form).
cudaError_t rows_to_fp32(const double* src, float* dst, int64_t count, cudaStream_t st);
// FP64 copy of count floats (observation vectors given in FP32 storage).
cudaError_t rows_to_fp64(const float* src, double* dst, int64_t count, cudaStream_t st);
// zone_gram_fp64 on augmented observation rows so.HSt = [HS_q | B_q] (N columns, the first nx
// weighted): the products for the SMWCovar Woodbury reduction (zone_smw.cu).
cudaError_t zone_gram_fp64_aug(const CellGrid& g, const SortedObs& so, int N, int nx,
                               LocParams lp, int32_t z0, int32_t nzc, const double* zone_xyzt,
                               const double* corr_len, const double* max_len, double* d_G,
                               double* d_g, int32_t* d_nobs, int brute, int32_t* d_work,
                               cudaStream_t st);
// exclusive scan of n int32 values (out[n] = total), one block
cudaError_t scan_exclusive_i32(const int32_t* d_in, int64_t n, int32_t* d_out, cudaStream_t st);
// ---- zone_layout.cu: the zone layout of initPartition and the rectilinear-grid observation
// operator of genObservationOper / cinterp
// zone layout of a partition vector (1-based zone numbers): zone sizes, zone_index (sorted
// position -> element, stable), its inverse (optional); *d_bad |= 1 for a zone number outside
// 1..nzones, |= 2 for an empty zone. d_work: zone_layout_work(n, nzones) int32 of scratch.
int64_t zone_layout_work(int64_t n, int32_t nzones);
cudaError_t zone_layout(int64_t n, const int32_t* d_partition, int32_t nzones, int32_t* d_work,
                        int32_t* d_zone_size, int32_t* d_zone_index, int32_t* d_inv_index,
                        int32_t* d_bad, cudaStream_t st);
// the reference's unique(partition, n, ind2 = partition) (assimilation.F90:420-424): every
// label replaced by its rank (1-based) among the distinct labels in ascending order; the number
// of distinct labels is d_work[5 n] afterwards
int64_t partition_compact_work(int64_t n);
cudaError_t partition_compact(int64_t n, const int32_t* d_labels, int32_t* d_work,
                              int32_t* d_out, cudaStream_t st);
// index[t] = inv[index[t]] for 0 <= index[t] < n; *d_bad |= 1 for an entry >= n
cudaError_t remap_index(int64_t count, int64_t* d_index, const int32_t* d_inv, int64_t n,
                        int32_t* d_bad, cudaStream_t st);
// Y(i, :) = X(index(i), :); an index outside [0, n) sets *d_bad and leaves the row 0
cudaError_t permute_rows(int64_t n, int ncols, const int32_t* d_index, const double* X,
                         int64_t ldX, double* Y, int64_t ldY, int32_t* d_bad, cudaStream_t st);
// packed index of the unmasked points (-1 for masked ones); d_tiles: 2 (sea_index_tiles + 1)
// int32 of scratch, d_tiles[2 tiles + 1] the unmasked count afterwards
int64_t sea_index_tiles(int64_t npts);
cudaError_t sea_index(int64_t npts, const uint8_t* d_mask, int32_t* d_tiles, int64_t* d_sea,
                      cudaStream_t st);
cudaError_t rectilinear_oper(int ndim, const int32_t* shape, const double* d_coords,
                             const int64_t* d_sea, const double* d_simplex, int nsimplex,
                             int64_t m, const double* d_pos, int64_t offset, int64_t* d_index,
                             double* d_weight, cudaStream_t st);
// ---- zone_smw.cu: SMWCovar (R = diag(C) + B B^T) support. smw_rows writes the augmented
// cell-sorted rows [HSt_q | B_perm(q)] (m x (N + k)); smw_reduce turns each zone's augmented
// products (NA = N + k) into G = X^T X - X^T Y (Y^T Y + I)^-1 Y^T X and the matching g.
cudaError_t smw_rows(int64_t m, int N, int k, const double* HSt, const int32_t* perm,
                     const double* B, int64_t ldB, double* HStA, cudaStream_t st);
cudaError_t smw_reduce(int N, int k, int32_t nzc, const double* Ga, const double* ga,
                       const int32_t* nobs, double* G, double* gv, cudaStream_t st);
// Same as zone_gram_fp64 for the zones listed in zlist[0..nzc) (G, g slots in list order).
cudaError_t zone_gram_fp64_list(const CellGrid& g, const SortedObs& so, int N, LocParams lp,
                                const int32_t* zlist, int32_t nzc, const double* zone_xyzt,
                                const double* corr_len, const double* max_len, double* d_G,
                                double* d_g, int32_t* d_nobs, int brute, int32_t* d_work,
                                cudaStream_t st);
// Adjoint of the analysis mean for the zones in zlist (see zone_adjoint.cu).
cudaError_t zone_adjoint_fp64(const CellGrid& g, const SortedObs& so, int N, LocParams lp,
                              const int32_t* zlist, int32_t nzc, const double* zone_xyzt,
                              const double* corr_len, const double* max_len,
                              const int64_t* zone_start, const double* Sf, int64_t ldS,
                              const double* seed, double infl, const double* d_G,
                              const double* d_g, const int32_t* d_nobs, double* dyo, double* dr,
                              double* dscal, int brute, int32_t* d_work, cudaStream_t st);
cudaError_t zone_active_list(const double* seed, const int64_t* zone_start, int32_t Z,
                             int32_t* d_flag, int32_t* d_pos, int32_t* d_list,
                             cudaStream_t st);
// Global analysis Gram over all m observations (weights 1): G, g accumulated atomically.
cudaError_t global_gram_fp64(int64_t m, int N, const double* HSf, int64_t ldH,
                             const double* yo, const double* Hxf, const double* r, double* d_G,
                             double* d_g, cudaStream_t st);

// ---- zone_eig.cu
// For zones [0, nzc) of a chunk with nobs > 0: eigen-decomposition of G (d_GT, N x N per
// zone), T = U (I+L)^-1/2 U^T Omega written over G, ampl (N per zone), status per zone.
// d_nobs/d_ampl/d_status are chunk-relative.
// d_aux holds zone_eig_aux(N) elements per zone, d_Z N*N elements per zone;
// d_work two counters. FP64 with tc_products and N <= gram_oz_max_n(): T_sym = U (I+L)^-1/2 U^T
// as exact slice products on the tensor cores (zone_tsym_oz), else on the FP64 CUDA cores.
cudaError_t zone_eig_fp64(int N, int32_t nzc, double* d_GT, const double* d_g,
                          const int32_t* d_nobs, int rotate, double* d_ampl, int32_t* d_status,
                          double* d_aux, double* d_Z, int32_t* d_work, cudaStream_t st,
                          int tc_products = 1);
cudaError_t zone_eig_fp32(int N, int32_t nzc, float* d_GT, const float* d_g,
                          const int32_t* d_nobs, int rotate, float* d_ampl, int32_t* d_status,
                          float* d_aux, float* d_Z, int32_t* d_work, cudaStream_t st);
size_t zone_eig_aux(int N);
// zone_eig_fp32 with the FP32 eigenpairs refined to FP64 accuracy (Ogita-Aishima) before T and
// the amplitudes are formed (zone_refine.cu): d_G0 (N x N floats a zone) keeps G, d_S holds
// zone_refine_scratch(N) floats a zone; N <= 128.
cudaError_t zone_eig_fp32_refined(int N, int32_t nzc, float* d_GT, const float* d_g,
                                  const int32_t* d_nobs, int rotate, float* d_ampl,
                                  int32_t* d_status, float* d_aux, float* d_Z, int32_t* d_work,
                                  float* d_G0, float* d_S, cudaStream_t st);
size_t zone_refine_scratch(int N);
cudaError_t zone_eig_refine(int N, int32_t nzc, const float* d_G0, float* d_Z, float* d_aux,
                            const int32_t* d_nobs, float* d_S, cudaStream_t st);

// ---- zone_eig32.cu: FP32 stages for N <= eig32_max_n() (one block per zone), used by
// zone_eig_fp32 (same arguments as its stages)
int eig32_max_n();
cudaError_t eig32_tridiag(int N, int32_t nzc, float* d_GT, float* d_aux, const int32_t* d_nobs,
                          cudaStream_t st);
cudaError_t eig32_values(int N, int32_t nzc, float* d_aux, const int32_t* d_nobs,
                         int32_t* d_status, cudaStream_t st);
cudaError_t eig32_vectors(int N, int32_t nzc, const float* d_aux, float* d_Z,
                          const int32_t* d_nobs, cudaStream_t st);
cudaError_t eig32_transform(int N, int32_t nzc, float* d_GT, const float* d_aux, float* d_Z,
                            const float* d_g, const int32_t* d_nobs, int rotate, float* d_ampl,
                            int32_t* d_status, cudaStream_t st, int mode = 0);
// E1 and E3 for eig32_max_n() < N <= eig128_max_n() (one 128-thread block per zone; E2 is the
// generic one)
int eig128_max_n();
cudaError_t eig128_tridiag(int N, int32_t nzc, float* d_GT, float* d_aux, const int32_t* d_nobs,
                           cudaStream_t st);
cudaError_t eig128_transform(int N, int32_t nzc, float* d_GT, const float* d_aux, float* d_Z,
                             const float* d_g, const int32_t* d_nobs, int rotate, float* d_ampl,
                             int32_t* d_status, cudaStream_t st, int mode = 0);

// ---- ensemble.cu: the ensemble prologue (mean, anomalies, sparse H E + Hshift) and epilogue
// (inflation, correction clip, reconstruction); HEf_scratch holds m x N values.
cudaError_t ensemble_prologue(int64_t n, int N, const double* Ef, int64_t ldE, int64_t m, int K,
                              const int64_t* idx, const double* w, const double* shift,
                              double* xf, double* Sf, int64_t ldS, double* Hxf, double* HSf,
                              int64_t ldH, double* HEf_scratch, cudaStream_t st);
// ens2sqrt: mean and N - 1 anomaly columns of an ensemble; sqrt2ens: E = mean + S Om^T with
// Om (N x N-1, row-major); the bias-aware steps ba = bf - gamma inc, ux = xf - ba; y = a x + b z.
cudaError_t ensemble_ens2sqrt(int64_t n, int N, const double* E, int64_t ldE, double* mean,
                              double* S, int64_t ldS, cudaStream_t st);
cudaError_t ensemble_sqrt2ens(int64_t n, int N, const double* mean, const double* S, int64_t ldS,
                              const double* Om, double* E, int64_t ldE, cudaStream_t st);
// sqrt2ens with Theta = I in closed form (one read of S, one write of E); E(:, j) = mean
cudaError_t ensemble_sqrt2ens_identity(int64_t n, int N, const double* mean, const double* S,
                                       int64_t ldS, double* E, int64_t ldE, cudaStream_t st);
cudaError_t ensemble_fill_columns(int64_t n, int N, const double* mean, double* E, int64_t ldE,
                                  cudaStream_t st);
// y = H x + shift for one state vector (the sparse operator of ensemble_prologue)
cudaError_t obsoper_apply(int64_t m, int K, const int64_t* idx, const double* w,
                          const double* shift, const double* x, int64_t ldx, double* y,
                          cudaStream_t st);
cudaError_t bias_update(int64_t n, double gamma, const double* bf, const double* inc,
                        const double* xf, double* ba, double* ux, cudaStream_t st);
cudaError_t axpby(int64_t n, double a, const double* x, double b, const double* z, double* y,
                  cudaStream_t st);
cudaError_t ensemble_epilogue(int64_t n, int N, const double* xf, const double* xa,
                              const double* Sa, int64_t ldS, double inflation,
                              const double* maxcorr, double* Ea, int64_t ldE, cudaStream_t st);

// ---- zone_update.cu
// xa = xf + Sf ampl, Sa = Sf T per zone; zones with nobs == 0 copy (xa = xf, Sa = Sf).
cudaError_t zone_update_fp64(int N, int32_t z0, int32_t nzc, const int64_t* d_zone_start,
                             int32_t zone_max, const double* xf, const double* Sf,
                             int64_t ldS, const double* d_T, const double* d_ampl,
                             const int32_t* d_nobs, double* xa, double* Sa, cudaStream_t st);
cudaError_t write_amplitudes(int N, int32_t z0, int32_t nzc, const double* d_ampl,
                             const int32_t* d_nobs, int all_zones, double* ampl_out,
                             cudaStream_t st);
cudaError_t zone_update_fp32(int N, int32_t z0, int32_t nzc, const int64_t* d_zone_start,
                             int32_t zone_max, const double* xf, const double* Sf,
                             int64_t ldS, const float* d_T, const float* d_ampl,
                             const int32_t* d_nobs, double* xa, double* Sa, cudaStream_t st);
cudaError_t write_amplitudes_fp32(int N, int32_t z0, int32_t nzc, const float* d_ampl,
                                  const int32_t* d_nobs, int all_zones, double* ampl_out,
                                  cudaStream_t st);
// The same with FP32 storage of xf, Sf, xa, Sa and the amplitudes at the boundary.
cudaError_t zone_update_fp64(int N, int32_t z0, int32_t nzc, const int64_t* d_zone_start,
                             int32_t zone_max, const float* xf, const float* Sf, int64_t ldS,
                             const double* d_T, const double* d_ampl, const int32_t* d_nobs,
                             float* xa, float* Sa, cudaStream_t st);
cudaError_t write_amplitudes(int N, int32_t z0, int32_t nzc, const double* d_ampl,
                             const int32_t* d_nobs, int all_zones, float* ampl_out,
                             cudaStream_t st);
cudaError_t zone_update_fp32(int N, int32_t z0, int32_t nzc, const int64_t* d_zone_start,
                             int32_t zone_max, const float* xf, const float* Sf, int64_t ldS,
                             const float* d_T, const float* d_ampl, const int32_t* d_nobs,
                             float* xa, float* Sa, cudaStream_t st);
cudaError_t write_amplitudes_fp32(int N, int32_t z0, int32_t nzc, const float* d_ampl,
                                  const int32_t* d_nobs, int all_zones, float* ampl_out,
                                  cudaStream_t st);

// Mixed form on the tensor cores (zone_update_tc.cu), N <= 128: the same update with
// Sa = Sf T and Sf ampl as one 3xTF32 product; d_err receives ZST_TIMEOUT (OR) if a bounded
// device wait expired.
cudaError_t zone_update_tc(int N, int32_t z0, int32_t nzc, const int64_t* d_zone_start,
                           const double* xf, const double* Sf, int64_t ldS, const float* d_T,
                           const float* d_ampl, const int32_t* d_nobs, double* xa, double* Sa,
                           int32_t* d_err, cudaStream_t st);
cudaError_t zone_update_tc(int N, int32_t z0, int32_t nzc, const int64_t* d_zone_start,
                           const float* xf, const float* Sf, int64_t ldS, const float* d_T,
                           const float* d_ampl, const int32_t* d_nobs, float* xa, float* Sa,
                           int32_t* d_err, cudaStream_t st);

int max_fp64_ensemble();  // largest N the FP64 kernels accept
int max_ensemble();       // largest N of the mixed-precision form

// ---- oakg_api.cu
void count_launches(int k);       // kernel-launch accounting (oakg_launch_count)
int64_t launch_total();
cudaStream_t current_stream();    // stream of the current device's context

}  // namespace oakg
