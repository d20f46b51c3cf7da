/*
 * oakg.h -- C ABI of the GB300 (sm_103a) local ensemble square-root analysis.
 *
 * Drop-in boundary for OAK's analysis path (gher-uliege/OAK 1.7). Two groups of entry points:
 *
 *  1. OAK's existing C interface, same names and signatures
 *     (assimilation.F90:4911-4933, compiled there under CINTERFACE, bind(C)):
 *        void oak_init(const char* fname);            assimilation.F90:4911-4916
 *        void oak_assim(int ntime, int n, int r,      assimilation.F90:4919-4927
 *                       double* Ef, double* Ea);
 *        void oak_done(void);                         assimilation.F90:4929-4933
 *     The reference stops the process on error (ERROR_STOP, ppdef.h:22); these return
 *     nothing either, but record the failure for oakg_last_error()/oakg_last_status()
 *     instead of exiting.
 *
 *  2. Kernel-level entry points replacing the Fortran routines the reference calls
 *     directly (test/test_rrsqrt.F90:65,144,154,174; assimilation.F90:3235,3288):
 *        oakg_analysis      <- analysis(xf,Hxf,yo,Sf,HSf,R,xa,Sa,amplitudes)
 *                              rrsqrt.F90:196-208 (R = DiagCovar, covariance.F90:70-79)
 *        oakg_locanalysis   <- locAnalysis(zoneSize,selectObservations,xf,Hxf,yo,Sf,HSf,
 *                              R,xa,Sa,amplitudes,localise_obs) rrsqrt.F90:433-466, with
 *                              selectObservations (assimilation.F90:3683-3771) replaced by
 *                              zone/observation geometry and a built-in weight kind.
 *
 * Conventions (all entry points):
 *  - Arrays are Fortran column-major, as in the reference: Sf/Sa are (n, N) with leading
 *    dimension ldS >= n; HSf is (m, N) with leading dimension ldH >= m; amplitudes is
 *    (N, nzones). Values are double precision (real(c_double)).
 *  - All pointers are borrowed for the duration of the call only. They are host pointers
 *    (mem = OAKG_MEM_HOST; copies to and from the GPU happen inside the call) or device
 *    pointers of the current CUDA device (mem = OAKG_MEM_DEVICE).
 *  - Outputs Sa and amplitudes may be NULL (the reference's optional arguments).
 *  - Return value: OAKG_OK (0) or one of the OAKG_ERR_* codes; oakg_last_error() gives a
 *    message. Calls are serialised by an internal lock (one call at a time per process).
 *  - The library keeps per-device buffers between calls; oakg_release() frees them.
 */
#ifndef OAKG_H
#define OAKG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define OAKG_OK 0
#define OAKG_ERR_ARGS 1     /* invalid sizes, pointers or options                        */
#define OAKG_ERR_CUDA 2     /* CUDA runtime error (no device, launch failure, ...)       */
#define OAKG_ERR_NAN 3      /* NaN analysis amplitudes (rrsqrt.F90:145-149)              */
#define OAKG_ERR_EIG 4      /* symmetric eigensolver did not converge                    */
#define OAKG_ERR_NOMEM 5    /* device allocation failed                                  */
#define OAKG_ERR_TIMEOUT 6  /* a bounded device-side wait ran out                        */
#define OAKG_ERR_INIT 7     /* init file / configuration error (oak_init, oak_assim)     */
#define OAKG_ERR_NOTIMPL 8  /* option not supported by this build                        */

/* where array pointers live */
#define OAKG_MEM_HOST 0
#define OAKG_MEM_DEVICE 1

/* observation weight kinds */
#define OAKG_WEIGHT_GAUSS_CUTOFF 0 /* w = exp(-(d/L)^2), d <= maxLength (assimilation.F90:3756-3767) */
#define OAKG_WEIGHT_GASPARI_COHN 1 /* w = locfun(d/L), d <= maxLength, w /= 0 (covariance.F90:645-667) */

/* metrics (metrictype, assimilation.F90:108-112, 3635-3672) */
#define OAKG_METRIC_CARTESIAN 0
#define OAKG_METRIC_SPHERICAL 1
#define OAKG_METRIC_SPHERICAL_APPROX 2

/* precision of the local analysis */
#define OAKG_PREC_FP64 0  /* every product in FP64 (the plain form)                     */
#define OAKG_PREC_MIXED 1 /* FP64 selection and (1+lambda)^-1/2, (1+lambda)^-1 scalings;
                             Gram (tensor cores, chunked FP32 accumulation), eigensolve and
                             update (tensor cores, 3xTF32) in FP32, compensated innovation
                             sums (relative analysis error ~1e-5). All forms take N <= 128. */
#define OAKG_PREC_MIXED_FP64EIG 2 /* OAKG_PREC_MIXED with the FP32 eigenpairs refined to
                             FP64 accuracy (Ogita-Aishima iterative refinement, exact
                             products of the FP32 eigenvectors and G) before T and the
                             amplitudes are formed: FP64 accuracy kept for the eigensolve
                             and the (1+lambda) scalings only                              */

/* oakg_loc.flags */
#define OAKG_FLAG_AMPL_ALWAYS 1 /* write amplitudes for every analysed zone (the reference
                                   writes them only when localise_obs is false, :375-384) */
#define OAKG_FLAG_BRUTE_SEARCH 2 /* test every observation for every zone (the reference's
                                    O(Z m) loop, assimilation.F90:3745-3757) instead of the
                                    cell-grid search; same results, for validation         */
#define OAKG_FLAG_SIMT_UPDATE 4  /* mixed form: the ensemble update on the CUDA cores (FP32
                                    FMA) instead of the tensor cores (3xTF32, used when the
                                    longest zone has at least 48 elements); both give
                                    FP32-level products                                    */
#define OAKG_FLAG_SIMT_GRAM 8    /* plain form: the Gram and square-root-transform
                                    (U (I+L)^-1/2 U^T) products on the FP64 CUDA cores
                                    instead of the tensor cores (exact 8-bit slice products,
                                    used for N <= 64); both give FP64-level products       */

typedef struct {
  int64_t n;        /* state vector size                                        */
  int32_t N;        /* ensemble size / error-space dimension (columns of Sf)    */
  int32_t pad0;
  int64_t m;        /* number of observations                                   */
  int64_t ldS;      /* leading dimension of Sf and Sa (>= n)                    */
  int64_t ldH;      /* leading dimension of HSf (>= m)                          */
  int32_t mem;      /* OAKG_MEM_HOST or OAKG_MEM_DEVICE                         */
  int32_t pad1;
} oakg_dims;

typedef struct {
  int32_t weight;       /* OAKG_WEIGHT_*                                          */
  int32_t metric;       /* OAKG_METRIC_* (metrictype)                             */
  int32_t loctype;      /* 1 horizontal (x,y), 2 |dz|, 3 |dt| (assimilation.F90:3748-3754) */
  int32_t localise_obs; /* localise_obs argument (default true, rrsqrt.F90:318-320) */
  int32_t rotate;       /* ROTATE_ENSEMBLE (rrsqrt.F90:24): 1 = rotate (reference default) */
  int32_t precision;    /* OAKG_PREC_*                                            */
  int32_t flags;        /* OAKG_FLAG_*                                            */
  int32_t pad0;
  double cell_size;     /* search-cell edge in coordinate units; <= 0 picks one   */
} oakg_loc;

/* analysis (rrsqrt.F90:196-208) with diagonal R = diag(r_diag):
 *   xf(n), Hxf(m), yo(m), Sf(n,N), HSf(m,N), r_diag(m) -> xa(n), Sa(n,N), ampl(N). */
int oakg_analysis(const oakg_dims* dims, const double* xf, const double* Hxf,
                  const double* yo, const double* Sf, const double* HSf,
                  const double* r_diag, double* xa, double* Sa, double* ampl);

/* locAnalysis (rrsqrt.F90:433-466): zones are consecutive blocks of the state vector,
 * zone_size(nzones) long (rrsqrt.F90:291-300). selectObservations (assimilation.F90:
 * 3683-3771) is evaluated on the device from:
 *   zone_xyzt(4, nzones)  column-major: x,y,z,t of each zone's first element (:3713-3740)
 *   obs_x, obs_y, obs_z, obs_t (m)      obsGridX/Y/Z/T (assimilation.F90:228);
 *                                        unused coordinates may be NULL
 *   corr_len, max_len (nzones)          hCorrLengthToObs / hMaxCorrLengthToObs at the
 *                                        zone's first element (assimilation.F90:229)
 * Outputs: xa(n), Sa(n,N) (may be NULL), ampl(N,nzones) (may be NULL), nobs(nzones)
 * (may be NULL; the number of relevant observations of each zone). */
int oakg_locanalysis(const oakg_dims* dims, const oakg_loc* loc, int32_t nzones,
                     const int32_t* zone_size, const double* xf, const double* Hxf,
                     const double* yo, const double* Sf, const double* HSf,
                     const double* r_diag, const double* zone_xyzt, const double* obs_x,
                     const double* obs_y, const double* obs_z, const double* obs_t,
                     const double* corr_len, const double* max_len, double* xa, double* Sa,
                     double* ampl, int32_t* nobs);

/* locAnalysis of the reference's single-precision build (PRECISION = single,
 * config.mk.template:17: real is real(4)): oakg_locanalysis with the state and observation
 * arrays xf, Hxf, yo, Sf, HSf, r_diag, xa, Sa and ampl in FP32 (real(c_float)); the geometry
 * (zone_xyzt, obs_*, corr_len, max_len) stays double, so the selection decisions are those of
 * oakg_locanalysis. Both precision modes: OAKG_PREC_FP64 widens the FP32 inputs and computes
 * in FP64 (rounding only the outputs); OAKG_PREC_MIXED reads and writes FP32 directly, half
 * the state bytes of the FP64 arrays. */
int oakg_locanalysis_f32(const oakg_dims* dims, const oakg_loc* loc, int32_t nzones,
                         const int32_t* zone_size, const float* xf, const float* Hxf,
                         const float* yo, const float* Sf, const float* HSf, const float* r_diag,
                         const double* zone_xyzt, const double* obs_x, const double* obs_y,
                         const double* obs_z, const double* obs_t, const double* corr_len,
                         const double* max_len, float* xa, float* Sa, float* ampl,
                         int32_t* nobs);

/* Adjoint of the local analysis mean -- no counterpart in the reference (it has no derivative
 * code). For a scalar cost J(xa) given by its gradient dJ_dxa(n) at the analysis of
 * oakg_locanalysis with the same inputs, where the prior anomalies are inflated by
 * `inflation` (Sf and HSf multiplied by it, the ErrorSpace.scale of assimilation.F90:1201):
 *   dJ_dyo(m), dJ_dr(m)   gradients w.r.t. the observations and their error variances
 *                          (original order; memory kind per dims->mem; may be NULL)
 *   *dJ_dlen              derivative w.r.t. a common factor on corr_len and max_len, at 1
 *                          (host pointer; the set of selected observations is held fixed,
 *                          exact for Gaspari-Cohn weights which vanish at the cut-off)
 *   *dJ_dinfl             derivative w.r.t. `inflation` (host pointer)
 * Only zones where dJ_dxa is non-zero are recomputed (Cholesky of I + G per zone, no stored
 * eigensystem). FP64. Sf and HSf are the anomalies before inflation. */
int oakg_locanalysis_adjoint(const oakg_dims* dims, const oakg_loc* loc, int32_t nzones,
                             const int32_t* zone_size, const double* Hxf, const double* yo,
                             const double* Sf, const double* HSf, const double* r_diag,
                             const double* zone_xyzt, const double* obs_x, const double* obs_y,
                             const double* obs_z, const double* obs_t, const double* corr_len,
                             const double* max_len, double inflation, const double* dJ_dxa,
                             double* dJ_dyo, double* dJ_dr, double* dJ_dlen, double* dJ_dinfl);

/* oakg_analysis for callers that cannot allocate device memory -- no counterpart in the
 * reference. Host programs that reserve all GPU memory for their own pool before loading this
 * library (model couplers often do), or that must not call cudaMalloc/cudaFree inside a
 * forecast-analysis cycle because those calls can synchronise the device, use this entry:
 * it calls no allocating routine. All temporaries live in one static device array of 256 KiB
 * that every GPU loading the library holds until the process exits.
 *   - Same arguments and results as oakg_analysis, plus the CUDA stream (cudaStream_t, NULL
 *     for the legacy default stream) the work is queued on; returns after it completed.
 *   - dims->mem must be OAKG_MEM_DEVICE; N (dims->N) must be <= 112, else OAKG_ERR_ARGS.
 *   - Calls share the array: calls that overlap on the GPU race, so serialise them.
 *   - The first call on a device also looks up the array's device address; make that first
 *     call before any stream capture. The address is kept until the process exits: do not
 *     reset the device's primary context (cudaDeviceReset) while the library is loaded. */
int oakg_analysis_noalloc(const oakg_dims* dims, const double* xf, const double* Hxf,
                          const double* yo, const double* Sf, const double* HSf,
                          const double* r_diag, double* xa, double* Sa, double* ampl,
                          void* stream);

/* Sparse observation operator H (m x n) in row form: observation j is
 *   sum_{t < K} weight[j*K + t] * x[index[j*K + t]] + (shift ? shift[j] : 0),
 * the reference's obsoper(H, x) + Hshift (assimilation.F90:3110-3114); a negative index
 * marks an unused pair (rows with fewer than K non-zeros). */
typedef struct oakg_obsoper {
  int64_t m;             /* rows (observations); must equal dims->m */
  int32_t K, pad0;       /* pairs per row */
  const int64_t* index;  /* [m*K] state rows */
  const double* weight;  /* [m*K] */
  const double* shift;   /* [m] Hshift, or NULL */
} oakg_obsoper;

/* Ensemble prologue of Assim (assimilation.F90:3110-3134, ASSIM_SCALING = 1): from the
 * ensemble Ef (n x N, leading dimension ldE) and H, the mean xf (n), the scaled anomalies
 * Sf = (Ef - xf)/sqrt(N-1) (n x N, dims->ldS), and the same for HEf = H Ef + Hshift: Hxf (m),
 * HSf (m x N, dims->ldH). Host or device arrays per dims->mem. */
int oakg_ensemble_prologue(const oakg_dims* dims, const double* Ef, int64_t ldE,
                           const oakg_obsoper* H, double* xf, double* Sf, double* Hxf,
                           double* HSf);

/* Ensemble epilogue (assimilation.F90:3299-3312, 3558-3565): Sa scaled by the posterior
 * inflation factor, xa clipped to xf +- max_correction (NULL: no clip), then
 * Ea(:,k) = xa + sqrt(N-1) Sa(:,k) (n x N, leading dimension ldE). */
int oakg_ensemble_epilogue(const oakg_dims* dims, const double* xf, const double* xa,
                           const double* Sa, double inflation, const double* max_correction,
                           double* Ea, int64_t ldE);

/* The local and global analyses with the non-diagonal observation error covariance of the
 * SMWCovar kind (covariance.F90:464-570): R = diag(r_diag) + B B^T, B (m x k, leading
 * dimension ldB, host or device per dims->mem). As in the reference, the zone covariance is R
 * packed to the zone's relevant observations with the localisation weights outside
 * (DCDCovar(w, R), rrsqrt.F90:395), solved by Sherman-Morrison-Woodbury with the k x k matrix
 * of the packed rows. FP64 form only (loc->precision = OAKG_PREC_FP64); N + k <= 128. Other
 * arguments and results as for oakg_locanalysis / oakg_analysis. */
int oakg_locanalysis_smw(const oakg_dims* dims, const oakg_loc* loc, int32_t nzones,
                         const int32_t* zone_size, const double* xf, const double* Hxf,
                         const double* yo, const double* Sf, const double* HSf,
                         const double* r_diag, int32_t k, const double* B, int64_t ldB,
                         const double* zone_xyzt, const double* obs_x, const double* obs_y,
                         const double* obs_z, const double* obs_t, const double* corr_len,
                         const double* max_len, double* xa, double* Sa, double* ampl,
                         int32_t* nobs);
int oakg_analysis_smw(const oakg_dims* dims, const double* xf, const double* Hxf,
                      const double* yo, const double* Sf, const double* HSf,
                      const double* r_diag, int32_t k, const double* B, int64_t ldB, double* xa,
                      double* Sa, double* ampl);

/* ens2sqrt (rrsqrt.F90:786-806, Pham 2001): the mean (n) and N - 1 anomaly columns
 * S (dims->ldS x (N-1)) of the ensemble E (n x N, leading dimension ldE):
 * alpha = (sqrt(N) - 1)/(N - 1), shift = (1 - alpha) mean + alpha E(:,N),
 * S(:,i) = (E(:,i) - shift)/sqrt(N - 1); S S^T is the ensemble covariance. N = dims->N. */
int oakg_ens2sqrt(const oakg_dims* dims, const double* E, int64_t ldE, double* mean, double* S);

/* sqrt2ens (rrsqrt.F90:815-839): the N-member ensemble E (n x N, leading dimension ldE) with
 * mean `mean` and covariance S S^T from N - 1 columns S (dims->ldS): E = mean + S Om^T,
 * Om = sqrt(N - 1) perpSpace(w) Theta, w = 1/sqrt(N) (perpSpace: matoper.F90:509-535). The
 * reference draws Theta with randOrthMatrix; here theta is the caller's (N-1) x (N-1)
 * orthogonal matrix (column-major, memory kind of dims->mem), or NULL for the identity. */
int oakg_sqrt2ens(const oakg_dims* dims, const double* mean, const double* S,
                  const double* theta, double* E, int64_t ldE);

/* ensAnalysis (rrsqrt.F90:613-671): the global analysis of an ensemble Ef (n x N, ldE) with
 * observed ensemble HEf (m x N, ldHE): mean and scaled anomalies of both, oakg_analysis,
 * Ea = xa + sqrt(N-1) Sa (n x N, ldE; may alias Ef). xa (n) and ampl (N) are optional. */
int oakg_ens_analysis(const oakg_dims* dims, const double* Ef, int64_t ldE, const double* HEf,
                      int64_t ldHE, const double* yo, const double* r_diag, double* Ea,
                      double* xa, double* ampl);

/* biasedLocAnalysis (rrsqrt.F90:476-546), the bias-aware local analysis: inc = the local
 * analysis increment of (Hxf, yo, Sf, HSf, R); ba = bf - gamma inc; the unbiased forecast
 * ux = xf - ba and H ux + Hshift (the operator H, shift included); xa = ux + the local analysis
 * increment of (H ux + Hshift, yo, Sf, HSf, (1 - gamma) R) (the reference's DCDCovar with
 * D = 1/sqrt(1 - gamma)); Sa = Sf (NULL: not written). 0 <= gamma < 1. Geometry arguments as
 * for oakg_locanalysis. */
int oakg_biased_locanalysis(const oakg_dims* dims, const oakg_loc* loc, int32_t nzones,
                            const int32_t* zone_size, double gamma, const oakg_obsoper* H,
                            const double* xf, const double* bf, const double* Hxf,
                            const double* yo, const double* Sf, const double* HSf,
                            const double* r_diag, const double* zone_xyzt, const double* obs_x,
                            const double* obs_y, const double* obs_z, const double* obs_t,
                            const double* corr_len, const double* max_len, double* xa,
                            double* ba, double* Sa);

/* ---- layout builders (the host preprocessing of the reference, on the device) ---------- */

/* initPartition (assimilation.F90:578-641): the zone layout of a partition vector.
 * partition (n): the zone number, 1..nzones, of every state element. Results: zone_size
 * (nzones); zone_index (n): the elements of zone 1, then of zone 2, ..., each zone's elements
 * in ascending order (0-based; the reference's zoneIndex minus 1); inv_index (n, optional):
 * position of every element in zone_index (invZoneIndex minus 1). A zone number outside
 * 1..nzones, or a zone without elements, is OAKG_ERR_ARGS (the reference stops on both,
 * :605-617). Arrays on the host or the device per mem (OAKG_MEM_*). */
int oakg_zone_layout(int64_t n, const int32_t* partition, int32_t nzones, int32_t mem,
                     int32_t* zone_size, int32_t* zone_index, int32_t* inv_index);

/* The zone numbering of globalInit (assimilation.F90:416-424): the partition file's labels (any
 * int32 values, gaps allowed) replaced by their rank, 1-based, among the distinct labels in
 * ascending order (unique(..., ind2 = partition), matoper.F90:1821-1882); *nzones (optional)
 * = the number of distinct labels. The result is a partition for oakg_zone_layout. labels and
 * partition must not alias. */
int oakg_partition_compact(int64_t n, const int32_t* labels, int32_t mem, int32_t* partition,
                           int32_t* nzones);

/* Y(i, :) = X(index(i), :) for i < n and ncols columns (column-major, leading dimensions ldX,
 * ldY >= n; X and Y must not alias): with index = zone_index it puts a state vector or an
 * ensemble in zone order (permute, matoper.F90:1166-1183, as in assimilation.F90:766, 4040),
 * with inv_index it puts it back (ipermute, matoper.F90:1187-1205; assimilation.F90:3994). */
int oakg_permute_rows(int64_t n, int32_t ncols, const int32_t* index, const double* X,
                      int64_t ldX, double* Y, int64_t ldY, int32_t mem);

/* The sea packing of a masked grid of npts points (the state vector holds the unmasked points
 * only: StateVectorSizeSea): sea[i] = number of unmasked points before point i, or -1 where
 * mask[i] != 0; *nsea (optional) = the number of unmasked points. */
int oakg_sea_index(int64_t npts, const uint8_t* mask, int32_t mem, int64_t* sea, int64_t* nsea);

/* The observation operator on the zone-ordered state (assimilation.F90:2404-2407,
 * H%j = invZoneIndex(H%j)): index[t] = inv_index[index[t]] in place for the count entries with
 * 0 <= index[t] < n; negative entries (unused pairs) stay; an entry >= n is OAKG_ERR_ARGS
 * (those entries are left as they were). */
int oakg_obsoper_to_zone_order(int64_t count, int64_t* index, const int32_t* inv_index,
                               int64_t n, int32_t mem);

/* genObservationOper (assimilation.F90:2471-2656) for one variable on a rectilinear grid of
 * ndim = 1..4 axes: shape[ndim] points per axis (each >= 2, host array), coords = the axes'
 * coordinates one after the other (shape[0] + ... values, each axis strictly monotone, either
 * direction), points in Fortran order (axis 0 fastest). sea: the sea packing of the grid's
 * points (oakg_sea_index) or NULL for an unmasked grid; offset: the variable's first row in the
 * state vector. For observation j at pos[k*m + j] (k < ndim), cinterp (ndgrid.F90:1183-1257):
 * the grid cell holding it, and if none of its 2^ndim corners is masked, the first simplex of
 * the cell's split (split, :357-435) whose barycentric coordinates lie in [-1e-8, 1 + 1e-8]
 * (interp_tetrahedron, :464-629), giving the corner weights. Row j of the operator:
 * index[j*2^ndim + c] = offset + sea[corner c], weight[...] its weight (corner c: bit k set =
 * upper side of axis k), in the oakg_obsoper row form. An observation outside the grid or next
 * to a masked point: index -1, weight 0 in all its pairs (the reference's out-of-domain
 * entry). A cell whose simplices have |det| <= 1e-8 (cell volume <= 2^(ndim-1) 1e-8, where the
 * reference falls back to an SVD solve): index -2, weight 0. */
int oakg_obsoper_rectilinear(int32_t ndim, const int32_t* shape, const double* coords,
                             const int64_t* sea, int64_t offset, int64_t m, const double* pos,
                             int32_t mem, int64_t* index, double* weight);

/* The local analysis of an ensemble, all on the device: prologue, oakg_locanalysis (dims->ldS
 * and dims->ldH are ignored: the anomalies are the library's), epilogue. Ea may alias Ef. The
 * numerical core of oak_assim for schemetype = 1 without the file I/O. */
int oakg_ens_locanalysis(const oakg_dims* dims, const oakg_loc* loc, int32_t nzones,
                         const int32_t* zone_size, const double* Ef, int64_t ldE,
                         const oakg_obsoper* H, const double* yo, const double* r_diag,
                         const double* zone_xyzt, const double* obs_x, const double* obs_y,
                         const double* obs_z, const double* obs_t, const double* corr_len,
                         const double* max_len, double inflation, const double* max_correction,
                         double* Ea);

/* Prepared local analysis -- no counterpart in the reference; for the repeated analyses of a
 * forecast-analysis cycle whose buffers stay in place (the cycle of assim.F90:71-99 calling
 * locAnalysis each step). oakg_plan_locanalysis takes the arguments of oakg_locanalysis (device
 * pointers only: dims->mem must be OAKG_MEM_DEVICE) and runs it once; it keeps the zone
 * offsets, the observation cell grid and every scratch buffer, and captures the device work
 * (observation binning, selection + Gram, eigensolve, update, status) as one CUDA graph.
 * oakg_plan_execute replays it on `stream` (NULL: the plan's own stream) against the current
 * contents of the same buffers -- new observation values and positions are honoured, the
 * sizes and pointers are those of the plan -- and waits for it: same status codes as
 * oakg_locanalysis. With tune != 0 (and loc->cell_size <= 0) the cell edge of the observation
 * grid is chosen among 0.25, 0.35, 0.5, 0.7 and 1 times the localisation reach by timing the
 * selection + Gram stage on the data; then the zone schedule of that stage: its persistent
 * blocks take zones off a counter in index order, or in descending observation count of the
 * tuning run (longest tasks first), whichever measures faster. oakg_plan_info reports the
 * chosen edge, the graph's node count and up to ntune (edge, ms) tuning samples; it returns
 * the number of samples. oakg_plan_schedule reports the zone schedule: 1 for the
 * descending-count order, 0 for index order, and the two measured stage times (ms, either may
 * be NULL; both 0 without tuning).
 * A plan holds the caller's pointers: keep the buffers alive until oakg_plan_destroy. */
typedef struct oakg_plan oakg_plan;
int oakg_plan_locanalysis(oakg_plan** plan, const oakg_dims* dims, const oakg_loc* loc,
                          int32_t nzones, const int32_t* zone_size, const double* xf,
                          const double* Hxf, const double* yo, const double* Sf,
                          const double* HSf, const double* r_diag, const double* zone_xyzt,
                          const double* obs_x, const double* obs_y, const double* obs_z,
                          const double* obs_t, const double* corr_len, const double* max_len,
                          double* xa, double* Sa, double* ampl, int32_t* nobs, int32_t tune);
int oakg_plan_execute(oakg_plan* plan, void* stream);
int oakg_plan_info(const oakg_plan* plan, double* cell_size, int64_t* graph_nodes,
                   double* tune_cell, double* tune_ms, int32_t ntune);
int oakg_plan_schedule(const oakg_plan* plan, double* index_order_ms, double* count_order_ms);
void oakg_plan_destroy(oakg_plan* plan);

/* Message of the last failed call on this thread (empty if none); returns its length. */
size_t oakg_last_error(char* buf, size_t len);

/* Status of the last call of any entry point (oak_* entry points return void). */
int oakg_last_status(void);

/* Device buffers kept between calls are freed. */
int oakg_release(void);

/* Per-stage device times of the last oakg_locanalysis call, in milliseconds, measured with
 * CUDA events on the library's stream: [0] observation preparation, [1] selection + Gram,
 * [2] eigensolve + transform, [3] ensemble update, [4] whole call (device). Returns the
 * number of values written (<= n). */
int oakg_last_timings(double* ms, int n);

/* CUDA stream (a cudaStream_t) the library launches on for the current device; NULL
 * restores the library's own stream. Calls still return only after their work is done.
 * No reference counterpart (the reference has no device). */
int oakg_set_stream(void* stream);

/* Number of kernel launches the library has made in this process (all devices).
 * No reference counterpart; used to account for device work in benchmarks. */
int64_t oakg_launch_count(void);

/* Diagnostic: measured FP64 FMA throughput of the current device in TFLOP/s (a
 * dependent-FMA loop over all SMs, ~0.1 s). No reference counterpart; it is the roofline
 * denominator of the FP64 kernels. */
int oakg_fp64_peak(double* tflops);

/* The data-file reader of the oak_init / oak_assim driver, as the reference's uload
 * (ufileformat.F90:555-745) reads a file:
 *  - spec "file.nc#var": a NetCDF variable (classic, 64-bit-offset or CDF-5 format;
 *    NetCDF-4 / HDF5 is not read);
 *  - spec "file" without '#': a GHER binary file in either byte order.
 * Outputs:
 *  - values: the values in Fortran order (first dimension fastest), capacity elements; NULL
 *    asks for the sizes only;
 *  - *count: the number of values;
 *  - shape[0..*ndim): the shape in Fortran order (at most 8 written);
 *  - *valex: the missing value. For NetCDF, the missing_value or _FillValue attribute, else
 *    -9999; for GHER, the header's.
 * scale_factor / add_offset are applied to the other values. The compact forms (the "shape"
 * attribute, negative GHER extents) are expanded as uexplo does, with 1-based indices. Host
 * only: no GPU is needed. */
int oakg_read_variable(const char* spec, double* values, int64_t capacity, int64_t* count,
                       int64_t* shape, int32_t* ndim, double* valex);

/* OAK's C interface (assimilation.F90:4885-4935), same names and signatures, with the
 * init-file driver of globalInit / Assim for the global (schemetype 0) and local (1) schemes:
 *  - oak_init(fname) (globalInit, assimilation.F90:253-493) reads the init file. From it:
 *    - the model's layout from Model.mask (a point is in the state where the mask value is not
 *      the file's missing value; Model.variables names the variables);
 *    - the model grids from Model.gridX/Y/Z/T (rectilinear: each coordinate array must be
 *      separable into one axis per dimension, else OAKG_ERR_NOTIMPL);
 *    - Model.hres, Model.maxCorrection and inflation.mult;
 *    - for schemetype 1, the zones: Zones.partition renumbered as the reference does, the zone
 *      layout, and Zones.corrLength / Zones.maxLength (files or .const) at each zone's first
 *      element.
 *    It creates the library's device context.
 *  - oak_assim(ntime, n, r, Ef, Ea) (Assim, :2977-3574) analyses the n x r ensemble Ef
 *    (column-major) with the observations ObsNNN.* of time index ntime. Those are: mask,
 *    variables, value, gridX/Y[/Z/T], rmse (or .const) or SMWCovar.SqrtDiag /
 *    SMWCovar.ErrorSpace / SMWCovar.dimension, and shift. The steps are:
 *    - the observation operator is generated on the model grids (oakg_obsoper_rectilinear);
 *    - observations outside every grid are excluded;
 *    - on the GPU: H Ef, mean and anomalies, the global or local analysis (the local one in
 *      zone order), inflation, the maxCorrection clip and Ea = xa + sqrt(r - 1) Sa.
 *    runtype 0 or 1 returns Ea = Ef.
 *  - oak_done frees the driver state and the device buffers (as oakg_release).
 * Files: NetCDF classic variables ("file.nc#var") and GHER binary files (names without '#').
 * Not done: diagnostics files (Diag*), biastype, anamorphosis, other schemetypes and operators
 * read from files (OAKG_ERR_NOTIMPL where the init file asks for them). The reference's
 * functions return nothing and stop the process on error; these record the status for
 * oakg_last_status() / oakg_last_error() and leave Ea unchanged. Call them from one thread. */
void oak_init(const char* fname);
void oak_assim(int ntime, int n, int r, double* Ef, double* Ea);
void oak_done(void);

#ifdef __cplusplus
}
#endif
#endif /* OAKG_H */
