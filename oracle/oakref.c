/*
 * C restatement of OAK's local ensemble square-root analysis -- TEST INFRASTRUCTURE.
 *
 * This file is the parity oracle at sizes NumPy loops cannot reach and the timed CPU
 * baseline (kind "port"). Only tests/, __graft_entry__.smoke() and bench.py's CPU leg load
 * it; the product library never links or calls it.
 *
 * It follows the reference (gher-uliege/OAK 1.7) routine by routine:
 *   oakref_locanalysis  <- rrsqrt.F90:258-466 (locAnalysisIncrement + locAnalysis):
 *       xa_xf = 0, Sa = Sf (:322-326); zone ranges by prefix sum (:328-335);
 *       OpenMP dynamic schedule over zones (:357); selectObservations (:368);
 *       p = 0 -> skip (:371); DCDCovar with D = weight (:395, covariance.F90:612-619);
 *       row-gather of the selected observations in ascending order (:397-404).
 *   select_zone         <- assimilation.F90:3683-3771 (d <= maxLength, w = exp(-(d/L)^2)),
 *                          distance() assimilation.F90:3635-3672, Gaspari-Cohn weights
 *                          covariance.F90:645-667 as used by test/test_rrsqrt.F90:254-271.
 *   analysis_increment  <- rrsqrt.F90:100-190, with the same sequence of products:
 *       temp = HSf^T (R^-1 HSf) (dgemm 't','n', matoper_inc.F90:420-439), symeig ->
 *       dsyev('V','L') (matoper_inc.F90:986-1005), clamp, lambda = 1/(1+lambda), ampl,
 *       xa_xf = Sf ampl, Sa = Sf (U (sqrt_lambda .dx. (U^T RotateVector(w,v)))).
 *   perp_space          <- matoper.F90:509-535;  RotateVector/normate <- rrsqrt.F90:737-756.
 *   oakref_analysis     <- rrsqrt.F90:196-208.
 *
 * dsyev/dgemm are taken as function pointers (the host passes LAPACK's, e.g. the ones
 * SciPy exports); with NULL pointers an internal eigensolver
 * (cyclic Jacobi, Golub & Van Loan, "Matrix Computations", 4th ed., 8.5) and plain loops are
 * used.
 *
 * Build: see oracle/build_oracle.py (gcc -O2 -fopenmp -ffp-contract=off -shared -fPIC).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef void (*dsyev_fn)(const char* jobz, const char* uplo, const int* n, double* a,
                         const int* lda, double* w, double* work, const int* lwork, int* info);
typedef void (*dgemm_fn)(const char* ta, const char* tb, const int* m, const int* n,
                         const int* k, const double* alpha, const double* a, const int* lda,
                         const double* b, const int* ldb, const double* beta, double* c,
                         const int* ldc);

static dsyev_fn g_dsyev = NULL;
static dgemm_fn g_dgemm = NULL;

void oakref_set_lapack(void* dsyev_ptr, void* dgemm_ptr) {
  g_dsyev = (dsyev_fn)dsyev_ptr;
  g_dgemm = (dgemm_fn)dgemm_ptr;
}

/* ---------------------------------------------------------------- small dense helpers */

/* C(m,n) = op(A) op(B), column-major, through BLAS when available. */
static void gemm(char ta, char tb, int m, int n, int k, const double* A, int lda,
                 const double* B, int ldb, double* C, int ldc) {
  if (g_dgemm) {
    const double one = 1.0, zero = 0.0;
    g_dgemm(&ta, &tb, &m, &n, &k, &one, A, &lda, B, &ldb, &zero, C, &ldc);
    return;
  }
  for (int j = 0; j < n; j++)
    for (int i = 0; i < m; i++) {
      double s = 0.0;
      for (int l = 0; l < k; l++) {
        double a = (ta == 'T') ? A[l + (size_t)i * lda] : A[i + (size_t)l * lda];
        double b = (tb == 'T') ? B[j + (size_t)l * ldb] : B[l + (size_t)j * ldb];
        s += a * b;
      }
      C[i + (size_t)j * ldc] = s;
    }
}

/* Symmetric eigensolver fallback (no LAPACK available): cyclic Jacobi rotations on the full
 * matrix, each annihilating one off-diagonal pair (Golub & Van Loan, "Matrix Computations",
 * 4th ed., 8.5.2-8.5.3), repeated until the off-diagonal mass is below eps * ||A||_F.
 * A (n x n, column-major, both triangles read from the lower one) is overwritten with the
 * eigenvectors (columns); w receives the eigenvalues in ascending order, as dsyev returns
 * them. scratch must hold n*n doubles. Returns 0, or 1 if 100 sweeps did not converge. */
static int sym_eig_internal(int n, double* A, double* w, double* V) {
  for (int j = 0; j < n; j++)
    for (int i = 0; i < j; i++) A[i + (size_t)j * n] = A[j + (size_t)i * n];
  for (int j = 0; j < n; j++)
    for (int i = 0; i < n; i++) V[i + (size_t)j * n] = (i == j) ? 1.0 : 0.0;
  double fro = 0.0;
  for (size_t k = 0; k < (size_t)n * n; k++) fro += A[k] * A[k];
  int converged = 0;
  for (int sweep = 0; sweep < 100 && !converged; sweep++) {
    double off = 0.0;
    for (int j = 0; j < n; j++)
      for (int i = 0; i < j; i++) off += 2.0 * A[i + (size_t)j * n] * A[i + (size_t)j * n];
    if (off <= 1e-30 * fro || off == 0.0) {
      converged = 1;
      break;
    }
    for (int p = 0; p < n - 1; p++)
      for (int q = p + 1; q < n; q++) {
        double apq = A[p + (size_t)q * n];
        if (apq == 0.0) continue;
        double app = A[p + (size_t)p * n], aqq = A[q + (size_t)q * n];
        /* rotation angle: tan(2 theta) = 2 apq / (aqq - app), smaller root for t */
        double tau = (aqq - app) / (2.0 * apq);
        double t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
        double c = 1.0 / sqrt(1.0 + t * t), s = t * c;
        for (int k = 0; k < n; k++) { /* columns p, q of A */
          double akp = A[k + (size_t)p * n], akq = A[k + (size_t)q * n];
          A[k + (size_t)p * n] = c * akp - s * akq;
          A[k + (size_t)q * n] = s * akp + c * akq;
        }
        for (int k = 0; k < n; k++) { /* rows p, q of A */
          double apk = A[p + (size_t)k * n], aqk = A[q + (size_t)k * n];
          A[p + (size_t)k * n] = c * apk - s * aqk;
          A[q + (size_t)k * n] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; k++) { /* accumulate V <- V J */
          double vkp = V[k + (size_t)p * n], vkq = V[k + (size_t)q * n];
          V[k + (size_t)p * n] = c * vkp - s * vkq;
          V[k + (size_t)q * n] = s * vkp + c * vkq;
        }
      }
  }
  for (int k = 0; k < n; k++) w[k] = A[k + (size_t)k * n];
  /* selection sort into ascending order, moving eigenvector columns along */
  for (int i = 0; i < n; i++) {
    int k = i;
    for (int j = i + 1; j < n; j++)
      if (w[j] < w[k]) k = j;
    if (k != i) {
      double t = w[i];
      w[i] = w[k];
      w[k] = t;
      for (int r = 0; r < n; r++) {
        double x = V[r + (size_t)i * n];
        V[r + (size_t)i * n] = V[r + (size_t)k * n];
        V[r + (size_t)k * n] = x;
      }
    }
  }
  memcpy(A, V, (size_t)n * n * sizeof(double));
  return converged ? 0 : 1;
}

/* symeig (matoper_inc.F90:939-1005): dsyev('V','L') on A (n x n); A <- U, w <- lambda. */
static int symeig(int n, double* A, double* w, double* work, int lwork) {
  if (g_dsyev) {
    int info = 0;
    g_dsyev("V", "L", &n, A, &n, w, work, &lwork, &info);
    return info;
  }
  return sym_eig_internal(n, A, w, work); /* work holds >= n*n doubles */
}

/* perpSpace(w) (matoper.F90:509-535): H (n x n-1), column-major. */
static void perp_space(int n, const double* w, double* H) {
  double alpha = -1.0 / (fabs(w[n - 1]) + 1.0);
  double sgn = signbit(w[n - 1]) ? -1.0 : 1.0;
  for (int j = 0; j < n - 1; j++) {
    for (int i = 0; i < n - 1; i++) {
      double h = alpha * w[i] * w[j];
      if (i == j) h += 1.0;
      H[i + (size_t)j * n] = h;
    }
    H[(n - 1) + (size_t)j * n] = alpha * (w[n - 1] + sgn) * w[j];
  }
}

/* Per-thread workspace for one analysisIncrement call. */
typedef struct {
  int N, pmax, nzmax, lwork;
  double *temp, *lam, *work, *ampl, *tmpv, *v, *w, *Pv, *Pw, *Om, *M, *T;
  double *HSz, *Wz, *dz, *rz;
  int* sel;
  double* dist;
} ws_t;

static void ws_init(ws_t* s, int N, int pmax, int nzmax, int m) {
  s->N = N;
  s->pmax = pmax;
  s->nzmax = nzmax;
  s->lwork = 64 * N + 64 > N * N ? 64 * N + 64 : N * N;
  size_t NN = (size_t)N * N;
  s->temp = malloc(NN * sizeof(double));
  s->lam = malloc(N * sizeof(double));
  s->work = malloc((size_t)s->lwork * sizeof(double));
  s->ampl = malloc(N * sizeof(double));
  s->tmpv = malloc(N * sizeof(double));
  s->v = malloc(N * sizeof(double));
  s->w = malloc(N * sizeof(double));
  s->Pv = malloc(NN * sizeof(double));
  s->Pw = malloc(NN * sizeof(double));
  s->Om = malloc(NN * sizeof(double));
  s->M = malloc(NN * sizeof(double));
  s->T = malloc(NN * sizeof(double));
  s->HSz = malloc((size_t)pmax * N * sizeof(double));
  s->Wz = malloc((size_t)pmax * N * sizeof(double));
  s->dz = malloc((size_t)pmax * sizeof(double));
  s->rz = malloc((size_t)pmax * sizeof(double));
  s->sel = malloc((size_t)(m > 0 ? m : 1) * sizeof(int));
  s->dist = malloc((size_t)(m > 0 ? m : 1) * sizeof(double));
}

static void ws_free(ws_t* s) {
  free(s->temp); free(s->lam); free(s->work); free(s->ampl); free(s->tmpv); free(s->v);
  free(s->w); free(s->Pv); free(s->Pw); free(s->Om); free(s->M); free(s->T); free(s->HSz);
  free(s->Wz); free(s->dz); free(s->rz); free(s->sel); free(s->dist);
}

/* analysisIncrement (rrsqrt.F90:100-190) on p gathered observations.
 * HSz (p x N, ld p), innov = yo - Hxf (p), rinv = R%mldivide diagonal (p),
 * Sf (nz rows of an ld-strided matrix), outputs xa_xf (nz), Sa (nz rows, ld), ampl (N).
 * Returns 0, or 1 on NaN amplitudes (:145-149), 2 on eigensolver failure. */
static int analysis_increment(ws_t* s, int p, const double* HSz, const double* innov,
                              const double* rinv, int nz, const double* Sf, size_t ldS,
                              double* xa_xf, double* Sa, size_t ldA, double* ampl_out,
                              int rotate) {
  const int N = s->N;
  /* temp = HSf^T (rinv .* HSf)   (:135) */
  for (int k = 0; k < N; k++)
    for (int j = 0; j < p; j++) s->Wz[j + (size_t)k * p] = rinv[j] * HSz[j + (size_t)k * p];
  gemm('T', 'N', N, N, p, HSz, p, s->Wz, p, s->temp, N);
  if (symeig(N, s->temp, s->lam, s->work, s->lwork) != 0) return 2; /* :136 */
  double* U = s->temp;
  for (int k = 0; k < N; k++) {
    double l = s->lam[k];
    if (l < 0) l = 0;             /* :137 */
    s->lam[k] = 1.0 / (1.0 + l);  /* :140 */
  }
  /* ampl = U (lambda .* (U^T (HSf^T (rinv .* (yo-Hxf)))))   (:142) */
  for (int k = 0; k < N; k++) {
    double acc = 0.0;
    for (int j = 0; j < p; j++) acc += HSz[j + (size_t)k * p] * (rinv[j] * innov[j]);
    s->v[k] = acc;
  }
  for (int k = 0; k < N; k++) {
    double acc = 0.0;
    for (int i = 0; i < N; i++) acc += U[i + (size_t)k * N] * s->v[i];
    s->tmpv[k] = s->lam[k] * acc;
  }
  for (int i = 0; i < N; i++) {
    double acc = 0.0;
    for (int k = 0; k < N; k++) acc += U[i + (size_t)k * N] * s->tmpv[k];
    s->ampl[i] = acc;
  }
  for (int i = 0; i < N; i++)
    if (s->ampl[i] != s->ampl[i]) return 1;
  /* xa_xf = Sf ampl   (:151) */
  for (int r = 0; r < nz; r++) {
    double acc = 0.0;
    for (int k = 0; k < N; k++) acc += Sf[r + k * ldS] * s->ampl[k];
    xa_xf[r] = acc;
  }
  if (ampl_out) memcpy(ampl_out, s->ampl, N * sizeof(double));
  if (!Sa) return 0;
  /* sqrt_lambda (:162) */
  for (int k = 0; k < N; k++) s->lam[k] = sqrt(s->lam[k]);
  /* M = U^T Omega with Omega = RotateVector(w, v) (:165-185), or U^T without rotation */
  if (rotate) {
    double wv = 1.0 / sqrt(1.0 * N);
    for (int i = 0; i < N; i++) s->w[i] = wv;
    /* v = U (sum(U,1) / sqrt_lambda); v = normate(v) */
    for (int k = 0; k < N; k++) {
      double cs = 0.0;
      for (int i = 0; i < N; i++) cs += U[i + (size_t)k * N];
      s->tmpv[k] = cs / s->lam[k];
    }
    double nrm = 0.0;
    for (int i = 0; i < N; i++) {
      double acc = 0.0;
      for (int k = 0; k < N; k++) acc += U[i + (size_t)k * N] * s->tmpv[k];
      s->v[i] = acc;
      nrm += acc * acc;
    }
    nrm = sqrt(nrm);
    for (int i = 0; i < N; i++) s->v[i] /= nrm;
    /* Omega = v w^T + perpSpace(v) perpSpace(w)^T */
    perp_space(N, s->v, s->Pv);
    perp_space(N, s->w, s->Pw);
    gemm('N', 'T', N, N, N - 1, s->Pv, N, s->Pw, N, s->Om, N);
    for (int j = 0; j < N; j++)
      for (int i = 0; i < N; i++) s->Om[i + (size_t)j * N] += s->v[i] * s->w[j];
    gemm('T', 'N', N, N, N, U, N, s->Om, N, s->M, N);
  } else {
    for (int j = 0; j < N; j++)
      for (int i = 0; i < N; i++) s->M[i + (size_t)j * N] = U[j + (size_t)i * N];
  }
  for (int j = 0; j < N; j++)
    for (int i = 0; i < N; i++) s->M[i + (size_t)j * N] *= s->lam[i];
  gemm('N', 'N', N, N, N, U, N, s->M, N, s->T, N);
  /* Sa = Sf T */
  if (g_dgemm) {
    int ldsi = (int)ldS, ldai = (int)ldA, Ni = N, nzi = nz;
    const double one = 1.0, zero = 0.0;
    g_dgemm("N", "N", &nzi, &Ni, &Ni, &one, Sf, &ldsi, s->T, &Ni, &zero, Sa, &ldai);
  } else {
    for (int c = 0; c < N; c++)
      for (int r = 0; r < nz; r++) {
        double acc = 0.0;
        for (int k = 0; k < N; k++) acc += Sf[r + k * ldS] * s->T[k + (size_t)c * N];
        Sa[r + c * ldA] = acc;
      }
  }
  return 0;
}

/* ------------------------------------------------------------------- selection */

#define OAKREF_PI 3.141592653589793238462643383279502884197
#define OAKREF_EARTH_RADIUS 6378137.0

/* distance() (assimilation.F90:3635-3672) */
static double distance(double x0, double y0, double x1, double y1, int metric) {
  if (metric == 0) {
    double dx = x1 - x0, dy = y1 - y0;
    return sqrt(dx * dx + dy * dy);
  } else if (metric == 2) {
    double coeff = OAKREF_PI * OAKREF_EARTH_RADIUS / 180.0;
    double a = coeff * cos((y0 + y1) * (OAKREF_PI / 360.0)) * (x1 - x0);
    double b = coeff * (y1 - y0);
    return sqrt(a * a + b * b);
  } else {
    double d2r = OAKREF_PI / 180.0;
    double a = y0 * d2r, b = y1 * d2r, C = (x1 - x0) * d2r;
    double coeff = sin(b) * sin(a) + cos(b) * cos(a) * cos(C);
    if (coeff > 1.0) coeff = 1.0;
    if (coeff < -1.0) coeff = -1.0;
    return OAKREF_EARTH_RADIUS * acos(coeff);
  }
}

/* locfun (covariance.F90:645-667) */
double oakref_locfun(double r) {
  if (r <= 1.0) return (((-r / 4.0 + 1.0 / 2.0) * r + 5.0 / 8.0) * r - 5.0 / 3.0) * (r * r) + 1.0;
  if (r <= 2.0)
    return ((((r / 12.0 - 1.0 / 2.0) * r + 5.0 / 8.0) * r + 5.0 / 3.0) * r - 5.0) * r + 4.0 -
           2.0 / (3.0 * r);
  return 0.0;
}

/* Selection parameters shared by all zones (mirrors the oakg_loc struct of the product). */
typedef struct {
  int metric;   /* 0 Cartesian, 1 spherical, 2 approx. spherical */
  int loctype;  /* 1 horizontal, 2 |dz|, 3 |dt| */
  int kind;     /* 0 Gaussian with cut-off, 1 Gaspari-Cohn */
  int localise; /* localise_obs */
  int rotate;   /* ROTATE_ENSEMBLE */
} oakref_loc;

/* selectObservations for one zone: returns p and fills sel (ascending indices) and dist
 * (the weight of each selected observation, replacing the distance). For the
 * non-localised branch all m observations are returned with their weights. */
static int select_zone(const oakref_loc* L, int m, const double* zpos, const double* ox,
                       const double* oy, const double* oz, const double* ot, double corr,
                       double maxl, int* sel, double* wsel, int* any_relevant) {
  int p = 0, nrel = 0;
  for (int l = 0; l < m; l++) {
    double d;
    if (L->loctype == 1)
      d = distance(ox[l], oy[l], zpos[0], zpos[1], L->metric); /* p0 = obs, p1 = zone */
    else if (L->loctype == 2)
      d = fabs(oz[l] - zpos[2]);
    else
      d = fabs(ot[l] - zpos[3]);
    double w;
    int rel;
    if (L->kind == 0) {
      rel = d <= maxl;
      w = exp(-(d / corr) * (d / corr));
    } else {
      w = oakref_locfun(d / corr);
      rel = (d <= maxl) && (w != 0.0);
    }
    nrel += rel;
    if (rel || !L->localise) {
      sel[p] = l;
      wsel[p] = w;
      p++;
    }
  }
  *any_relevant = nrel;
  return p;
}

/* locAnalysis (rrsqrt.F90:258-466) with geometric selection.
 * Sf (n x N, ld n), HSf (m x N, ld m) column-major; zpos (Z x 4, row-major);
 * obs coordinates ox/oy/oz/ot (m); corr/maxl (Z).
 * Outputs xa (n), Sa (n x N, may be NULL), ampl (N x Z, may be NULL), nobs (Z, may be
 * NULL). nthreads <= 0 keeps the OpenMP default. Returns 0 or the first error code. */
int oakref_locanalysis(int n, int N, int m, int Z, const int* zone_size, const double* xf,
                       const double* Hxf, const double* yo, const double* Sf,
                       const double* HSf, const double* r_diag, const double* zpos,
                       const double* ox, const double* oy, const double* oz,
                       const double* ot, const double* corr, const double* maxl,
                       const oakref_loc* L, double* xa, double* Sa, double* ampl, int* nobs,
                       int nthreads) {
  long* start = malloc((size_t)(Z + 1) * sizeof(long));
  start[0] = 0;
  for (int z = 0; z < Z; z++) start[z + 1] = start[z] + zone_size[z];
  int nzmax = 0;
  for (int z = 0; z < Z; z++)
    if (zone_size[z] > nzmax) nzmax = zone_size[z];
  /* xa_xf = 0; Sa = Sf; amplitudes = 0  (:322-326) */
  for (int i = 0; i < n; i++) xa[i] = 0.0;
  if (Sa) memcpy(Sa, Sf, (size_t)n * N * sizeof(double));
  if (ampl) memset(ampl, 0, (size_t)N * Z * sizeof(double));
  int err = 0;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel
  {
    ws_t s;
    ws_init(&s, N, m > 0 ? m : 1, nzmax, m);
#pragma omp for schedule(dynamic)
    for (int z = 0; z < Z; z++) {
      int nrel = 0;
      int p = select_zone(L, m, zpos + 4 * (size_t)z, ox, oy, oz, ot, corr[z], maxl[z],
                          s.sel, s.dist, &nrel);
      if (nobs) nobs[z] = nrel;
      if (nrel == 0) continue; /* :371 */
      for (int j = 0; j < p; j++) {
        int l = s.sel[j];
        for (int k = 0; k < N; k++) s.HSz[j + (size_t)k * p] = HSf[l + (size_t)k * m];
        s.dz[j] = yo[l] - Hxf[l];
        s.rz[j] = s.dist[j] * (s.dist[j] / r_diag[l]); /* D * C^-1 (D x) */
      }
      long i1 = start[z];
      int nz = zone_size[z];
      double* az = (ampl && !L->localise) ? ampl + (size_t)z * N : NULL;
      int rc = analysis_increment(&s, p, s.HSz, s.dz, s.rz, nz, Sf + i1, (size_t)n, xa + i1,
                                  Sa ? Sa + i1 : NULL, (size_t)n, az, L->rotate);
      if (rc) {
#pragma omp critical
        if (!err) err = rc;
      }
    }
    ws_free(&s);
  }
  /* xa = xf + xa_xf (:462-464) */
  for (int i = 0; i < n; i++) xa[i] += xf[i];
  free(start);
  return err;
}

/* analysis (rrsqrt.F90:196-208) with diagonal R. */
int oakref_analysis(int n, int N, int m, const double* xf, const double* Hxf, const double* yo,
                    const double* Sf, const double* HSf, const double* r_diag, double* xa,
                    double* Sa, double* ampl, int rotate) {
  ws_t s;
  ws_init(&s, N, m > 0 ? m : 1, n, m);
  for (int j = 0; j < m; j++) {
    s.dz[j] = yo[j] - Hxf[j];
    s.rz[j] = 1.0 / r_diag[j];
  }
  int rc = analysis_increment(&s, m, HSf, s.dz, s.rz, n, Sf, (size_t)n, xa, Sa, (size_t)n,
                              ampl, rotate);
  for (int i = 0; i < n; i++) xa[i] += xf[i];
  ws_free(&s);
  return rc;
}
