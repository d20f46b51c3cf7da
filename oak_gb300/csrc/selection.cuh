// Device-side observation selection shared by the forward (zone_gram.cu) and adjoint
// (zone_adjoint.cu) kernels: the reference's distance() and Gaspari-Cohn locfun() with
// explicit rounding, and the cell ranges a zone has to visit.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

#include "oakg_internal.cuh"

namespace oakg {
namespace sel {

constexpr double kPi = 3.141592653589793238462643383279502884197;
constexpr double kEarthRadius = 6378137.0;

// Gaspari-Cohn (covariance.F90:645-667), evaluated in the reference's Horner order with every
// product and sum rounded separately (no FMA contraction). Near r = 2 the value is a
// cancellation of order (2-r)^3, so the `w /= 0` relevance test is only reproducible when the
// operations round exactly as a plain IEEE evaluation does.
static __device__ __forceinline__ double locfun(double r) {
  if (r <= 1.0) {
    double t = __dadd_rn(__ddiv_rn(-r, 4.0), 0.5);
    t = __dadd_rn(__dmul_rn(t, r), 5.0 / 8.0);
    t = __dsub_rn(__dmul_rn(t, r), 5.0 / 3.0);
    return __dadd_rn(__dmul_rn(t, __dmul_rn(r, r)), 1.0);
  }
  if (r <= 2.0) {
    double t = __dsub_rn(__ddiv_rn(r, 12.0), 0.5);
    t = __dadd_rn(__dmul_rn(t, r), 5.0 / 8.0);
    t = __dadd_rn(__dmul_rn(t, r), 5.0 / 3.0);
    t = __dsub_rn(__dmul_rn(t, r), 5.0);
    t = __dadd_rn(__dmul_rn(t, r), 4.0);
    return __dsub_rn(t, __ddiv_rn(2.0, __dmul_rn(3.0, r)));
  }
  return 0.0;
}

// locfun's value with FMA and reciprocal constants (one division): for weight values, where an
// ulp or two of difference from the reference's rounding does not matter; relevance decisions
// use locfun above
static __device__ __forceinline__ double locfun_value(double r) {
  if (r <= 1.0) {
    const double t = fma(fma(fma(-0.25, r, 0.5), r, 0.625), r, -5.0 / 3.0);
    return fma(t, r * r, 1.0);
  }
  if (r <= 2.0) {
    const double t = fma(fma(fma(fma(r, 1.0 / 12.0, -0.5), r, 0.625), r, 5.0 / 3.0), r, -5.0);
    return fma(t, r, 4.0) - (2.0 / 3.0) / r;
  }
  return 0.0;
}

// distance(p0 = observation, p1 = zone) (assimilation.F90:3635-3672). Products and sums are
// rounded one by one (no FMA contraction), so the Cartesian value is the correctly rounded
// result of the reference expression and the d <= maxLength test matches a CPU evaluation.
static __device__ __forceinline__ double distance(double x0, double y0, double x1, double y1,
                                           int metric) {
  if (metric == OAKG_METRIC_CARTESIAN) {
    double dx = __dsub_rn(x1, x0), dy = __dsub_rn(y1, y0);
    return sqrt(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
  } else if (metric == OAKG_METRIC_SPHERICAL_APPROX) {
    const double coeff = kPi * kEarthRadius / 180.0;
    double a = __dmul_rn(__dmul_rn(coeff, cos(__dmul_rn(__dadd_rn(y0, y1), kPi / 360.0))),
                         __dsub_rn(x1, x0));
    double b = __dmul_rn(coeff, __dsub_rn(y1, y0));
    return sqrt(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)));
  } else {
    const double d2r = kPi / 180.0;
    double a = __dmul_rn(y0, d2r), b = __dmul_rn(y1, d2r), C = __dmul_rn(__dsub_rn(x1, x0), d2r);
    double coeff = __dadd_rn(__dmul_rn(sin(b), sin(a)),
                             __dmul_rn(__dmul_rn(cos(b), cos(a)), cos(C)));
    coeff = fmax(fmin(coeff, 1.0), -1.0);
    return __dmul_rn(kEarthRadius, acos(coeff));
  }
}

// Cell-relative FP32 coordinates of a zone for the Cartesian and 1-D distances: its cell indices
// along u and v (not clamped) and its FP32 offsets inside that cell. The distance to an
// observation of cell indices (cq, cvq) and offsets (rq, rvq) is then, per axis,
// (cq - cu) csu + (rq - ru) in FP32: every term is below maxLength + 2 csu in magnitude, so
// with cell edges of at most 2 maxLength its relative error at d = maxLength stays below
// 1e-6 (about 12 roundings of 2^-24), whatever the magnitude of the coordinates, and no FP64
// operation is spent on a candidate. ok is false for periodic grids and wider cells.
struct ZoneCell32 {
  int cu, cv;
  float ru, rv, csu, csv;
  bool ok;
};

static __device__ __forceinline__ ZoneCell32 zone_cell32(const CellGrid& g, double zu, double zv,
                                                         double Rmax) {
  ZoneCell32 z;
  const double fu = floor((zu - g.u0) / g.csu), fv = floor((zv - g.v0) / g.csv);
  z.ok = !g.periodic_u && g.csu <= 2.0 * Rmax && g.csv <= 2.0 * Rmax && fabs(fu) < 1e8 &&
         fabs(fv) < 1e8;
  z.cu = z.ok ? (int)fu : 0;
  z.cv = z.ok ? (int)fv : 0;
  z.ru = (float)(zu - (g.u0 + z.cu * g.csu));
  z.rv = (float)(zv - (g.v0 + z.cv * g.csv));
  z.csu = (float)g.csu;
  z.csv = (float)g.csv;
  return z;
}

// FP32 distance between the zone and observation q of cell row cv (see ZoneCell32)
static __device__ __forceinline__ float cell_distance32(const ZoneCell32& z, const SortedObs& so,
                                                        int32_t q, int cv, bool two_d) {
  const float du = fmaf((float)(so.cu[q] - z.cu), z.csu, so.ru[q] - z.ru);
  float D2 = du * du;
  if (two_d) {
    const float dv = fmaf((float)(cv - z.cv), z.csv, so.rv[q] - z.rv);
    D2 = fmaf(dv, dv, D2);
  }
  return sqrtf(D2);
}

// Cell-index ranges a zone has to visit. Rows are v cells [cv0, cv1]; in each row the u cells
// [cu0, cu1] (unclamped for a periodic axis; iterate modulo nu). all_u: visit every u cell.
struct ScanRange {
  int cu0, cu1, cv0, cv1, all_u;
};

static __device__ ScanRange zone_scan_range(const CellGrid& g, int metric, int loctype, double zu,
                                     double zv, double R) {
  ScanRange s;
  double du, dv;
  int all_u = 0;
  if (loctype != 1 || metric == OAKG_METRIC_CARTESIAN) {
    du = R;
    dv = (loctype == 1) ? R : 0.0;
  } else if (metric == OAKG_METRIC_SPHERICAL_APPROX) {
    const double coeff = kPi * kEarthRadius / 180.0;
    dv = R / coeff;  // |dlat| bound, degrees
    double a = (zv - 0.5 * dv) * (kPi / 180.0), b = (zv + 0.5 * dv) * (kPi / 180.0);
    double cmin = fmin(fabs(cos(a)), fabs(cos(b)));
    if ((zv - 0.5 * dv) <= 0.0 && (zv + 0.5 * dv) >= 0.0) cmin = fmin(cmin, 1.0);
    if (fabs(zv) + 0.5 * dv >= 90.0 || cmin < 1e-12) {
      all_u = 1;
      du = 0.0;
    } else {
      du = R / (coeff * cmin);
    }
  } else {
    double rho = R / kEarthRadius;  // angular radius, radians
    dv = rho * (180.0 / kPi);
    if (rho >= kPi || fabs(zv) + dv >= 90.0) {
      all_u = 1;
      du = 0.0;
    } else {
      double sl = sin(rho) / cos(zv * (kPi / 180.0));
      du = (sl >= 1.0) ? 180.0 : asin(sl) * (180.0 / kPi);
      if (du >= 180.0) all_u = 1;
    }
  }
  // relative + absolute safety margins: candidates are a superset, the exact test decides
  du = du * (1.0 + 1e-9) + 1e-9 * (fabs(zu) + du + g.csu);
  dv = dv * (1.0 + 1e-9) + 1e-9 * (fabs(zv) + dv + g.csv);
  double zuu = zu;
  if (g.periodic_u) zuu = zu - 360.0 * floor(zu / 360.0);
  double fu0 = floor((zuu - du - g.u0) / g.csu), fu1 = floor((zuu + du - g.u0) / g.csu);
  if (g.periodic_u) {  // one extra cell each side absorbs rounding of the wrap-around
    fu0 -= 1.0;
    fu1 += 1.0;
  }
  // Ranges are clamped to the grid, never emptied: observations outside the grid are binned
  // into its edge cells, so a zone whose window lies beyond an edge still scans that edge
  // (the exact distance test decides). This keeps a grid valid when observations later move
  // outside the bounds it was built for.
  double fv0 = floor((zv - dv - g.v0) / g.csv), fv1 = floor((zv + dv - g.v0) / g.csv);
  fv0 = fmin(fmax(fv0, 0.0), (double)(g.nv - 1));
  fv1 = fmin(fmax(fv1, 0.0), (double)(g.nv - 1));
  s.cv0 = (int)fv0;
  s.cv1 = (int)fv1;
  if (g.periodic_u) {
    if (all_u || fu1 - fu0 + 1.0 >= (double)g.nu) {
      all_u = 1;
    } else {
      s.cu0 = (int)fu0;
      s.cu1 = (int)fu1;
    }
  } else {
    fu0 = fmin(fmax(fu0, 0.0), (double)(g.nu - 1));
    fu1 = fmin(fmax(fu1, 0.0), (double)(g.nu - 1));
    s.cu0 = (int)fu0;
    s.cu1 = (int)fu1;
  }
  if (all_u) {
    s.cu0 = 0;
    s.cu1 = g.nu - 1;
  }
  s.all_u = all_u;
  return s;
}


// d locfun / dr (the derivative of the Gaspari-Cohn polynomial pieces, covariance.F90:645-667).
static __device__ __forceinline__ double locfun_deriv(double r) {
  if (r <= 1.0) return (((-5.0 / 4.0 * r + 2.0) * r + 15.0 / 8.0) * r - 10.0 / 3.0) * r;
  if (r <= 2.0)
    return (((5.0 / 12.0 * r - 2.0) * r + 15.0 / 8.0) * r + 10.0 / 3.0) * r - 5.0 +
           2.0 / (3.0 * r * r);
  return 0.0;
}

}  // namespace sel
}  // namespace oakg
