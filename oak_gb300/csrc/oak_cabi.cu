// OAK's C interface (assimilation.F90:4885-4935): oak_init / oak_assim / oak_done, with the
// init-file driver behind them for the analysis schemes this library computes.
//
// oak_init (globalInit, assimilation.F90:253-493): the init file; the model's memory layout
// from its mask files (MemoryLayout, :1620-1775: a point is in the state where the mask value
// is not the file's missing value); the model grids (Model.gridX/Y/Z/T: rectilinear grids,
// the coordinate arrays separable into one axis per dimension); for schemetype = 1 the zones
// (Zones.partition renumbered as unique(...) does, :416-424; zone layout of initPartition;
// Zones.corrLength / Zones.maxLength at each zone's first element, as selectObservations reads
// them, :3713-3767); Model.maxCorrection; inflation.mult.
//
// oak_assim (Assim, :2977-3574, with ASSIM_SCALING = 1): the observations of time index ntime
// (ObsNNN.*: layout from ObsNNN.mask, values, coordinates, rmse or SMWCovar.SqrtDiag with
// SMWCovar.ErrorSpace, optional shift), the observation operator generated on the model grids
// (genObservationOper, :2471-2656; the finest-resolution grid that holds the observation,
// Model.hres), observations outside every grid excluded (loadObservationOper, :2395-2398);
// then on the GPU: H Ef, mean and anomalies, the global analysis (schemetype 0) or the local
// analysis in zone order (schemetype 1), inflation, the maxCorrection clip and
// Ea = xa + sqrt(N - 1) Sa. runtype 0 and 1 return Ea = Ef (no analysis).
//
// Files are NetCDF classic-format variables ("file.nc#var") or GHER binary files (oak_io.cpp).
// Not done here: diagnostics files (Diag*), biastype / anamorphosis / other schemetypes
// (refused with OAKG_ERR_NOTIMPL), curvilinear model grids (OAKG_ERR_NOTIMPL), operators read
// from files (OAKG_ERR_NOTIMPL).
// The reference stops the process on an error; these functions record it for
// oakg_last_status() / oakg_last_error() and leave Ea unchanged.
#include <math.h>
#include <stdio.h>

#include <algorithm>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "oak_io.h"
#include "oakg_internal.cuh"

namespace oakg {
int record_failure(int code, const char* msg);
int context_init_impl();
int release_impl();
void set_ok();
std::mutex& api_mutex();
int& last_status();

namespace {

struct Fail {
  int code;
  std::string msg;
};

// the reference's MemLayout with removeLandPoints = .true. (:55, :129)
struct Layout {
  std::vector<std::string> names;
  std::vector<std::vector<int64_t>> shape;  // per variable, Fortran order, ndim entries
  std::vector<int64_t> start, size, start_sea, size_sea;
  std::vector<uint8_t> sea;  // per point of all variables: 1 = in the state
  int64_t total = 0, total_sea = 0;
  int nvar() const { return (int)names.size(); }
};

struct ModelGrid {
  std::vector<std::vector<double>> axes;  // one per dimension
  std::vector<int64_t> sea;               // grid point -> state row (packed, all variables)
};

struct State {
  io::InitFile cfg;
  int runtype = 2, schemetype = 0, metrictype = 1, loctype = 1;
  Layout model;
  std::vector<ModelGrid> grid;
  std::vector<double> hres;
  std::vector<int64_t> invindex;  // state row -> (variable's grid point) linear index
  std::vector<int32_t> row_var;   // state row -> variable
  // schemetype 1
  int32_t nzones = 0;
  std::vector<int32_t> zone_size, zone_index, inv_index;
  std::vector<double> zone_xyzt, corr, maxl;
  std::vector<double> max_correction;  // per state row; empty = none
  double inflation = 1.0;
};

std::mutex g_drv_mutex;
std::unique_ptr<State> g_state;

void check(int rc) {
  if (rc != OAKG_OK) {
    char buf[512];
    oakg_last_error(buf, sizeof buf);
    throw Fail{rc, buf};
  }
}

void need(bool ok, const std::string& err, int code = OAKG_ERR_INIT) {
  if (!ok) throw Fail{code, err};
}

std::string prefix_of(const std::string& key) {
  const size_t p = key.rfind('.');
  return p == std::string::npos ? std::string() : key.substr(0, p + 1);
}

io::Array read(const State& s, const std::string& path, const std::string& spec) {
  io::Array a;
  std::string err;
  need(io::read_array(path, spec, a, err), err);
  return a;
}

std::vector<double> replicate(const io::Array& a, const std::vector<int64_t>& t,
                              const std::string& what) {
  std::vector<double> out;
  std::string err;
  need(io::replicate(a, t, out, err), what + ": " + err);
  return out;
}

// MemoryLayout_byinitval (:1753-1775)
Layout load_layout(const State& s, const std::string& prefix) {
  std::string err;
  Layout L;
  std::vector<std::string> masks;
  need(s.cfg.strs(prefix + "mask", masks, err), err);
  need(s.cfg.strs(prefix + "variables", L.names, err), err);
  need(L.names.size() == masks.size(),
       prefix + "variables and " + prefix + "mask have different lengths");
  const std::string path = s.cfg.str_or(prefix + "path", "");
  for (size_t v = 0; v < masks.size(); v++) {
    io::Array a = read(s, path, masks[v]);
    std::vector<int64_t> sh = a.shape;
    if (sh.size() == 4 && sh[3] == 1) sh.resize(3);
    else if (sh.size() == 3 && sh[2] == 1) sh.resize(2);
    need(sh.size() <= 4, masks[v] + ": more than 4 dimensions", OAKG_ERR_NOTIMPL);
    L.shape.push_back(sh);
    L.start.push_back(L.total);
    L.size.push_back((int64_t)a.v.size());
    L.start_sea.push_back(L.total_sea);
    int64_t ns = 0;
    for (double x : a.v) {
      const uint8_t in = x != a.valex;
      L.sea.push_back(in);
      ns += in;
    }
    L.size_sea.push_back(ns);
    L.total += (int64_t)a.v.size();
    L.total_sea += ns;
  }
  return L;
}

// loadVector_byinitval (:916-958): the variables' files (or KEY.const per variable), packed
std::vector<double> load_vector(const State& s, const std::string& key, const Layout& L) {
  std::string err;
  std::vector<double> out((size_t)L.total_sea, 0.0);
  if (s.cfg.has(key)) {
    std::vector<std::string> files;
    need(s.cfg.strs(key, files, err), err);
    need((int)files.size() == L.nvar(),
         key + ": expected " + std::to_string(L.nvar()) + " file names");
    const std::string path = s.cfg.str_or(prefix_of(key) + "path", "");
    for (int v = 0; v < L.nvar(); v++) {
      std::vector<double> x = replicate(read(s, path, files[v]), L.shape[v], files[v]);
      int64_t q = L.start_sea[v];
      for (int64_t e = 0; e < L.size[v]; e++)
        if (L.sea[L.start[v] + e]) out[q++] = x[e];
    }
  } else {
    std::vector<double> c;
    need(s.cfg.nums(key + ".const", c, err), key + " (or " + key + ".const) is missing");
    need((int)c.size() == L.nvar(), key + ".const: expected " + std::to_string(L.nvar()) +
                                        " values");
    for (int v = 0; v < L.nvar(); v++)
      std::fill(out.begin() + L.start_sea[v], out.begin() + L.start_sea[v] + L.size_sea[v], c[v]);
  }
  return out;
}

std::string fortran_format(const std::string& fmt, int k) {
  std::string out, err;
  need(io::fortran_format(fmt, k, out, err), err, OAKG_ERR_NOTIMPL);
  return out;
}

// loadVectorSpace (:1166-1265): dimension columns, ensemble members (type 2) turned into
// scaled anomalies
std::vector<double> load_space(const State& s, const std::string& key, const Layout& L,
                               int* dim_out) {
  std::string err;
  const std::string pre = prefix_of(key);
  double dimd;
  need(s.cfg.num(pre + "dimension", dimd, err), err);
  const int dim = (int)dimd;
  need(dim >= 1, pre + "dimension must be positive");
  std::vector<std::string> fmts;
  need(s.cfg.strs(key, fmts, err), err);
  need((int)fmts.size() == L.nvar(), key + ": one format per variable");
  const std::string path = s.cfg.str_or(pre + "path", "");
  const double scale = s.cfg.num_or(pre + "scale", 1.0);
  const int type = (int)s.cfg.num_or(pre + "type", 1.0);
  need(!s.cfg.has(pre + "spaceScale"), pre + "spaceScale is not supported", OAKG_ERR_NOTIMPL);
  const int64_t n = L.total_sea;
  std::vector<double> S((size_t)(n * dim));
  for (int k = 1; k <= dim; k++)
    for (int v = 0; v < L.nvar(); v++) {
      const std::string file = fortran_format(fmts[v], k);
      std::vector<double> x = replicate(read(s, path, file), L.shape[v], file);
      int64_t q = L.start_sea[v];
      for (int64_t e = 0; e < L.size[v]; e++)
        if (L.sea[L.start[v] + e]) S[(size_t)(k - 1) * n + q++] = x[e];
    }
  if (type == 2) {
    for (int64_t i = 0; i < n; i++) {
      double mu = 0.0;
      for (int k = 0; k < dim; k++) mu += S[(size_t)k * n + i];
      mu /= dim;
      for (int k = 0; k < dim; k++)
        S[(size_t)k * n + i] = (S[(size_t)k * n + i] - mu) / sqrt((double)dim - 1.0);
    }
  }
  if (scale != 1.0)
    for (double& x : S) x *= scale;
  *dim_out = dim;
  return S;
}

// grid point (Fortran linear index of variable v) -> coordinate along dimension k
double coord(const State& s, int v, int64_t lin, int k) {
  const std::vector<int64_t>& sh = s.model.shape[v];
  int64_t r = lin;
  for (int q = 0; q < k; q++) r /= sh[q];
  return s.grid[v].axes[k][r % sh[k]];
}

void init_state(State& s, const char* fname) {
  std::string err;
  need(fname != nullptr, "oak_init: file name is NULL");
  need(s.cfg.load(fname, err), err);
  s.runtype = (int)s.cfg.num_or("runtype", 2.0);
  s.metrictype = (int)s.cfg.num_or("metrictype", 1.0);
  if (s.runtype == 0) return;  // FreeRun: nothing else is read (:284)
  s.schemetype = (int)s.cfg.num_or("schemetype", 0.0);
  s.loctype = (int)s.cfg.num_or("loctype", 1.0);
  need(s.schemetype == 0 || s.schemetype == 1,
       "schemetype " + std::to_string(s.schemetype) + " is not supported (0 global, 1 local)",
       OAKG_ERR_NOTIMPL);
  need((int)s.cfg.num_or("biastype", 0.0) == 0, "biastype != 0 is not supported by oak_assim",
       OAKG_ERR_NOTIMPL);
  need((int)s.cfg.num_or("anamorphosistype", 0.0) == 0, "anamorphosis is not supported",
       OAKG_ERR_NOTIMPL);
  need(s.metrictype >= 0 && s.metrictype <= 2, "metrictype must be 0, 1 or 2");
  need(s.loctype >= 1 && s.loctype <= 3, "loctype must be 1, 2 or 3");
  s.model = load_layout(s, "Model.");
  const Layout& L = s.model;
  const std::string path = s.cfg.str_or("Model.path", "");
  static const char* gkeys[4] = {"Model.gridX", "Model.gridY", "Model.gridZ", "Model.gridT"};
  std::vector<std::vector<std::string>> gfiles(4);
  s.grid.resize(L.nvar());
  s.invindex.assign((size_t)L.total_sea, 0);
  s.row_var.assign((size_t)L.total_sea, 0);
  for (int v = 0; v < L.nvar(); v++) {
    const std::vector<int64_t>& sh = L.shape[v];
    const int nd = (int)sh.size();
    ModelGrid& g = s.grid[v];
    for (int k = 0; k < nd; k++) {
      if (gfiles[k].empty()) need(s.cfg.strs(gkeys[k], gfiles[k], err), err);
      need((int)gfiles[k].size() == L.nvar(), std::string(gkeys[k]) + ": one file per variable");
      std::vector<double> full = replicate(read(s, path, gfiles[k][v]), sh, gfiles[k][v]);
      int64_t stride = 1;
      for (int q = 0; q < k; q++) stride *= sh[q];
      std::vector<double> ax((size_t)sh[k]);
      for (int64_t i = 0; i < sh[k]; i++) ax[i] = full[(size_t)(i * stride)];
      for (int64_t e = 0; e < (int64_t)full.size(); e++)
        need(full[e] == ax[(e / stride) % sh[k]],
             gfiles[k][v] + ": the model grid is not rectilinear (curvilinear grids are not "
                            "supported by this library's operator generation)",
             OAKG_ERR_NOTIMPL);
      g.axes.push_back(ax);
    }
    g.sea.assign((size_t)L.size[v], -1);
    int64_t q = L.start_sea[v];
    for (int64_t e = 0; e < L.size[v]; e++)
      if (L.sea[L.start[v] + e]) {
        g.sea[e] = q;
        s.invindex[q] = e;
        s.row_var[q] = v;
        q++;
      }
  }
  s.hres.assign(L.nvar(), 0.0);
  if (s.cfg.has("Model.hres")) {
    need(s.cfg.nums("Model.hres", s.hres, err), err);
    need((int)s.hres.size() == L.nvar(), "Model.hres: one value per variable");
  }
  const int64_t n = L.total_sea;
  if (s.cfg.has("Model.maxCorrection")) {
    std::vector<double> mc;
    need(s.cfg.nums("Model.maxCorrection", mc, err), err);
    need((int)mc.size() == L.nvar(), "Model.maxCorrection: one value per variable");
    s.max_correction.assign((size_t)n, 0.0);
    for (int64_t r = 0; r < n; r++) s.max_correction[r] = mc[s.row_var[r]];
  }
  s.inflation = s.cfg.num_or("inflation.mult", 1.0);
  if (s.schemetype == 1) {
    // zones (:400-451): partition labels rounded, renumbered 1..Z, laid out on the GPU
    std::vector<double> pf = load_vector(s, "Zones.partition", L);
    std::vector<int32_t> lab((size_t)n), part((size_t)n);
    for (int64_t r = 0; r < n; r++) lab[r] = (int32_t)(pf[r] + 0.5);
    check(oakg_partition_compact(n, lab.data(), OAKG_MEM_HOST, part.data(), &s.nzones));
    s.zone_size.resize(s.nzones);
    s.zone_index.resize((size_t)n);
    s.inv_index.resize((size_t)n);
    check(oakg_zone_layout(n, part.data(), s.nzones, OAKG_MEM_HOST, s.zone_size.data(),
                           s.zone_index.data(), s.inv_index.data()));
    std::vector<double> corr = load_vector(s, "Zones.corrLength", L);
    std::vector<double> maxl = load_vector(s, "Zones.maxLength", L);
    s.corr.resize(s.nzones);
    s.maxl.resize(s.nzones);
    s.zone_xyzt.assign((size_t)4 * s.nzones, 0.0);
    int64_t pos = 0;
    for (int32_t z = 0; z < s.nzones; z++) {
      const int64_t r = s.zone_index[pos];  // the zone's first element
      pos += s.zone_size[z];
      s.corr[z] = corr[r];
      s.maxl[z] = maxl[r];
      const int v = s.row_var[r];
      for (int k = 0; k < (int)L.shape[v].size(); k++)
        s.zone_xyzt[(size_t)4 * z + k] = coord(s, v, s.invindex[r], k);
    }
  }
}

// the analysis of time index ntime (Assim, :2977-3574)
void assim_state(const State& s, int ntime, int n, int r, const double* Ef, double* Ea) {
  std::string err;
  need(Ef != nullptr && Ea != nullptr, "oak_assim: Ef and Ea are required", OAKG_ERR_ARGS);
  need(n >= 1 && r >= 1, "oak_assim: n and r must be positive", OAKG_ERR_ARGS);
  if (s.runtype != 2) {
    // FreeRun (0) and compare-only (1): the ensemble is returned unchanged
    if (Ea != Ef) std::copy(Ef, Ef + (size_t)n * r, Ea);
    return;
  }
  need(n == s.model.total_sea, "oak_assim: n = " + std::to_string(n) +
                                   " but the model's state vector has " +
                                   std::to_string(s.model.total_sea) + " elements",
       OAKG_ERR_ARGS);
  need(r >= 2 && r <= 128, "oak_assim: the ensemble size must be in [2, 128]", OAKG_ERR_ARGS);
  char pre[64];
  if (ntime < 999) snprintf(pre, sizeof pre, "Obs%03d.", ntime);
  else snprintf(pre, sizeof pre, "Obs%d.", ntime);
  const std::string P(pre);
  for (const char* k : {"operator", "HperObs", "shiftMod", "filterMod"})
    need(!s.cfg.has(P + k), P + k + ": operators read from files are not supported (the "
                                      "operator is generated on the model grids)",
         OAKG_ERR_NOTIMPL);
  const Layout O = load_layout(s, P);
  const int64_t m0 = O.total_sea;
  std::vector<double> yo = load_vector(s, P + "value", O);
  std::vector<double> rv, B;
  int kB = 0;
  if (s.cfg.has(P + "rmse") || s.cfg.has(P + "rmse.const")) {
    rv = load_vector(s, P + "rmse", O);
    for (double& x : rv) {
      need(x > 0, P + "rmse: zero or negative value (:2101-2106)");
      x = x * x;
    }
  } else if (s.cfg.has(P + "SMWCovar.SqrtDiag")) {
    B = load_space(s, P + "SMWCovar.ErrorSpace", O, &kB);
    rv = load_vector(s, P + "SMWCovar.SqrtDiag", O);
    for (double& x : rv) x = x * x;
  } else {
    throw Fail{OAKG_ERR_INIT, "cannot determine the observation error covariance: expected " +
                                  P + "rmse or " + P + "SMWCovar.SqrtDiag"};
  }
  std::vector<std::vector<double>> opos(4);
  static const char* ck[4] = {"gridX", "gridY", "gridZ", "gridT"};
  for (int k = 0; k < 4; k++)
    if (k < 2 || s.cfg.has(P + ck[k]) || s.cfg.has(P + ck[k] + ".const"))
      opos[k] = load_vector(s, P + ck[k], O);
  std::vector<double> shift;
  if (s.cfg.has(P + "shift") || s.cfg.has(P + "shift.const")) shift = load_vector(s, P + "shift", O);

  // observation operator on the model grids (genObservationOper): per observation variable,
  // each model variable of the same name in turn while its hres is not above the best so far
  const int K = 16;
  std::vector<int64_t> Hi((size_t)m0 * K, -1);
  std::vector<double> Hw((size_t)m0 * K, 0.0);
  std::vector<uint8_t> valid((size_t)m0, 0);
  for (int ov = 0; ov < O.nvar(); ov++) {
    const int64_t o0 = O.start_sea[ov], mo = O.size_sea[ov];
    if (mo == 0) continue;
    std::vector<double> minres((size_t)mo, INFINITY);
    for (int v = 0; v < s.model.nvar(); v++) {
      if (s.model.names[v] != O.names[ov]) continue;
      const int nd = (int)s.model.shape[v].size(), Kv = 1 << nd;
      std::vector<int32_t> shape(s.model.shape[v].begin(), s.model.shape[v].end());
      std::vector<double> coords, pos((size_t)nd * mo);
      for (int k = 0; k < nd; k++) {
        coords.insert(coords.end(), s.grid[v].axes[k].begin(), s.grid[v].axes[k].end());
        need(!opos[k].empty(), P + ck[k] + " is needed for the " + std::to_string(nd) +
                                   "-dimensional variable " + s.model.names[v]);
        std::copy(opos[k].begin() + o0, opos[k].begin() + o0 + mo, pos.begin() + (size_t)k * mo);
      }
      std::vector<int64_t> idx((size_t)mo * Kv);
      std::vector<double> w((size_t)mo * Kv);
      check(oakg_obsoper_rectilinear(nd, shape.data(), coords.data(), s.grid[v].sea.data(), 0,
                                     mo, pos.data(), OAKG_MEM_HOST, idx.data(), w.data()));
      for (int64_t j = 0; j < mo; j++) {
        if (!(minres[j] >= s.hres[v])) continue;
        need(idx[(size_t)j * Kv] != -2,
             "an observation of " + O.names[ov] + " lies in a model grid cell below the 1e-8 "
             "determinant tolerance (the reference's SVD branch is not reproduced)",
             OAKG_ERR_NOTIMPL);
        if (idx[(size_t)j * Kv] < 0) continue;
        minres[j] = s.hres[v];
        valid[o0 + j] = 1;
        for (int c = 0; c < K; c++) {
          Hi[(size_t)(o0 + j) * K + c] = c < Kv ? idx[(size_t)j * Kv + c] : -1;
          Hw[(size_t)(o0 + j) * K + c] = c < Kv ? w[(size_t)j * Kv + c] : 0.0;
        }
      }
    }
  }
  // observations outside every grid are excluded (zero weight in the reference: DCDCovar with
  // D = 0, :3088-3092); they are left out of the arrays here
  std::vector<int64_t> keep;
  for (int64_t j = 0; j < m0; j++)
    if (valid[j]) keep.push_back(j);
  const int64_t m = (int64_t)keep.size();
  int Kused = 1;
  for (int v = 0; v < s.model.nvar(); v++)
    Kused = std::max(Kused, 1 << (int)s.model.shape[v].size());
  std::vector<int64_t> hi((size_t)m * Kused);
  std::vector<double> hw((size_t)m * Kused), y((size_t)m), rr((size_t)m), sh,
      ox((size_t)m), oy((size_t)m), oz, ot, Bk;
  if (!shift.empty()) sh.resize((size_t)m);
  if (!opos[2].empty()) oz.resize((size_t)m);
  if (!opos[3].empty()) ot.resize((size_t)m);
  if (kB > 0) Bk.resize((size_t)m * kB);
  for (int64_t q = 0; q < m; q++) {
    const int64_t j = keep[q];
    for (int c = 0; c < Kused; c++) {
      hi[(size_t)q * Kused + c] = Hi[(size_t)j * K + c];
      hw[(size_t)q * Kused + c] = Hw[(size_t)j * K + c];
    }
    y[q] = yo[j];
    rr[q] = rv[j];
    ox[q] = opos[0][j];
    oy[q] = opos[1][j];
    if (!oz.empty()) oz[q] = opos[2][j];
    if (!ot.empty()) ot[q] = opos[3][j];
    if (!sh.empty()) sh[q] = shift[j];
    for (int c = 0; c < kB; c++) Bk[(size_t)c * m + q] = B[(size_t)c * m0 + j];
  }

  oakg_dims d{};
  d.n = n;
  d.N = r;
  d.m = m;
  d.ldS = n;
  d.ldH = m > 0 ? m : 1;
  d.mem = OAKG_MEM_HOST;
  oakg_obsoper H{};
  H.m = m;
  H.K = Kused;
  H.index = hi.data();
  H.weight = hw.data();
  H.shift = sh.empty() ? nullptr : sh.data();
  const double* mc = s.max_correction.empty() ? nullptr : s.max_correction.data();
  std::vector<double> xf((size_t)n), xa((size_t)n), Sf((size_t)n * r), Sa((size_t)n * r),
      Hxf((size_t)std::max<int64_t>(m, 1)), HSf((size_t)std::max<int64_t>(m, 1) * r);

  if (s.schemetype == 0) {
    check(oakg_ensemble_prologue(&d, Ef, n, &H, xf.data(), Sf.data(), Hxf.data(), HSf.data()));
    if (kB > 0)
      check(oakg_analysis_smw(&d, xf.data(), Hxf.data(), y.data(), Sf.data(), HSf.data(),
                              rr.data(), kB, Bk.data(), m, xa.data(), Sa.data(), nullptr));
    else
      check(oakg_analysis(&d, xf.data(), Hxf.data(), y.data(), Sf.data(), HSf.data(), rr.data(),
                          xa.data(), Sa.data(), nullptr));
    check(oakg_ensemble_epilogue(&d, xf.data(), xa.data(), Sa.data(), s.inflation, mc, Ea, n));
    return;
  }
  // local: the state in zone order (permute(zoneIndex, ...), :766, :4040), the operator's
  // rows mapped to it (:2404-2407), the zone geometry of selectObservations
  std::vector<double> Ez((size_t)n * r), Eaz((size_t)n * r), mcz;
  check(oakg_permute_rows(n, r, s.zone_index.data(), Ef, n, Ez.data(), n, OAKG_MEM_HOST));
  if (m > 0)
    check(oakg_obsoper_to_zone_order(m * Kused, hi.data(), s.inv_index.data(), n, OAKG_MEM_HOST));
  if (mc) {
    mcz.resize((size_t)n);
    check(oakg_permute_rows(n, 1, s.zone_index.data(), mc, n, mcz.data(), n, OAKG_MEM_HOST));
  }
  oakg_loc loc{};
  loc.weight = OAKG_WEIGHT_GAUSS_CUTOFF;
  loc.metric = s.metrictype;
  loc.loctype = s.loctype;
  loc.localise_obs = 1;
  loc.rotate = 1;
  loc.precision = OAKG_PREC_FP64;
  const double* oxp = m > 0 ? ox.data() : nullptr;
  const double* oyp = m > 0 ? oy.data() : nullptr;
  const double* ozp = oz.empty() ? nullptr : oz.data();
  const double* otp = ot.empty() ? nullptr : ot.data();
  if (kB > 0) {
    check(oakg_ensemble_prologue(&d, Ez.data(), n, &H, xf.data(), Sf.data(), Hxf.data(),
                                 HSf.data()));
    check(oakg_locanalysis_smw(&d, &loc, s.nzones, s.zone_size.data(), xf.data(), Hxf.data(),
                               y.data(), Sf.data(), HSf.data(), rr.data(), kB, Bk.data(), m,
                               s.zone_xyzt.data(), oxp, oyp, ozp, otp, s.corr.data(),
                               s.maxl.data(), xa.data(), Sa.data(), nullptr, nullptr));
    check(oakg_ensemble_epilogue(&d, xf.data(), xa.data(), Sa.data(), s.inflation,
                                 mcz.empty() ? nullptr : mcz.data(), Eaz.data(), n));
  } else {
    check(oakg_ens_locanalysis(&d, &loc, s.nzones, s.zone_size.data(), Ez.data(), n, &H,
                               y.data(), rr.data(), s.zone_xyzt.data(), oxp, oyp, ozp, otp,
                               s.corr.data(), s.maxl.data(), s.inflation,
                               mcz.empty() ? nullptr : mcz.data(), Eaz.data()));
  }
  check(oakg_permute_rows(n, r, s.inv_index.data(), Eaz.data(), n, Ea, n, OAKG_MEM_HOST));
}

}  // namespace
}  // namespace oakg

extern "C" {
int oakg_read_variable(const char* spec, double* values, int64_t capacity, int64_t* count,
                       int64_t* shape, int32_t* ndim, double* valex) {
  oakg::io::Array a;
  std::string err;
  int rc = OAKG_OK;
  if (!spec || !count) {
    rc = oakg::record_failure(OAKG_ERR_ARGS, "oakg_read_variable: spec and count are required");
  } else if (!oakg::io::read_array("", spec, a, err)) {
    rc = oakg::record_failure(OAKG_ERR_INIT, err.c_str());
  } else {
    *count = (int64_t)a.v.size();
    if (ndim) *ndim = (int32_t)a.shape.size();
    if (shape)
      for (size_t k = 0; k < a.shape.size() && k < 8; k++) shape[k] = a.shape[k];
    if (valex) *valex = a.valex;
    if (values) {
      if (capacity < (int64_t)a.v.size())
        rc = oakg::record_failure(OAKG_ERR_ARGS, "oakg_read_variable: capacity too small");
      else
        std::copy(a.v.begin(), a.v.end(), values);
    }
  }
  oakg::last_status() = rc;
  return rc;
}

void oak_init(const char* fname) {
  std::lock_guard<std::mutex> lk(oakg::g_drv_mutex);
  std::unique_ptr<oakg::State> st(new oakg::State());
  int rc = OAKG_OK;
  try {
    {
      std::lock_guard<std::mutex> lk2(oakg::api_mutex());
      oakg::set_ok();
      rc = oakg::context_init_impl();
    }
    if (rc == OAKG_OK) oakg::init_state(*st, fname);
  } catch (const oakg::Fail& f) {
    rc = oakg::record_failure(f.code, ("oak_init: " + f.msg).c_str());
  }
  if (rc == OAKG_OK) oakg::g_state = std::move(st);
  oakg::last_status() = rc;
}

void oak_assim(int ntime, int n, int r, double* Ef, double* Ea) {
  std::lock_guard<std::mutex> lk(oakg::g_drv_mutex);
  int rc = OAKG_OK;
  try {
    if (!oakg::g_state) throw oakg::Fail{OAKG_ERR_INIT, "oak_init has not succeeded"};
    oakg::assim_state(*oakg::g_state, ntime, n, r, Ef, Ea);
  } catch (const oakg::Fail& f) {
    rc = oakg::record_failure(f.code, ("oak_assim: " + f.msg).c_str());
  }
  oakg::last_status() = rc;
}

void oak_done(void) {
  std::lock_guard<std::mutex> lk(oakg::g_drv_mutex);
  oakg::g_state.reset();
  std::lock_guard<std::mutex> lk2(oakg::api_mutex());
  oakg::set_ok();
  oakg::last_status() = oakg::release_impl();
}
}
