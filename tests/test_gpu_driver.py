"""oak_init / oak_assim / oak_done, the reference's C interface, driven by init files and
NetCDF classic files written here with SciPy.

1. test/test_assim.F90's own case (3 x 3 grid, two variables, N = 10, one observation at node
   (2, 2), Ef = sin(3 i)): the analysis ensemble's mean and covariance against the Kalman
   formulas, with the diagonal R = 2 and with the SMWCovar R = 2 + RC RC^T (the reference checks
   1e-5; here 1e-10).
2. A local-scheme case (temperature 12 x 9 x 3 and sea level 12 x 9 with land, zones = columns
   with gapped labels, observations of both variables, some outside the grid or next to land,
   maxCorrection, inflation): oak_assim against the oracle's restatement of Assim (layout,
   cinterp operator, initPartition, zone order, ensemble prologue, localised analysis,
   epilogue) at 1e-9.
"""
import numpy as np
import pytest

from oracle import oakref as R

pytestmark = pytest.mark.gpu
netcdf = pytest.importorskip("scipy.io").netcdf_file
FILL = -9999.0


def _write(path, **vars_):
    """vars_: name -> Fortran-ordered array (written with reversed dimensions, as the
    Fortran NetCDF interface stores them), with missing_value = -9999."""
    with netcdf(str(path), "w") as nc:
        for name, a in vars_.items():
            a = np.asarray(a, dtype=np.float64)
            dims = []
            for k, s in enumerate(reversed(a.shape)):
                dn = f"{name}_d{k}"
                nc.createDimension(dn, s)
                dims.append(dn)
            v = nc.createVariable(name, "d", tuple(dims))
            v[:] = a.T
            v.missing_value = FILL


def _init(path, lines):
    path.write_text("\n".join(lines) + "\n")
    return path


def _reference_case(tmp_path, smw):
    imax = jmax = 3
    x, y = np.meshgrid(np.arange(1, imax + 1.0), np.arange(1, jmax + 1.0), indexing="ij")
    d = tmp_path / "data"
    d.mkdir()
    _write(d / "domain.nc", lon=x, lat=y, z=np.zeros_like(x), mask=np.ones_like(x))
    obs = dict(lon=[2.0], lat=[2.0], z=[0.0], var1=[1.0], rmse=[np.sqrt(2.0)])
    _write(d / "obs1.nc", **obs)
    n, Nens, m = imax * jmax * 2, 10, 1
    RC = np.sin(3.0 * np.arange(1, m * 10 + 1)).reshape((m, 10), order="F")
    lines = ["# test/test_assim.F90's case",
             "Model.variables = ['var1', 'var2']",
             "Model.gridX = ['domain.nc#lon', 'domain.nc#lon']",
             "Model.gridY = ['domain.nc#lat', 'domain.nc#lat']",
             "Model.gridZ = ['domain.nc#z', 'domain.nc#z']",
             "Model.mask = ['domain.nc#mask', 'domain.nc#mask']",
             f"Model.path = '{d}/'",
             "runtype = 2", "schemetype = 0",
             f"Obs001.path = '{d}/'",
             "Obs001.variables = ['var1']",
             "Obs001.gridX = ['obs1.nc#lon']", "Obs001.gridY = ['obs1.nc#lat']",
             "Obs001.gridZ = ['obs1.nc#z']", "Obs001.value = ['obs1.nc#var1']",
             "Obs001.mask = ['obs1.nc#var1']"]
    if smw:
        for k in range(10):
            _write(d / f"S{k + 1:03d}-obs.nc", var1=RC[:, k])
        lines += ["Obs001.SMWCovar.SqrtDiag = ['obs1.nc#rmse']",
                  "Obs001.SMWCovar.dimension = 10",
                  "Obs001.SMWCovar.ErrorSpace = ['(\"S\",I3.3,\"-obs.nc#var1\")']",
                  f"Obs001.SMWCovar.path = '{d}/'"]
        Rm = 2.0 * np.eye(m) + RC @ RC.T
    else:
        lines += ["Obs001.rmse = ['obs1.nc#rmse']"]
        Rm = 2.0 * np.eye(m)
    Ef = np.sin(3.0 * np.arange(1, n * Nens + 1)).reshape((n, Nens), order="F")
    H = np.zeros((m, n))
    H[0, 1 + imax * 1] = 1.0
    return _init(tmp_path / "test.init", lines), Ef, H, Rm, np.ones(m)


@pytest.mark.parametrize("smw", [False, True])
def test_reference_test_assim_case(oakg, tmp_path, smw):
    fname, Ef, H, Rm, yo = _reference_case(tmp_path, smw)
    Nens = Ef.shape[1]
    xf = Ef.mean(axis=1)
    Efp = Ef - xf[:, None]
    Pf = Efp @ Efp.T / (Nens - 1)
    K = Pf @ H.T @ np.linalg.inv(H @ Pf @ H.T + Rm)
    Pa = Pf - K @ H @ Pf
    xa = xf + K @ (yo - H @ xf)
    oakg.oak_init(fname)
    Ea = oakg.oak_assim(1, Ef)
    oakg.oak_done()
    xa_g = Ea.mean(axis=1)
    Eap = Ea - xa_g[:, None]
    assert np.abs(xa_g - xa).max() < 1e-10
    assert np.abs(Eap @ Eap.T / (Nens - 1) - Pa).max() < 1e-10


def _local_case(tmp_path, rng):
    nx, ny, nz = 12, 9, 3
    lon = np.linspace(0.0, 11.0 * 0.8, nx)
    lat = np.linspace(40.0, 40.0 + 8 * 0.6, ny)
    dep = np.array([0.0, 10.0, 50.0])
    X3, Y3, Z3 = np.meshgrid(lon, lat, dep, indexing="ij")
    land = np.zeros((nx, ny), dtype=bool)
    land[0:3, 0:2] = True
    land[7, 5] = True
    m3 = np.where(np.repeat(land[:, :, None], nz, axis=2), FILL, 1.0)
    m3[4, 4, 2] = FILL  # a deep point on land only at depth
    m2 = np.where(land, FILL, 1.0)
    col = (np.arange(nx)[:, None] + nx * np.arange(ny)[None, :]) * 10 + 5  # gapped labels
    d = tmp_path / "data"
    d.mkdir()
    _write(d / "model.nc", lon3=X3, lat3=Y3, dep3=Z3, mask3=m3, lon2=X3[:, :, 0],
           lat2=Y3[:, :, 0], mask2=m2, part3=np.repeat(col[:, :, None], nz, axis=2),
           part2=col)
    # observations: temperature at 3-D points, sea level at 2-D points; a few outside the grid
    mt, ms = 70, 40
    ot = np.stack([rng.uniform(-0.5, 9.3, mt), rng.uniform(39.8, 45.0, mt),
                   rng.uniform(0.0, 50.0, mt)])
    os_ = np.stack([rng.uniform(-0.5, 9.3, ms), rng.uniform(39.8, 45.0, ms)])
    vt = rng.normal(size=mt)
    vt[3] = FILL  # a missing observation (masked in the observation layout)
    vs = rng.normal(size=ms)
    _write(d / "obs.nc", tx=ot[0], ty=ot[1], tz=ot[2], tv=vt, tr=rng.uniform(0.3, 1.0, mt),
           sx=os_[0], sy=os_[1], sz=np.zeros(ms), sv=vs, sr=rng.uniform(0.3, 1.0, ms))
    lines = ["Model.variables = ['temp', 'ssh']",
             "Model.mask = ['model.nc#mask3', 'model.nc#mask2']",
             "Model.gridX = ['model.nc#lon3', 'model.nc#lon2']",
             "Model.gridY = ['model.nc#lat3', 'model.nc#lat2']",
             "Model.gridZ = ['model.nc#dep3', 'model.nc#lon2']",
             f"Model.path = '{d}/'",
             "Model.maxCorrection = [0.4, 0.25]",
             "inflation.mult = 1.03",
             "runtype = 2", "schemetype = 1", "metrictype = 0", "loctype = 1",
             f"Zones.path = '{d}/'",
             "Zones.partition = ['model.nc#part3', 'model.nc#part2']",
             "Zones.corrLength.const = [1.5, 1.5]",
             "Zones.maxLength.const = [3.0, 3.0]   ! a comment",
             f"Obs002.path = '{d}/'",
             "Obs002.variables = ['temp', 'ssh']",
             "Obs002.mask = ['obs.nc#tv', 'obs.nc#sv']",
             "Obs002.value = ['obs.nc#tv', 'obs.nc#sv']",
             "Obs002.rmse = ['obs.nc#tr', 'obs.nc#sr']",
             "Obs002.gridX = ['obs.nc#tx', 'obs.nc#sx']",
             "Obs002.gridY = ['obs.nc#ty', 'obs.nc#sy']",
             "Obs002.gridZ = ['obs.nc#tz', 'obs.nc#sz']"]
    geo = dict(lon=lon, lat=lat, dep=dep, m3=m3 != FILL, m2=m2 != FILL, col=col, ot=ot,
               os=os_, vt=vt, vs=vs)
    return _init(tmp_path / "local.init", lines), geo


def _oracle_assim_local(geo, Ef, cfg, d):
    """Assim for schemetype 1 restated with the oracle: sea packing (Fortran order), the
    cinterp operator per observation variable, observations outside the grid dropped, zones
    from the renumbered partition, the state in zone order, prologue, localised analysis with
    the Gaussian weight, epilogue with inflation and the maxCorrection clip."""
    m3 = geo["m3"].reshape(-1, order="F")
    m2 = geo["m2"].reshape(-1, order="F")
    sea3, n3 = R.sea_index(~m3)
    sea2, n2 = R.sea_index(~m2)
    n = n3 + n2
    ax3 = [geo["lon"], geo["lat"], geo["dep"]]
    ax2 = [geo["lon"], geo["lat"]]
    rd = netcdf(str(d / "obs.nc"), "r", mmap=False)
    tr = rd.variables["tr"][:].copy()
    sr = rd.variables["sr"][:].copy()
    rd.close()
    okt = geo["vt"] != FILL
    it, wt = R.obsoper_rectilinear(ax3, [p[okt] for p in geo["ot"]], sea=sea3)
    is_, ws = R.obsoper_rectilinear(ax2, list(geo["os"]), sea=sea2, offset=n3)
    K = 8
    idx = np.full((it.shape[0] + is_.shape[0], K), -1, dtype=np.int64)
    w = np.zeros(idx.shape)
    idx[:it.shape[0]] = it
    w[:it.shape[0]] = wt
    idx[it.shape[0]:, :4] = is_
    w[it.shape[0]:, :4] = ws
    yo = np.concatenate([geo["vt"][okt], geo["vs"]])
    r = np.concatenate([tr[okt], sr]) ** 2
    ox = np.concatenate([geo["ot"][0][okt], geo["os"][0]])
    oy = np.concatenate([geo["ot"][1][okt], geo["os"][1]])
    keep = idx[:, 0] >= 0
    idx, w, yo, r, ox, oy = idx[keep], w[keep], yo[keep], r[keep], ox[keep], oy[keep]
    nzd = len(geo["dep"])
    col3 = np.repeat(geo["col"][:, :, None], nzd, axis=2).reshape(-1, order="F")[m3]
    col2 = geo["col"].reshape(-1, order="F")[m2]
    part, Z = R.partition_compact(np.concatenate([col3, col2]))
    zsize, zidx, inv = R.init_partition(part)
    # coordinates of every state row, then of each zone's first element
    X3, Y3 = np.meshgrid(geo["lon"], geo["lat"], indexing="ij")
    X3 = np.repeat(X3[:, :, None], nzd, axis=2).reshape(-1, order="F")[m3]
    Y3 = np.repeat(Y3[:, :, None], nzd, axis=2).reshape(-1, order="F")[m3]
    X2 = np.meshgrid(geo["lon"], geo["lat"], indexing="ij")[0].reshape(-1, order="F")[m2]
    Y2 = np.meshgrid(geo["lon"], geo["lat"], indexing="ij")[1].reshape(-1, order="F")[m2]
    xs, ys = np.concatenate([X3, X2]), np.concatenate([Y3, Y2])
    first = zidx[np.concatenate([[0], np.cumsum(zsize)[:-1]])]
    zpos = np.zeros((Z, 4))
    zpos[:, 0], zpos[:, 1] = xs[first], ys[first]
    Ez = Ef[zidx]
    idx_z = np.where(idx >= 0, inv[np.maximum(idx, 0)], -1)
    HEf = np.stack([R.sparse_apply(idx_z, w, Ez[:, k]) for k in range(Ez.shape[1])], axis=1)
    xf, Hxf, Sf, HSf = R.ensemble_prologue(Ez, HEf)
    sel = R.geometric_selector(zpos, (ox, oy), np.full(Z, cfg["corr"]), np.full(Z, cfg["maxl"]),
                               R.CARTESIAN, 1, R.GAUSS_CUTOFF)
    xa, Sa, _, _ = R.loc_analysis(zsize, sel, xf, Hxf, yo, Sf, HSf, r)
    mc = np.concatenate([np.full(n3, 0.4), np.full(n2, 0.25)])[zidx]
    Eaz = R.ensemble_epilogue(xf, xa, Sa, cfg["infl"], mc)
    Ea = np.empty_like(Eaz)
    Ea[zidx] = Eaz
    return Ea, n, (keep.sum(), keep.size)


def test_local_scheme_matches_oracle_assim(oakg, tmp_path):
    rng = np.random.default_rng(21)
    fname, geo = _local_case(tmp_path, rng)
    d = tmp_path / "data"
    n = int(geo["m3"].sum() + geo["m2"].sum())
    N = 16
    Ef = rng.normal(size=(n, N)) * 0.7 + 3.0
    Ea_o, n_o, (kept, total) = _oracle_assim_local(geo, Ef, dict(corr=1.5, maxl=3.0,
                                                                 infl=1.03), d)
    assert n_o == n and 0 < kept < total  # some observations fall outside the grid or by land
    oakg.oak_init(fname)
    Ea = oakg.oak_assim(2, Ef)
    oakg.oak_done()
    assert np.abs(Ea - Ea_o).max() < 1e-9 * np.abs(Ea_o).max()
    assert np.abs(Ea - Ef).max() > 1e-3  # the analysis did something


def test_driver_errors(oakg, tmp_path):
    fname, Ef, *_ = _reference_case(tmp_path, False)
    with pytest.raises(oakg.OakError) as ei:
        oakg.oak_init(tmp_path / "missing.init")
    assert ei.value.code == oakg.ERR_INIT
    oakg.oak_init(fname)
    with pytest.raises(oakg.OakError) as ei:
        oakg.oak_assim(1, Ef[:10])  # wrong state size
    assert ei.value.code == oakg.ERR_ARGS
    with pytest.raises(oakg.OakError) as ei:
        oakg.oak_assim(7, Ef)  # no Obs007 entries
    assert ei.value.code == oakg.ERR_INIT and "Obs007" in str(ei.value)
    oakg.oak_done()
    bad = tmp_path / "bad.init"
    bad.write_text(fname.read_text().replace("schemetype = 0", "schemetype = 2"))
    with pytest.raises(oakg.OakError) as ei:
        oakg.oak_init(bad)
    assert ei.value.code == oakg.ERR_NOTIMPL
    op = tmp_path / "op.init"
    op.write_text(fname.read_text() + "Obs001.operator = 'H.nc#H'" + chr(10))
    oakg.oak_init(op)
    with pytest.raises(oakg.OakError) as ei:
        oakg.oak_assim(1, Ef)
    assert ei.value.code == oakg.ERR_NOTIMPL and "operator" in str(ei.value)
    oakg.oak_done()


def test_nested_grids_take_the_finest(oakg, tmp_path):
    """Two model variables of the same name: a coarse grid (Model.hres 1) and a nested fine
    one (hres 0.25). genObservationOper keeps, per observation, the finest grid that holds it
    (assimilation.F90:2557-2590); observations outside both are excluded. Global scheme: the
    analysis ensemble's mean and covariance against the Kalman formulas with that operator."""
    rng = np.random.default_rng(5)
    d = tmp_path / "data"
    d.mkdir()
    cx, cy = np.arange(0.0, 11.0), np.arange(0.0, 9.0)
    fx, fy = np.arange(2.0, 5.01, 0.25), np.arange(2.0, 4.01, 0.25)
    CX, CY = np.meshgrid(cx, cy, indexing="ij")
    FX, FY = np.meshgrid(fx, fy, indexing="ij")
    _write(d / "grids.nc", clon=CX, clat=CY, cmask=np.ones_like(CX), flon=FX, flat=FY,
           fmask=np.ones_like(FX))
    m = 40
    ox = rng.uniform(0.0, 10.0, m)
    oy = rng.uniform(0.0, 8.0, m)
    ox[:12] = rng.uniform(2.0, 5.0, 12)
    oy[:12] = rng.uniform(2.0, 4.0, 12)
    ox[-1] = 11.5  # outside both grids
    yo = rng.normal(size=m)
    rmse = rng.uniform(0.5, 1.0, m)
    _write(d / "obs.nc", x=ox, y=oy, v=yo, r=rmse)
    lines = ["Model.variables = ['temp', 'temp']",
             "Model.mask = ['grids.nc#cmask', 'grids.nc#fmask']",
             "Model.gridX = ['grids.nc#clon', 'grids.nc#flon']",
             "Model.gridY = ['grids.nc#clat', 'grids.nc#flat']",
             "Model.hres = [1.0, 0.25]",
             f"Model.path = '{d}/'", "schemetype = 0",
             f"Obs001.path = '{d}/'", "Obs001.variables = ['temp']",
             "Obs001.mask = ['obs.nc#v']", "Obs001.value = ['obs.nc#v']",
             "Obs001.rmse = ['obs.nc#r']", "Obs001.gridX = ['obs.nc#x']",
             "Obs001.gridY = ['obs.nc#y']"]
    fname = _init(tmp_path / "nested.init", lines)
    nc, nf = CX.size, FX.size
    ic, wc = R.obsoper_rectilinear([cx, cy], [ox, oy])
    i_f, wf = R.obsoper_rectilinear([fx, fy], [ox, oy], offset=nc)
    fine = i_f[:, 0] >= 0
    idx = np.where(fine[:, None], i_f, ic)
    w = np.where(fine[:, None], wf, wc)
    keep = idx[:, 0] >= 0
    assert fine.sum() >= 12 and (~keep).sum() == 1
    n, Nens = nc + nf, 12
    H = np.zeros((keep.sum(), n))
    for q, j in enumerate(np.nonzero(keep)[0]):
        for c in range(4):
            H[q, idx[j, c]] += w[j, c]
    Ef = rng.normal(size=(n, Nens))
    xf = Ef.mean(axis=1)
    Efp = Ef - xf[:, None]
    Pf = Efp @ Efp.T / (Nens - 1)
    Rm = np.diag(rmse[keep] ** 2)
    K = Pf @ H.T @ np.linalg.inv(H @ Pf @ H.T + Rm)
    xa = xf + K @ (yo[keep] - H @ xf)
    Pa = Pf - K @ H @ Pf
    oakg.oak_init(fname)
    Ea = oakg.oak_assim(1, Ef)
    oakg.oak_done()
    Eap = Ea - Ea.mean(axis=1)[:, None]
    assert np.abs(Ea.mean(axis=1) - xa).max() < 1e-10
    assert np.abs(Eap @ Eap.T / (Nens - 1) - Pa).max() < 1e-10
