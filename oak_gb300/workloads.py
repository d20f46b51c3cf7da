"""Seeded synthetic workloads with the shapes and value distributions of the benchmark
configurations (the reference publishes no dataset for this path; these stand in for it).

* ``global_case``  -- one 2-D field 100 x 80, N = 30 members, m = 500 observations at distinct
  uniform cells, y = x_true + N(0, 0.1^2), R = 0.01 I (global analysis, rrsqrt.F90:196-208).
* ``batched_case`` -- 5-variable state (temp, salt, u, v on 30 levels and the 2-D ssh) on a
  720 x 360 grid, zone = one column of 4 * 30 + 1 = 121 elements, N = 100 members with
  per-variable sd (temp 1.0, salt 0.2, ssh 0.05, u 0.1, v 0.1), m = 200,000 observations
  (ssh 50 %, temp 30 %, salt 20 %) through bilinear interpolation (4 columns, nearest level),
  70 % of them on 8 track segments so that zones near them select up to ~3,000, noise sd 0.1
  of the variable's sd, Gaspari-Cohn support radius 12 cells.
* ``large_case``   -- 2 variables (temp, salt) on 1440 x 720 x 50 (zone = 100 elements),
  N = 128, m = 1,000,000 clustered bilinear point observations with error sd ~ U(0.05, 0.5),
  Gaspari-Cohn support radius 10 cells.
* ``local_case``   -- 3-D grid 360 x 180 x 20, one variable, N = 64 members (Gaussian
  random fields, horizontal length 8 cells, vertical 3 levels), m = 50,000 observations
  (70 % on 40 great-circle-like tracks, 30 % uniform, noise sd 0.1), zones = the 64,800
  vertical columns, Gaspari-Cohn localisation with support radius 12 cells
  (locfun(d/6), maxLength = 12), Cartesian cell-index coordinates (metrictype = 0).
  ``scale`` shrinks the horizontal grid and observation count for tests.

Random fields: white N(0,1) noise convolved (FFT, periodic) with g(r) = exp(-(r/l)^2)
per axis, renormalised to sample standard deviation 1. Seeds are 1000*config + role
(0 truth, 1..N members, 900 positions, 901 noise, 902 tracks).

State layout: zones are vertical columns, so the state vector is ordered column by column
(the partition-sorted order the reference builds with initPartition/zoneIndex,
assimilation.F90:578-641): element (i, j, k) sits at ((j*nx + i) * nz + k).
"""
from __future__ import annotations

import dataclasses

import numpy as np


@dataclasses.dataclass
class Case:
    name: str
    xf: np.ndarray          # (n,)
    Hxf: np.ndarray         # (m,)
    yo: np.ndarray          # (m,)
    Sf: np.ndarray          # (n, N) Fortran order
    HSf: np.ndarray         # (m, N) Fortran order
    r_diag: np.ndarray      # (m,)
    x_true: np.ndarray      # (n,)
    zone_size: np.ndarray | None = None   # (Z,) int32
    zone_pos: np.ndarray | None = None    # (Z, 4)
    obs_pos: tuple | None = None          # (x, y, z, t)
    corr_len: np.ndarray | None = None    # (Z,)
    max_len: np.ndarray | None = None     # (Z,)
    weight: int = 1                       # Gaspari-Cohn
    metric: int = 0
    loctype: int = 1
    obs_index: np.ndarray | None = None   # (m,) state index observed (nearest cell H)
    H_index: np.ndarray | None = None     # (m, K) state indices of an interpolating H
    H_weight: np.ndarray | None = None    # (m, K) their weights
    Ef: np.ndarray | None = None          # (n, N) ensemble, when kept
    HEf: np.ndarray | None = None

    @property
    def n(self):
        return self.xf.size

    @property
    def N(self):
        return self.Sf.shape[1]

    @property
    def m(self):
        return self.yo.size

    @property
    def Z(self):
        return 0 if self.zone_size is None else self.zone_size.size


def gaussian_field(shape, lengths, rng, dtype=np.float64):
    """White noise convolved with exp(-(r/l)^2) per axis (periodic FFT), sd renormalised to 1."""
    noise = rng.standard_normal(shape)
    F = np.fft.rfftn(noise)
    for ax, (nax, l) in enumerate(zip(shape, lengths)):
        if l <= 0:
            continue
        if ax == len(shape) - 1:
            k = np.fft.rfftfreq(nax)
        else:
            k = np.fft.fftfreq(nax)
        # Fourier transform of exp(-(x/l)^2) (up to a constant): exp(-(pi l k)^2)
        tf = np.exp(-((np.pi * l * k) ** 2))
        sh = [1] * len(shape)
        sh[ax] = tf.size
        F = F * tf.reshape(sh)
    f = np.fft.irfftn(F, s=shape, axes=tuple(range(len(shape))))
    f = f / f.std()
    return f.astype(dtype, copy=False)


def _anomalies(Ef, HEf):
    N = Ef.shape[1]
    xf = Ef.mean(axis=1)
    Hxf = HEf.mean(axis=1)
    s = np.sqrt(N - 1.0)
    Sf = np.asfortranarray((Ef - xf[:, None]) / s)
    HSf = np.asfortranarray((HEf - Hxf[:, None]) / s)
    return xf, Hxf, Sf, HSf


def global_case(keep_ensemble=False) -> Case:
    """Config: global analysis, 100 x 80 field, N = 30, m = 500, R = 0.01 I."""
    cfg = 0
    nx, ny, N, m, ell = 100, 80, 30, 500, 10.0
    truth = gaussian_field((ny, nx), (ell, ell), np.random.default_rng(1000 * cfg + 0)).reshape(-1)
    Ef = np.empty((nx * ny, N), order="F")
    for k in range(N):
        Ef[:, k] = gaussian_field((ny, nx), (ell, ell),
                                  np.random.default_rng(1000 * cfg + 1 + k)).reshape(-1)
    idx = np.random.default_rng(1000 * cfg + 900).choice(nx * ny, size=m, replace=False)
    noise = np.random.default_rng(1000 * cfg + 901).standard_normal(m) * 0.1
    yo = truth[idx] + noise
    HEf = Ef[idx, :]
    xf, Hxf, Sf, HSf = _anomalies(Ef, HEf)
    c = Case("global 100x80 N=30 m=500", xf, Hxf, yo, Sf, HSf, np.full(m, 0.01), truth,
             obs_index=idx)
    if keep_ensemble:
        c.Ef, c.HEf = Ef, HEf
    return c


def _track_obs(nx, ny, m_track, ntracks, rng):
    """Observation (i, j) cells on great-circle-like tracks
    j = ny/2 + (ny/2) atan(tan(a) sin(2 pi (i - i0)/nx)) / (pi/2)."""
    per = np.full(ntracks, m_track // ntracks)
    per[: m_track - per.sum()] += 1
    ii, jj = [], []
    for t in range(ntracks):
        a = np.deg2rad(rng.uniform(10.0, 80.0))
        i0 = rng.uniform(0.0, nx)
        i = rng.uniform(0.0, nx, per[t])
        j = ny / 2 + (ny / 2) * np.arctan(np.tan(a) * np.sin(2 * np.pi * (i - i0) / nx)) / (np.pi / 2)
        ii.append(np.clip(np.rint(i), 0, nx - 1).astype(np.int64))
        jj.append(np.clip(np.rint(j), 0, ny - 1).astype(np.int64))
    return np.concatenate(ii), np.concatenate(jj)


def local_case(scale=1.0, N=64, nz=20, m=50_000, radius=12.0, seed_cfg=1, track_frac=0.7,
               ntracks=40, dtype=np.float64, keep_ensemble=False) -> Case:
    """Config: local analysis 360 x 180 x 20, N = 64, m = 50,000, GC radius 12 cells.

    ``scale`` < 1 shrinks nx, ny by ``scale`` and m by ``scale**2`` (observation density kept).
    """
    nx = max(4, int(round(360 * scale)))
    ny = max(4, int(round(180 * scale)))
    if scale != 1.0:
        m = max(1, int(round(m * scale * scale)))
    cfg = seed_cfg
    shape = (ny, nx, nz)
    lengths = (8.0, 8.0, 3.0)
    n = nx * ny * nz
    truth = gaussian_field(shape, lengths, np.random.default_rng(1000 * cfg + 0)).reshape(-1)
    Ef = np.empty((n, N), order="F", dtype=np.float64)
    for k in range(N):
        Ef[:, k] = gaussian_field(shape, lengths,
                                  np.random.default_rng(1000 * cfg + 1 + k)).reshape(-1)
    # observations: track part + uniform part, nearest cell, random level
    rng_pos = np.random.default_rng(1000 * cfg + 900)
    m_track = int(round(track_frac * m))
    ti, tj = _track_obs(nx, ny, m_track, ntracks, np.random.default_rng(1000 * cfg + 902))
    ui = rng_pos.integers(0, nx, m - m_track)
    uj = rng_pos.integers(0, ny, m - m_track)
    oi = np.concatenate([ti, ui])
    oj = np.concatenate([tj, uj])
    ok = rng_pos.integers(0, nz, m)
    idx = (oj * nx + oi) * nz + ok   # state index (column-ordered layout)
    noise = np.random.default_rng(1000 * cfg + 901).standard_normal(m) * 0.1
    yo = truth[idx] + noise
    HEf = Ef[idx, :]
    xf, Hxf, Sf, HSf = _anomalies(Ef, HEf)
    Z = nx * ny
    zone_size = np.full(Z, nz, dtype=np.int32)
    zc = np.arange(Z)
    zone_pos = np.zeros((Z, 4))
    zone_pos[:, 0] = zc % nx   # x = i
    zone_pos[:, 1] = zc // nx  # y = j
    obs_pos = (oi.astype(np.float64), oj.astype(np.float64), ok.astype(np.float64),
               np.zeros(m))
    corr = np.full(Z, radius / 2.0)
    maxl = np.full(Z, radius)
    c = Case(f"local {nx}x{ny}x{nz} N={N} m={m} GC radius {radius:g}", xf, Hxf, yo,
             Sf.astype(dtype, copy=False), HSf.astype(dtype, copy=False), np.full(m, 0.01),
             truth, zone_size, zone_pos, obs_pos, corr, maxl, weight=1, metric=0, loctype=1,
             obs_index=idx)
    if keep_ensemble:
        c.Ef, c.HEf = Ef, HEf
    return c


# variables of the batched state: (name, sd); the first four have nz levels, the last (ssh) one
BATCHED_VARS = (("temp", 1.0), ("salt", 0.2), ("u", 0.1), ("v", 0.1), ("ssh", 0.05))
# variables of the large state: two 3-D variables
LARGE_VARS = (("temp", 1.0), ("salt", 0.2))


def _column_obs(nx, ny, nz, n3, zsz, m, cfg, track_frac, ntracks, obs_split, obs_sd):
    """Observations of a column workload (numpy, seeded): positions in cell units, 70 %
    (track_frac) on track segments a quarter of the grid long, the observed variable and
    level, the bilinear operator (4 columns at the level; H_index into the column-ordered
    state, H_weight), each observation's error sd and its noise draw."""
    rng_pos = np.random.default_rng(1000 * cfg + 900)
    m_track = int(round(track_frac * m))
    rng_t = np.random.default_rng(1000 * cfg + 902)
    per = np.full(ntracks, m_track // ntracks)
    per[: m_track - per.sum()] += 1
    xs, ys = [], []
    for t in range(ntracks):
        a = np.deg2rad(rng_t.uniform(10.0, 80.0))
        i0 = rng_t.uniform(0.0, nx)
        s0 = rng_t.uniform(0.0, 0.75 * (nx - 1))
        i = rng_t.uniform(s0, s0 + 0.25 * (nx - 1), per[t])
        j = ny / 2 + (ny / 2) * np.arctan(np.tan(a) * np.sin(2 * np.pi * (i - i0) / nx)) / (np.pi / 2)
        xs.append(i)
        ys.append(np.clip(j, 0.0, ny - 1.0))
    xs.append(rng_pos.uniform(0.0, nx - 1, m - m_track))
    ys.append(rng_pos.uniform(0.0, ny - 1, m - m_track))
    ox, oy = np.concatenate(xs), np.concatenate(ys)
    u = rng_pos.uniform(0.0, 1.0, m)
    var = np.asarray(obs_split[0])[np.searchsorted(np.asarray(obs_split[1]), u, side="right")]
    is2 = var == n3
    lev = np.where(is2, 0, rng_pos.integers(0, nz, m))
    off = np.where(is2, n3 * nz, var * nz + lev)
    ix = np.minimum(np.floor(ox).astype(np.int64), nx - 2)
    iy = np.minimum(np.floor(oy).astype(np.int64), ny - 2)
    fx, fy = ox - ix, oy - iy
    cols = np.stack([iy * nx + ix, iy * nx + ix + 1, (iy + 1) * nx + ix, (iy + 1) * nx + ix + 1], 1)
    H_index = cols * zsz + off[:, None]
    H_weight = np.stack([(1 - fx) * (1 - fy), fx * (1 - fy), (1 - fx) * fy, fx * fy], 1)
    sd_obs = obs_sd(var, np.random.default_rng(1000 * cfg + 903))
    noise = np.random.default_rng(1000 * cfg + 901).standard_normal(m) * sd_obs
    return {"ox": ox, "oy": oy, "lev": lev, "var": var, "H_index": H_index,
            "H_weight": H_weight, "sd_obs": sd_obs, "noise": noise}


def _column_case(name, gx, gy, scale, N, nz, vars3, var2, m, radius, cfg, track_frac, ntracks,
                 obs_split, obs_sd, keep_ensemble):
    """Columns of several variables (zone = one horizontal column), bilinear observations.

    vars3: (name, sd) of the 3-D variables (nz levels each), var2: (name, sd) of a 2-D variable
    or None. Column (i, j) is zone j*nx + i; inside it the 3-D variables' levels 0..nz-1 in
    order, then the 2-D one. obs_split = (variables, bounds): observation l observes
    variables[searchsorted(bounds, u_l)] (u_l uniform, bounds the cumulative fractions but the
    last; variable index into vars3 + var2); obs_sd(var, rng) gives each observation's error
    sd. Observations sit
    at continuous (x, y) in cell units, 70 % (track_frac) on track segments a quarter of the
    grid long; H interpolates the 4 surrounding columns bilinearly at the observation's level.
    ``scale`` shrinks the grid by ``scale``, m by ``scale**2`` and the number of tracks by
    ``scale`` (the density along a track, and with it the largest per-zone counts, stay those
    of the full grid).
    """
    nx = max(4, int(round(gx * scale)))
    ny = max(4, int(round(gy * scale)))
    if scale != 1.0:
        m = max(1, int(round(m * scale * scale)))
        ntracks = max(1, int(round(ntracks * scale)))
    Z = nx * ny
    n3 = len(vars3)
    zsz = n3 * nz + (1 if var2 else 0)
    n = Z * zsz
    lengths3, lengths2 = (8.0, 8.0, 3.0), (8.0, 8.0)

    def draw(seed):
        x = np.empty((Z, zsz))
        rng = np.random.default_rng(seed)
        for v, (_, sd) in enumerate(vars3):
            x[:, v * nz:(v + 1) * nz] = sd * gaussian_field((ny, nx, nz), lengths3, rng).reshape(Z, nz)
        if var2:
            x[:, n3 * nz] = var2[1] * gaussian_field((ny, nx), lengths2, rng).reshape(Z)
        return x.reshape(-1)

    truth = draw(1000 * cfg + 0)
    Ef = np.empty((n, N), order="F")
    for k in range(N):
        Ef[:, k] = draw(1000 * cfg + 1 + k)
    ob = _column_obs(nx, ny, nz, n3, zsz, m, cfg, track_frac, ntracks, obs_split, obs_sd)
    ox, oy, lev, H_index, H_weight = ob["ox"], ob["oy"], ob["lev"], ob["H_index"], ob["H_weight"]
    HEf = np.einsum("mk,mkn->mn", H_weight, Ef[H_index.reshape(-1), :].reshape(m, 4, N))
    sd_obs = ob["sd_obs"]
    yo = np.einsum("mk,mk->m", H_weight, truth[H_index]) + ob["noise"]
    xf, Hxf, Sf, HSf = _anomalies(Ef, HEf)
    zone_size = np.full(Z, zsz, dtype=np.int32)
    zc = np.arange(Z)
    zone_pos = np.zeros((Z, 4))
    zone_pos[:, 0] = zc % nx
    zone_pos[:, 1] = zc // nx
    obs_pos = (ox, oy, lev.astype(np.float64), np.zeros(m))
    c = Case(f"{name} {nx}x{ny}x{nz} N={N} m={m} GC radius {radius:g}", xf, Hxf, yo, Sf, HSf,
             sd_obs ** 2, truth, zone_size, zone_pos, obs_pos, np.full(Z, radius / 2.0),
             np.full(Z, radius), weight=1, metric=0, loctype=1, H_index=H_index,
             H_weight=H_weight)
    if keep_ensemble:
        c.Ef, c.HEf = Ef, HEf
    return c


def batched_case(scale=0.25, N=100, nz=30, m=200_000, radius=12.0, seed_cfg=2,
                 track_frac=0.7, ntracks=8, keep_ensemble=False) -> Case:
    """Config: batched mixed-precision local analysis, 720 x 360 columns of temp, salt, u, v
    (nz levels) and ssh, N = 100, m = 200,000 bilinear observations clustered on 8 track
    segments (ssh 50 %, temp 30 %, salt 20 %; noise sd 0.1 of the variable's sd)."""
    sds = np.array([sd for _, sd in BATCHED_VARS])
    return _column_case("batched 5 variables", 720, 360, scale, N, nz, BATCHED_VARS[:4],
                        BATCHED_VARS[4], m, radius, seed_cfg, track_frac, ntracks,
                        ((4, 0, 1), (0.5, 0.8)), lambda var, rng: 0.1 * sds[var],
                        keep_ensemble)


def large_case(scale=0.125, N=128, nz=50, m=1_000_000, radius=10.0, seed_cfg=4,
               track_frac=0.7, ntracks=16, keep_ensemble=False) -> Case:
    """Config: large mixed-precision analysis, 1440 x 720 columns of 2 variables (temp, salt) on
    nz = 50 levels (100 elements a zone), N = 128, m = 1,000,000 clustered point observations
    (bilinear, half per variable) with error sd drawn uniformly from 0.05-0.5, Gaspari-Cohn
    support radius 10 cells."""
    return _column_case("large 2 variables", 1440, 720, scale, N, nz, LARGE_VARS, None, m,
                        radius, seed_cfg, track_frac, ntracks, ((0, 1), (0.5,)),
                        lambda var, rng: rng.uniform(0.05, 0.5, var.size), keep_ensemble)


# ------------------------------------------------------------------------------------------
# The column workloads at full size, generated on the GPU with FP32 storage: the state of the
# large configuration is 104M values x 128 members (53 GB in FP32), which host-side NumPy FFTs
# cannot generate in reasonable time. Same recipe as _column_case (Gaussian random fields by
# FFT, seeded per member; observations from _column_obs), with torch's CUDA generator seeded
# 1000*config + role and FP32 FFTs.

@dataclasses.dataclass
class DeviceCase:
    """A workload whose state and observation arrays live on the GPU in FP32 (torch tensors):
    xf (n), Sf (n, N) column-major, x_true (n), Hxf, yo, r_diag (m), HSf (m, N) column-major.
    Geometry stays on the host in FP64 (zone_size, zone_pos, obs_pos, corr_len, max_len)."""
    name: str
    xf: object
    Hxf: object
    yo: object
    Sf: object
    HSf: object
    r_diag: object
    x_true: object
    zone_size: np.ndarray
    zone_pos: np.ndarray
    obs_pos: tuple
    corr_len: np.ndarray
    max_len: np.ndarray
    nx: int = 0
    ny: int = 0
    weight: int = 1
    metric: int = 0
    loctype: int = 1

    @property
    def n(self):
        return int(self.xf.shape[0])

    @property
    def N(self):
        return int(self.Sf.shape[1])

    @property
    def m(self):
        return int(self.yo.shape[0])

    @property
    def Z(self):
        return int(self.zone_size.size)


def gaussian_field_torch(shape, lengths, gen, device):
    """gaussian_field on the GPU in FP32: white noise from `gen`, the same spectral filter
    exp(-(pi l k)^2) per axis, sd renormalised to 1."""
    import math

    import torch
    noise = torch.randn(shape, generator=gen, device=device, dtype=torch.float32)
    F = torch.fft.rfftn(noise)
    del noise
    for ax, (nax, l) in enumerate(zip(shape, lengths)):
        if l <= 0:
            continue
        if ax == len(shape) - 1:
            k = torch.fft.rfftfreq(nax, device=device)
        else:
            k = torch.fft.fftfreq(nax, device=device)
        tf = torch.exp(-((math.pi * l * k) ** 2))
        sh = [1] * len(shape)
        sh[ax] = tf.numel()
        F *= tf.reshape(sh)
    f = torch.fft.irfftn(F, s=shape)
    del F
    f /= f.std()
    return f


def _column_case_device(name, gx, gy, scale, N, nz, vars3, var2, m, radius, cfg, track_frac,
                        ntracks, obs_split, obs_sd, device):
    import torch
    nx = max(4, int(round(gx * scale)))
    ny = max(4, int(round(gy * scale)))
    if scale != 1.0:
        m = max(1, int(round(m * scale * scale)))
        ntracks = max(1, int(round(ntracks * scale)))
    Z = nx * ny
    n3 = len(vars3)
    zsz = n3 * nz + (1 if var2 else 0)
    n = Z * zsz
    lengths3, lengths2 = (8.0, 8.0, 3.0), (8.0, 8.0)
    gen = torch.Generator(device=device)

    def draw(seed, out):  # out: (Z, zsz) view of one member (or the truth)
        gen.manual_seed(seed)
        for v, (_, sd) in enumerate(vars3):
            out[:, v * nz:(v + 1) * nz] = sd * gaussian_field_torch(
                (ny, nx, nz), lengths3, gen, device).reshape(Z, nz)
        if var2:
            out[:, n3 * nz] = var2[1] * gaussian_field_torch((ny, nx), lengths2, gen,
                                                             device).reshape(Z)

    f32 = torch.float32
    truth = torch.empty(n, dtype=f32, device=device)
    draw(1000 * cfg + 0, truth.view(Z, zsz))
    E = torch.empty((N, n), dtype=f32, device=device)   # member k = row k; E.t() is (n, N)
    for k in range(N):
        draw(1000 * cfg + 1 + k, E[k].view(Z, zsz))
    # mean and scaled anomalies (ASSIM_SCALING: (Ef - xf)/sqrt(N-1)), in FP64, stored in FP32
    xf = torch.empty(n, dtype=f32, device=device)
    s = float(np.sqrt(N - 1.0))
    step = max(1, (1 << 29) // (8 * N))
    for c0 in range(0, n, step):
        c1 = min(n, c0 + step)
        blk = E[:, c0:c1].double()
        mu = blk.mean(0)
        xf[c0:c1] = mu.float()
        E[:, c0:c1] = ((blk - mu) / s).float()
        del blk, mu
    Sf = E.t()
    ob = _column_obs(nx, ny, nz, n3, zsz, m, cfg, track_frac, ntracks, obs_split, obs_sd)
    idx = torch.as_tensor(ob["H_index"], device=device)
    w = torch.as_tensor(ob["H_weight"], device=device)
    # H is linear: H xf and H Sf are the mean and anomalies of H Ef
    Hxf = (w * xf.double()[idx]).sum(1).float()
    HSt = torch.empty((N, m), dtype=f32, device=device)  # HSt.t() is HSf (m, N) column-major
    mstep = max(1, (1 << 28) // (8 * 4 * N))
    for j0 in range(0, m, mstep):
        j1 = min(m, j0 + mstep)
        rows = E[:, idx[j0:j1].reshape(-1)].double().reshape(N, j1 - j0, 4)
        HSt[:, j0:j1] = (rows * w[j0:j1].unsqueeze(0)).sum(2).float()
        del rows
    yo = ((w * truth.double()[idx]).sum(1)
          + torch.as_tensor(ob["noise"], device=device)).float()
    r = torch.as_tensor(ob["sd_obs"] ** 2, device=device).float()
    zone_size = np.full(Z, zsz, dtype=np.int32)
    zc = np.arange(Z)
    zone_pos = np.zeros((Z, 4))
    zone_pos[:, 0] = zc % nx
    zone_pos[:, 1] = zc // nx
    obs_pos = (ob["ox"], ob["oy"], ob["lev"].astype(np.float64), np.zeros(m))
    return DeviceCase(f"{name} {nx}x{ny}x{nz} N={N} m={m} GC radius {radius:g} (FP32)", xf, Hxf,
                      yo, Sf, HSt.t(), r, truth, zone_size, zone_pos, obs_pos,
                      np.full(Z, radius / 2.0), np.full(Z, radius), nx=nx, ny=ny)


def batched_case_device(scale=1.0, device="cuda", N=100, nz=30, m=200_000, radius=12.0,
                        seed_cfg=2, track_frac=0.7, ntracks=8) -> DeviceCase:
    """batched_case generated on the GPU with FP32 storage (default: the full 720 x 360 grid,
    259,200 zones of 121 elements, N = 100: 12.5 GB per ensemble array)."""
    sds = np.array([sd for _, sd in BATCHED_VARS])
    return _column_case_device("batched 5 variables", 720, 360, scale, N, nz, BATCHED_VARS[:4],
                               BATCHED_VARS[4], m, radius, seed_cfg, track_frac, ntracks,
                               ((4, 0, 1), (0.5, 0.8)), lambda var, rng: 0.1 * sds[var],
                               device)


def large_case_device(scale=1.0, device="cuda", N=128, nz=50, m=1_000_000, radius=10.0,
                      seed_cfg=4, track_frac=0.7, ntracks=16) -> DeviceCase:
    """large_case generated on the GPU with FP32 storage (default: the full 1440 x 720 grid,
    1,036,800 zones of 100 elements, N = 128: 53 GB per ensemble array)."""
    return _column_case_device("large 2 variables", 1440, 720, scale, N, nz, LARGE_VARS, None,
                               m, radius, seed_cfg, track_frac, ntracks, ((0, 1), (0.5,)),
                               lambda var, rng: rng.uniform(0.05, 0.5, var.size), device)


def rrsqrt_test_case():
    """The known-answer case of test/test_rrsqrt.F90:277-322: n = 10, m = 5, N = 12,
    Ef(i) = sin(3 i^2) (column-major fill), H = reshape(1..50, [5, 10]), y = 1..5, R = 2 I."""
    n, m, N = 10, 5, 12
    i = np.arange(1, n * N + 1, dtype=np.float64)
    Ef = np.sin(3.0 * i * i).reshape(N, n).T.copy()
    H = np.arange(1, m * n + 1, dtype=np.float64).reshape(n, m).T.copy()
    y = np.arange(1, m + 1, dtype=np.float64)
    xf = Ef.sum(axis=1) / N
    Sf = (Ef - xf[:, None]) / np.sqrt(N - 1.0)
    return xf, Sf, H, y, np.full(m, 2.0)
