"""The oak_init / oak_assim driver's data-file reader (oakg_read_variable, host only): NetCDF
classic and 64-bit-offset files written by SciPy's independent NetCDF-3 writer, and GHER
binary files written here record by record, read back as the reference's uload returns them
(ufileformat.F90:555-745): Fortran order and shape, the missing value from missing_value /
_FillValue (else -9999, or the GHER header's), scale_factor / add_offset on the other values,
record variables, and the compact forms."""
import struct
import numpy as np
import pytest

from oak_gb300 import build

netcdf = pytest.importorskip("scipy.io").netcdf_file


@pytest.fixture(scope="module")
def oakg():
    build.build()
    import oak_gb300
    return oak_gb300


@pytest.mark.parametrize("version", [1, 2])
def test_types_fill_and_scaling(oakg, tmp_path, version):
    f = tmp_path / "a.nc"
    rng = np.random.default_rng(version)
    d = rng.normal(size=(4, 5, 3))
    fl = rng.normal(size=(5, 3)).astype(np.float32)
    fl[1, 2] = -1e10
    sh = rng.integers(-300, 300, size=(5, 3)).astype(np.int16)
    sh[0, 0] = -32767
    with netcdf(str(f), "w", version=version) as nc:
        nc.createDimension("z", 4)
        nc.createDimension("y", 5)
        nc.createDimension("x", 3)
        v = nc.createVariable("d", "d", ("z", "y", "x"))
        v[:] = d
        v = nc.createVariable("fl", "f", ("y", "x"))
        v[:] = fl
        v._FillValue = np.float32(-1e10)
        v = nc.createVariable("sh", "h", ("y", "x"))
        v[:] = sh
        v.missing_value = np.int16(-32767)
        v.scale_factor = 0.5
        v.add_offset = 10.0
        v = nc.createVariable("b", "b", ("x",))
        v[:] = np.array([-3, 0, 7], dtype=np.int8)
        v = nc.createVariable("i", "i", ("y",))
        v[:] = np.arange(5, dtype=np.int32) * 1000
    x, valex = oakg.read_variable(f"{f}#d")
    assert x.shape == (3, 5, 4) and valex == -9999.0
    assert np.array_equal(x, d.T)
    x, valex = oakg.read_variable(f"{f}#fl")
    assert valex == np.float32(-1e10) and np.array_equal(x, fl.T.astype(np.float64))
    x, valex = oakg.read_variable(f"{f}#sh")
    exp = np.where(sh == -32767, -32767.0, sh * 0.5 + 10.0)
    assert valex == -32767.0 and np.array_equal(x, exp.T)
    x, _ = oakg.read_variable(f"{f}#b")
    assert list(x) == [-3.0, 0.0, 7.0]
    x, _ = oakg.read_variable(f"{f}#i")
    assert list(x) == [0.0, 1000.0, 2000.0, 3000.0, 4000.0]


def test_record_variables_interleaved(oakg, tmp_path):
    f = tmp_path / "r.nc"
    a = np.arange(3 * 2 * 4, dtype=np.float64).reshape(3, 2, 4)
    b = -np.arange(3 * 5, dtype=np.float32).reshape(3, 5)
    with netcdf(str(f), "w") as nc:
        nc.createDimension("t", None)
        nc.createDimension("y", 2)
        nc.createDimension("x", 4)
        nc.createDimension("w", 5)
        va = nc.createVariable("a", "d", ("t", "y", "x"))
        vb = nc.createVariable("b", "f", ("t", "w"))
        va[:] = a
        vb[:] = b
    x, _ = oakg.read_variable(f"{f}#a")
    assert x.shape == (4, 2, 3) and np.array_equal(x, a.T)
    x, _ = oakg.read_variable(f"{f}#b")
    assert np.array_equal(x, b.T.astype(np.float64))


def test_compact_shape_form(oakg, tmp_path):
    """A variable with a "shape" attribute holds x0 and one increment per dimension, expanded
    with 1-based indices as uexplo does (ufileformat.F90:2300-2337)."""
    f = tmp_path / "c.nc"
    with netcdf(str(f), "w") as nc:
        nc.createDimension("n", 3)
        v = nc.createVariable("lon", "d", ("n",))
        v[:] = np.array([10.0, 0.5, 2.0])
        v.shape = np.array([4, 3], dtype=np.int32)
    x, _ = oakg.read_variable(f"{f}#lon")
    i, j = np.meshgrid(np.arange(4), np.arange(3), indexing="ij")
    assert x.shape == (4, 3) and np.array_equal(x, 10.0 + 0.5 * (i + 1) + 2.0 * (j + 1))


def test_errors(oakg, tmp_path):
    f = tmp_path / "e.nc"
    with netcdf(str(f), "w") as nc:
        nc.createDimension("n", 2)
        nc.createVariable("v", "d", ("n",))[:] = [1.0, 2.0]
    with pytest.raises(oakg.OakError, match="no variable"):
        oakg.read_variable(f"{f}#w")
    (tmp_path / "t.nc").write_text("not a netcdf file")
    with pytest.raises(oakg.OakError, match="classic"):
        oakg.read_variable(f"{tmp_path / 't.nc'}#v")
    with pytest.raises(oakg.OakError, match="cannot open"):
        oakg.read_variable(f"{tmp_path / 'missing.nc'}#v")


def _gher(path, data, valex=-99.0, prec=4, nbmots=7, big=False, degen=None):
    """A GHER file as the reference's writer lays it out: 10 empty records, the header record
    (imax, jmax, kmax, iprec, nbmots, valex), then records of nbmots values (4-byte record
    markers, one byte order)."""
    e = ">" if big else "<"
    fl = "f" if prec == 4 else "d"

    def rec(payload):
        return struct.pack(e + "i", len(payload)) + payload + struct.pack(e + "i", len(payload))

    if degen is not None:
        shape, coeffs = degen
        ext = [-s for s in shape] + [1] * (3 - len(shape))
        vals = list(coeffs)
    else:
        a = np.asarray(data, dtype=np.float64)
        ext = list(a.shape) + [1] * (3 - a.ndim)
        vals = list(a.reshape(-1, order="F"))
    out = b"".join(rec(b"") for _ in range(10))
    out += rec(struct.pack(e + "5if", ext[0], ext[1], ext[2], prec, nbmots, valex))
    for q in range(0, len(vals), nbmots):
        chunk = vals[q:q + nbmots]
        out += rec(struct.pack(e + fl * len(chunk), *chunk))
    path.write_bytes(out)


@pytest.mark.parametrize("big", [False, True])
@pytest.mark.parametrize("prec", [4, 8])
def test_gher_files(oakg, tmp_path, big, prec):
    rng = np.random.default_rng(prec + big)
    a = rng.normal(size=(5, 4, 3)).astype(np.float32 if prec == 4 else np.float64)
    a[1, 2, 0] = -99.0
    f = tmp_path / "field.TEM"
    _gher(f, a, prec=prec, big=big)
    x, valex = oakg.read_variable(str(f))
    assert valex == -99.0 and x.shape == (5, 4, 3)
    assert np.array_equal(x, a.astype(np.float64))
    # a 2-D field (kmax = 1) and a 1-D one (jmax = kmax = 1)
    _gher(f, a[:, :, 0], prec=prec, big=big)
    x, _ = oakg.read_variable(str(f))
    assert x.shape == (5, 4) and np.array_equal(x, a[:, :, 0].astype(np.float64))
    _gher(f, a[:, 0, 0], prec=prec, big=big, nbmots=5)
    x, _ = oakg.read_variable(str(f))
    assert x.shape == (5,) and np.array_equal(x, a[:, 0, 0].astype(np.float64))


def test_gher_compact_form(oakg, tmp_path):
    """Negative extents: c0, dci, dcj, dck expanded with 1-based indices (uexplo)."""
    f = tmp_path / "lon.TEM"
    _gher(f, None, prec=8, degen=((6, 4), (-10.0, 0.25, 1.5, 0.0)))
    x, _ = oakg.read_variable(str(f))
    i, j = np.meshgrid(np.arange(1, 7), np.arange(1, 5), indexing="ij")
    assert x.shape == (6, 4) and np.array_equal(x, -10.0 + 0.25 * i + 1.5 * j)


def test_gher_damaged(oakg, tmp_path):
    f = tmp_path / "bad.TEM"
    _gher(f, np.arange(12.0).reshape(3, 4))
    f.write_bytes(f.read_bytes()[:-6])
    with pytest.raises(oakg.OakError, match="GHER"):
        oakg.read_variable(str(f))

