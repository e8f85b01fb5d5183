"""NetCDF classic initial conditions and field dumps (ampe_gb300.fields_io),
with the reference's variable names and checks (FieldsInitializer.cc:77-362,
685-707; FieldsWriter.cc:55-489): round trips, files written by an
independent implementation of the format (scipy.io.netcdf_file) read here
and ours read there, the 2D slice of a 3D file, and the refusal of a file
whose dimensions are not the level's."""
import os

import numpy as np
import pytest

from ampe_gb300 import configs, fields_io as F


def _fields(shape, rng, qlen=4):
    q = rng.standard_normal((qlen,) + shape)
    q /= np.linalg.norm(q, axis=0, keepdims=True)
    return (rng.uniform(0, 1, shape), rng.uniform(0.2, 0.4, shape), q,
            rng.uniform(1400, 1500, shape))


def test_round_trip_3d(tmp_path):
    m = configs.calphad3d(8, seed=3, T_run=1500.0)
    m.n[1], m.n[2] = 6, 5
    rng = np.random.default_rng(1)
    phi, c, q, T = _fields(m.interior_shape(), rng)
    p = os.path.join(tmp_path, "ic.nc")
    F.write_fields(p, phi, concentration=c, quat=q, temperature=T, time=0.25)
    out = F.read_initial_conditions(p, m)
    assert np.array_equal(out["phase"], phi.astype(np.float32))
    assert np.array_equal(out["concentration"][0], c.astype(np.float32))
    assert np.array_equal(out["quat"], q.astype(np.float32))
    assert np.array_equal(out["temperature"], T.astype(np.float32))
    dims, var, atts = F.read(p)
    assert dims == {"x": 8, "y": 6, "z": 5, "qlen": 4}
    assert abs(float(atts["time"][0]) - 0.25) < 1e-15
    assert var["phase"].dtype == np.float32


def test_several_compositions_and_double_precision(tmp_path):
    m = configs.dilute2d(10)
    rng = np.random.default_rng(2)
    shp = m.interior_shape()
    a, b, ph = rng.uniform(size=shp), rng.uniform(size=shp), rng.uniform(size=shp)
    p = os.path.join(tmp_path, "two.nc")
    F.write(p, {"phase": (("z", "y", "x"), ph), "concentration0": (("z", "y", "x"), a),
                "concentration1": (("z", "y", "x"), b)})
    out = F.read_initial_conditions(p, m, ncompositions=2)
    assert np.array_equal(out["phase"], ph)  # doubles stay doubles
    assert np.array_equal(out["concentration"][1], b)
    # one composition named concentration0 is accepted
    p1 = os.path.join(tmp_path, "one.nc")
    F.write(p1, {"phase": (("z", "y", "x"), ph), "concentration0": (("z", "y", "x"), a)})
    assert np.array_equal(F.read_initial_conditions(p1, m)["concentration"][0], a)


def test_2d_level_takes_a_slice(tmp_path):
    m = configs.dilute2d(6)
    rng = np.random.default_rng(3)
    phi3 = rng.uniform(size=(5, 6, 6)).astype(np.float32)
    c3 = rng.uniform(size=(5, 6, 6)).astype(np.float32)
    p = os.path.join(tmp_path, "slab.nc")
    F.write_fields(p, phi3, concentration=c3)
    out = F.read_initial_conditions(p, m)
    assert np.array_equal(out["phase"][0], phi3[2])  # the middle slice by default
    out = F.read_initial_conditions(p, m, slice_index=4)
    assert np.array_equal(out["concentration"][0][0], c3[4])


def test_dimension_mismatch_refused(tmp_path):
    m = configs.calphad3d(8, seed=3, T_run=1500.0)
    p = os.path.join(tmp_path, "bad.nc")
    F.write_fields(p, np.zeros((8, 8, 7)), concentration=np.zeros((8, 8, 7)))
    with pytest.raises(F.NetcdfError, match="dimensions are incorrect"):
        F.read_initial_conditions(p, m)


def test_interoperates_with_scipy(tmp_path):
    netcdf = pytest.importorskip("scipy.io").netcdf_file
    rng = np.random.default_rng(4)
    phi = rng.uniform(size=(3, 4, 5))
    # ours -> scipy
    p = os.path.join(tmp_path, "ours.nc")
    F.write_fields(p, phi, concentration=2 * phi, time=1.5)
    with netcdf(p, "r", mmap=False) as f:
        assert np.array_equal(f.variables["phase"][:], phi.astype(np.float32))
        assert np.array_equal(f.variables["concentration"][:], (2 * phi).astype(np.float32))
        assert f.dimensions["x"] == 5 and abs(f.time - 1.5) < 1e-15
    # scipy (classic and 64-bit offset) -> ours
    for version in (1, 2):
        q = os.path.join(tmp_path, "scipy%d.nc" % version)
        with netcdf(q, "w", version=version) as f:
            f.createDimension("z", 3)
            f.createDimension("y", 4)
            f.createDimension("x", 5)
            v = f.createVariable("phase", "d", ("z", "y", "x"))
            v[:] = phi
            w = f.createVariable("concentration", "f", ("z", "y", "x"))
            w[:] = phi / 3
        dims, var, _ = F.read(q)
        assert dims == {"z": 3, "y": 4, "x": 5}
        assert np.array_equal(var["phase"], phi)
        assert np.array_equal(var["concentration"], (phi / 3).astype(np.float32))
