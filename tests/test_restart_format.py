"""CPU tests of the netCDF classic encoder and decoder the restart files use
(mom5_gb300/csrc/ncfile.h), against scipy's independent reader and writer of
the same format (scipy.io.netcdf_file, CDF-1 and CDF-2)."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
netcdf = pytest.importorskip("scipy.io").netcdf_file


@pytest.fixture(scope="module")
def drv(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("nc") / "libncdrv.so")
    subprocess.run(["g++", "-O1", "-std=c++17", "-shared", "-fPIC", "-o", out, os.path.join(HERE, "nc", "nc_driver.cpp")],
                   check=True)
    lib = C.CDLL(out)
    lib.nc_read_var.restype = C.c_long
    return lib


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def test_our_file_reads_in_scipy(drv, tmp_path):
    ni, nj, nk, nv = 7, 5, 3, 2
    rng = np.random.default_rng(1)
    data = np.ascontiguousarray(rng.standard_normal((nv, nk, nj, ni)))
    path = str(tmp_path / "a.nc")
    assert drv.nc_write_fields(path.encode(), ni, nj, nk, nv, _p(data)) == 0
    with open(path, "rb") as fh:
        assert fh.read(4) == b"CDF\x02"
    with netcdf(path, "r", mmap=False) as f:
        assert f.dimensions["xaxis_1"] == ni and f.dimensions["zaxis_1"] == nk and f.dimensions["Time"] is None
        assert f._attributes["filename"] == b"test.res.nc"
        assert np.array_equal(f.variables["xaxis_1"][:], np.arange(1, ni + 1))
        assert np.array_equal(f.variables["Time"][:], [1.0])
        for q in range(nv):
            v = f.variables[f"field{q}"]
            assert v.dimensions == ("Time", "zaxis_1", "yaxis_1", "xaxis_1")
            assert np.array_equal(v[0], data[q])
            assert v.long_name == f"field{q}".encode()


@pytest.mark.parametrize("version", [1, 2])
def test_scipy_file_reads_in_ours(drv, tmp_path, version):
    ni, nj, nk = 6, 4, 2
    rng = np.random.default_rng(2)
    a = rng.standard_normal((2, nk, nj, ni))
    b = rng.standard_normal((nj, ni)).astype(np.float32)
    path = str(tmp_path / f"s{version}.nc")
    with netcdf(path, "w", version=version) as f:
        f.history = "written by scipy"
        f.createDimension("Time", None)
        f.createDimension("zaxis_1", nk)
        f.createDimension("yaxis_1", nj)
        f.createDimension("xaxis_1", ni)
        t = f.createVariable("Time", "d", ("Time",))
        v = f.createVariable("temp", "d", ("Time", "zaxis_1", "yaxis_1", "xaxis_1"))
        v.checksum = "        DEADBEEF"
        w = f.createVariable("eta", "f", ("yaxis_1", "xaxis_1"))
        s = f.createVariable("salt", "d", ("Time", "zaxis_1", "yaxis_1", "xaxis_1"))
        t[0:2] = [1.0, 2.0]
        v[0:2] = a
        s[0:2] = a[::-1] * 2.0
        w[:] = b
    out = np.zeros(ni * nj * nk)
    for rec in (0, 1):
        assert drv.nc_read_var(path.encode(), b"temp", rec, _p(out), out.size) == out.size
        assert np.array_equal(out.reshape(nk, nj, ni), a[rec])
        assert drv.nc_read_var(path.encode(), b"salt", rec, _p(out), out.size) == out.size
        assert np.array_equal(out.reshape(nk, nj, ni), a[1 - rec] * 2.0)
    assert drv.nc_read_var(path.encode(), b"eta", 0, _p(out), out.size) == ni * nj
    assert np.array_equal(out[:ni * nj].reshape(nj, ni), b.astype(np.float64))
    buf = C.create_string_buffer(64)
    assert drv.nc_read_text_att(path.encode(), b"temp", b"checksum", buf, 64) == 16
    assert buf.value == b"        DEADBEEF"
    assert drv.nc_read_text_att(path.encode(), b"", b"history", buf, 64) > 0
    assert drv.nc_read_var(path.encode(), b"missing", 0, _p(out), out.size) == -3


def test_truncated_or_foreign_file_is_refused(drv, tmp_path):
    p = tmp_path / "bad.nc"
    p.write_bytes(b"CDF\x05" + bytes(100))
    out = np.zeros(4)
    assert drv.nc_read_var(str(p).encode(), b"x", 0, _p(out), 4) == -2
    p.write_bytes(b"HDF5" + bytes(100))
    assert drv.nc_read_var(str(p).encode(), b"x", 0, _p(out), 4) == -2
