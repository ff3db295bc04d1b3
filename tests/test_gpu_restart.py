"""Restart files through the C ABI: fms_io layout (read back by scipy's netCDF
reader), checksum verification on read, and the reference's restart identity
(N steps == N/2 steps, write, fresh domain, read, N/2 steps; bit for bit)."""
import numpy as np
import pytest

from mom5_gb300 import grid

pytestmark = pytest.mark.gpu
netcdf = pytest.importorskip("scipy.io").netcdf_file

DT = 1800.0


def _spec():
    return grid.DomainSpec(ni=36, nj=28, nk=10, lon0=0.0, lon1=36.0, lat0=-30.0, lat1=30.0, cyclic_x=True,
                           continent=(10, 8, 6, 5), hmin=1200.0, wavelength_cells=6.0, ntracers=3, seed=21)


def _make(capi, dom):
    from mom5_gb300 import harness
    opts = capi.default_options(barotropic_time_stepping_B=1)
    d = harness.load(dom, options=opts)
    d.set_tracer_scheme(3, capi.ADVECT_PSOM, capi.ADVECT_PSOM, -1.0e10, 1.0e10)
    d.set_psom_limit(3, True)
    d.set_tracer_name(1, "temp", "ocean_temp_salt.res.nc")
    d.set_tracer_name(2, "salt", "ocean_temp_salt.res.nc")
    d.set_tracer_name(3, "passive", "ocean_passive.res.nc")
    d.barotropic_init(dtuv=DT, dtbt=60.0)
    return d


def _step(d, tau, itt0):
    d.set_itt0(itt0)
    d.tracer_advection_step(tau, tau, 3 - tau, DT)
    d.update_ocean_barotropic(tau, 3 - tau)
    return 3 - tau


def _inner(a, shape):
    return a.reshape(shape)[..., 1:-1, 1:-1]


def test_restart_identity_and_layout(gpu_lib, tmp_path):
    capi = gpu_lib
    F = capi.F
    sp = _spec()
    dom = grid.make_domain(sp)
    shp3, shp2 = dom["T"][0].shape, dom["eta_t"].shape
    # straight run of 4 steps
    a = _make(capi, dom)
    tau_a = 1
    for s in range(4):
        tau_a = _step(a, tau_a, s)
    # 2 steps, restart files, a fresh domain, 2 steps
    b = _make(capi, dom)
    tau = 1
    for s in range(2):
        tau = _step(b, tau, s)
    b.write_restart(str(tmp_path), tau)
    # the files as fms_io lays them out
    with netcdf(str(tmp_path / "ocean_temp_salt.res.nc"), "r", mmap=False) as f:
        assert [f.dimensions[k] for k in ("xaxis_1", "yaxis_1", "zaxis_1")] == [sp.ni, sp.nj, sp.nk]
        assert f.dimensions["Time"] is None
        for n, name in ((1, "temp"), (2, "salt")):
            v = f.variables[name]
            assert v.dimensions == ("Time", "zaxis_1", "yaxis_1", "xaxis_1")
            ref = _inner(b.get(F.TRACER, n=n, level=tau), shp3)
            assert np.array_equal(v[0], ref)
            ck = int(np.sum(ref.view(np.uint64), dtype=np.uint64))
            assert v.checksum == ("%16X" % ck).encode()
            assert v.units == b"none" and v.long_name == name.encode()
    with netcdf(str(tmp_path / "ocean_barotropic.res.nc"), "r", mmap=False) as f:
        assert "zaxis_1" not in f.dimensions
        for name, fid in (("eta_t_bar", F.ETA_T_BAR), ("udrho", F.UDRHO_U), ("vdrho", F.UDRHO_V)):
            assert np.array_equal(f.variables[name][0], _inner(b.get(fid, level=tau), shp2))
    with netcdf(str(tmp_path / "ocean_psom_moments.res.nc"), "r", mmap=False) as f:
        assert np.array_equal(f.variables["passive_prather_sxy"][0], _inner(b.get(F.PSOM_SXY, n=3), shp3))
        assert np.abs(f.variables["passive_prather_sx"][0]).max() > 0
    b.close()
    c = _make(capi, dom)
    c.read_restart(str(tmp_path), tau)
    for s in range(2, 4):
        tau = _step(c, tau, s)
    assert tau == tau_a
    for n in (1, 2, 3):
        x, y = _inner(a.get(F.TRACER, n=n, level=tau), shp3), _inner(c.get(F.TRACER, n=n, level=tau), shp3)
        assert np.array_equal(x, y), f"tracer {n}"
    for q in range(10):
        x, y = _inner(a.get(F.PSOM_S0 + q, n=3), shp3), _inner(c.get(F.PSOM_S0 + q, n=3), shp3)
        assert np.array_equal(x, y), f"moment {q}"
    for fid in (F.ETA_T_BAR, F.UDRHO_U, F.UDRHO_V, F.CONV_RHO_UD_T, F.ETA_U):
        assert np.array_equal(a.get(fid, level=tau), c.get(fid, level=tau)), fid
    a.close()
    c.close()


def test_restart_checksum_and_shape_are_checked(gpu_lib, tmp_path):
    capi = gpu_lib
    sp = _spec()
    dom = grid.make_domain(sp)
    d = _make(capi, dom)
    d.write_restart(str(tmp_path), 1)
    p = tmp_path / "ocean_temp_salt.res.nc"
    raw = bytearray(p.read_bytes())
    raw[-1] ^= 0x01  # last mantissa byte of the last value of "salt"
    p.write_bytes(bytes(raw))
    with pytest.raises(capi.Mom5GpuError) as e:
        d.read_restart(str(tmp_path), 1)
    assert e.value.status == capi.ENUMERIC
    # a domain of another size refuses the files
    sp2 = grid.DomainSpec(ni=30, nj=28, nk=10, lon0=0.0, lon1=30.0, lat0=-30.0, lat1=30.0, cyclic_x=True,
                          continent=None, hmin=1200.0, ntracers=3, seed=2)
    d2 = _make(capi, grid.make_domain(sp2))
    d.write_restart(str(tmp_path), 1)
    with pytest.raises(capi.Mom5GpuError) as e:
        d2.read_restart(str(tmp_path), 1)
    assert e.value.status == capi.EINVAL
    # a missing tracer file is an error
    (tmp_path / "ocean_passive.res.nc").unlink()
    with pytest.raises(capi.Mom5GpuError):
        d.read_restart(str(tmp_path), 1)
    d.close()
    d2.close()


def test_copy_field_async_on_caller_streams(gpu_lib):
    """mom5gpu_copy_field_async: host -> device on one stream, device -> host on
    another after an event; the values arrive unchanged (pinned buffers)."""
    import torch
    capi = gpu_lib
    F = capi.F
    dom = grid.make_domain(_spec())
    d = _make(capi, dom)
    n3 = d.count(F.TRACER)
    src = torch.randn(n3, dtype=torch.float64).pin_memory()
    dst = torch.zeros(n3, dtype=torch.float64).pin_memory()
    up, down = torch.cuda.Stream(), torch.cuda.Stream()
    d.copy_field_async(F.TRACER, src.data_ptr(), 1, up.cuda_stream, n=2, level=3)
    e = torch.cuda.Event()
    e.record(up)
    down.wait_event(e)
    d.copy_field_async(F.TRACER, dst.data_ptr(), 0, down.cuda_stream, n=2, level=3)
    down.synchronize()
    assert torch.equal(src, dst)
    assert np.array_equal(d.get(F.TRACER, n=2, level=3), src.numpy())
    with pytest.raises(capi.Mom5GpuError):
        d.copy_field_async(F.TRACER, src.data_ptr(), 1, up.cuda_stream, n=9, level=1)
    d.close()


def test_run_configuration_drives_a_domain(gpu_lib, tmp_path):
    """A JSON run configuration (namelists and field_table choices) sets the
    domain's options, schemes, limiters and restart names."""
    capi = gpu_lib
    from mom5_gb300 import config
    doc = {"ocean_barotropic_nml": {"barotropic_time_stepping_B": True},
           "tracers": [{"name": "temp", "horiz_advect_scheme": "quickMOM3", "vert_advect_scheme": "quicker",
                        "restart_file": "ocean_temp_salt.res.nc"},
                       {"name": "salt", "horiz_advect_scheme": "mdppm", "vert_advect_scheme": "mdppm",
                        "ppm_hlimiter": 3, "restart_file": "ocean_temp_salt.res.nc"},
                       {"name": "age", "horiz_advect_scheme": "psom", "vert_advect_scheme": "psom",
                        "psom_limit": True}]}
    cfg = config.parse(doc)
    dom = grid.make_domain(_spec())
    d = config.load_domain(dom, cfg)
    d.barotropic_init(dtuv=DT, dtbt=60.0)
    _step(d, 1, 0)
    assert d.check_finite(0, 2)
    d.write_restart(str(tmp_path), 2)
    with netcdf(str(tmp_path / "ocean_temp_salt.res.nc"), "r", mmap=False) as f:
        assert {"temp", "salt"} <= set(f.variables)
    with netcdf(str(tmp_path / "ocean_psom_moments.res.nc"), "r", mmap=False) as f:
        assert "age_prather_sxx" in f.variables
    d.close()
