"""ocean_advection_velocity (ocean_advection_velocity.F90:568-672), T-cell
part, through mom5gpu_ocean_advection_velocity against the C restatement:
uhrho_et, vhrho_nt, diverge_t and wrho_bt equal value for value on B and C
grids, cyclic and walled, with a non-zero surface flux, thickness tendency and
mass source."""
import numpy as np
import pytest

from mom5_gb300 import grid

pytestmark = pytest.mark.gpu


def _inputs(sp, seed):
    rng = np.random.default_rng(seed)
    shp3 = (sp.nk, sp.nj + 2, sp.ni + 2)
    shp2 = shp3[1:]
    r = lambda shape, s=1.0: rng.standard_normal(shape) * s
    return {"u": r(shp3, 0.3), "v": r(shp3, 0.3), "rho_dzu": 1035.0 * (10.0 + 50.0 * rng.random(shp3)),
            "rho_dzten_e": 1035.0 * (10.0 + 50.0 * rng.random(shp3)),
            "rho_dzten_n": 1035.0 * (10.0 + 50.0 * rng.random(shp3)),
            "dxt_dxter": 0.9 + 0.2 * rng.random(shp2), "dyt_dyter": 0.9 + 0.2 * rng.random(shp2),
            "dxt_dxtnr": 0.9 + 0.2 * rng.random(shp2), "dyt_dytnr": 0.9 + 0.2 * rng.random(shp2),
            "rho_dzt_tendency": r(shp3, 1e-3), "mass_source": r(shp3, 1e-4), "pme": r(shp2, 1e-4),
            "river": np.abs(r(shp2, 1e-4))}


@pytest.mark.parametrize("cgrid", [False, True])
@pytest.mark.parametrize("cyclic_x", [False, True])
def test_advection_velocity_matches(gpu_lib, oracle_lib, cgrid, cyclic_x):
    capi, O = gpu_lib, oracle_lib
    from mom5_gb300 import harness
    F = capi.F
    sp = grid.DomainSpec(ni=37, nj=26, nk=9, lon0=0.0, lon1=37.0, lat0=-30.0, lat1=30.0, cyclic_x=cyclic_x,
                         continent=(10, 8, 6, 5), wavelength_cells=6.0, ntracers=1, seed=41)
    dom = grid.make_domain(sp)
    d = harness.load(dom, horz_grid=capi.CGRID if cgrid else capi.BGRID)
    x = _inputs(sp, 7)
    tau = 2
    d.set(F.U_VEL, x["u"], level=tau)
    d.set(F.V_VEL, x["v"], level=tau)
    d.set(F.RHO_DZU, x["rho_dzu"], level=tau)
    for fid, k in ((F.RHO_DZTEN_E, "rho_dzten_e"), (F.RHO_DZTEN_N, "rho_dzten_n"), (F.DXT_DXTER, "dxt_dxter"),
                   (F.DYT_DYTER, "dyt_dyter"), (F.DXT_DXTNR, "dxt_dxtnr"), (F.DYT_DYTNR, "dyt_dytnr"),
                   (F.RHO_DZT_TENDENCY, "rho_dzt_tendency"), (F.MASS_SOURCE, "mass_source"), (F.PME, "pme"),
                   (F.RIVER, "river")):
        d.set(fid, x[k])
    d.ocean_advection_velocity(tau)
    g = O.domain_arrays(dom)
    g.update({k: x[k] for k in ("dxt_dxter", "dyt_dyter", "dxt_dxtnr", "dyt_dytnr")})
    ue, vn, dv, w = O.ocean_advection_velocity(O.dims(sp), g, x["u"], x["v"], rho_dzu=x["rho_dzu"],
                                               rho_dzten_e=x["rho_dzten_e"], rho_dzten_n=x["rho_dzten_n"],
                                               cgrid=cgrid, rho_dzt_tendency=x["rho_dzt_tendency"],
                                               mass_source=x["mass_source"], pme=x["pme"], river=x["river"])
    for fid, ref, name in ((F.UHRHO_ET, ue, "uhrho_et"), (F.VHRHO_NT, vn, "vhrho_nt"), (F.DIVERGE_T, dv, "diverge_t"),
                           (F.WRHO_BT, w, "wrho_bt")):
        got = d.get(fid)
        assert np.all(got == ref.ravel()), f"{name}: max diff {np.abs(got - ref.ravel()).max()}"
    # the tracer path then runs on the new velocities
    d.tracer_advection_step(1, 1, 2, 3600.0)
    assert d.check_finite(1, 2)
    d.close()
