"""The rest of the explicit tracer and barotropic step on the device, against
the C restatement, value for value:
- surface and bottom source terms of the tracer step (ocean_tracer.F90:2318-2336)
  through mom5gpu_tracer_boundary_terms;
- ocean_barotropic_forcing (ocean_barotropic.F90:3058-3141) through
  mom5gpu_ocean_barotropic_forcing, with its zero_nonlinear_forcing_bt and
  zero_forcing_bt options, on cyclic and walled domains."""
import numpy as np
import pytest

from mom5_gb300 import grid

pytestmark = pytest.mark.gpu


def _spec(cyclic_x, ntr=3):
    return grid.DomainSpec(ni=35, nj=27, nk=8, lon0=0.0, lon1=35.0, lat0=-30.0, lat1=30.0, cyclic_x=cyclic_x,
                           continent=(9, 8, 6, 5), wavelength_cells=6.0, ntracers=ntr, seed=57)


@pytest.mark.parametrize("cyclic_x", [False, True])
def test_tracer_boundary_terms_match(gpu_lib, oracle_lib, cyclic_x):
    capi, O = gpu_lib, oracle_lib
    from mom5_gb300 import harness
    F = capi.F
    sp = _spec(cyclic_x)
    dom = grid.make_domain(sp)
    d = harness.load(dom)
    g = O.domain_arrays(dom)
    rng = np.random.default_rng(4)
    shp2 = (sp.nj + 2, sp.ni + 2)
    pme = rng.standard_normal(shp2) * 1e-4
    d.set(F.PME, pme)
    kmt = dom["kmt"].numpy()
    for n in range(1, sp.ntracers + 1):
        tp, es, pb = rng.standard_normal(shp2), rng.standard_normal(shp2) * 1e-3, rng.standard_normal(shp2) * 1e-3
        th0 = rng.standard_normal(g["tmask"].shape)
        d.set(F.TPME, tp, n=n)
        d.set(F.TRACER_ETA_SMOOTH, es, n=n)
        d.set(F.PBOT_SMOOTH, pb, n=n)
        d.set(F.TH_TENDENCY, th0, n=n)
        ref = O.tracer_boundary_terms(O.dims(sp), g, kmt, pme, tp, es, pb, th0)
        if n == sp.ntracers:
            d.tracer_boundary_terms(0)  # every tracer; the others are checked below
        else:
            d.tracer_boundary_terms(n)
            got = d.get(F.TH_TENDENCY, n=n)
            assert np.all(got == ref.ravel()), f"tracer {n}"
    got = d.get(F.TH_TENDENCY, n=sp.ntracers)
    assert np.all(got == ref.ravel())
    d.close()


@pytest.mark.parametrize("opt", ["default", "zero_nonlinear", "zero_forcing"])
@pytest.mark.parametrize("cyclic_x", [False, True])
def test_barotropic_forcing_matches(gpu_lib, oracle_lib, cyclic_x, opt):
    capi, O = gpu_lib, oracle_lib
    from mom5_gb300 import harness
    F = capi.F
    sp = _spec(cyclic_x)
    dom = grid.make_domain(sp)
    opts = capi.default_options(zero_nonlinear_forcing_bt=int(opt == "zero_nonlinear"),
                                zero_forcing_bt=int(opt == "zero_forcing"))
    d = harness.load(dom, options=opts)
    rng = np.random.default_rng(8)
    tm = dom["tmask"].numpy()
    shp3, shp2 = tm.shape, tm.shape[1:]
    ten = tm * (rng.random(shp3) > 0.1)
    tnn = tm * (rng.random(shp3) > 0.1)
    d.set(F.TMASKEN_E, ten)
    d.set(F.TMASKEN_N, tnn)
    x = {k: rng.standard_normal(shp3) for k in ("au", "av")}
    x.update({k: rng.standard_normal(shp2) * 0.1 for k in ("su", "sv", "bu", "bv")})
    x["bu"][3, 4] = x["su"][3, 4]  # exact cancellation: -0/+0 handling
    for fid, k in ((F.ACCEL_U, "au"), (F.ACCEL_V, "av"), (F.SMF_U, "su"), (F.SMF_V, "sv"), (F.BMF_U, "bu"),
                   (F.BMF_V, "bv")):
        d.set(fid, x[k])
    d.ocean_barotropic_forcing()
    dims = O.dims(sp)
    kw = dict(zero_nonlinear=opt == "zero_nonlinear", zero_forcing=opt == "zero_forcing")
    ru = O.ocean_barotropic_forcing(dims, ten, x["au"], x["su"], x["bu"], **kw)
    rv = O.ocean_barotropic_forcing(dims, tnn, x["av"], x["sv"], x["bv"], **kw)
    for fid, ref in ((F.FORCING_BT_U, ru), (F.FORCING_BT_V, rv)):
        got = d.get(fid)
        assert np.array_equal(got.view(np.uint64), ref.ravel().view(np.uint64)), f"{fid}: bits differ"
    d.close()


@pytest.mark.parametrize("case", [(1, False, False, False), (1, True, False, True), (2, False, False, False),
                                  (2, True, True, False), (5, True, False, False), (3, False, True, False),
                                  (6, True, False, False)])
def test_update_ucell_thickness_matches(gpu_lib, oracle_lib, case):
    """update_ucell_thickness (ocean_thickness.F90:3507-3886) through
    mom5gpu_update_ucell_thickness: the geopotential branch (also with
    linear_free_surface), the minimum-of-neighbours branch of zstar and pstar
    (also with update_dzwu_k0 off, on cyclic and walled domains) and the sigma
    copies; every field it writes equal to the restatement on the data domain."""
    capi, O = gpu_lib, oracle_lib
    from mom5_gb300 import harness
    F = capi.F
    vcoord, cyclic, cyclic_y, linear = case
    sp = grid.DomainSpec(ni=35, nj=27, nk=8, lon0=0.0, lon1=35.0, lat0=-30.0, lat1=30.0, cyclic_x=cyclic,
                         cyclic_y=cyclic_y, continent=None, wavelength_cells=6.0, ntracers=1, seed=61)
    dom = grid.make_domain(sp)
    d = harness.load(dom)
    st = grid.thickness_state(sp.ni, sp.nj, sp.nk, cyclic_x=cyclic, cyclic_y=cyclic_y, seed=7 + vcoord)
    dzwu_k0 = vcoord != 5
    taup1 = 2
    fields = {"umask": (F.UMASK, 0), "tmasken_e": (F.TMASKEN_E, 0), "tmasken_n": (F.TMASKEN_N, 0),
              "dzt": (F.DZT, 0), "dzwt": (F.DZWT, 0), "rho_dzt": (F.RHO_DZT, taup1), "depth_zt": (F.DEPTH_ZT, 0),
              "depth_zwt": (F.DEPTH_ZWT, 0), "eta_u": (F.ETA_U, taup1), "dzu": (F.DZU, 0), "dzwu": (F.DZWU, 0),
              "rho_dzu": (F.RHO_DZU, taup1), "rho_dzur": (F.RHO_DZUR, 0), "dzten_e": (F.DZTEN_E, 0),
              "dzten_n": (F.DZTEN_N, 0), "rho_dzten_e": (F.RHO_DZTEN_E, 0), "rho_dzten_n": (F.RHO_DZTEN_N, 0),
              "depth_zu": (F.DEPTH_ZU, 0), "depth_zwu": (F.DEPTH_ZWU, 0)}
    for k, (fid, lev) in fields.items():
        d.set(fid, np.ascontiguousarray(st[k]), level=lev)
    d.update_ucell_thickness(taup1, vcoord, linear_free_surface=linear, update_dzwu_k0=dzwu_k0)
    ref = O.update_ucell_thickness(O.dims(sp), vcoord, st, rho0=1035.0, linear_free_surface=linear,
                                   update_dzwu_k0=dzwu_k0)
    outs = dict(fields)
    outs.update({"thicku": (F.THICKU, taup1), "thicken_e": (F.THICKEN_E, 0), "thicken_n": (F.THICKEN_N, 0),
                 "mass_u": (F.MASS_U, taup1), "mass_en_e": (F.MASS_EN_E, 0), "mass_en_n": (F.MASS_EN_N, 0)})
    for k in ref:
        fid, lev = outs[k]
        got = d.get(fid, level=lev)
        assert np.array_equal(got, ref[k].ravel()), f"{k}: {np.abs(got - ref[k].ravel()).max():.3e}"
    d.close()
