"""The rest of the explicit tracer and barotropic step on the device, against
the C restatement, value for value:
- surface and bottom source terms of the tracer step (ocean_tracer.F90:2318-2336)
  through mom5gpu_tracer_boundary_terms;
- ocean_barotropic_forcing (ocean_barotropic.F90:3058-3141) through
  mom5gpu_ocean_barotropic_forcing, with its zero_nonlinear_forcing_bt and
  zero_forcing_bt options, on cyclic and walled domains, and with the
  barotropic friction on udrho(tau) through mom5gpu_ocean_barotropic_forcing_tau."""
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


@pytest.mark.parametrize("which", ["lap", "bih", "both", "none", "both_zero_forcing"])
@pytest.mark.parametrize("cyc", [(False, False), (True, False), (True, True)])
def test_barotropic_friction_matches(gpu_lib, oracle_lib, which, cyc):
    """The barotropic friction of ocean_barotropic_forcing (ocean_barotropic.F90:
    3105-3120) through mom5gpu_ocean_barotropic_forcing_tau: the background
    viscosities (:1306-1341), lap_friction_barotropic (ocean_lap_friction.F90:
    423-446) and bih_friction_barotropic (ocean_bih_friction.F90:416-454) of
    udrho(tau), and forcing_bt with the frictions added (also under
    zero_forcing_bt), every field equal to the restatement bit for bit on the
    data domain; walled, x-periodic and doubly periodic domains, the lateral
    friction modules' viscosities random."""
    capi, O = gpu_lib, oracle_lib
    from mom5_gb300 import harness
    F = capi.F
    cx, cy = cyc
    sp = grid.DomainSpec(ni=35, nj=27, nk=8, lon0=0.0, lon1=35.0, lat0=-30.0, lat1=30.0, cyclic_x=cx,
                         cyclic_y=cy, continent=(9, 8, 6, 5), wavelength_cells=6.0, ntracers=1, seed=57)
    dom = grid.make_domain(sp)
    lap, bih = which.startswith(("lap", "both")), which.startswith(("bih", "both"))
    zf = which.endswith("zero_forcing")
    vl, vb = 0.07, 0.013
    opts = capi.default_options(udrho_lap=int(lap), udrho_bih=int(bih), udrho_lap_vel_micom=vl,
                                udrho_bih_vel_micom=vb, zero_forcing_bt=int(zf))
    d = harness.load(dom, options=opts)
    rng = np.random.default_rng(21)
    tm = dom["tmask"].numpy()
    shp3, shp2 = tm.shape, tm.shape[1:]
    jit = lambda a: a * (1.0 + 0.01 * rng.standard_normal(shp2))
    dxu, dyu, um = (dom[k].numpy().copy() for k in ("dxu", "dyu", "umask1"))
    met = [jit(dyu), 1.0 / jit(dxu), jit(dxu), 1.0 / jit(dyu), dom["daur"].numpy().copy(), um]
    for fid, a in zip((F.DYUE, F.DXUER, F.DXUN, F.DYUNR), met[:4]):
        d.set(fid, a)
    visc = [2e3 * rng.random(shp2) for _ in range(4)]
    for fid, a in zip((F.LAP_VISC_CEU, F.LAP_VISC_CNU, F.BIH_VISC_CEU, F.BIH_VISC_CNU), visc):
        d.set(fid, a)
    tau = 2
    ud = [1e3 * rng.standard_normal(shp2) for _ in range(2)]
    d.set(F.UDRHO_U, ud[0], level=tau)
    d.set(F.UDRHO_V, ud[1], level=tau)
    ten, tnn = tm * (rng.random(shp3) > 0.1), tm * (rng.random(shp3) > 0.1)
    d.set(F.TMASKEN_E, ten)
    d.set(F.TMASKEN_N, tnn)
    x = {k: rng.standard_normal(shp3) for k in ("au", "av")}
    x.update({k: rng.standard_normal(shp2) * 0.1 for k in ("su", "sv", "bu", "bv")})
    for fid, k in ((F.ACCEL_U, "au"), (F.ACCEL_V, "av"), (F.SMF_U, "su"), (F.SMF_V, "sv"), (F.BMF_U, "bu"),
                   (F.BMF_V, "bv")):
        d.set(fid, x[k])
    d.ocean_barotropic_forcing(tau)

    def same(fid, ref):
        got = d.get(fid)
        assert np.array_equal(got.view(np.uint64), np.ascontiguousarray(ref).ravel().view(np.uint64)), \
            f"field {fid}: bits differ"

    dims = O.dims(sp)
    back = O.bt_friction_back(dims, dxu, dyu, um, vl, vb)
    if lap or bih:
        for fid, ref in zip((F.LAP_CEU_BACK, F.LAP_CNU_BACK, F.BIH_CEU_BACK, F.BIH_CNU_BACK), back):
            same(fid, ref)
    coefs = [back[0], back[1], visc[0], visc[1], back[2], back[3], visc[2], visc[3]]
    for comp, (te, ak, sk, bk) in enumerate(((ten, "au", "su", "bu"), (tnn, "av", "sv", "bv"))):
        fl, fb, del2 = O.bt_friction(dims, lap, bih, met, coefs, ud[comp])
        same((F.LAP_FRICTION_BT_U, F.LAP_FRICTION_BT_V)[comp], fl)
        same((F.BIH_FRICTION_BT_U, F.BIH_FRICTION_BT_V)[comp], fb)
        if bih:
            same((F.BIH_DEL2_VEL_U, F.BIH_DEL2_VEL_V)[comp], del2)
            assert np.abs(fb).max() > 0
        if lap:
            assert np.abs(fl).max() > 0
        ref = O.ocean_barotropic_forcing(dims, te, x[ak], x[sk], x[bk], zero_forcing=zf,
                                         friction_lap=fl if (lap or bih) else None,
                                         friction_bih=fb if (lap or bih) else None)
        same((F.FORCING_BT_U, F.FORCING_BT_V)[comp], ref)
    d.close()


def test_barotropic_friction_needs_tau(gpu_lib):
    """With udrho_lap set, the entry point without tau refuses (the friction acts
    on udrho(tau)), and tau must be a time level."""
    capi = gpu_lib
    from mom5_gb300 import harness
    dom = grid.make_domain(_spec(False, ntr=1))
    d = harness.load(dom, options=capi.default_options(udrho_lap=1))
    with pytest.raises(capi.Mom5GpuError):
        d.ocean_barotropic_forcing()
    with pytest.raises(capi.Mom5GpuError):
        d.ocean_barotropic_forcing(4)
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
