"""Precision form (MOM5GPU_PRECISION_MIXED): FP32 fluxes and limiters, FP64
tracer state.  Checked against the FP64 drop-in, itself equal value for value to
the restatement of advect_tracer_mdfl_sweby (ocean_tracer_advect.F90:3806-4066).

Tolerance: relative tracer error max|a-b| / max|b| <= 1e-6 against FP64.

The reference's MDFL Sweby limiter is not contractive on rough tracer fields (the
reference itself warns that this legacy routine's limiters can misbehave,
ocean_tracer_advect.F90:3755-3760): in FP64, a 1e-12 relative perturbation of
the initial temperature of config C0 grows to ~1e-4 in 100 steps.  Any
arithmetic other than the reference's exact operation sequence therefore
departs from it at that rate, so the 1e-6 bound is checked over the first 10
steps (the predictability horizon of the reference trajectory), and at 100 steps
the precision form is required to stay within a small multiple of the
reference's own response to a 1e-12 perturbation.
"""
import numpy as np
import pytest

from mom5_gb300 import grid

pytestmark = pytest.mark.gpu

REL_TOL = 1e-6


def run(capi, harness, dom, precision, nsteps, dt, perturb=0.0):
    opts = capi.default_options(precision=precision)
    d = harness.load(dom, options=opts)
    if perturb:
        rng = np.random.default_rng(123)
        for n in range(1, dom.spec.ntracers + 1):
            T = d.get(capi.F.TRACER, n=n, level=1)
            d.set(capi.F.TRACER, np.ascontiguousarray(T * (1.0 + perturb * rng.standard_normal(T.shape))), n=n, level=1)
    tau = 1
    c0 = [d.global_tracer_content(n, 1) for n in range(1, dom.spec.ntracers + 1)]
    for _ in range(nsteps):
        d.tracer_advection_step(tau, tau, 3 - tau, dt)
        tau = 3 - tau
    T = [d.get(capi.F.TRACER, n=n, level=tau) for n in range(1, dom.spec.ntracers + 1)]
    c1 = [d.global_tracer_content(n, tau) for n in range(1, dom.spec.ntracers + 1)]
    d.close()
    return T, c0, c1


def rel_err(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.mark.parametrize("cyclic_x", [False, True])
@pytest.mark.parametrize("nsteps", [1, 10])
def test_mixed_against_fp64_c0(gpu_lib, cyclic_x, nsteps):
    capi = gpu_lib
    from mom5_gb300 import harness
    sp = grid.config_c0()
    sp.cyclic_x = cyclic_x
    dom = grid.make_domain(sp)
    T64, _, _ = run(capi, harness, dom, capi.PRECISION_FP64, nsteps, 3600.0)
    Tmx, c0, c1 = run(capi, harness, dom, capi.PRECISION_MIXED, nsteps, 3600.0)
    for n in range(sp.ntracers):
        err = rel_err(Tmx[n], T64[n])
        assert err <= REL_TOL, f"tracer {n + 1}: relative error {err:.3e} after {nsteps} steps"
        drift = abs(c1[n] - c0[n]) / abs(c0[n])
        print(f"tracer {n + 1}: {nsteps} steps, relative error {err:.3e}, content drift {drift:.3e}")
        assert drift <= 1e-10 * nsteps, f"tracer {n + 1}: content drift {drift:.3e}"


def test_mixed_hundred_steps_within_reference_sensitivity(gpu_lib):
    """C0, 100 steps: the precision form's departure from the FP64 trajectory is
    bounded by a small multiple of the FP64 path's own response to a 1e-12
    relative perturbation of the initial tracers."""
    capi = gpu_lib
    from mom5_gb300 import harness
    sp = grid.config_c0()
    dom = grid.make_domain(sp)
    T64, c064, c164 = run(capi, harness, dom, capi.PRECISION_FP64, 100, 3600.0)
    Tpe, _, _ = run(capi, harness, dom, capi.PRECISION_FP64, 100, 3600.0, perturb=1e-12)
    Tmx, c0, c1 = run(capi, harness, dom, capi.PRECISION_MIXED, 100, 3600.0)
    for n in range(sp.ntracers):
        sens = rel_err(Tpe[n], T64[n])
        err = rel_err(Tmx[n], T64[n])
        drift = abs(c1[n] - c0[n]) / abs(c0[n])
        drift64 = abs(c164[n] - c064[n]) / abs(c064[n])
        print(f"tracer {n + 1}: mixed error {err:.3e}, FP64 response to a 1e-12 perturbation {sens:.3e}, "
              f"content drift mixed {drift:.3e} / FP64 {drift64:.3e}")
        assert err <= max(REL_TOL, 10.0 * sens)
        assert drift <= 1e-8


def test_mixed_tendency_form(gpu_lib):
    """horz_advect_tracer in the precision form adds rho_dzt*dT/dtime to th_tendency."""
    capi = gpu_lib
    from mom5_gb300 import harness
    sp = grid.DomainSpec(ni=40, nj=30, nk=12, lon0=0.0, lon1=40.0, lat0=-30.0, lat1=30.0, cyclic_x=True,
                         continent=(12, 9, 7, 5), wavelength_cells=6.0, ntracers=3, seed=5)
    dom = grid.make_domain(sp)
    outs = []
    for prec in (capi.PRECISION_FP64, capi.PRECISION_MIXED):
        d = harness.load(dom, options=capi.default_options(precision=prec))
        th = []
        for n in range(1, 4):
            d.zero_th_tendency(n)
            d.horz_advect_tracer(n, 1, 1, 6 * 3600.0)
            th.append(d.get(capi.F.TH_TENDENCY, n=n))
        outs.append(th)
        d.close()
    for n in range(3):
        a, b = outs[1][n], outs[0][n]
        # the tendency is a small difference: compare against rho_dzt*T/dt, the scale it is taken from
        scale = (np.abs(dom["T"][n].numpy()).max() * dom["rho_dzt"].max().item()) / (6 * 3600.0)
        assert np.abs(a - b).max() <= 1e-6 * scale, n


@pytest.mark.parametrize("case", [(False, False, 61, 45), (True, False, 57, 30), (True, True, 30, 29)])
def test_mixed_multi_tile_and_partial_tiles(gpu_lib, case):
    """Domains that are not multiples of the 28x28 tile, several tiles, both halo modes."""
    capi = gpu_lib
    from mom5_gb300 import harness
    cx, cy, ni, nj = case
    sp = grid.DomainSpec(ni=ni, nj=nj, nk=7, lon0=0.0, lon1=float(ni), lat0=-20.0, lat1=20.0, cyclic_x=cx,
                         cyclic_y=cy, continent=(10, 8, 5, 6), wavelength_cells=6.0, ntracers=2, seed=ni)
    dom = grid.make_domain(sp)
    T64, _, _ = run(capi, harness, dom, capi.PRECISION_FP64, 3, 6 * 3600.0)
    Tmx, _, _ = run(capi, harness, dom, capi.PRECISION_MIXED, 3, 6 * 3600.0)
    for n in range(2):
        err = rel_err(Tmx[n], T64[n])
        assert err <= REL_TOL, (ni, nj, cx, cy, n, err)


@pytest.mark.parametrize("case", [(False, False, 62, 45, 10), (True, True, 30, 29, 3), (True, False, 57, 30, 1),
                                  (True, False, 88, 50, 4), (False, False, 61, 33, 2)])
def test_precision_form_launch_shapes_agree(gpu_lib, case):
    """Every launch shape of the precision form (tile height 32, 64, 24, 16, 16 with the
    tracer prefetch through cp.async, and heights 16 and 24 staged by TMA with the
    tracer levels carried down the column, height 16 also with at most 5 tracers per
    block) gives the same tracers bit for bit; an odd ni takes the plain kernel for
    the TMA shapes."""
    capi = gpu_lib
    from mom5_gb300 import harness
    cx, cy, ni, nj, ntr = case
    sp = grid.DomainSpec(ni=ni, nj=nj, nk=7, lon0=0.0, lon1=float(ni), lat0=-20.0, lat1=20.0, cyclic_x=cx,
                         cyclic_y=cy, continent=(10, 8, 5, 6), wavelength_cells=6.0, ntracers=ntr, seed=ni + 1)
    dom = grid.make_domain(sp)
    out = {}
    for shape in ((32, 0, 0), (64, 0, 0), (24, 0, 0), (16, 0, 0), (16, 1, 0), (16, 2, 0), (24, 2, 0), (16, 3, 0)):
        d = harness.load(dom, options=capi.default_options(precision=capi.PRECISION_MIXED))
        d.tuning = shape
        assert d.tuning == shape
        tau = 1
        for _ in range(3):
            d.tracer_advection_step(tau, tau, 3 - tau, 6 * 3600.0)
            tau = 3 - tau
        out[shape] = [d.get(capi.F.TRACER, n=n, level=tau) for n in range(1, ntr + 1)]
        d.close()
    for shape, T in out.items():
        for n in range(ntr):
            assert np.array_equal(T[n], out[(32, 0, 0)][n]), (shape, n)
    with pytest.raises(capi.Mom5GpuError):
        d = harness.load(dom, options=capi.default_options(precision=capi.PRECISION_MIXED))
        try:
            d.tuning = (32, 1, 0)
        finally:
            d.close()


@pytest.mark.parametrize("stepping_B", [True, False])
@pytest.mark.parametrize("cyclic_x", [True, False])
def test_precision_form_barotropic_is_fp64_accurate(gpu_lib, oracle_lib, cyclic_x, stepping_B):
    """The precision form keeps the barotropic state in FP64 and forms each
    subcycle's increments in FP32 (bt_fast_body.cuh): over three baroclinic
    steps of 20 subcycles every output field stays within the form's 1e-6
    (relative to the field's maximum) of the restatement of
    update_ocean_barotropic (ocean_barotropic.F90:2763-3033)."""
    capi, O = gpu_lib, oracle_lib
    from mom5_gb300 import harness
    sp = grid.DomainSpec(ni=48, nj=36, nk=1, lon0=0.0, lon1=48.0, lat0=-60.0, lat1=60.0, cyclic_x=cyclic_x,
                         hmin=None, ridge_amp=1500.0, ntracers=0, seed=9,
                         continent=None if cyclic_x else (10, 10, 6, 4))
    dom = grid.make_domain(sp)
    opts = capi.default_options(barotropic_time_stepping_A=int(not stepping_B),
                                barotropic_time_stepping_B=int(stepping_B), precision=capi.PRECISION_MIXED)
    d = harness.load(dom, options=opts)
    dtbt = 30.0
    nts = d.barotropic_init(dtuv=20 * dtbt / 2, dtbt=dtbt)
    g = O.domain_arrays(dom)
    dims = O.dims(sp)
    st = {k: dom[k].numpy().copy() for k in ("eta_t", "eta_t_bar", "udrho_u", "udrho_v")}
    names = {"eta_t_bar": capi.F.ETA_T_BAR, "udrho_u": capi.F.UDRHO_U, "udrho_v": capi.F.UDRHO_V,
             "conv_rho_ud_t": capi.F.CONV_RHO_UD_T, "eta_u": capi.F.ETA_U}
    tau = 1
    worst = 0.0
    for step in range(3):
        taup1 = 3 - tau
        d.update_ocean_barotropic(tau, taup1)
        out = O.update_ocean_barotropic(dims, g, st, nts, dtbt, time_stepping_B=stepping_B)
        for k, fid in names.items():
            got = d.get(fid, level=taup1)
            ref = out[k].ravel()
            err = np.abs(got - ref).max() / max(np.abs(ref).max(), 1e-300)
            worst = max(worst, err)
            print(f"precision-form barotropic, step {step} {k}: {err:.2e}")
            assert err <= 1e-6, f"step {step} {k}: relative error {err:.3e}"
        st = {"eta_t": st["eta_t"], "eta_t_bar": out["eta_t_bar"], "udrho_u": out["udrho_u"],
              "udrho_v": out["udrho_v"]}
        d.set(capi.F.ETA_T, np.ascontiguousarray(st["eta_t"]), level=taup1)
        # continue from the oracle's state so the bound is per step
        for k, fid in (("eta_t_bar", capi.F.ETA_T_BAR), ("udrho_u", capi.F.UDRHO_U), ("udrho_v", capi.F.UDRHO_V)):
            d.set(fid, np.ascontiguousarray(out[k]), level=taup1)
        tau = taup1
    print(f"precision-form barotropic: worst relative error {worst:.2e}")


@pytest.mark.parametrize("cyclic_x,cyclic_y,stepping_B", [(True, False, True), (False, False, False),
                                                         (True, True, True), (False, True, False)])
def test_precision_form_barotropic_one_launch_equals_three(gpu_lib, cyclic_x, cyclic_y, stepping_B):
    """The precision-form subcycle as one launch per subcycle (each 64x8 tile
    recomputing the surface pressure and transports of its ring) gives the same
    bits as the three launches per subcycle, on a domain of several tiles with
    partial ones, over three baroclinic steps, also when the form changes
    between steps."""
    capi = gpu_lib
    from mom5_gb300 import harness
    sp = grid.DomainSpec(ni=150, nj=29, nk=1, lon0=0.0, lon1=150.0, lat0=-55.0, lat1=55.0, cyclic_x=cyclic_x,
                         cyclic_y=cyclic_y, hmin=None, ridge_amp=1200.0, ntracers=0, seed=73,
                         continent=None if cyclic_y else (40, 8, 9, 6))
    dom = grid.make_domain(sp)
    per_level = (capi.F.ETA_T_BAR, capi.F.UDRHO_U, capi.F.UDRHO_V, capi.F.CONV_RHO_UD_T, capi.F.ETA_U)
    names = per_level + (capi.F.PS, capi.F.GRAD_PS_X, capi.F.GRAD_PS_Y)
    outs = {}
    for forms in ((0, 0, 0), (1, 1, 1), (1, 0, 1)):
        opts = capi.default_options(barotropic_time_stepping_A=int(not stepping_B),
                                    barotropic_time_stepping_B=int(stepping_B), precision=capi.PRECISION_MIXED)
        d = harness.load(dom, options=opts)
        d.barotropic_init(dtuv=600.0, dtbt=30.0)
        tau, got = 1, []
        for mode in forms:
            d.set_barotropic_fusion(mode)
            d.update_ocean_barotropic(tau, 3 - tau)
            tau = 3 - tau
            got.append([d.get(f, level=tau) if f in per_level else d.get(f) for f in names])
        d.close()
        outs[forms] = got
    ref = outs[(0, 0, 0)]
    assert np.abs(ref[-1][0]).max() > 0 and np.abs(ref[-1][1]).max() > 0
    for forms in ((1, 1, 1), (1, 0, 1)):
        for step in range(3):
            for f, a, b in zip(names, outs[forms][step], ref[step]):
                assert np.array_equal(a, b), f"forms {forms} step {step} field {f}: max diff {np.abs(a - b).max()}"
