"""Precision form (MOM5GPU_PRECISION_MIXED): FP32 fluxes and limiters, FP64
tracer state.  Checked against the FP64 drop-in (itself equal to the
restatement of advect_tracer_mdfl_sweby, ocean_tracer_advect.F90:3806-4066).

Tolerance (stated by the specification of this form): relative tracer error
<= 1e-6 against FP64, here after 100 steps of config C0; the error of a field is
max|a-b| / max|b|.  Global content drift is reported and bounded.
"""
import numpy as np
import pytest

from mom5_gb300 import grid

pytestmark = pytest.mark.gpu

REL_TOL = 1e-6


def run(capi, harness, dom, precision, nsteps, dt):
    opts = capi.default_options(precision=precision)
    d = harness.load(dom, options=opts)
    tau = 1
    c0 = [d.global_tracer_content(n, 1) for n in range(1, dom.spec.ntracers + 1)]
    for _ in range(nsteps):
        d.tracer_advection_step(tau, tau, 3 - tau, dt)
        tau = 3 - tau
    T = [d.get(capi.F.TRACER, n=n, level=tau) for n in range(1, dom.spec.ntracers + 1)]
    c1 = [d.global_tracer_content(n, tau) for n in range(1, dom.spec.ntracers + 1)]
    d.close()
    return T, c0, c1


@pytest.mark.parametrize("cyclic_x", [False, True])
def test_mixed_against_fp64_c0(gpu_lib, cyclic_x):
    capi = gpu_lib
    from mom5_gb300 import harness
    sp = grid.config_c0()
    sp.cyclic_x = cyclic_x
    if cyclic_x:
        sp.continent = (50, 33, 20, 15)
    dom = grid.make_domain(sp)
    T64, c064, c164 = run(capi, harness, dom, capi.PRECISION_FP64, 100, 3600.0)
    Tmx, c0mx, c1mx = run(capi, harness, dom, capi.PRECISION_MIXED, 100, 3600.0)
    for n in range(sp.ntracers):
        err = np.abs(Tmx[n] - T64[n]).max() / np.abs(T64[n]).max()
        assert err <= REL_TOL, f"tracer {n + 1}: relative error {err:.3e}"
        drift = abs(c1mx[n] - c0mx[n]) / abs(c0mx[n])
        assert drift <= 1e-9, f"tracer {n + 1}: content drift {drift:.3e}"


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


def test_mixed_multi_tile_and_partial_tiles(gpu_lib):
    """Domains that are not multiples of the 28x28 tile, several tiles, both halo modes."""
    capi = gpu_lib
    from mom5_gb300 import harness
    for cx, cy, ni, nj in ((False, False, 61, 45), (True, False, 57, 30), (True, True, 30, 29)):
        sp = grid.DomainSpec(ni=ni, nj=nj, nk=7, lon0=0.0, lon1=float(ni), lat0=-20.0, lat1=20.0, cyclic_x=cx,
                             cyclic_y=cy, continent=(10, 8, 5, 6), wavelength_cells=6.0, ntracers=2, seed=ni)
        dom = grid.make_domain(sp)
        T64, _, _ = run(capi, harness, dom, capi.PRECISION_FP64, 10, 6 * 3600.0)
        Tmx, _, _ = run(capi, harness, dom, capi.PRECISION_MIXED, 10, 6 * 3600.0)
        for n in range(2):
            err = np.abs(Tmx[n] - T64[n]).max() / np.abs(T64[n]).max()
            assert err <= REL_TOL, (ni, nj, cx, cy, n, err)
