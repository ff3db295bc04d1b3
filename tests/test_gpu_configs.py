"""The workload configurations themselves, value for value against the C
restatement of the reference routines:

* the 0.25 degree grid at its poleward edge (the global config's geometry:
  lat 12.5..80, periodic in x, 10 tracers, 50 levels), two whole FP64 steps
  of MDFL Sweby advection + explicit update + a 60-subcycle barotropic step;
* the barotropic config as stated: 360x300, 1 degree, lat -75..75, ridge
  bathymetry, 80 predictor-corrector subcycles of 67.5 s per baroclinic step
  (dtuv = 2700 s), 50 steps, with the eta tendency and update between them;
* a batched FP64 ensemble of uneven domains, each domain compared with the
  restatement directly (not with the one-domain library path).

Equality is IEEE value equality on every compared array.
"""
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

from mom5_gb300 import grid

pytestmark = pytest.mark.gpu


def equal(a, b):
    a = np.asarray(a).ravel()
    b = np.asarray(b).ravel()
    return a.shape == b.shape and bool(np.all((a == b) | (np.isnan(a) & np.isnan(b))))


def diff_report(a, b):
    a = np.asarray(a).ravel()
    b = np.asarray(b).ravel()
    bad = np.nonzero(a != b)[0]
    if bad.size == 0:
        return "identical"
    d = np.abs(a - b)
    return f"{bad.size} differ; max abs {d.max():.3e}; first at flat index {bad[0]}"


def _pool():
    # the restatement's C routines release the GIL inside ctypes calls
    return ThreadPoolExecutor(max_workers=max(1, min(10, os.cpu_count() or 1)))


BARO_OUT = ("eta_t_bar", "udrho_u", "udrho_v", "conv_rho_ud_t", "eta_u")


def _baro_fields(capi):
    return {"eta_t_bar": capi.F.ETA_T_BAR, "udrho_u": capi.F.UDRHO_U, "udrho_v": capi.F.UDRHO_V,
            "conv_rho_ud_t": capi.F.CONV_RHO_UD_T, "eta_u": capi.F.ETA_U}


def test_c2_polar_block_two_full_steps(gpu_lib, oracle_lib):
    """Config C2's geometry (0.25 deg to 80 deg, periodic in x, 10 tracers, 50
    levels) on a 360x270 block: two whole FP64 steps (dtts = 600 s, 60
    subcycles of 20 s) -- every tracer value, every barotropic output, the
    compensated content equal to the restatement's and conserved."""
    capi, O = gpu_lib, oracle_lib
    from mom5_gb300 import harness
    sp = grid.config_c2_polar_block()
    dom = grid.make_domain(sp)
    assert grid.barotropic_cfl_limit(dom) >= 20.0
    d = harness.load(dom, options=capi.default_options(barotropic_time_stepping_B=1))
    dtts, dtbt = 600.0, 20.0
    nts = d.barotropic_init(dtuv=dtts, dtbt=dtbt)
    assert nts == 60
    g = O.domain_arrays(dom)
    dims = O.dims(sp)
    ntr = sp.ntracers
    T = [g["T"][n].copy() for n in range(ntr)]
    c0 = [O.total_tracer(dims, g, T[n])[0] for n in range(ntr)]
    st = {k: g[k].copy() for k in ("eta_t", "eta_t_bar", "udrho_u", "udrho_v")}
    names = _baro_fields(capi)

    def oracle_tracer(n):
        return O.update_tracer(dims, g, T[n], O.advect_mdfl_sweby(dims, g, T[n], dtts), dtts)

    tau = 1
    with _pool() as pool:
        for step in range(2):
            taup1 = 3 - tau
            d.tracer_advection_step(tau, tau, taup1, dtts)
            d.update_ocean_barotropic(tau, taup1)
            T = list(pool.map(oracle_tracer, range(ntr)))
            out = O.update_ocean_barotropic(dims, g, st, nts, dtbt)
            for n in range(1, ntr + 1):
                got = d.get(capi.F.TRACER, n=n, level=taup1)
                assert equal(got, T[n - 1]), f"step {step} tracer {n}: {diff_report(got, T[n - 1])}"
            for k, fid in names.items():
                got = d.get(fid, level=taup1)
                assert equal(got, out[k]), f"step {step} {k}: {diff_report(got, out[k])}"
            for k, fid in (("ps", capi.F.PS), ("grad_ps_x", capi.F.GRAD_PS_X), ("grad_ps_y", capi.F.GRAD_PS_Y)):
                got = d.get(fid)
                assert equal(got, out[k]), f"step {step} {k}: {diff_report(got, out[k])}"
            st = {"eta_t": st["eta_t"], "eta_t_bar": out["eta_t_bar"], "udrho_u": out["udrho_u"],
                  "udrho_v": out["udrho_v"]}
            tau = taup1
    for n in range(1, ntr + 1):
        got = d.global_tracer_content(n, tau)
        ref = O.total_tracer(dims, g, T[n - 1])[0]
        assert abs(got - ref) <= 1e-14 * abs(ref), (n, got, ref)
        assert abs(got - c0[n - 1]) <= 1e-12 * abs(c0[n - 1]), (n, got, c0[n - 1])
    d.close()


def test_c1_as_stated_fifty_steps(gpu_lib, oracle_lib):
    """Config C1 exactly: 360x300 at 1 degree, lat -75..75, ridge bathymetry,
    barotropic_init(dtuv = 2700 s, dtbt = 67.5 s) -> 80 subcycles per step,
    50 steps of eta_and_pbot_tendency, update_ocean_barotropic and
    eta_and_pbot_update (ocean_barotropic.F90:2668-2734, :2763-3033,
    :2290-2385); every output equal at steps 1, 10, 20, ..., 50."""
    capi, O = gpu_lib, oracle_lib
    from mom5_gb300 import harness
    sp = grid.config_c1()
    dom = grid.make_domain(sp)
    d = harness.load(dom, options=capi.default_options(barotropic_time_stepping_B=1))
    dtts, dtbt = 2700.0, 67.5
    nts = d.barotropic_init(dtuv=dtts, dtbt=dtbt)
    assert nts == 80
    g = O.domain_arrays(dom)
    dims = O.dims(sp)
    st = {k: g[k].copy() for k in ("eta_t", "eta_t_bar", "udrho_u", "udrho_v")}
    conv = g["conv_rho_ud_t"].copy()
    names = _baro_fields(capi)
    compute_rows = (slice(1, -1), slice(0, None))
    tau = 1
    for step in range(1, 51):
        taup1 = 3 - tau
        d.eta_and_pbot_tendency(tau)
        d.update_ocean_barotropic(tau, taup1)
        d.eta_and_pbot_update(tau, taup1, dtts)
        deta = O.eta_and_pbot_tendency(dims, g, conv)
        out = O.update_ocean_barotropic(dims, g, st, nts, dtbt)
        eta_new = O.eta_and_pbot_update(dims, st["eta_t"], deta, dtts)
        if step == 1 or step % 10 == 0:
            for k, fid in names.items():
                got = d.get(fid, level=taup1)
                assert equal(got, out[k]), f"step {step} {k}: {diff_report(got, out[k])}"
            got = d.get(capi.F.DETA_DT)
            assert equal(got, deta), f"step {step} deta_dt: {diff_report(got, deta)}"
            got = d.get(capi.F.ETA_T, level=taup1).reshape(eta_new.shape)
            assert equal(got[compute_rows], eta_new[compute_rows]), \
                f"step {step} eta_t: {diff_report(got[compute_rows], eta_new[compute_rows])}"
        st = {"eta_t": eta_new, "eta_t_bar": out["eta_t_bar"], "udrho_u": out["udrho_u"], "udrho_v": out["udrho_v"]}
        conv = out["conv_rho_ud_t"]
        tau = taup1
    # a live flow after 50 steps: the comparison is not of quiescent fields
    assert np.abs(st["udrho_u"]).max() > 0 and np.abs(st["eta_t_bar"]).max() > 1e-3
    d.close()


ENSEMBLE = [(40, 30, 8, False), (57, 23, 11, True), (29, 41, 6, False), (64, 64, 9, False), (18, 12, 5, True)]


def test_batched_fp64_ensemble_matches_restatement(gpu_lib, oracle_lib):
    """The batched FP64 form (mom5gpu_batch_step: work-list launches, then the
    CUDA-graph path) on five uneven domains, 3 tracers each: after every one
    of four steps each domain's tracers and barotropic outputs equal the
    restatement's own stepping of that domain."""
    capi, O = gpu_lib, oracle_lib
    from mom5_gb300 import harness
    dt, dtuv, dtbt = 3600.0 * 3, 200.0, 20.0
    doms, ref = [], []
    for n, (ni, nj, nk, cx) in enumerate(ENSEMBLE):
        sp = grid.DomainSpec(ni=ni, nj=nj, nk=nk, lon0=0.0, lon1=float(ni) * 0.5, lat0=-25.0, lat1=25.0,
                             cyclic_x=cx, continent=(ni // 3, nj // 3, max(2, ni // 8), max(2, nj // 8)),
                             wavelength_cells=6.0, ntracers=3, seed=140 + n)
        dom = grid.make_domain(sp)
        d = harness.load(dom, options=capi.default_options(barotropic_time_stepping_B=1))
        nts = d.barotropic_init(dtuv=dtuv, dtbt=dtbt)
        doms.append(d)
        g = O.domain_arrays(dom)
        ref.append({"dims": O.dims(sp), "g": g, "nts": nts, "T": [g["T"][m].copy() for m in range(3)],
                    "st": {k: g[k].copy() for k in ("eta_t", "eta_t_bar", "udrho_u", "udrho_v")}})
    b = capi.Batch(doms)
    names = _baro_fields(capi)
    every = list(range(len(doms)))
    for step in range(4):
        parity = step % 2
        if step < 2:
            b.step(dt, index=every, parity=[parity] * len(doms))
        else:
            b.step(dt, parity=parity)
        taup1 = 2 - parity
        for i, r in enumerate(ref):
            dims, g = r["dims"], r["g"]
            r["T"] = [O.update_tracer(dims, g, T, O.advect_mdfl_sweby(dims, g, T, dt), dt) for T in r["T"]]
            out = O.update_ocean_barotropic(dims, g, r["st"], r["nts"], dtbt)
            r["st"] = {"eta_t": r["st"]["eta_t"], "eta_t_bar": out["eta_t_bar"], "udrho_u": out["udrho_u"],
                       "udrho_v": out["udrho_v"]}
            for n in range(1, 4):
                got = doms[i].get(capi.F.TRACER, n=n, level=taup1)
                assert equal(got, r["T"][n - 1]), f"step {step} domain {i} tracer {n}: " \
                                                  f"{diff_report(got, r['T'][n - 1])}"
            for k, fid in names.items():
                got = doms[i].get(fid, level=taup1)
                assert equal(got, out[k]), f"step {step} domain {i} {k}: {diff_report(got, out[k])}"
    b.close()
    for d in doms:
        d.close()
