"""CPU tests of the C restatement (the oracle) itself.

The reference ships no golden vectors for these routines, so the restatement is
pinned by properties the reference algorithms must satisfy: conservation,
preservation of a uniform tracer, the documented reductions between schemes,
closed-form weights, exact one-cell shifts, symmetric gravity waves and the
restart identity.  Each test names the reference lines it checks.
"""
import math

import numpy as np
import pytest

from mom5_gb300 import grid


def small(ni=24, nj=18, nk=8, ntr=2, seed=1, cyclic_x=False, continent=(8, 6, 5, 4), **kw):
    return grid.DomainSpec(ni=ni, nj=nj, nk=nk, lon0=0.0, lon1=float(ni), lat0=-20.0, lat1=20.0,
                           cyclic_x=cyclic_x, continent=continent, wavelength_cells=6.0, ntracers=ntr, seed=seed, **kw)


@pytest.fixture(scope="module")
def O(oracle_lib):
    return oracle_lib


def load(O, sp):
    dom = grid.make_domain(sp)
    return dom, O.domain_arrays(dom), O.dims(sp)


@pytest.mark.parametrize("cyclic_x", [False, True])
def test_flow_is_divergence_free(O, cyclic_x):
    """Continuity (ocean_advection_velocity.F90:600-627) reproduces the generator's
    vertical mass flux, and it vanishes at the sea floor."""
    dom, g, d = load(O, small(cyclic_x=cyclic_x))
    w = O.continuity_w(d, g)
    assert np.allclose(w, g["wrho_bt"], rtol=0, atol=1e-9 * np.abs(g["uhrho_et"]).max())
    kmt = dom["kmt"].numpy()
    scale = np.abs(g["wrho_bt"]).max()
    assert scale > 0
    for j in range(1, d.nj + 1):
        for i in range(1, d.ni + 1):
            if kmt[j, i] > 0:
                assert abs(g["wrho_bt"][kmt[j, i], j, i]) <= 1e-10 * scale


def test_advection_velocity_restatements_agree(O):
    """The full ocean_advection_velocity restatement (ocean_advection_velocity.F90:
    600-627) and the continuity-only one give the same wrho_bt for the same face
    fluxes when the thickness tendency and mass source vanish; on the C grid with
    unit face-area ratios uhrho_et = u*rho_dzten exactly (:645-654)."""
    dom, g, d = load(O, small(seed=4))
    rng = np.random.default_rng(3)
    shp = g["uhrho_et"].shape
    u, v = rng.standard_normal(shp), rng.standard_normal(shp)
    rz = 1035.0 * (5.0 + rng.random(shp))
    ue, vn, dv, w = O.ocean_advection_velocity(d, g, u, v, rho_dzu=rz)
    g2 = dict(g, uhrho_et=ue, vhrho_nt=vn)
    assert np.array_equal(w, O.continuity_w(d, g2))
    # BAY / BAX vanish on the first row / column of the data domain
    assert np.all(ue[:, 0, :] == 0.0) and np.all(vn[:, :, 0] == 0.0)
    one = np.ones(shp[1:])
    g3 = dict(g, dxt_dxter=one, dyt_dyter=one, dxt_dxtnr=one, dyt_dytnr=one)
    ue, vn, dv, w = O.ocean_advection_velocity(d, g3, u, v, rho_dzten_e=rz, rho_dzten_n=2 * rz, cgrid=True)
    assert np.array_equal(ue, u * rz) and np.array_equal(vn, v * (2 * rz))


def test_step_terms_restatements(O):
    """Source terms of the tracer step (ocean_tracer.F90:2318-2336) add exactly
    tmask*(pme*tpme + eta_smooth) at k=1 and tmask*pbot_smooth at kmt; the
    barotropic forcing (ocean_barotropic.F90:3058-3141) of a fluid at rest with
    equal surface and bottom stress is +0 everywhere, halo included."""
    dom, g, d = load(O, small(seed=6))
    rng = np.random.default_rng(2)
    kmt = dom["kmt"].numpy()
    shp2 = kmt.shape
    pme, tp, es, pb = (rng.standard_normal(shp2) for _ in range(4))
    th = np.zeros_like(g["tmask"])
    out = O.tracer_boundary_terms(d, g, kmt, pme, tp, es, pb, th)
    exp = np.zeros_like(th)
    exp[0, 1:-1, 1:-1] = (g["tmask"][0] * (pme * tp + es))[1:-1, 1:-1]
    for j in range(1, d.nj + 1):
        for i in range(1, d.ni + 1):
            if kmt[j, i] > 0:
                exp[kmt[j, i] - 1, j, i] += g["tmask"][kmt[j, i] - 1, j, i] * pb[j, i]
    assert np.array_equal(out, exp)
    z3 = np.zeros_like(g["tmask"])
    s = rng.standard_normal(shp2)
    f = O.ocean_barotropic_forcing(d, g["tmask"], z3, s, s)
    assert np.all(f.view(np.uint64) == 0)


@pytest.mark.parametrize("scheme", ["mdfl", "dst", "all", "upwind", "quicker", "c2", "c4", "c6", "ppm1", "ppm2", "ppm3",
                                    "supb", "psom", "psom_prather", "psom_nolimit", "qm3"])
@pytest.mark.parametrize("cyclic_x", [False, True])
def test_uniform_tracer_stays_uniform(O, scheme, cyclic_x):
    """A uniform tracer in a non-divergent flow has zero advective tendency
    (to roundoff) under every scheme."""
    dom, g, d = load(O, small(cyclic_x=cyclic_x))
    U = np.ascontiguousarray(g["tmask"] * 7.25)
    if scheme == "mdfl":
        th = O.advect_mdfl_sweby(d, g, U, 3600.0)
    elif scheme == "dst":
        th = O.advect_mdfl_sweby(d, g, U, 3600.0, 0.0)
    elif scheme == "all":
        th = O.advect_sweby_all(d, g, np.ascontiguousarray(U[None]), 3600.0)[0]
    elif scheme == "upwind":
        th = O.horz_advect_upwind(d, g, U) + O.vert_advect_upwind(d, g, U)
    elif scheme.startswith("ppm"):
        th = O.advect_mdppm(d, g, U, 3600.0, int(scheme[3]))
    elif scheme == "supb":
        th = O.advect_mdfl_sup_b(d, g, U, 3600.0)
    elif scheme.startswith("psom"):
        th = psom_steps(O, d, g, U, 3600.0, scheme, 1)
    elif scheme == "qm3":
        q = O.quicker_init(d, g, dom.dzt.numpy())
        th = O.horz_advect_quickmom3(d, g, q, U, U) + O.vert_advect_quicker(d, g, q, U, U)
    elif scheme.startswith("c"):
        order = int(scheme[1])
        th = O.horz_advect_centred(d, g, U, order) + O.vert_advect_centred(d, g, U, order, dom["kmt"].numpy())
    else:
        q = O.quicker_init(d, g, dom.dzt.numpy())
        th = O.horz_advect_quicker(d, g, q, U, U) + O.vert_advect_quicker(d, g, q, U, U)
    scale = 7.25 * np.abs(g["wrho_bt"]).max() + 7.25 * np.abs(g["uhrho_et"]).max() * g["datr"].max() * 1e5
    assert np.abs(th).max() <= 1e-12 * scale


def psom_steps(O, d, g, T, dtime, scheme, nsteps, moments=None):
    """nsteps calls of advect_tracer_psom on the same T (itt0 = 0, 1, ...); the
    tendency of the last."""
    if moments is None:
        moments = np.zeros((9,) + T.shape)
    th = None
    for itt0 in range(nsteps):
        th, _ = O.advect_psom(d, g, T, dtime, moments, itt0=itt0, limit=scheme != "psom_nolimit",
                              prather=scheme == "psom_prather")
    return th


@pytest.mark.parametrize("scheme", ["mdfl", "upwind", "quicker", "c4", "ppm1", "ppm2", "ppm3", "supb", "psom",
                                    "psom_prather", "qm3"])
def test_global_content_conserved(O, scheme):
    """sum(dat*rho_dzt*T*tmask) (ocean_tracer_diag.F90:2395-2412) is unchanged by
    advection plus the explicit update, to FP64 roundoff."""
    dom, g, d = load(O, small(seed=7))
    q = O.quicker_init(d, g, dom.dzt.numpy())
    T = g["T"][0].copy()
    c0 = O.total_tracer(d, g, T)[0]
    moments = np.zeros((9,) + T.shape)
    for step in range(10):
        if scheme.startswith("psom"):
            th, _ = O.advect_psom(d, g, T, 3600.0 * 6, moments, itt0=step, prather=scheme == "psom_prather")
        elif scheme == "mdfl":
            th = O.advect_mdfl_sweby(d, g, T, 3600.0 * 6)
        elif scheme == "upwind":
            th = O.horz_advect_upwind(d, g, T) + O.vert_advect_upwind(d, g, T)
        elif scheme.startswith("ppm"):
            th = O.advect_mdppm(d, g, T, 3600.0 * 6, int(scheme[3]))
        elif scheme == "supb":
            th = O.advect_mdfl_sup_b(d, g, T, 3600.0 * 6)
        elif scheme == "c4":
            th = O.horz_advect_centred(d, g, T, 4) + O.vert_advect_centred(d, g, T, 4, dom["kmt"].numpy())
        elif scheme == "qm3":
            th = O.horz_advect_quickmom3(d, g, q, T, T) + O.vert_advect_quicker(d, g, q, T, T)
        else:
            th = O.horz_advect_quicker(d, g, q, T, T) + O.vert_advect_quicker(d, g, q, T, T)
        T = O.update_tracer(d, g, T, th, 3600.0 * 6)
    c1 = O.total_tracer(d, g, T)[0]
    assert abs(c1 - c0) <= 1e-13 * abs(c0)


def test_psom_limiters_on_a_square_pulse(O):
    """Torus pulse under PSOM for 20 steps through every sweep order: with the
    Merryfield-Holloway limiter (the default, ocean_tracer_advect.F90:112-117)
    and with Prather's limiter the tracer stays non-negative (Prather's limiter
    is documented as positive definite but not monotonic, :4542-4547); without
    a limiter the second-order moments undershoot below zero."""
    sp = small(ni=32, nj=24, nk=4, continent=None, ntr=1, seed=3, cyclic_x=True, hmin=None, depth=400.0,
               dz_top=80.0, dz_bot=120.0)
    dom, g, d = load(O, sp)
    T0 = np.zeros_like(g["T"][0])
    T0[:, 8:16, 10:20] = 1.0
    T0 *= g["tmask"]
    O.halo_update(d, T0)
    dt = 3600.0 * 6
    wet = g["tmask"] > 0
    ext = {}
    for mode in ("mh", "prather", "none"):
        T = T0.copy()
        mom = np.zeros((9,) + T.shape)
        for step in range(20):
            th, _ = O.advect_psom(d, g, T, dt, mom, itt0=step, limit=mode != "none", prather=mode == "prather")
            T = O.update_tracer(d, g, T, th, dt)
        ext[mode] = (T[wet].min(), T[wet].max())
    assert ext["mh"][0] >= 0.0 and ext["prather"][0] >= 0.0
    assert ext["none"][0] < -1e-3
    assert ext["mh"][1] < 1.01 and ext["mh"][1] < ext["prather"][1]


def test_sweby_is_monotone_and_quicker_is_not(O):
    """Torus pulse test (testcase_ocean_solo.pdf section 2), qualitative: Quicker
    over/undershoots a square pulse, MDFL Sweby's extrema are far smaller.  The
    reference documents that this legacy MDFL routine is not strictly monotone
    (ocean_tracer_advect.F90:3755-3760), so small extrema are expected."""
    sp = small(ni=32, nj=24, nk=4, continent=None, ntr=1, seed=3, cyclic_x=True, hmin=None, depth=400.0,
               dz_top=80.0, dz_bot=120.0)
    dom, g, d = load(O, sp)
    q = O.quicker_init(d, g, dom.dzt.numpy())
    T = np.zeros_like(g["T"][0])
    T[:, 8:16, 10:20] = 1.0
    T *= g["tmask"]
    O.halo_update(d, T)
    Ts, Tq = T.copy(), T.copy()
    dt = 3600.0 * 6
    for _ in range(20):
        Ts = O.update_tracer(d, g, Ts, O.advect_mdfl_sweby(d, g, Ts, dt), dt)
        th = O.horz_advect_quicker(d, g, q, Tq, Tq) + O.vert_advect_quicker(d, g, q, Tq, Tq)
        Tq = O.update_tracer(d, g, Tq, th, dt)
    wet = g["tmask"] > 0
    ext_s = max(-Ts[wet].min(), Ts[wet].max() - 1.0, 0.0)
    ext_q = max(-Tq[wet].min(), Tq[wet].max() - 1.0, 0.0)
    assert ext_q > 1e-3
    assert ext_s < 1e-3 and ext_s < 0.05 * ext_q


def test_sweby_all_equals_one_tracer_to_roundoff(O):
    """advect_tracer_sweby_all (:4104-4511) regroups the products of
    advect_tracer_mdfl_sweby (:3806-4066): same values to a few ulps."""
    dom, g, d = load(O, small(ntr=3, seed=9))
    dt = 3600.0 * 6
    allv = O.advect_sweby_all(d, g, np.ascontiguousarray(g["T"]), dt)
    for n in range(3):
        one = O.advect_mdfl_sweby(d, g, g["T"][n].copy(), dt)
        # the tendency is rho_dzt*(T_mdfl - T)/dt: roundoff of T_mdfl is amplified by rho_dzt/dt
        tol = 64 * np.finfo(float).eps * np.abs(g["T"][n]).max() * g["rho_dzt"].max() / dt
        assert np.abs(allv[n] - one).max() <= tol
        assert np.abs(allv[n] - one).max() > 0 or n > 0


def test_dst_linear_is_sweby_without_limiter(O):
    """sweby_limiter = 0 gives the linear DST scheme (:1960-1962): it differs from
    the limited scheme where the limiter is active, and is not monotone."""
    dom, g, d = load(O, small(ntr=1, seed=12))
    T = g["T"][0].copy()
    a = O.advect_mdfl_sweby(d, g, T, 3600.0 * 6, 1.0)
    b = O.advect_mdfl_sweby(d, g, T, 3600.0 * 6, 0.0)
    assert np.abs(a - b).max() > 0


def test_upwind_cfl_one_shifts_one_cell(O):
    """1-D upwind at Courant number 1 moves a profile exactly one cell (:2238-2294)."""
    sp = grid.DomainSpec(ni=16, nj=3, nk=1, lon0=0.0, lon1=16.0, lat0=-1.0, lat1=1.0, cyclic_x=True,
                         continent=None, hmin=None, ntracers=1, seed=0)
    dom, g, d = load(O, sp)
    u = 0.75  # m/s
    rdz = g["rho_dzt"][0, 1, 1]
    g["uhrho_et"][:] = u * rdz
    g["vhrho_nt"][:] = 0.0
    g["wrho_bt"][:] = 0.0
    g["tmask"][:] = 0.0
    g["tmask"][:, 1:-1, :] = 1.0
    dx = g["dxte"][2, 3]
    dt = dx / u
    T = np.zeros_like(g["T"][0])
    T[0, 2, 1:17] = np.arange(16, dtype=float) ** 2
    O.halo_update(d, T)
    th = O.horz_advect_upwind(d, g, T)
    Tn = O.update_tracer(d, g, T, th, dt)
    expect = np.roll(T[0, 2, 1:17], 1)
    assert np.allclose(Tn[0, 2, 1:17], expect, rtol=1e-12, atol=1e-9)


def _scheme_step(O, scheme, dom, dt):
    """One forward step of a scheme on a tracer at time level tau = taum1."""
    g, d = O.domain_arrays(dom), O.dims(dom.spec)
    T = g["T"][0]
    nk = dom.spec.nk
    if scheme == "mdfl_sweby":
        th = O.advect_mdfl_sweby(d, g, T, dt, 1.0)
    elif scheme == "upwind":
        th = O.horz_advect_upwind(d, g, T) + O.vert_advect_upwind(d, g, T)
    elif scheme == "quicker":
        q = O.quicker_init(d, g, dom.dzt.numpy())
        th = O.horz_advect_quicker(d, g, q, T, T) + O.vert_advect_quicker(d, g, q, T, T)
    else:
        order = int(scheme[-1])
        kmt = np.full(T.shape[1:], nk, dtype=np.int32)
        th = O.horz_advect_centred(d, g, T, order) + O.vert_advect_centred(d, g, T, order, kmt)
    return O.update_tracer(d, g, T, th, dt)


ANALYTIC_CASES = [("mdfl_sweby", "cubic"), ("upwind", "linear"), ("quicker", "quadratic"),
                  ("centred2", "quadratic"), ("centred4", "quadratic"), ("centred6", "quadratic")]


@pytest.mark.parametrize("vel", [(0.4, 0.0, 0.0), (0.0, -0.3, 0.0), (0.0, 0.0, 1e-3), (0.4, -0.3, 1e-3),
                                 (-0.2, 0.25, -2e-3)])
@pytest.mark.parametrize("scheme,kind", ANALYTIC_CASES)
def test_schemes_match_the_advection_equation(O, scheme, kind, vel):
    """Known answers from the advection equation on a uniform box in uniform
    flow (tests/analytic.py): MDFL Sweby (:3806-4066) translates a cubic
    exactly, upwind (:2238-2294, :2792-2824) a linear profile; centred
    2nd/4th/6th order (:2306-2529, :2836-2972) and Quicker (:2538-2653,
    :2981-3031) take the exact forward-Euler step of a quadratic."""
    import analytic as A
    u, v, w = vel
    dom, spacing = A.make_box(kind, u, v, w)
    dt = 2000.0
    Tn = _scheme_step(O, scheme, dom, dt)
    E = A.expected(kind, Tn.shape, u, v, w, dt, spacing)
    assert A.rel_err(Tn, E) < 2e-15
    # the profile did move, by far more than the tolerance
    assert A.rel_err(Tn, dom["T"][0].numpy()) > 1e-4


@pytest.mark.parametrize("axis", [2, 1, 0])
@pytest.mark.parametrize("case", ["line", "slope", "one", "zero", "slope_negative_u", "one_negative_u"])
def test_sweby_limiter_branches(O, case, axis):
    """Known answer (tests/analytic.py): on profiles whose differences along
    the flow form a geometric sequence, the limiter of advect_tracer_mdfl_sweby
    (ocean_tracer_advect.F90:3868-3878) takes one value at every face, on the
    DST3 line, on the slope bound (1-c)/c*theta, on the bound 1 or at 0, and one
    step equals the 1-D flux form with that value (x, y and z passes, either sign
    of the velocity; the z pass with k counting down)."""
    import analytic as A
    dom, E, psi = A.make_limiter_box(case, axis)
    Tn = _scheme_step(O, "mdfl_sweby", dom, 2000.0)
    vert = axis == 0
    assert A.rel_err_cells(Tn, E, vertical=vert) < 1e-12
    # the step moved the profile, and the limiter mattered: psi = 0 or the DST3 line would differ
    T0 = dom["T"][0].numpy()
    assert A.rel_err_cells(Tn, T0, vertical=vert) > 1e-3
    r, c, sign, branch = A.LIMITER_CASES[case]
    for other in {0.0, 1.0, A.limiter_psi(A.limiter_theta(r, sign), c)[1]} - {psi}:
        assert A.rel_err_cells(Tn, A.limiter_expected(T0, axis, c, sign, other), vertical=vert) > 1e-6


@pytest.mark.parametrize("vel", [(0.4, 0.0, 0.0), (0.0, -0.3, 0.0), (0.0, 0.0, 5e-4), (0.4, 0.3, 5e-4),
                                 (-0.4, -0.3, -5e-4)])
def test_mdfl_at_courant_one_moves_any_field_one_cell(O, vel):
    """At Courant number 1 the Sweby limiter (:3868-3878) and the DST3 terms
    vanish and each MDFL pass is upwind at Courant number 1: a random tracer
    moves exactly one cell along each velocity component (tests/analytic.py)."""
    import analytic as A
    u, v, w = vel
    dom, _, T0 = A.make_random_box(u, v, w)
    g, d = O.domain_arrays(dom), O.dims(dom.spec)
    T = g["T"][0]
    dt = A.CFL1_DT
    Tn = O.update_tracer(d, g, T, O.advect_mdfl_sweby(d, g, T, dt, 1.0), dt)
    assert np.abs(A.interior(Tn) - A.interior(A.shifted_one_cell(T0, u, v, w))).max() < 2e-15


@pytest.mark.parametrize("stepping_B", [False, True])
def test_barotropic_matches_the_momentum_equation(O, stepping_B):
    """Known answer (tests/analytic.py): with f = 0, no forcing, a flat bottom
    and a sea surface of uniform slope, pred_corr_tropic_depth_bgrid
    (ocean_barotropic.F90:3225-3579) accelerates the transports uniformly at
    -H rho0 g grad(eta), eta keeps its value, and update_ocean_barotropic
    (:2763-3033) returns the subcycles' time average."""
    import analytic as A
    sx, sy, u0, v0, nts, dtbt = 1e-3, -5e-4, 100.0, -50.0, 10, 20.0
    dom, spacing = A.make_baro_box(sx, sy, u0, v0)
    g, d = O.domain_arrays(dom), O.dims(dom.spec)
    st = {k: g[k].copy() for k in ("eta_t", "eta_t_bar", "udrho_u", "udrho_v")}
    out = O.update_ocean_barotropic(d, g, st, nts, dtbt, time_stepping_B=stepping_B)
    eu, ev = A.baro_expected(sx, sy, u0, v0, nts, dtbt, spacing, stepping_B)
    assert np.abs(A.interior2(out["udrho_u"]) - eu).max() <= 1e-10 * abs(eu)
    assert np.abs(A.interior2(out["udrho_v"]) - ev).max() <= 1e-10 * abs(ev)
    assert np.abs(A.interior2(out["eta_t_bar"]) - A.interior2(g["eta_t"])).max() <= 1e-12
    assert np.abs(A.interior2(out["conv_rho_ud_t"])).max() <= 1e-10 * abs(eu) / spacing[0]


@pytest.mark.parametrize("cgrid", [False, True])
@pytest.mark.parametrize("stepping_B", [False, True])
def test_barotropic_inertial_oscillation(O, stepping_B, cgrid):
    """Known answer (tests/analytic.py): a flat sea surface and uniform
    transports on an f-plane only rotate.  The B-grid subcycle
    (pred_corr_tropic_depth_bgrid, ocean_barotropic.F90:3225-3579) is the
    Crank-Nicolson rotation, the C-grid one (pred_corr_tropic_depth_cgrid,
    :3601-3965) the Adams-Bashforth-3 extrapolation of the Coriolis force; the
    step returns the subcycles' time average and eta stays flat (a doubly
    periodic domain: no walls, so no waves)."""
    import analytic as A
    f, u0, v0, nts, dtbt = 1.4e-4, 100.0, -50.0, 20, 20.0
    dom, spacing = A.make_baro_box(0.0, 0.0, u0, v0, f=f, periodic=True)
    g, d = O.domain_arrays(dom), O.dims(dom.spec)
    st = {k: g[k].copy() for k in ("eta_t", "eta_t_bar", "udrho_u", "udrho_v")}
    out = O.update_ocean_barotropic(d, g, st, nts, dtbt, time_stepping_B=stepping_B, cgrid=cgrid)
    eu, ev = A.baro_inertial_expected(f, u0, v0, nts, dtbt, stepping_B, cgrid)
    amp = np.hypot(eu, ev)
    assert np.abs(A.interior2(out["udrho_u"]) - eu).max() <= 1e-12 * amp
    assert np.abs(A.interior2(out["udrho_v"]) - ev).max() <= 1e-12 * amp
    assert np.abs(A.interior2(out["eta_t_bar"]) - 0.5).max() <= 1e-13


def test_quicker_weights_uniform_grid(O):
    """On a uniform grid quicker_init (:1510-1578) gives quick = 1/2 and the
    curvature weights 1/8, -1/4 (relative form of the classic 3/8, 6/8, -1/8)."""
    sp = grid.DomainSpec(ni=10, nj=8, nk=5, lon0=0.0, lon1=10.0, lat0=-0.5, lat1=0.5, continent=None, hmin=None,
                         ntracers=1, seed=0, dz_top=50.0, dz_bot=50.0, depth=250.0)
    dom, g, d = load(O, sp)
    g["dxt"][:] = 1000.0
    g["dyt"][:] = 1000.0
    q = O.quicker_init(d, g, np.full(5, 50.0))
    inner = (slice(None), slice(2, -2), slice(2, -2))
    assert np.allclose(q["quick_x"][inner], 0.5) and np.allclose(q["quick_y"][inner], 0.5)
    assert np.allclose(q["curv_xp"][0][2:-2, 2:-2], 1.0 / 8.0)
    assert np.allclose(q["curv_xp"][1][2:-2, 2:-2], -1.0 / 4.0)
    assert np.allclose(q["curv_xp"][2][2:-2, 2:-2], 1.0 / 8.0)
    assert np.allclose(q["quick_z"], 0.5)
    assert np.allclose(q["curv_zp"][:, 1:-2], np.array([[1 / 8.0], [-1 / 4.0], [1 / 8.0]]))


def _flat_basin(O, n=40, f0=0.0, cyclic=False):
    sp = grid.DomainSpec(ni=n, nj=n, nk=1, lon0=0.0, lon1=float(n) * 0.1, lat0=-0.1 * n / 2, lat1=0.1 * n / 2,
                         cyclic_x=cyclic, continent=None, hmin=None, ntracers=0, seed=0)
    dom, g, d = load(O, sp)
    g["f"][:] = f0
    g["forcing_u"][:] = 0.0
    g["forcing_v"][:] = 0.0
    g["dxu"][:] = g["dxu"][2, 2]
    g["dxt"][:] = g["dxt"][2, 2]
    g["dxur"][:] = 1.0 / (g["dxu"] + 1e-40)
    g["dat"][:] = g["dxt"] * g["dyt"]
    g["datr"][:] = 1.0 / (g["dat"] + 1e-40)
    return dom, g, d


def test_barotropic_mass_conserved_and_symmetric(O):
    """Flat bottom, f = 0, a centred eta bump: the subcycle (:3225-3579) keeps
    sum(dat*eta_t_bar) (no sources) and the solution stays symmetric under i ->
    mirror and j -> mirror."""
    n = 40
    dom, g, d = _flat_basin(O, n)
    x = np.arange(n + 2) - (n + 1) / 2.0
    bump = np.exp(-(x[None, :] ** 2 + x[:, None] ** 2) / 18.0) * 0.1
    eta = np.ascontiguousarray(bump * g["tmask1"])
    st = {"eta_t": eta, "eta_t_bar": eta.copy(), "udrho_u": np.zeros_like(eta), "udrho_v": np.zeros_like(eta)}
    m0 = O.area_integral(d, g, eta)
    for _ in range(4):
        out = O.update_ocean_barotropic(d, g, st, 40, 20.0)
        st = {"eta_t": eta, "eta_t_bar": out["eta_t_bar"], "udrho_u": out["udrho_u"], "udrho_v": out["udrho_v"]}
    e = out["eta_t_bar"][1:-1, 1:-1]
    assert abs(O.area_integral(d, g, out["eta_t_bar"]) - m0) <= 1e-12 * abs(m0)
    assert np.abs(e - e[:, ::-1]).max() <= 1e-6 * np.abs(e).max() * 10 + 1e-12
    assert np.abs(e - e[::-1, :]).max() <= 1e-6 * np.abs(e).max() * 10 + 1e-12
    assert np.abs(e - bump[1:-1, 1:-1]).max() > 1e-4  # the waves moved


def test_barotropic_gamma0_nts1_is_forward_backward(O):
    """With pred_corr_gamma = 0 and nts = 1 the subcycle is one forward-backward
    step: eta from the old transport divergence is not used for the pressure."""
    n = 20
    dom, g, d = _flat_basin(O, n, f0=1e-4)
    rng = np.random.default_rng(1)
    eta = np.ascontiguousarray(rng.normal(size=g["tmask1"].shape) * 0.01 * g["tmask1"])
    st = {"eta_t": eta, "eta_t_bar": eta.copy(), "udrho_u": np.zeros_like(eta), "udrho_v": np.zeros_like(eta)}
    out = O.update_ocean_barotropic(d, g, st, 1, 10.0, gamma=0.0, time_stepping_B=False)
    # by hand: ps from eta, momentum from the pressure gradient, eta from the new transport
    ps = g["rho_g"] * eta + g["patm"]
    gx, gy = O.grad_baro_p(d, g, ps)
    c1 = 0.5 * 10.0 * g["f"]
    c2 = 1.0 / (1.0 + c1 * c1)
    t1 = 10.0 * (-g["thicku"] * gx)
    t2 = 10.0 * (-g["thicku"] * gy)
    u = c2 * (t1 + c1 * t2)
    v = c2 * (t2 - c1 * t1)
    dv = O.div_ud_bgrid(d, g, np.ascontiguousarray(u), np.ascontiguousarray(v))
    eta1 = eta + 10.0 / 1035.0 * (-dv * g["tmask1"])
    expect_bar = (eta + eta1) / 2.0
    inner = (slice(1, -1), slice(1, -1))
    assert np.allclose(out["eta_t_bar"][inner], expect_bar[inner], rtol=1e-12, atol=1e-15)
    assert np.allclose(out["udrho_u"][inner], u[inner], rtol=1e-12, atol=1e-12)


def test_barotropic_restart_identity(O):
    """N steps == N/2 steps, restart from the saved fields, N/2 steps (the
    reference's restart identity, testcase_ocean_solo.pdf section 1.1)."""
    sp = grid.DomainSpec(ni=30, nj=24, nk=1, cyclic_x=True, hmin=None, ridge_amp=800.0, ntracers=0, seed=4)
    dom, g, d = load(O, sp)
    st0 = {k: g[k].copy() for k in ("eta_t", "eta_t_bar", "udrho_u", "udrho_v")}

    def run(st, nsteps):
        for _ in range(nsteps):
            out = O.update_ocean_barotropic(d, g, st, 10, 30.0)
            st = {"eta_t": st["eta_t"], "eta_t_bar": out["eta_t_bar"], "udrho_u": out["udrho_u"],
                  "udrho_v": out["udrho_v"]}
        return st

    a = run(st0, 4)
    half = run(st0, 2)
    saved = {k: np.frombuffer(v.tobytes()).reshape(v.shape).copy() for k, v in half.items()}
    b = run(saved, 2)
    for k in a:
        assert np.array_equal(a[k], b[k])


def test_tmask_limit_flags_out_of_range(O):
    """compute_tmask_limit (ocean_tracer.F90:2804-2851) flags a wet cell whose own,
    east, north or lower neighbour is outside the tracer's range."""
    dom, g, d = load(O, small(ntr=1, seed=2, continent=None, hmin=None))
    T = np.full_like(g["T"][0], 10.0) * g["tmask"]
    T[3, 5, 7] = 50.0
    tl = O.compute_tmask_limit(d, g, T, 0.0, 20.0)
    assert tl[3, 5, 7] == 1 and tl[3, 5, 6] == 1 and tl[3, 4, 7] == 1 and tl[2, 5, 7] == 1
    assert tl[3, 5, 8] == 0 and tl[3, 6, 7] == 0 and tl[4, 5, 7] == 0
    assert tl.sum() == 4


def test_halo_update_semantics(O):
    """Single-PE mpp_update_domains: periodic copy in cyclic directions, halo
    untouched at walls, corners only when both directions are cyclic."""
    from oracle.oracle import Dims
    d = Dims(4, 3, 1, 1, 0)
    a = np.arange(6 * 5, dtype=float).reshape(1, 5, 6)
    b = a.copy()
    O.halo_update(d, b)
    assert np.array_equal(b[0, 1:4, 0], a[0, 1:4, 4]) and np.array_equal(b[0, 1:4, 5], a[0, 1:4, 1])
    assert np.array_equal(b[0, 0, :], a[0, 0, :]) and np.array_equal(b[0, 4, :], a[0, 4, :])


@pytest.mark.parametrize("vcoord", [1, 2, 3])
def test_ucell_thickness_rules(O, vcoord):
    """update_ucell_thickness (ocean_thickness.F90:3507-3886): the geopotential
    branch moves only the top U cell with eta_u (:3617-3635); the sigma branch
    copies the T-cell thicknesses (:3663-3683); the others take the minimum of
    the neighbouring T cells (:3735-3763); depths are cumulative sums
    (:3811-3827), thicku the depth of the bottom U level (:3817-3826), mass_u
    and thicken vertical sums (:3829-3858)."""
    ni, nj, nk = 10, 8, 5
    st = grid.thickness_state(ni, nj, nk, seed=4)
    d = O.dims(small(ni=ni, nj=nj, nk=nk))
    out = O.update_ucell_thickness(d, vcoord, st)
    rho0 = 1035.0
    sl = (slice(None), slice(0, nj + 1), slice(0, ni + 1))  # computed by the min loops (isd:iec, jsd:jec)
    if vcoord == 1:
        assert np.array_equal(out["dzu"][0], st["depth_zwt"][0] + st["eta_u"])
        assert np.array_equal(out["dzwu"][0], st["depth_zt"][0] + st["eta_u"])
        assert np.array_equal(out["dzu"][1:], st["dzu"][1:]) and np.array_equal(out["depth_zwu"], st["depth_zwu"])
        assert np.array_equal(out["rho_dzur"][0], 1.0 / (rho0 * out["dzu"][0] + 1e-20))
    elif vcoord == 3:
        assert np.array_equal(out["dzu"], st["dzt"]) and np.array_equal(out["rho_dzu"], st["rho_dzt"])
        assert np.array_equal(out["dzwu"], st["dzwt"]) and np.array_equal(out["rho_dzten_e"], st["rho_dzten_e"])
    else:
        t = st["dzt"]
        m4 = np.minimum(np.minimum(np.minimum(t[:, :-1, :-1], t[:, :-1, 1:]), t[:, 1:, :-1]), t[:, 1:, 1:])
        assert np.array_equal(out["dzu"][sl], m4)
        assert np.array_equal(out["dzten_e"][sl], np.minimum(t[:, :-1, :-1], t[:, :-1, 1:]))
        assert np.array_equal(out["dzu"][:, :, ni + 1], st["dzu"][:, :, ni + 1])  # walled halo kept
    if vcoord != 1:
        assert np.allclose(out["depth_zwu"], np.cumsum(out["dzu"], axis=0), rtol=1e-14, atol=0)
        assert np.array_equal(out["rho_dzur"], st["umask"] / (out["rho_dzu"] + 1e-20))
    kmu = st["kmu"]
    want = np.where(kmu > 1, np.take_along_axis(out["depth_zwu"], np.maximum(kmu - 1, 0)[None], 0)[0], 0.0)
    assert np.array_equal(out["thicku"], want)
    assert np.allclose(out["mass_u"], (st["umask"] * out["rho_dzu"]).sum(0), rtol=1e-14, atol=0)
    assert np.allclose(out["thicken_n"], out["dzten_n"].sum(0), rtol=1e-14, atol=0)


def _uniform_friction_metrics(ni, nj, dx, dy):
    one = np.ones((nj + 2, ni + 2))
    # dyue, dxuer, dxun, dyunr, daur, umask1 of a uniform B grid, every U cell wet
    return [dy * one, one / dx, dx * one, one / dy, one / (dx * dy), one.copy()]


@pytest.mark.parametrize("axis", ["x", "y"])
def test_barotropic_friction_of_a_parabola(O, axis):
    """Barotropic friction on a uniform grid (dx = 2, dy = 4) with constant
    viscosities (back + visc = 0.75 east, 0.625 north; every value and operation
    exact): the Laplacian (ocean_lap_friction.F90:423-446) of u = x^2 is 2*c_e at
    every compute point and of u = y^2 is 2*c_n; the biharmonic
    (ocean_bih_friction.F90:416-454) of the same u has del2_vel = 2*c and a second
    iteration that vanishes where all the neighbours are compute points (walled
    box: zero halo)."""
    from oracle.oracle import Dims
    ni, nj, dx, dy = 10, 8, 2.0, 4.0
    d = Dims(ni, nj, 1, 0, 0)
    m = _uniform_friction_metrics(ni, nj, dx, dy)
    shp = (nj + 2, ni + 2)
    ce, cn = 0.75, 0.625
    coefs = [np.full(shp, 0.5), np.full(shp, 0.5), np.full(shp, ce - 0.5), np.full(shp, cn - 0.5),
             np.full(shp, 0.25), np.full(shp, 0.125), np.full(shp, ce - 0.25), np.full(shp, cn - 0.125)]
    j, i = np.meshgrid(np.arange(nj + 2), np.arange(ni + 2), indexing="ij")
    u = (i * dx) ** 2 if axis == "x" else (j * dy) ** 2
    c = ce if axis == "x" else cn
    lap, bih, del2 = O.bt_friction(d, True, True, m, coefs, u.astype(float))
    assert np.all(lap[1:-1, 1:-1] == 2 * c)
    assert np.all(del2[1:-1, 1:-1] == 2 * c)
    assert np.all(bih[2:-2, 2:-2] == 0.0)
    assert np.all(lap[0, :] == 0) and np.all(bih[:, 0] == 0)  # walls: the halo stays 0.0
    # a linear u: no Laplacian friction
    lin = (3.0 * i * dx + 5.0 * j * dy).astype(float)
    lap2, _, _ = O.bt_friction(d, True, False, m, coefs, lin)
    assert np.all(lap2[1:-1, 1:-1] == 0.0)


def test_barotropic_friction_background_viscosity(O):
    """lap/bih_c*u_back of ocean_barotropic_init (ocean_barotropic.F90:1306-1341) on
    square U cells of side 4: the MICOM viscosity vel*4 (Laplacian) and
    sqrt(vel*4^3) (biharmonic) on the compute domain, zero in a walled halo, the
    periodic copy in a cyclic one."""
    from oracle.oracle import Dims
    ni, nj = 6, 5
    for cyclic in (0, 1):
        d = Dims(ni, nj, 1, cyclic, 0)
        one = np.ones((nj + 2, ni + 2))
        le, ln, be, bn = O.bt_friction_back(d, 4.0 * one, 4.0 * one, one, 0.05, 0.01)
        for a, want in ((le, 0.05 * 4.0), (ln, 0.05 * 4.0), (be, math.sqrt(0.01 * 64.0)), (bn, math.sqrt(0.01 * 64.0))):
            assert np.allclose(a[1:-1, 1:-1], want, rtol=1e-15, atol=0)
            assert np.all(a[0, :] == 0) and np.all(a[-1, :] == 0)
            assert np.all(a[1:-1, 0] == (a[1:-1, ni] if cyclic else 0.0))
