"""Parity of the CUDA path (through the C ABI) with the C restatement of the
reference routines, on seeded synthetic domains.

The FP64 drop-in is required to agree with the restatement value for value
(IEEE equality, so +0 == -0); each test says which reference routine it
covers.
"""
import numpy as np
import pytest

from mom5_gb300 import grid

pytestmark = pytest.mark.gpu


def spec(ni=40, nj=30, nk=12, cyclic_x=False, cyclic_y=False, ntr=3, seed=5, continent=(12, 9, 7, 5), hmin=1500.0,
         lat=(-30.0, 30.0)):
    return grid.DomainSpec(ni=ni, nj=nj, nk=nk, lon0=0.0, lon1=float(ni), lat0=lat[0], lat1=lat[1],
                           cyclic_x=cyclic_x, cyclic_y=cyclic_y, continent=continent, hmin=hmin,
                           wavelength_cells=6.0, ntracers=ntr, seed=seed)


def equal(a, b):
    """IEEE value equality, element by element."""
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
    return f"{bad.size} differ; max abs {d.max():.3e}; max rel {(d / np.maximum(np.abs(b), 1e-300)).max():.3e}"


@pytest.fixture(scope="module")
def env(gpu_lib, oracle_lib):
    return gpu_lib, oracle_lib


def setup(env, sp, scheme=9, options=None, limits=None):
    capi, O = env
    from mom5_gb300 import harness
    dom = grid.make_domain(sp)
    d = harness.load(dom, options=options, scheme=scheme, tracer_limits=limits)
    return dom, d, O.domain_arrays(dom), O.dims(sp)


@pytest.mark.parametrize("cyclic_x", [False, True])
@pytest.mark.parametrize("limiter", [1.0, 0.0])
def test_mdfl_one_tracer_matches(env, cyclic_x, limiter):
    """horz_advect_tracer with ADVECT_MDFL_SWEBY / ADVECT_DST_LINEAR
    (ocean_tracer_advect.F90:1953-1962 -> advect_tracer_mdfl_sweby :3806-4066)."""
    capi, O = env
    scheme = capi.ADVECT_MDFL_SWEBY if limiter == 1.0 else capi.ADVECT_DST_LINEAR
    sp = spec(cyclic_x=cyclic_x)
    dom, d, g, dims = setup(env, sp, scheme=scheme)
    dt = 6 * 3600.0
    for n in range(1, sp.ntracers + 1):
        d.zero_th_tendency(n)
        d.horz_advect_tracer(n, 1, 1, dt)
        d.vert_advect_tracer(n, 1, 1, dt)
        got = d.get(capi.F.TH_TENDENCY, n=n)
        ref = O.advect_mdfl_sweby(dims, g, g["T"][n - 1].copy(), dt, limiter)
        assert equal(got, ref), f"tracer {n}: {diff_report(got, ref)}"


@pytest.mark.parametrize("cyclic_x", [False, True])
def test_sweby_all_matches(env, cyclic_x):
    """advect_tracer_sweby_all (ocean_tracer_advect.F90:4104-4511)."""
    capi, O = env
    sp = spec(cyclic_x=cyclic_x, ntr=4, seed=11)
    opts = capi.default_options(advect_sweby_all=1)
    dom, d, g, dims = setup(env, sp, options=opts)
    dt = 6 * 3600.0
    d.zero_th_tendency(0)
    for n in range(1, sp.ntracers + 1):  # the reference runs the all-tracer routine from n == 1 only
        d.horz_advect_tracer(n, 1, 1, dt)
        d.vert_advect_tracer(n, 1, 1, dt)
    ref = O.advect_sweby_all(dims, g, np.ascontiguousarray(g["T"]), dt)
    for n in range(1, sp.ntracers + 1):
        got = d.get(capi.F.TH_TENDENCY, n=n)
        assert equal(got, ref[n - 1]), f"tracer {n}: {diff_report(got, ref[n - 1])}"


@pytest.mark.parametrize("cyclic_x", [False, True])
def test_upwind_matches(env, cyclic_x):
    """ADVECT_UPWIND horizontal (:2238-2294) and vertical (:2792-2824)."""
    capi, O = env
    sp = spec(cyclic_x=cyclic_x, ntr=2, seed=3)
    dom, d, g, dims = setup(env, sp, scheme=capi.ADVECT_UPWIND)
    for n in (1, 2):
        d.zero_th_tendency(n)
        d.horz_advect_tracer(n, 1, 1, 3600.0)
        got_h = d.get(capi.F.TH_TENDENCY, n=n)
        T = g["T"][n - 1].copy()
        ref_h = O.horz_advect_upwind(dims, g, T)
        assert equal(got_h, ref_h), diff_report(got_h, ref_h)
        d.vert_advect_tracer(n, 1, 1, 3600.0)
        got = d.get(capi.F.TH_TENDENCY, n=n)
        ref = ref_h + O.vert_advect_upwind(dims, g, T)
        assert equal(got, ref), diff_report(got, ref)


@pytest.mark.parametrize("order", [2, 4, 6])
@pytest.mark.parametrize("cyclic_x,cyclic_y", [(False, False), (True, False), (True, True)])
def test_centred_schemes_match(env, order, cyclic_x, cyclic_y):
    """ADVECT_2ND/4TH/6TH_ORDER (ocean_tracer_advect.F90:2306-2529 horizontal,
    :2836-2972 vertical) on T(tau), with the 4th/6th-order land substitutions
    next to the continent and the halo-2/3 copies of cyclic domains."""
    capi, O = env
    scheme = {2: capi.ADVECT_2ND_ORDER, 4: capi.ADVECT_4TH_ORDER, 6: capi.ADVECT_6TH_ORDER}[order]
    sp = spec(cyclic_x=cyclic_x, cyclic_y=cyclic_y, ntr=2, seed=13 + order)
    dom, d, g, dims = setup(env, sp, scheme=scheme)
    rng = np.random.default_rng(order)
    kmt = dom["kmt"].numpy()
    for n in (1, 2):
        T0 = np.ascontiguousarray(g["T"][n - 1] * (1.0 + 0.01 * rng.standard_normal(g["T"][n - 1].shape)))
        d.set(capi.F.TRACER, T0, n=n, level=2)  # tau = 2 differs from taum1 = 1
        d.zero_th_tendency(n)
        d.horz_advect_tracer(n, 1, 2, 3600.0)
        got_h = d.get(capi.F.TH_TENDENCY, n=n)
        ref_h = O.horz_advect_centred(dims, g, T0, order)
        assert equal(got_h, ref_h), f"horz tracer {n}: {diff_report(got_h, ref_h)}"
        d.vert_advect_tracer(n, 1, 2, 3600.0)
        got = d.get(capi.F.TH_TENDENCY, n=n)
        ref = ref_h + O.vert_advect_centred(dims, g, T0, order, kmt)
        assert equal(got, ref), f"vert tracer {n}: {diff_report(got, ref)}"


@pytest.mark.parametrize("cyclic_x,cyclic_y", [(False, False), (True, False), (True, True)])
def test_mdfl_sup_b_matches(env, cyclic_x, cyclic_y):
    """ADVECT_MDFL_SUP_B (advect_tracer_mdfl_sup_b, ocean_tracer_advect.F90:3189-3466):
    the tendency of two tracers, then three whole steps, every value equal."""
    capi, O = env
    sp = spec(cyclic_x=cyclic_x, cyclic_y=cyclic_y, ntr=2, seed=44)
    dom, d, g, dims = setup(env, sp, scheme=capi.ADVECT_MDFL_SUP_B)
    dt = 6 * 3600.0
    for n in (1, 2):
        d.zero_th_tendency(n)
        d.horz_advect_tracer(n, 1, 1, dt)
        d.vert_advect_tracer(n, 1, 1, dt)
        got = d.get(capi.F.TH_TENDENCY, n=n)
        ref = O.advect_mdfl_sup_b(dims, g, g["T"][n - 1].copy(), dt)
        assert equal(got, ref), f"tracer {n}: {diff_report(got, ref)}"
    tau = 1
    T = [g["T"][n].copy() for n in range(2)]
    for s in range(3):
        d.tracer_advection_step(tau, tau, 3 - tau, dt)
        tau = 3 - tau
        for n in range(2):
            T[n] = O.update_tracer(dims, g, T[n], O.advect_mdfl_sup_b(dims, g, T[n], dt), dt)
    for n in (1, 2):
        got = d.get(capi.F.TRACER, n=n, level=tau)
        assert equal(got, T[n - 1]), f"step 3 tracer {n}: {diff_report(got, T[n - 1])}"


@pytest.mark.parametrize("limiter", [1, 2, 3])
@pytest.mark.parametrize("cyclic_x,cyclic_y", [(False, False), (True, False), (True, True)])
def test_mdppm_matches(env, limiter, cyclic_x, cyclic_y):
    """ADVECT_MDPPM (advect_tracer_mdppm, ocean_tracer_advect.F90:5990-6507) with
    each edge limiter (ppm_hlimiter 1, 2, 3: :6510-6660): the tendency of two
    tracers, then three whole steps, every value equal."""
    capi, O = env
    sp = spec(cyclic_x=cyclic_x, cyclic_y=cyclic_y, ntr=2, seed=30 + limiter)
    dom, d, g, dims = setup(env, sp, scheme=capi.ADVECT_MDPPM)
    dt = 6 * 3600.0
    for n in (1, 2):
        d.set_ppm_limiter(n, limiter)
        d.zero_th_tendency(n)
        d.horz_advect_tracer(n, 1, 1, dt)
        d.vert_advect_tracer(n, 1, 1, dt)
        got = d.get(capi.F.TH_TENDENCY, n=n)
        ref = O.advect_mdppm(dims, g, g["T"][n - 1].copy(), dt, limiter)
        assert equal(got, ref), f"tracer {n}: {diff_report(got, ref)}"
    tau = 1
    T = [g["T"][n].copy() for n in range(2)]
    for s in range(3):
        d.tracer_advection_step(tau, tau, 3 - tau, dt)
        tau = 3 - tau
        for n in range(2):
            th = O.advect_mdppm(dims, g, T[n], dt, limiter)
            T[n] = O.update_tracer(dims, g, T[n], th, dt)
    for n in (1, 2):
        got = d.get(capi.F.TRACER, n=n, level=tau)
        assert equal(got, T[n - 1]), f"step 3 tracer {n}: {diff_report(got, T[n - 1])}"


@pytest.mark.parametrize("mode", ["merryfield_holloway", "prather", "unlimited"])
@pytest.mark.parametrize("cyclic_x,cyclic_y", [(False, False), (True, False), (True, True)])
def test_psom_matches(env, mode, cyclic_x, cyclic_y):
    """ADVECT_PSOM (advect_tracer_psom, ocean_tracer_advect.F90:4549-4660; psom_x/y/z
    :4662-5420) with the Merryfield-Holloway limiter, Prather's limiter
    (psom_limit_prather) or none: the tendency of two tracers at itt0 = 0, then
    six whole steps through every sweep order (mod(itt0, 6)), every tracer value
    and every moment equal."""
    capi, O = env
    opts = capi.default_options(psom_limit_prather=int(mode == "prather"))
    sp = spec(cyclic_x=cyclic_x, cyclic_y=cyclic_y, ntr=2, seed=50 + cyclic_x + 2 * cyclic_y)
    dom, d, g, dims = setup(env, sp, scheme=capi.ADVECT_PSOM, options=opts)
    limit, prather = mode != "unlimited", mode == "prather"
    dt = 6 * 3600.0
    mom = [np.zeros((9,) + g["T"][0].shape) for _ in range(2)]
    for n in (1, 2):
        d.set_psom_limit(n, limit)
        d.zero_th_tendency(n)
        d.horz_advect_tracer(n, 1, 1, dt)
        d.vert_advect_tracer(n, 1, 1, dt)
        got = d.get(capi.F.TH_TENDENCY, n=n)
        ref, _ = O.advect_psom(dims, g, g["T"][n - 1].copy(), dt, mom[n - 1], itt0=0, limit=limit, prather=prather)
        assert equal(got, ref), f"tracer {n}: {diff_report(got, ref)}"
    tau = 1
    T = [g["T"][n].copy() for n in range(2)]
    s0 = [None, None]
    for itt0 in range(1, 7):
        d.set_itt0(itt0)
        d.tracer_advection_step(tau, tau, 3 - tau, dt)
        tau = 3 - tau
        for n in range(2):
            th, s0[n] = O.advect_psom(dims, g, T[n], dt, mom[n], itt0=itt0, limit=limit, prather=prather)
            T[n] = O.update_tracer(dims, g, T[n], th, dt)
    inner = (slice(None), slice(1, -1), slice(1, -1))
    shp = g["T"][0].shape
    for n in (1, 2):
        got = d.get(capi.F.TRACER, n=n, level=tau)
        assert equal(got, T[n - 1]), f"step 6 tracer {n}: {diff_report(got, T[n - 1])}"
        got = d.get(capi.F.PSOM_S0, n=n).reshape(shp)[inner]
        assert equal(got, s0[n - 1][inner]), f"s0 tracer {n}: {diff_report(got, s0[n - 1][inner])}"
        for q, name in enumerate(O.PSOM_MOMENTS):
            got = d.get(capi.F.PSOM_SX + q, n=n).reshape(shp)[inner]
            ref = mom[n - 1][q][inner]
            assert equal(got, ref), f"{name} tracer {n}: {diff_report(got, ref)}"


@pytest.mark.parametrize("limit_with_upwind", [0, 1])
@pytest.mark.parametrize("cyclic_x", [False, True])
def test_quicker_matches(env, cyclic_x, limit_with_upwind):
    """ADVECT_QUICKER (quicker_init :1442-1586, horz :2538-2653, vert :2981-3031)
    with tmask_limit from compute_tmask_limit (ocean_tracer.F90:2788-2892)."""
    capi, O = env
    sp = spec(cyclic_x=cyclic_x, ntr=2, seed=4)
    opts = capi.default_options(limit_with_upwind=limit_with_upwind)
    limits = [(2.0, 20.0), (34.6, 35.3)]  # makes tmask_limit non-trivial
    dom, d, g, dims = setup(env, sp, scheme=capi.ADVECT_QUICKER, options=opts, limits=limits)
    q = O.quicker_init(dims, g, dom.dzt.numpy())
    d.compute_tmask_limit(1, 1, 2)
    tl = [O.compute_tmask_limit(dims, g, g["T"][n].copy(), *limits[n]) for n in range(2)]
    O.tmask_limit_ts_same(dims, tl[0], tl[1])
    for n in (1, 2):
        got_tl = d.get(capi.F.TMASK_LIMIT, n=n)
        assert equal(got_tl, tl[n - 1]), diff_report(got_tl, tl[n - 1])
        assert 0 < tl[n - 1].sum() < tl[n - 1].size
    # two distinct time levels: tau != taum1 exercises the centred/upwind split
    T0 = g["T"] * 1.01 + 0.003
    for n in (1, 2):
        d.set(capi.F.TRACER, np.ascontiguousarray(T0[n - 1]), n=n, level=2)
    for n in (1, 2):
        Tm1 = g["T"][n - 1].copy()
        Tt = np.ascontiguousarray(T0[n - 1])
        d.zero_th_tendency(n)
        d.horz_advect_tracer(n, 1, 2, 3600.0)
        got_h = d.get(capi.F.TH_TENDENCY, n=n)
        ref_h = O.horz_advect_quicker(dims, g, q, Tm1, Tt, tl[n - 1], bool(limit_with_upwind))
        assert equal(got_h, ref_h), diff_report(got_h, ref_h)
        d.vert_advect_tracer(n, 1, 2, 3600.0)
        got = d.get(capi.F.TH_TENDENCY, n=n)
        ref = ref_h + O.vert_advect_quicker(dims, g, q, Tm1, Tt, tl[n - 1])
        assert equal(got, ref), diff_report(got, ref)


@pytest.mark.parametrize("case", [(6, 5, 1, False, False), (2, 3, 2, True, True), (5, 4, 3, True, False),
                                  (130, 7, 33, True, False)])
def test_psom_small_and_odd_domains(env, case):
    """PSOM on one-level columns, two-cell periodic rings, and a row longer than one
    x segment with more levels than one z segment: every value equal after three calls."""
    capi, O = env
    ni, nj, nk, cx, cy = case
    sp = spec(ni=ni, nj=nj, nk=nk, cyclic_x=cx, cyclic_y=cy, ntr=1, seed=ni * 7 + nk, continent=None)
    dom, d, g, dims = setup(env, sp, scheme=capi.ADVECT_PSOM)
    d.set_psom_limit(1, True)
    mom = np.zeros((9,) + g["T"][0].shape)
    for itt0 in range(3):
        d.set_itt0(itt0)
        d.zero_th_tendency(1)
        d.horz_advect_tracer(1, 1, 1, 3600.0)
        got = d.get(capi.F.TH_TENDENCY, n=1)
        ref, _ = O.advect_psom(dims, g, g["T"][0].copy(), 3600.0, mom, itt0=itt0)
        assert equal(got, ref), f"call {itt0}: {diff_report(got, ref)}"
    inner = (slice(None), slice(1, -1), slice(1, -1))
    for q in range(9):
        got = d.get(capi.F.PSOM_SX + q, n=1).reshape(g["T"][0].shape)[inner]
        assert equal(got, mom[q][inner]), q


@pytest.mark.parametrize("limit_with_upwind", [0, 1])
@pytest.mark.parametrize("cyclic_x,cyclic_y", [(False, False), (True, False), (True, True)])
def test_quickmom3_matches(env, cyclic_x, cyclic_y, limit_with_upwind):
    """Horizontal ADVECT_QUICKMOM3 (horz_advect_tracer_quickmom3, ocean_tracer_advect.F90:
    2665-2780; the northern second neighbour clamped to jec) with vertical Quicker,
    tmask_limit non-trivial; the vertical QuickMOM3 is refused (undefined at k = nk)."""
    capi, O = env
    sp = spec(cyclic_x=cyclic_x, cyclic_y=cyclic_y, ntr=2, seed=6)
    opts = capi.default_options(limit_with_upwind=limit_with_upwind)
    limits = [(2.0, 20.0), (34.6, 35.3)]
    dom, d, g, dims = setup(env, sp, scheme=capi.ADVECT_QUICKER, options=opts, limits=limits)
    for n, lim in zip((1, 2), limits):
        d.set_tracer_scheme(n, capi.ADVECT_QUICKMOM3, capi.ADVECT_QUICKER, *lim)
    with pytest.raises(capi.Mom5GpuError) as e:
        d.set_tracer_scheme(1, capi.ADVECT_QUICKMOM3, capi.ADVECT_QUICKMOM3, *limits[0])
    assert e.value.status == capi.EUNSUPPORTED
    q = O.quicker_init(dims, g, dom.dzt.numpy())
    d.compute_tmask_limit(1, 1, 2)
    tl = [O.compute_tmask_limit(dims, g, g["T"][n].copy(), *limits[n]) for n in range(2)]
    O.tmask_limit_ts_same(dims, tl[0], tl[1])
    T0 = g["T"] * 1.01 + 0.003
    for n in (1, 2):
        d.set(capi.F.TRACER, np.ascontiguousarray(T0[n - 1]), n=n, level=2)
    for n in (1, 2):
        Tm1 = g["T"][n - 1].copy()
        Tt = np.ascontiguousarray(T0[n - 1])
        d.zero_th_tendency(n)
        d.horz_advect_tracer(n, 1, 2, 3600.0)
        got_h = d.get(capi.F.TH_TENDENCY, n=n)
        ref_h = O.horz_advect_quickmom3(dims, g, q, Tm1, Tt, tl[n - 1], bool(limit_with_upwind))
        assert equal(got_h, ref_h), diff_report(got_h, ref_h)
        d.vert_advect_tracer(n, 1, 2, 3600.0)
        got = d.get(capi.F.TH_TENDENCY, n=n)
        ref = ref_h + O.vert_advect_quicker(dims, g, q, Tm1, Tt, tl[n - 1])
        assert equal(got, ref), diff_report(got, ref)


def _oracle_steps(O, dims, g, nsteps, dt, limiter=1.0):
    T = [g["T"][n].copy() for n in range(g["T"].shape[0])]
    for _ in range(nsteps):
        for n in range(len(T)):
            th = O.advect_mdfl_sweby(dims, g, T[n], dt, limiter)
            T[n] = O.update_tracer(dims, g, T[n], th, dt)
    return T


@pytest.mark.parametrize("cyclic_x", [False, True])
def test_multistep_advection_matches(env, cyclic_x):
    """20 two-level steps of update_advection_only (ocean_tracer.F90:2618-2649)
    with the explicit update (:2341-2350) and halo update; every value equal."""
    capi, O = env
    sp = spec(cyclic_x=cyclic_x, ntr=3, seed=21)
    dom, d, g, dims = setup(env, sp)
    dt = 6 * 3600.0
    nsteps = 20
    tau = 1
    for s in range(nsteps):
        taup1 = 3 - tau
        d.tracer_advection_step(tau, tau, taup1, dt)
        tau = taup1
    ref = _oracle_steps(O, dims, g, nsteps, dt)
    for n in range(1, sp.ntracers + 1):
        got = d.get(capi.F.TRACER, n=n, level=tau)
        assert equal(got, ref[n - 1]), f"tracer {n}: {diff_report(got, ref[n - 1])}"


@pytest.mark.parametrize("ntr", [7, 10, 13])
def test_tracer_chunks_match(env, ntr):
    """Whole-step advection of many tracers: one launch set covers up to 10
    tracers, more are split into equal chunks (13 -> 7 + 6); 3 steps, every
    value equal to the oracle."""
    capi, O = env
    sp = spec(ni=33, nj=21, nk=7, cyclic_x=True, ntr=ntr, seed=31)
    dom, d, g, dims = setup(env, sp)
    dt = 6 * 3600.0
    tau = 1
    for s in range(3):
        d.tracer_advection_step(tau, tau, 3 - tau, dt)
        tau = 3 - tau
    ref = _oracle_steps(O, dims, g, 3, dt)
    for n in range(1, ntr + 1):
        got = d.get(capi.F.TRACER, n=n, level=tau)
        assert equal(got, ref[n - 1]), f"tracer {n}: {diff_report(got, ref[n - 1])}"


def test_autotune_keeps_parity(env):
    """mom5gpu_autotune changes only launch shapes: after it, steps still equal
    the oracle (its trials overwrite time level 2, which the next step rewrites)."""
    capi, O = env
    sp = spec(cyclic_x=True, ntr=3, seed=23)
    dom, d, g, dims = setup(env, sp)
    dt = 6 * 3600.0
    report = d.autotune(dt)
    assert "chosen tj=" in report, report
    tau = 1
    for s in range(4):
        d.tracer_advection_step(tau, tau, 3 - tau, dt)
        tau = 3 - tau
    ref = _oracle_steps(O, dims, g, 4, dt)
    for n in range(1, sp.ntracers + 1):
        got = d.get(capi.F.TRACER, n=n, level=tau)
        assert equal(got, ref[n - 1]), f"tracer {n}: {diff_report(got, ref[n - 1])}"


def test_c0_hundred_steps_matches_and_conserves(env):
    """Config C0 (120x80x30, 2 tracers, MDFL Sweby, dt = 3600 s, 100 steps):
    identical to the restatement, global content conserved to roundoff."""
    capi, O = env
    sp = grid.config_c0()
    dom, d, g, dims = setup(env, sp)
    dt = 3600.0
    c0 = [d.global_tracer_content(n, 1) for n in (1, 2)]
    tau = 1
    for s in range(100):
        taup1 = 3 - tau
        d.tracer_advection_step(tau, tau, taup1, dt)
        tau = taup1
    ref = _oracle_steps(O, dims, g, 100, dt)
    for n in (1, 2):
        got = d.get(capi.F.TRACER, n=n, level=tau)
        assert equal(got, ref[n - 1]), f"tracer {n}: {diff_report(got, ref[n - 1])}"
        c1 = d.global_tracer_content(n, tau)
        assert abs(c1 - c0[n - 1]) <= 1e-12 * abs(c0[n - 1]), (c0[n - 1], c1)
        # the device's compensated sum agrees with the restatement's
        ro = O.total_tracer(dims, g, ref[n - 1])[0]
        assert abs(c1 - ro) <= 1e-14 * abs(ro)


def _baro_state(dom):
    return {k: dom[k].numpy().copy() for k in ("eta_t", "eta_t_bar", "udrho_u", "udrho_v")}


@pytest.mark.parametrize("cgrid", [False, True])
@pytest.mark.parametrize("stepping_B", [True, False])
@pytest.mark.parametrize("cyclic_x", [True, False])
def test_barotropic_matches(env, cyclic_x, stepping_B, cgrid):
    """update_ocean_barotropic, splitting branch (ocean_barotropic.F90:2763-3033)
    with pred_corr_tropic_depth_bgrid (:3225-3579) or _cgrid (:3601-3965):
    three baroclinic steps, every output field equal on the whole data domain."""
    capi, O = env
    sp = grid.DomainSpec(ni=48, nj=36, nk=1, lon0=0.0, lon1=48.0, lat0=-60.0, lat1=60.0, cyclic_x=cyclic_x,
                         hmin=None, ridge_amp=1500.0, ntracers=0, seed=9,
                         continent=None if cyclic_x else (10, 10, 6, 4))
    from mom5_gb300 import harness
    dom = grid.make_domain(sp)
    opts = capi.default_options(barotropic_time_stepping_A=int(not stepping_B),
                                barotropic_time_stepping_B=int(stepping_B))
    d = harness.load(dom, options=opts, horz_grid=capi.CGRID if cgrid else capi.BGRID)
    dtbt = 30.0
    nts = d.barotropic_init(dtuv=20 * dtbt / 2, dtbt=dtbt)
    assert nts == 20
    g = O.domain_arrays(dom)
    dims = O.dims(sp)
    st = _baro_state(dom)
    tau = 1
    names = {"eta_t_bar": capi.F.ETA_T_BAR, "udrho_u": capi.F.UDRHO_U, "udrho_v": capi.F.UDRHO_V,
             "conv_rho_ud_t": capi.F.CONV_RHO_UD_T, "eta_u": capi.F.ETA_U}
    for step in range(3):
        taup1 = 3 - tau
        d.update_ocean_barotropic(tau, taup1)
        out = O.update_ocean_barotropic(dims, g, st, nts, dtbt, time_stepping_B=stepping_B, cgrid=cgrid)
        for k, fid in names.items():
            got = d.get(fid, level=taup1)
            assert equal(got, out[k]), f"step {step} {k}: {diff_report(got, out[k])}"
        for k, fid in (("ps", capi.F.PS), ("grad_ps_x", capi.F.GRAD_PS_X), ("grad_ps_y", capi.F.GRAD_PS_Y)):
            got = d.get(fid)
            assert equal(got, out[k]), f"step {step} {k}: {diff_report(got, out[k])}"
        # next step starts from these (eta_t is not advanced by the barotropic routine)
        st = {"eta_t": st["eta_t"], "eta_t_bar": out["eta_t_bar"], "udrho_u": out["udrho_u"],
              "udrho_v": out["udrho_v"]}
        d.set(capi.F.ETA_T, np.ascontiguousarray(st["eta_t"]), level=taup1)
        tau = taup1
    assert np.abs(out["eta_t_bar"]).max() > 0 and np.abs(out["udrho_u"]).max() > 0


@pytest.mark.parametrize("fusion", [0, 1, 2])
@pytest.mark.parametrize("cyclic_x,cyclic_y,stepping_B", [(True, False, True), (False, False, False),
                                                         (True, True, True)])
def test_barotropic_subcycle_forms_match(env, fusion, cyclic_x, cyclic_y, stepping_B):
    """The exact B-grid subcycle as three launches, as one launch per subcycle
    (ring of pressure and transports recomputed per tile), as one cooperative
    launch for all subcycles (grid barriers between the phases), on a domain of
    several tiles with partial ones: every output equal to the restatement over
    three baroclinic steps, also when the form changes between steps."""
    capi, O = env
    sp = grid.DomainSpec(ni=150, nj=29, nk=1, lon0=0.0, lon1=150.0, lat0=-55.0, lat1=55.0, cyclic_x=cyclic_x,
                         cyclic_y=cyclic_y, hmin=None, ridge_amp=1200.0, ntracers=0, seed=71,
                         continent=None if cyclic_y else (40, 8, 9, 6))
    from mom5_gb300 import harness
    dom = grid.make_domain(sp)
    opts = capi.default_options(barotropic_time_stepping_A=int(not stepping_B),
                                barotropic_time_stepping_B=int(stepping_B))
    d = harness.load(dom, options=opts)
    nts = d.barotropic_init(dtuv=300.0, dtbt=30.0)
    g = O.domain_arrays(dom)
    dims = O.dims(sp)
    st = _baro_state(dom)
    tau = 1
    for step, mode in enumerate((fusion, fusion, (fusion + 2) % 3)):
        d.set_barotropic_fusion(mode)
        taup1 = 3 - tau
        d.update_ocean_barotropic(tau, taup1)
        out = O.update_ocean_barotropic(dims, g, st, nts, 30.0, time_stepping_B=stepping_B)
        for k, fid in (("eta_t_bar", capi.F.ETA_T_BAR), ("udrho_u", capi.F.UDRHO_U), ("udrho_v", capi.F.UDRHO_V),
                       ("conv_rho_ud_t", capi.F.CONV_RHO_UD_T), ("eta_u", capi.F.ETA_U)):
            got = d.get(fid, level=taup1)
            assert equal(got, out[k]), f"step {step} form {mode} {k}: {diff_report(got, out[k])}"
        st = {"eta_t": st["eta_t"], "eta_t_bar": out["eta_t_bar"], "udrho_u": out["udrho_u"],
              "udrho_v": out["udrho_v"]}
        d.set(capi.F.ETA_T, np.ascontiguousarray(st["eta_t"]), level=taup1)
        tau = taup1
    for bad in (-1, 3):
        with pytest.raises(capi.Mom5GpuError):
            d.set_barotropic_fusion(bad)


def test_barotropic_graph_follows_arguments(env):
    """The subcycle loop is replayed from a CUDA graph keyed by its kernel
    arguments: repeated level pairs replay, a new dtbt (new nts and step
    constants) captures a new graph; every call equals the restatement."""
    capi, O = env
    sp = grid.DomainSpec(ni=40, nj=30, nk=1, lon0=0.0, lon1=40.0, lat0=-50.0, lat1=50.0, cyclic_x=True,
                         hmin=None, ridge_amp=1000.0, ntracers=0, seed=21)
    from mom5_gb300 import harness
    dom = grid.make_domain(sp)
    d = harness.load(dom, options=capi.default_options(barotropic_time_stepping_B=1))
    g = O.domain_arrays(dom)
    dims = O.dims(sp)
    st = _baro_state(dom)
    tau = 1
    for step, dtbt in enumerate((30.0, 30.0, 30.0, 20.0, 20.0, 30.0)):
        nts = d.barotropic_init(dtuv=300.0, dtbt=dtbt)
        taup1 = 3 - tau
        d.update_ocean_barotropic(tau, taup1)
        out = O.update_ocean_barotropic(dims, g, st, nts, dtbt, time_stepping_B=True)
        for k, fid in (("eta_t_bar", capi.F.ETA_T_BAR), ("udrho_u", capi.F.UDRHO_U), ("udrho_v", capi.F.UDRHO_V)):
            got = d.get(fid, level=taup1)
            assert equal(got, out[k]), f"step {step} dtbt {dtbt} {k}: {diff_report(got, out[k])}"
        st = {"eta_t": st["eta_t"], "eta_t_bar": out["eta_t_bar"], "udrho_u": out["udrho_u"],
              "udrho_v": out["udrho_v"]}
        d.set(capi.F.ETA_T, np.ascontiguousarray(st["eta_t"]), level=taup1)
        tau = taup1


def test_barotropic_cfl_check(env):
    """The gravity-wave check of ocean_barotropic_init (:1595-1662) rejects a
    step above the limit and accepts one below it."""
    capi, O = env
    sp = grid.config_c1()
    from mom5_gb300 import harness
    dom = grid.make_domain(sp)
    opts = capi.default_options(barotropic_time_stepping_B=1)
    d = harness.load(dom, options=opts)
    lim = grid.barotropic_cfl_limit(dom)
    assert 60.0 < lim < 200.0
    with pytest.raises(capi.Mom5GpuError) as e:
        d.barotropic_init(dtuv=80 * (lim + 20) / 2, dtbt=lim + 20)
    assert e.value.status == capi.ECFL
    assert d.barotropic_init(dtuv=2700.0, dtbt=67.5) == 80


def test_eta_tendency_and_update(env):
    """eta_and_pbot_tendency (:2683-2690) and eta_and_pbot_update (:2314-2330)."""
    capi, O = env
    sp = grid.DomainSpec(ni=30, nj=20, nk=1, cyclic_x=True, hmin=None, ridge_amp=1000.0, ntracers=0, seed=2)
    from mom5_gb300 import harness
    dom = grid.make_domain(sp)
    d = harness.load(dom)
    g = O.domain_arrays(dom)
    dims = O.dims(sp)
    rng = np.random.default_rng(0)
    conv = rng.normal(size=g["eta_t"].shape) * 1e-3
    pme = rng.normal(size=g["eta_t"].shape) * 1e-4
    g["pme"] = pme
    d.set(capi.F.CONV_RHO_UD_T, conv, level=1)
    d.set(capi.F.PME, pme)
    d.eta_and_pbot_tendency(1)
    ref = O.eta_and_pbot_tendency(dims, g, conv)
    assert equal(d.get(capi.F.DETA_DT), ref)
    d.eta_and_pbot_update(1, 2, 5400.0)
    ref_e = O.eta_and_pbot_update(dims, g["eta_t"].copy(), ref, 5400.0)
    got = d.get(capi.F.ETA_T, level=2)
    sl = (slice(1, -1), slice(0, None))  # compute rows; halo columns follow the cyclic update
    assert equal(got.reshape(ref_e.shape)[sl], ref_e[sl])


@pytest.mark.parametrize("case", ["tiny", "strip", "column1", "all_land", "deep_only"])
def test_edge_domains(env, case):
    """Small and degenerate domains: 6x5x4, a one-cell land strip, kmt = 1
    columns, an all-land box, and a single-level ocean."""
    capi, O = env
    if case == "tiny":
        sp = spec(ni=6, nj=5, nk=4, continent=None, ntr=2, seed=31)
    elif case == "strip":
        sp = spec(ni=16, nj=12, nk=5, continent=(7, 0, 1, 12), ntr=2, seed=32, cyclic_x=True)
    elif case == "column1":
        sp = spec(ni=14, nj=10, nk=6, continent=None, ntr=2, seed=33, hmin=5.0)
    elif case == "all_land":
        sp = spec(ni=8, nj=6, nk=3, continent=(0, 0, 8, 6), ntr=1, seed=34)
    else:
        sp = spec(ni=12, nj=10, nk=1, continent=(3, 3, 2, 2), ntr=2, seed=35)
    dom, d, g, dims = setup(env, sp)
    dt = 3600.0 * 4
    tau = 1
    for s in range(3):
        d.tracer_advection_step(tau, tau, 3 - tau, dt)
        tau = 3 - tau
    ref = _oracle_steps(O, dims, g, 3, dt)
    for n in range(1, sp.ntracers + 1):
        got = d.get(capi.F.TRACER, n=n, level=tau)
        assert equal(got, ref[n - 1]), f"{case} tracer {n}: {diff_report(got, ref[n - 1])}"
        assert d.check_finite(n, tau)


def test_errors_are_status_codes(env):
    """Bad arguments come back as negative status codes with a message; nothing aborts."""
    capi, O = env
    sp = spec(ni=8, nj=6, nk=3, ntr=1, continent=None)
    dom, d, g, dims = setup(env, sp)
    with pytest.raises(capi.Mom5GpuError) as e:
        d.horz_advect_tracer(2, 1, 1, 100.0)
    assert e.value.status == capi.EINVAL and "tracer" in str(e.value)
    with pytest.raises(capi.Mom5GpuError) as e:
        d.update_tracer(1, 0, 2, 100.0)
    assert e.value.status == capi.EINVAL
    with pytest.raises(capi.Mom5GpuError) as e:
        d.update_ocean_barotropic(1, 2)
    assert e.value.status == capi.ESTATE
    with pytest.raises(capi.Mom5GpuError) as e:
        d.set_tracer_scheme(1, capi.ADVECT_MDFL_SWEBY, capi.ADVECT_UPWIND)
    assert e.value.status == capi.EINVAL
    with pytest.raises(capi.Mom5GpuError) as e:
        d.barotropic_init(1000.0, 100.0)  # neither time-stepping flag set
    assert e.value.status == capi.EINVAL
