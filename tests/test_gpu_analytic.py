"""Known answers from the advection equation through the C ABI (tests/analytic.py):
on a uniform box in uniform flow, one mom5gpu_tracer_advection_step of MDFL
Sweby translates a cubic exactly, upwind a linear profile, and the centred
2nd/4th/6th-order and Quicker schemes take the exact forward-Euler step of a
quadratic -- to FP64 roundoff on the drop-in path, within the precision form's
FP32 tolerance for MDFL in that form; and from the barotropic momentum equation
(a uniform surface slope; an inertial oscillation on an f-plane)."""
import numpy as np
import pytest

import analytic as A

pytestmark = pytest.mark.gpu

CASES = [("mdfl_sweby", "cubic"), ("upwind", "linear"), ("quicker", "quadratic"), ("centred2", "quadratic"),
         ("centred4", "quadratic"), ("centred6", "quadratic")]


def _scheme_id(capi, name):
    return {"mdfl_sweby": capi.ADVECT_MDFL_SWEBY, "upwind": capi.ADVECT_UPWIND, "quicker": capi.ADVECT_QUICKER,
            "centred2": capi.ADVECT_2ND_ORDER, "centred4": capi.ADVECT_4TH_ORDER,
            "centred6": capi.ADVECT_6TH_ORDER}[name]


def _step(capi, dom, scheme, dt, precision=None):
    from mom5_gb300 import harness
    opts = capi.default_options(precision=precision) if precision is not None else None
    d = harness.load(dom, options=opts, scheme=_scheme_id(capi, scheme))
    d.tracer_advection_step(1, 1, 2, dt)
    T = d.get(capi.F.TRACER, n=1, level=2).reshape(tuple(dom["T"][0].shape))
    d.close()
    return T


@pytest.mark.parametrize("vel", [(0.4, -0.3, 1e-3), (-0.2, 0.25, -2e-3), (0.0, 0.0, 1e-3)])
@pytest.mark.parametrize("scheme,kind", CASES)
def test_drop_in_matches_the_advection_equation(gpu_lib, scheme, kind, vel):
    capi = gpu_lib
    u, v, w = vel
    dom, spacing = A.make_box(kind, u, v, w)
    dt = 2000.0
    T = _step(capi, dom, scheme, dt)
    E = A.expected(kind, T.shape, u, v, w, dt, spacing)
    assert A.rel_err(T, E) < 2e-15
    assert A.rel_err(T, dom["T"][0].numpy()) > 1e-4


@pytest.mark.parametrize("vel", [(0.4, 0.3, 5e-4), (-0.4, -0.3, -5e-4)])
def test_mdfl_at_courant_one_moves_any_field_one_cell(gpu_lib, vel):
    """Drop-in MDFL at Courant number 1: a random tracer moves exactly one cell."""
    capi = gpu_lib
    u, v, w = vel
    dom, _, T0 = A.make_random_box(u, v, w)
    T = _step(capi, dom, "mdfl_sweby", A.CFL1_DT)
    assert abs(A.interior(T) - A.interior(A.shifted_one_cell(T0, u, v, w))).max() < 2e-15


@pytest.mark.parametrize("vel", [(0.4, -0.3, 1e-3), (-0.2, 0.25, -2e-3)])
def test_precision_form_matches_the_advection_equation(gpu_lib, vel):
    capi = gpu_lib
    u, v, w = vel
    dom, spacing = A.make_box("cubic", u, v, w, ni=62, nj=40)  # several TMA tiles (ni even)
    dt = 2000.0
    T = _step(capi, dom, "mdfl_sweby", dt, precision=capi.PRECISION_MIXED)
    E = A.expected("cubic", T.shape, u, v, w, dt, spacing)
    assert A.rel_err(T, E) < 1e-6


@pytest.mark.parametrize("fusion", [0, 1, 2])
@pytest.mark.parametrize("stepping_B", [False, True])
def test_barotropic_matches_the_momentum_equation(gpu_lib, stepping_B, fusion):
    """A sea surface of uniform slope, f = 0, no forcing, flat bottom: the
    exact B-grid subcycles (each form) accelerate the transports uniformly at
    -H rho0 g grad(eta) and the step returns their time average; eta keeps its
    value away from the walls."""
    capi = gpu_lib
    from mom5_gb300 import harness
    sx, sy, u0, v0, nts, dtbt = 1e-3, -5e-4, 100.0, -50.0, 10, 20.0
    dom, spacing = A.make_baro_box(sx, sy, u0, v0)
    opts = capi.default_options(barotropic_time_stepping_A=int(not stepping_B),
                                barotropic_time_stepping_B=int(stepping_B))
    d = harness.load(dom, options=opts)
    assert d.barotropic_init(dtuv=nts * dtbt / 2, dtbt=dtbt) == nts
    d.set_barotropic_fusion(fusion)
    d.update_ocean_barotropic(1, 2)
    shape = tuple(dom["eta_t"].shape)
    get = lambda fid: d.get(fid, level=2).reshape(shape)
    eu, ev = A.baro_expected(sx, sy, u0, v0, nts, dtbt, spacing, stepping_B)
    assert abs(A.interior2(get(capi.F.UDRHO_U)) - eu).max() <= 1e-10 * abs(eu)
    assert abs(A.interior2(get(capi.F.UDRHO_V)) - ev).max() <= 1e-10 * abs(ev)
    assert abs(A.interior2(get(capi.F.ETA_T_BAR)) - A.interior2(dom["eta_t"].numpy())).max() <= 1e-12
    d.close()


@pytest.mark.parametrize("grid_kind,fusion,precision", [("b", 0, 0), ("b", 1, 0), ("b", 2, 0), ("c", 0, 0),
                                                        ("b", 0, 1), ("b", 1, 1)])
@pytest.mark.parametrize("stepping_B", [False, True])
def test_barotropic_inertial_oscillation(gpu_lib, grid_kind, fusion, precision, stepping_B):
    """A flat sea surface and uniform transports on an f-plane (doubly periodic):
    the transports only rotate, Crank-Nicolson on the B grid (every subcycle
    form), Adams-Bashforth-3 on the C grid, and the step returns their time
    average (tests/analytic.py); 1e-12 of the amplitude for the exact path,
    1e-6 for the precision form."""
    capi = gpu_lib
    from mom5_gb300 import harness
    f, u0, v0, nts, dtbt = 1.4e-4, 100.0, -50.0, 20, 20.0
    dom, spacing = A.make_baro_box(0.0, 0.0, u0, v0, f=f, periodic=True)
    opts = capi.default_options(barotropic_time_stepping_A=int(not stepping_B),
                                barotropic_time_stepping_B=int(stepping_B),
                                precision=capi.PRECISION_MIXED if precision else capi.PRECISION_FP64)
    d = harness.load(dom, options=opts, horz_grid=capi.CGRID if grid_kind == "c" else capi.BGRID)
    assert d.barotropic_init(dtuv=nts * dtbt / 2, dtbt=dtbt) == nts
    d.set_barotropic_fusion(fusion)
    d.update_ocean_barotropic(1, 2)
    shape = tuple(dom["eta_t"].shape)
    get = lambda fid: d.get(fid, level=2).reshape(shape)
    eu, ev = A.baro_inertial_expected(f, u0, v0, nts, dtbt, stepping_B, cgrid=grid_kind == "c")
    tol = (1e-6 if precision else 1e-12) * np.hypot(eu, ev)
    assert abs(A.interior2(get(capi.F.UDRHO_U)) - eu).max() <= tol
    assert abs(A.interior2(get(capi.F.UDRHO_V)) - ev).max() <= tol
    assert abs(A.interior2(get(capi.F.ETA_T_BAR)) - 0.5).max() <= (1e-9 if precision else 1e-13)
    d.close()


@pytest.mark.parametrize("axis", [2, 1, 0])
@pytest.mark.parametrize("case", ["line", "slope", "one", "zero", "slope_negative_u", "one_negative_u"])
def test_sweby_limiter_branches(gpu_lib, case, axis):
    """The Sweby limiter on each of its branches (tests/analytic.py): one step
    of the drop-in equals the 1-D flux form with the branch's limiter value to
    1e-12 per cell (x, y and z passes)."""
    capi = gpu_lib
    dom, E, _ = A.make_limiter_box(case, axis)
    T = _step(capi, dom, "mdfl_sweby", 2000.0)
    assert A.rel_err_cells(T, E, vertical=axis == 0) < 1e-12


@pytest.mark.parametrize("axis", [1, 0])
@pytest.mark.parametrize("case", ["line", "slope", "one", "zero", "slope_negative_u", "one_negative_u"])
def test_sweby_limiter_branches_precision_form(gpu_lib, case, axis):
    """The same limiter cases through the precision form's TMA-staged tiles
    (a box 62 wide; flow along y or z, 32 or 30 cells, so that the profile stays
    within FP32's range): within the form's 1e-6 of the field's maximum."""
    capi = gpu_lib
    dom, E, _ = A.make_limiter_box(case, axis, ni=62, nj=30)
    T = _step(capi, dom, "mdfl_sweby", 2000.0, precision=capi.PRECISION_MIXED)
    assert A.rel_err_side(T, E, vertical=axis == 0) < 1e-6
