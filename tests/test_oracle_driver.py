"""The CPU baseline's stepping loop (oracle/mom5_oracle.c orc_run_steps) does
exactly the arithmetic of the restatement's per-routine entry points: MDFL
Sweby + explicit update per tracer, then update_ocean_barotropic, with the
scheme scratch held across steps instead of allocated per call."""
import numpy as np
import pytest

from mom5_gb300 import grid


@pytest.mark.parametrize("cyclic_x,nsteps", [(True, 3), (False, 4)])
def test_run_steps_equals_routine_by_routine(oracle_lib, cyclic_x, nsteps):
    O = oracle_lib
    sp = grid.DomainSpec(ni=26, nj=19, nk=7, lon0=0.0, lon1=26.0, lat0=-30.0, lat1=30.0, cyclic_x=cyclic_x,
                         continent=(8, 6, 4, 3), wavelength_cells=6.0, ntracers=3, seed=17)
    dom = grid.make_domain(sp)
    g = O.domain_arrays(dom)
    dims = O.dims(sp)
    dt, nts, dtbt = 4 * 3600.0, 12, 25.0
    st = {k: g[k].copy() for k in ("eta_t", "eta_t_bar", "udrho_u", "udrho_v")}
    T = [g["T"][n].copy() for n in range(3)]
    for _ in range(nsteps):
        T = [O.update_tracer(dims, g, t, O.advect_mdfl_sweby(dims, g, t, dt), dt) for t in T]
        out = O.update_ocean_barotropic(dims, g, st, nts, dtbt)
        st = {"eta_t": st["eta_t"], "eta_t_bar": out["eta_t_bar"], "udrho_u": out["udrho_u"],
              "udrho_v": out["udrho_v"]}
    Tl = np.ascontiguousarray(g["T"]).copy()
    state = {k: g[k].copy() for k in ("eta_t", "eta_t_bar", "udrho_u", "udrho_v")}
    sec, res = O.run_steps(dims, g, Tl, dt, warmup=1, steps=nsteps - 1, nts=nts, dtbt=dtbt, state=state)
    assert sec >= 0.0
    for n in range(3):
        assert np.array_equal(Tl[n], T[n]), n
    for k in ("eta_t_bar", "udrho_u", "udrho_v", "conv_rho_ud_t", "eta_u", "ps", "grad_ps_x", "grad_ps_y"):
        assert np.array_equal(res[k], out[k]), k


def test_run_steps_barotropic_only(oracle_lib):
    O = oracle_lib
    sp = grid.DomainSpec(ni=30, nj=20, nk=1, cyclic_x=True, hmin=None, ridge_amp=1000.0, ntracers=0, seed=5)
    dom = grid.make_domain(sp)
    g = O.domain_arrays(dom)
    dims = O.dims(sp)
    st = {k: g[k].copy() for k in ("eta_t", "eta_t_bar", "udrho_u", "udrho_v")}
    for _ in range(2):
        out = O.update_ocean_barotropic(dims, g, st, 10, 30.0)
        st = {"eta_t": st["eta_t"], "eta_t_bar": out["eta_t_bar"], "udrho_u": out["udrho_u"],
              "udrho_v": out["udrho_v"]}
    state = {k: g[k].copy() for k in ("eta_t", "eta_t_bar", "udrho_u", "udrho_v")}
    sec, res = O.run_steps(dims, g, np.zeros((0, 1, 22, 32)), 0.0, warmup=0, steps=2, nts=10, dtbt=30.0,
                           state=state)
    for k in ("eta_t_bar", "udrho_u", "udrho_v", "eta_u"):
        assert np.array_equal(res[k], out[k]), k


def test_openmp_build_equals_serial(oracle_lib):
    """The CPU baseline's OpenMP build of the restatement gives the serial
    build's values bit for bit (its parallel loops have independent iterations)."""
    O = oracle_lib
    try:
        O.build_omp()
    except Exception as e:  # a compiler without OpenMP: the baseline falls back to processes
        pytest.skip(f"no OpenMP build: {e}")
    sp = grid.DomainSpec(ni=41, nj=23, nk=9, lon0=0.0, lon1=41.0, lat0=-30.0, lat1=30.0, cyclic_x=True,
                         continent=(8, 6, 4, 3), wavelength_cells=6.0, ntracers=2, seed=19)
    dom = grid.make_domain(sp)
    g = O.domain_arrays(dom)
    dims = O.dims(sp)
    st = {k: g[k].copy() for k in ("eta_t", "eta_t_bar", "udrho_u", "udrho_v")}
    T1 = np.ascontiguousarray(g["T"]).copy()
    T2 = T1.copy()
    _, r1 = O.run_steps(dims, g, T1, 7200.0, steps=3, nts=8, dtbt=25.0, state=dict(st))
    _, r2 = O.run_steps(dims, g, T2, 7200.0, steps=3, nts=8, dtbt=25.0, state=dict(st), threaded=True)
    assert np.array_equal(T1, T2)
    for k in r1:
        assert np.array_equal(r1[k], r2[k]), k
