"""ctypes front end of the C restatement in mom5_oracle.c.

TEST INFRASTRUCTURE ONLY: used by tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of bench.py to check the CUDA library.  The shipped library
never imports this module.

All arrays are numpy float64 in the reference's data-domain layout (halo 1,
Fortran column-major == C-ordered ``(nk, nj+2, ni+2)``).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Dict

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libmom5oracle.so")
_lib = None

DP = C.POINTER(C.c_double)


class Dims(C.Structure):
    _fields_ = [("ni", C.c_int), ("nj", C.c_int), ("nk", C.c_int), ("cyclic_x", C.c_int), ("cyclic_y", C.c_int)]


class Quicker(C.Structure):
    _fields_ = [(n, DP) for n in ("quick_x", "quick_y", "curv_xp", "curv_xn", "curv_yp", "curv_yn",
                                  "quick_z", "curv_zp", "curv_zn", "tmask_quick")]


class BaroParams(C.Structure):
    _fields_ = [("nts", C.c_int), ("dtbt", C.c_double), ("pred_corr_gamma", C.c_double), ("rho0", C.c_double),
                ("time_stepping_B", C.c_int), ("initsum_with_bar", C.c_int), ("cgrid", C.c_int)]


BARO_IO_FIELDS = ["tmask1", "umask1", "f", "dxu", "dyu", "dxur", "dyur", "dat", "datr", "dxter", "dytnr",
                  "tmasken_e1", "tmasken_n1", "dte", "dtw", "dus", "dun", "daur",
                  "patm", "pme", "river", "source", "eta_smooth", "thicku", "thicken_e", "thicken_n",
                  "forcing_u", "forcing_v", "rho_g",
                  "eta_t_tau", "eta_t_bar_tau", "udrho_u_tau", "udrho_v_tau",
                  "out_eta_t_bar", "out_udrho_u", "out_udrho_v", "out_conv_rho_ud_t", "out_eta_u", "out_ps",
                  "out_grad_ps_x", "out_grad_ps_y"]


class BaroIO(C.Structure):
    _fields_ = [(n, DP) for n in BARO_IO_FIELDS]


_OMP_PATH = os.path.join(_HERE, "_build", "libmom5oracle_omp.so")
_lib_omp = None


def build() -> str:
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def build_omp() -> str:
    """The OpenMP build of the same source (the CPU baseline's); raises if the
    compiler has no OpenMP."""
    subprocess.run(["make", "-s", "-C", _HERE, "omp"], check=True)
    return _OMP_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        _lib = C.CDLL(_LIB_PATH)
        _lib.orc_area_integral.restype = C.c_double
    return _lib


def lib_omp():
    global _lib_omp
    if _lib_omp is None:
        if not os.path.exists(_OMP_PATH):
            build_omp()
        _lib_omp = C.CDLL(_OMP_PATH)
    return _lib_omp


def p(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"], (a.dtype, a.flags)
    return a.ctypes.data_as(DP)


def dims(spec) -> Dims:
    return Dims(spec.ni, spec.nj, spec.nk, int(spec.cyclic_x), int(spec.cyclic_y))


def np64(t) -> np.ndarray:
    """torch tensor or array -> contiguous float64 numpy copy."""
    if hasattr(t, "detach"):
        t = t.detach().cpu().numpy()
    return np.ascontiguousarray(t, dtype=np.float64)


# ----------------------------------------------------------------------------- wrappers
def horz_advect_upwind(d: Dims, g: Dict[str, np.ndarray], T: np.ndarray) -> np.ndarray:
    out = np.zeros_like(T)
    lib().orc_horz_advect_upwind(C.byref(d), p(g["tmask"]), p(g["dyte"]), p(g["dxtn"]), p(g["datr"]),
                                 p(g["uhrho_et"]), p(g["vhrho_nt"]), p(T), p(out))
    return out


def vert_advect_upwind(d: Dims, g, T):
    out = np.zeros_like(T)
    lib().orc_vert_advect_upwind(C.byref(d), p(g["tmask"]), p(g["wrho_bt"]), p(T), p(out))
    return out


def horz_advect_centred(d: Dims, g, T, order):
    """wrk1 of the 2nd/4th/6th-order horizontal schemes (T at tau)."""
    out = np.zeros_like(T)
    lib().orc_horz_advect_centred(C.byref(d), int(order), p(g["tmask"]), p(g["dyte"]), p(g["dxtn"]), p(g["datr"]),
                                  p(g["uhrho_et"]), p(g["vhrho_nt"]), p(T), p(out))
    return out


def vert_advect_centred(d: Dims, g, T, order, kmt):
    out = np.zeros_like(T)
    k = np.ascontiguousarray(kmt, dtype=np.int32)
    lib().orc_vert_advect_centred(C.byref(d), int(order), p(g["tmask"]), k.ctypes.data_as(C.POINTER(C.c_int)),
                                  p(g["wrho_bt"]), p(T), p(out))
    return out


def advect_mdfl_sup_b(d: Dims, g, T, dtime):
    """wrk1 = -advect_tracer_mdfl_sup_b(...)."""
    out = np.zeros_like(T)
    lib().orc_advect_mdfl_sup_b(C.byref(d), C.c_double(dtime), p(g["tmask"]), p(g["dat"]), p(g["datr"]),
                                p(g["dxte"]), p(g["dyte"]), p(g["dxtn"]), p(g["dytn"]), p(g["uhrho_et"]),
                                p(g["vhrho_nt"]), p(g["wrho_bt"]), p(g["rho_dzt"]), p(np.ascontiguousarray(T)), p(out))
    return out


def advect_mdppm(d: Dims, g, T, dtime, limiter=2):
    """wrk1 = -advect_tracer_mdppm(...) for ppm_hlimiter = limiter (1 cw84, 2 ifc, 3 sh)."""
    out = np.zeros_like(T)
    lib().orc_advect_mdppm(C.byref(d), int(limiter), C.c_double(dtime), p(g["tmask"]), p(g["dat"]), p(g["datr"]),
                           p(g["dxte"]), p(g["dyte"]), p(g["dxtn"]), p(g["dytn"]), p(g["uhrho_et"]),
                           p(g["vhrho_nt"]), p(g["wrho_bt"]), p(g["rho_dzt"]), p(np.ascontiguousarray(T)), p(out))
    return out


PSOM_MOMENTS = ("sx", "sxx", "sy", "syy", "sz", "szz", "sxy", "sxz", "syz")


def advect_psom(d: Dims, g, T, dtime, moments, itt0=0, limit=True, prather=False, rho_dzt=None):
    """wrk1 = -advect_tracer_psom(...) (T and rho_dzt at taum1).  ``moments`` is the
    (9, nk, nj+2, ni+2) array of Tracer%sx..syz in PSOM_MOMENTS order, updated in
    place; returns (wrk1, s0)."""
    assert moments.dtype == np.float64 and moments.flags["C_CONTIGUOUS"] and moments.shape[0] == 9
    out = np.zeros_like(T)
    s0 = np.zeros_like(T)
    rdz = g["rho_dzt"] if rho_dzt is None else np.ascontiguousarray(rho_dzt)
    lib().orc_advect_psom(C.byref(d), C.c_long(int(itt0)), int(bool(limit)), int(bool(prather)), C.c_double(dtime),
                          p(g["tmask"]), p(g["dat"]), p(g["datr"]), p(g["dxtn"]), p(g["dyte"]), p(g["uhrho_et"]),
                          p(g["vhrho_nt"]), p(g["wrho_bt"]), p(rdz), p(np.ascontiguousarray(T)), p(s0),
                          p(moments), p(out))
    return out, s0


def quicker_init(d: Dims, g, dzt: np.ndarray):
    nxd, nyd, nk = d.ni + 2, d.nj + 2, d.nk
    q = {"quick_x": np.zeros((2, nyd, nxd)), "quick_y": np.zeros((2, nyd, nxd)),
         "curv_xp": np.zeros((3, nyd, nxd)), "curv_xn": np.zeros((3, nyd, nxd)),
         "curv_yp": np.zeros((3, nyd, nxd)), "curv_yn": np.zeros((3, nyd, nxd)),
         "quick_z": np.zeros((2, nk)), "curv_zp": np.zeros((3, nk)), "curv_zn": np.zeros((3, nk)),
         "tmask_quick": np.zeros((nk, d.nj + 4, d.ni + 4))}
    qs = Quicker(*[p(q[n]) for n, _ in Quicker._fields_])
    lib().orc_quicker_init(C.byref(d), p(g["dxt"]), p(g["dyt"]), p(np64(dzt)), p(g["tmask"]), C.byref(qs))
    q["_struct"] = qs
    return q


def horz_advect_quicker(d, g, q, Tm1, T0, tmask_limit=None, limit_with_upwind=False):
    out = np.zeros_like(Tm1)
    tl = tmask_limit if tmask_limit is not None else np.zeros_like(Tm1)
    lib().orc_horz_advect_quicker(C.byref(d), int(limit_with_upwind), C.byref(q["_struct"]), p(g["tmask"]), p(tl),
                                  p(g["dyte"]), p(g["dxtn"]), p(g["datr"]), p(g["uhrho_et"]), p(g["vhrho_nt"]),
                                  p(Tm1), p(T0), p(out))
    return out


def horz_advect_quickmom3(d, g, q, Tm1, T0, tmask_limit=None, limit_with_upwind=False):
    """wrk1 = -horz_advect_tracer_quickmom3(...) (weights from quicker_init)."""
    out = np.zeros_like(Tm1)
    tl = tmask_limit if tmask_limit is not None else np.zeros_like(Tm1)
    lib().orc_horz_advect_quickmom3(C.byref(d), int(limit_with_upwind), C.byref(q["_struct"]), p(g["tmask"]), p(tl),
                                    p(g["dyte"]), p(g["dxtn"]), p(g["datr"]), p(g["uhrho_et"]), p(g["vhrho_nt"]),
                                    p(Tm1), p(T0), p(out))
    return out


def vert_advect_quicker(d, g, q, Tm1, T0, tmask_limit=None):
    out = np.zeros_like(Tm1)
    tl = tmask_limit if tmask_limit is not None else np.zeros_like(Tm1)
    lib().orc_vert_advect_quicker(C.byref(d), C.byref(q["_struct"]), p(g["tmask"]), p(tl), p(g["wrho_bt"]),
                                  p(Tm1), p(T0), p(out))
    return out


def advect_mdfl_sweby(d, g, T, dtime, sweby_limiter=1.0):
    out = np.zeros_like(T)
    lib().orc_advect_mdfl_sweby(C.byref(d), C.c_double(sweby_limiter), C.c_double(dtime), p(g["tmask"]),
                                p(g["dat"]), p(g["datr"]), p(g["dxte"]), p(g["dyte"]), p(g["dxtn"]), p(g["dytn"]),
                                p(g["uhrho_et"]), p(g["vhrho_nt"]), p(g["wrho_bt"]), p(g["rho_dzt"]), p(T), p(out))
    return out


def advect_sweby_all(d, g, Tall, dtime):
    out = np.zeros_like(Tall)
    lib().orc_advect_sweby_all(C.byref(d), int(Tall.shape[0]), C.c_double(dtime), p(g["tmask"]), p(g["dat"]),
                               p(g["datr"]), p(g["dxte"]), p(g["dyte"]), p(g["dxtn"]), p(g["dytn"]),
                               p(g["uhrho_et"]), p(g["vhrho_nt"]), p(g["wrho_bt"]), p(g["rho_dzt"]), p(Tall), p(out))
    return out


def update_tracer(d, g, Tm1, th, dtime):
    out = Tm1.copy()
    lib().orc_update_tracer(C.byref(d), C.c_double(dtime), p(g["rho_dzt"]), p(g["rho_dztr"]), p(Tm1), p(th), p(out))
    lib().orc_halo_update_3d(C.byref(d), p(out), d.nk, 3)
    return out


def compute_tmask_limit(d, g, T, tmin, tmax):
    out = np.zeros_like(T)
    lib().orc_compute_tmask_limit(C.byref(d), p(g["tmask"]), p(T), C.c_double(tmin), C.c_double(tmax), p(out))
    return out


def tmask_limit_ts_same(d, tl_t, tl_s):
    lib().orc_tmask_limit_ts_same(C.byref(d), p(tl_t), p(tl_s))


def halo_update(d, a, flags=3):
    nlev = a.shape[0] if a.ndim == 3 else 1
    lib().orc_halo_update_3d(C.byref(d), p(a), nlev, flags)


def continuity_w(d, g):
    nk = d.nk
    w = np.zeros((nk + 1, d.nj + 2, d.ni + 2))
    z = np.zeros((d.nj + 2, d.ni + 2))
    lib().orc_continuity_w(C.byref(d), p(g["tmask"]), p(g["dyte"]), p(g["dxtn"]), p(g["datr"]), p(g["uhrho_et"]),
                           p(g["vhrho_nt"]), p(z), p(z), p(w))
    return w


def ocean_advection_velocity(d, g, u, v, rho_dzu=None, rho_dzten_e=None, rho_dzten_n=None, cgrid=False,
                             rho_dzt_tendency=None, mass_source=None, pme=None, river=None):
    """ocean_advection_velocity (T-cell part): returns uhrho_et, vhrho_nt, diverge_t, wrho_bt."""
    nk = d.nk
    shp3 = (nk, d.nj + 2, d.ni + 2)
    z3 = np.zeros(shp3)
    z2 = np.zeros(shp3[1:])
    ue, vn, dv = np.zeros(shp3), np.zeros(shp3), np.zeros(shp3)
    w = np.zeros((nk + 1,) + shp3[1:])
    # the arrays stay referenced by `keep` until the call returns
    keep = [np.ascontiguousarray(a if a is not None else z, dtype=np.float64) for a, z in (
        (u, z3), (v, z3), (rho_dzu, z3), (rho_dzten_e, z3), (rho_dzten_n, z3), (g["dxu"], z2), (g["dyu"], z2),
        (g["dyte"], z2), (g["dxtn"], z2), (g.get("dxt_dxter"), z2), (g.get("dyt_dyter"), z2),
        (g.get("dxt_dxtnr"), z2), (g.get("dyt_dytnr"), z2), (g["datr"], z2), (g["tmask"], z3),
        (rho_dzt_tendency, z3), (mass_source, z3), (pme, z2), (river, z2))]
    lib().orc_ocean_advection_velocity(C.byref(d), int(cgrid), *[p(a) for a in keep], p(ue), p(vn), p(dv), p(w))
    return ue, vn, dv, w


def tracer_boundary_terms(d, g, kmt, pme, tpme, eta_smooth, pbot_smooth, th):
    """th (one tracer) after the surface and bottom source terms; returns a new array."""
    out = np.ascontiguousarray(th, dtype=np.float64).copy()
    keep = [np.ascontiguousarray(a, dtype=np.float64) for a in (pme, tpme, eta_smooth, pbot_smooth)]
    k = np.ascontiguousarray(kmt, dtype=np.int32)
    lib().orc_tracer_boundary_terms(C.byref(d), p(g["tmask"]), k.ctypes.data_as(C.POINTER(C.c_int)),
                                    *[p(a) for a in keep], p(out))
    return out


def ocean_barotropic_forcing(d, tmasken, accel, smf, bmf, zero_nonlinear=False, zero_forcing=False,
                             friction_lap=None, friction_bih=None):
    """One component of forcing_bt (ocean_barotropic.F90:3058-3141); friction_lap /
    friction_bih: that component's barotropic frictions (None: 0.0)."""
    out = np.zeros((d.nj + 2, d.ni + 2))
    keep = [np.ascontiguousarray(a, dtype=np.float64) for a in (tmasken, accel, smf, bmf)]
    fr = [None if f is None else np.ascontiguousarray(f, dtype=np.float64) for f in (friction_lap, friction_bih)]
    lib().orc_ocean_barotropic_forcing_friction(C.byref(d), int(zero_nonlinear), int(zero_forcing),
                                                *[p(a) for a in keep], *[None if f is None else p(f) for f in fr],
                                                p(out))
    return out


def bt_friction_back(d, dxu, dyu, umask1, vel_lap=0.05, vel_bih=0.01):
    """(lap_ceu_back, lap_cnu_back, bih_ceu_back, bih_cnu_back) as ocean_barotropic_init
    forms them (ocean_barotropic.F90:1306-1341)."""
    keep = [np.ascontiguousarray(a, dtype=np.float64) for a in (dxu, dyu, umask1)]
    out = [np.zeros((d.nj + 2, d.ni + 2)) for _ in range(4)]
    lib().orc_bt_friction_back(C.byref(d), *[p(a) for a in keep], C.c_double(vel_lap), C.c_double(vel_bih),
                               *[p(o) for o in out])
    return tuple(out)


def bt_friction(d, lap, bih, metrics, coefs, a):
    """(friction_lap, friction_bih, del2_vel) of one udrho component
    (ocean_barotropic.F90:3105-3113).  metrics: dyue, dxuer, dxun, dyunr, daur, umask1;
    coefs: lap_ceu_back, lap_cnu_back, lap_visc_ceu, lap_visc_cnu, bih_ceu_back,
    bih_cnu_back, bih_visc_ceu, bih_visc_cnu."""
    m = [np.ascontiguousarray(x, dtype=np.float64) for x in metrics]
    c = [np.ascontiguousarray(x, dtype=np.float64) for x in coefs]
    assert len(m) == 6 and len(c) == 8
    mp, cp = (DP * 6)(*[p(x) for x in m]), (DP * 8)(*[p(x) for x in c])
    a = np.ascontiguousarray(a, dtype=np.float64)
    out = [np.zeros((d.nj + 2, d.ni + 2)) for _ in range(3)]
    lib().orc_bt_friction(C.byref(d), int(lap), int(bih), mp, cp, p(a), *[p(o) for o in out])
    return tuple(out)


def total_tracer(d, g, T):
    r = np.zeros(2)
    lib().orc_total_tracer(C.byref(d), p(g["tmask"]), p(g["dat"]), p(g["rho_dzt"]), p(T), p(r))
    return r


def area_integral(d, g, eta):
    return lib().orc_area_integral(C.byref(d), p(g["tmask1"]), p(g["dat"]), p(eta))


def div_ud_bgrid(d, g, u, v):
    out = np.zeros_like(u)
    lib().orc_div_ud_bgrid(C.byref(d), p(u), p(v), p(g["dyu"]), p(g["dxu"]), p(g["datr"]), p(out))
    return out


def grad_baro_p(d, g, press, cgrid=False):
    gx = np.zeros_like(press)
    gy = np.zeros_like(press)
    if cgrid:
        lib().orc_grad_baro_p(C.byref(d), 1, p(press), p(g["dxter"]), p(g["dytnr"]), p(g["tmasken_e1"]),
                              p(g["tmasken_n1"]), p(gx), p(gy))
    else:
        lib().orc_grad_baro_p(C.byref(d), 0, p(press), p(g["dxur"]), p(g["dyur"]), p(g["umask1"]), p(g["umask1"]),
                              p(gx), p(gy))
    return gx, gy


def eta_and_pbot_tendency(d, g, conv_tau, rho0=1035.0):
    out = np.zeros_like(conv_tau)
    lib().orc_eta_and_pbot_tendency(C.byref(d), C.c_double(rho0), p(g["tmask1"]), p(conv_tau), p(g["pme"]),
                                    p(g["river"]), p(g["source"]), p(out))
    return out


def eta_and_pbot_update(d, eta_taum1, deta_dt, dtime):
    out = eta_taum1.copy()
    lib().orc_eta_and_pbot_update(C.byref(d), C.c_double(dtime), p(eta_taum1), p(deta_dt), p(out))
    return out


def update_ocean_barotropic(d, g, state, nts, dtbt, gamma=0.2, rho0=1035.0, time_stepping_B=True,
                            initsum_with_bar=True, cgrid=False):
    """One barotropic step; ``state`` holds eta_t, eta_t_bar, udrho_u, udrho_v at tau.
    Returns the taup1 fields."""
    shp = g["tmask1"].shape
    out = {k: np.zeros(shp) for k in ("eta_t_bar", "udrho_u", "udrho_v", "conv_rho_ud_t", "eta_u", "ps",
                                      "grad_ps_x", "grad_ps_y")}
    src = dict(g)
    src["eta_t_tau"] = state["eta_t"]
    src["eta_t_bar_tau"] = state["eta_t_bar"]
    src["udrho_u_tau"] = state["udrho_u"]
    src["udrho_v_tau"] = state["udrho_v"]
    ptrs = []
    for n in BARO_IO_FIELDS:
        if n.startswith("out_"):
            ptrs.append(p(out[n[4:]]))
        else:
            ptrs.append(p(src[n]))
    io = BaroIO(*ptrs)
    prm = BaroParams(int(nts), float(dtbt), float(gamma), float(rho0), int(time_stepping_B), int(initsum_with_bar),
                     int(cgrid))
    lib().orc_update_ocean_barotropic(C.byref(d), C.byref(prm), C.byref(io))
    return out


def run_steps(d, g, T, dtts, warmup=0, steps=1, nts=0, dtbt=0.0, state=None, gamma=0.2, rho0=1035.0,
              threaded=False, threads=None):
    """The CPU baseline's loop (orc_run_steps): warmup + steps baroclinic steps of
    one block in C with the scheme scratch held across steps -- every tracer of
    ``T`` (ntr, nk, nj+2, ni+2) by MDFL Sweby with the explicit update, then,
    with nts > 0, update_ocean_barotropic from ``state`` (eta_t, eta_t_bar,
    udrho_u, udrho_v at tau).  ``T`` is updated in place.  threaded=True runs
    the OpenMP build on ``threads`` threads (default: every host core).  Returns (seconds of the timed
    steps, the last barotropic outputs or None)."""
    T = np.ascontiguousarray(T)
    assert T.dtype == np.float64 and T.ndim == 4
    ntr = int(T.shape[0])
    io = out = prm = None
    keep = []
    if nts > 0:
        shp = g["tmask1"].shape
        out = {k: np.zeros(shp) for k in ("eta_t_bar", "udrho_u", "udrho_v", "conv_rho_ud_t", "eta_u", "ps",
                                          "grad_ps_x", "grad_ps_y")}
        src = dict(g)
        src["eta_t_tau"] = state["eta_t"]
        for k in ("eta_t_bar", "udrho_u", "udrho_v"):
            src[k + "_tau"] = np.ascontiguousarray(state[k]).copy()
        keep = [src, out]
        io = BaroIO(*[p(out[n[4:]]) if n.startswith("out_") else p(src[n]) for n in BARO_IO_FIELDS])
        prm = BaroParams(int(nts), float(dtbt), float(gamma), float(rho0), 1, 1, 0)
    z = np.zeros(1)
    arr = lambda k: p(g[k]) if ntr > 0 else p(z)
    L = lib_omp() if threaded else lib()
    if threaded:
        L.orc_set_threads(int(os.cpu_count() if threads is None else threads))
    f = L.orc_run_steps
    f.restype = C.c_double
    sec = f(C.byref(d), ntr, int(warmup), int(steps), C.c_double(dtts), arr("tmask"), arr("dat"), arr("datr"),
            arr("dxte"), arr("dyte"), arr("dxtn"), arr("dytn"), arr("uhrho_et"), arr("vhrho_nt"), arr("wrho_bt"),
            arr("rho_dzt"), arr("rho_dztr"), p(T) if ntr > 0 else p(z),
            C.byref(prm) if prm is not None else None, C.byref(io) if io is not None else None)
    if nts > 0:
        # the last step's outputs sit in whichever buffer that step wrote
        last = (warmup + steps) % 2
        src = keep[0]
        res = dict(out)
        if last == 0:
            for k in ("eta_t_bar", "udrho_u", "udrho_v"):
                res[k] = src[k + "_tau"]
        return sec, res
    return sec, None


def domain_arrays(dom) -> Dict[str, np.ndarray]:
    """numpy copies of a grid.Domain's arrays (the oracle's inputs)."""
    return {k: np64(v) for k, v in dom.f.items() if k != "kmt"}


def update_ucell_thickness(d, vcoord, state, rho0=1035.0, linear_free_surface=False, update_dzwu_k0=True):
    """update_ucell_thickness (ocean_thickness.F90:3507-3886), no blobs.  state maps
    umask, tmasken_e, tmasken_n, dzt, dzwt (nk+1 levels), rho_dzt (level taup1),
    depth_zt, depth_zwt (level 1 used), eta_u (level taup1), kmu and the fields it
    updates: dzu, dzwu, rho_dzu (level taup1), rho_dzur, dzten_e/n, rho_dzten_e/n,
    depth_zu, depth_zwu.  Returns new arrays of those plus thicku, mass_u,
    thicken_e/n, mass_en_e/n."""
    f = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    out = {k: f(state[k]).copy() for k in ("dzu", "dzwu", "rho_dzu", "rho_dzur", "dzten_e", "dzten_n", "rho_dzten_e",
                                           "rho_dzten_n", "depth_zu", "depth_zwu")}
    n2 = (d.nj + 2, d.ni + 2)
    for k in ("thicku", "thicken_e", "thicken_n", "mass_u", "mass_en_e", "mass_en_n"):
        out[k] = np.zeros(n2)
    ins = [f(state[k]) for k in ("umask", "tmasken_e", "tmasken_n", "dzt", "dzwt", "rho_dzt")]
    ins += [f(np.asarray(state["depth_zt"]).reshape(d.nk, *n2)[0]), f(np.asarray(state["depth_zwt"]).reshape(d.nk, *n2)[0]),
            f(state["eta_u"])]
    kmu = np.ascontiguousarray(state["kmu"], dtype=np.int32)
    lib().orc_update_ucell_thickness(C.byref(d), int(vcoord), int(linear_free_surface), int(update_dzwu_k0),
                                     C.c_double(rho0), *[p(a) for a in ins], kmu.ctypes.data_as(C.POINTER(C.c_int)),
                                     *[p(out[k]) for k in ("dzu", "dzwu", "rho_dzu", "rho_dzur", "dzten_e", "dzten_n",
                                                           "rho_dzten_e", "rho_dzten_n", "depth_zu", "depth_zwu",
                                                           "thicku", "thicken_e", "thicken_n", "mass_u", "mass_en_e",
                                                           "mass_en_n")])
    return out
