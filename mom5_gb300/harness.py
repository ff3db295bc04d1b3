"""Loading synthetic domains into the library and driving whole steps.

The field map below is the correspondence between the arrays of
``grid.Domain`` (named after the reference's derived-type components) and the
field ids of the C ABI.
"""
from __future__ import annotations

from typing import Optional

from . import capi
from .capi import F
from .grid import Domain

GRID2D = {F.DXT: "dxt", F.DYT: "dyt", F.DXU: "dxu", F.DYU: "dyu", F.DXTE: "dxte", F.DYTE: "dyte", F.DXTN: "dxtn",
          F.DYTN: "dytn", F.DAT: "dat", F.DATR: "datr", F.DXUR: "dxur", F.DYUR: "dyur", F.DXTER: "dxter",
          F.DYTNR: "dytnr", F.DTE: "dte", F.DTW: "dtw", F.DUS: "dus", F.DUN: "dun", F.DAUR: "daur",
          F.CORIOLIS_F: "f", F.UMASK1: "umask1", F.TMASKEN_E1: "tmasken_e1", F.TMASKEN_N1: "tmasken_n1"}
GRID3D = {F.TMASK: "tmask", F.UHRHO_ET: "uhrho_et", F.VHRHO_NT: "vhrho_nt", F.WRHO_BT: "wrho_bt",
          F.RHO_DZTR: "rho_dztr"}
BARO2D = {F.FORCING_BT_U: "forcing_u", F.FORCING_BT_V: "forcing_v", F.PATM: "patm", F.PME: "pme",
          F.RIVER: "river", F.SOURCE: "source", F.ETA_SMOOTH: "eta_smooth", F.THICKEN_E: "thicken_e",
          F.THICKEN_N: "thicken_n", F.RHO_G: "rho_g"}
BARO_STATE = {F.ETA_T: "eta_t", F.ETA_T_BAR: "eta_t_bar", F.UDRHO_U: "udrho_u", F.UDRHO_V: "udrho_v",
              F.CONV_RHO_UD_T: "conv_rho_ud_t"}


def _c(t):
    return t.contiguous()


def load(dom: Domain, options: Optional[capi.Options] = None, horz_grid: int = capi.BGRID, tau: int = 1,
         scheme: int = capi.ADVECT_MDFL_SWEBY, tracer_limits=None, levels=(1, 2)) -> capi.Domain:
    """Create a library domain and copy every input of ``dom`` into it.

    ``tau`` is the time level that receives the state; ``levels`` are the levels
    whose thickness is set (two-level stepping alternates between two)."""
    s = dom.spec
    ntr = s.ntracers
    d = capi.Domain(s.ni, s.nj, s.nk, ntr, s.cyclic_x, s.cyclic_y, horz_grid, options)
    for fid, name in GRID2D.items():
        d.set(fid, _c(dom[name]))
    for fid, name in GRID3D.items():
        d.set(fid, _c(dom[name]))
    for lv in levels:
        d.set(F.RHO_DZT, _c(dom["rho_dzt"]), level=lv)
    d.set_vertical_grid(dom.dzt.numpy(), dom.zw.numpy(), dom["kmt"].cpu().numpy())
    for n in range(1, ntr + 1):
        lim = tracer_limits[n - 1] if tracer_limits else (-1.0e10, 1.0e10)
        d.set_tracer_scheme(n, scheme, scheme, lim[0], lim[1])
        d.set(F.TRACER, _c(dom["T"][n - 1]), n=n, level=tau)
    if "eta_t" in dom.f:
        for fid, name in BARO2D.items():
            d.set(fid, _c(dom[name]))
        for lv in levels:
            d.set(F.THICKU, _c(dom["thicku"]), level=lv)
        for fid, name in BARO_STATE.items():
            d.set(fid, _c(dom[name]), level=tau)
    if ntr > 0:
        d.tracer_advect_init()
    return d
