"""Seeded synthetic ocean domains for the advection + barotropic path.

MOM5 reads its grid from ``grid_spec.nc`` and its state from restart files;
neither is available here, so every workload is generated from a seed.  The
rules follow the reference's grid module where they matter for the path:

* spherical metrics, ``dat = dxt*dyt`` (ocean_grids.F90:844) and reciprocals
  ``1/(x + epsln)`` with ``epsln = 1e-40`` (ocean_grids.F90:956-965);
* ``tmask`` from ``kmt`` (ocean_grids.F90:1373-1388), face masks as products
  of the two neighbouring T masks (ocean_grids.F90:1390-1410);
* partial bottom cells (``dzt(kmt) = ht - zw(kmt-1)``);
* ``rho_dzt = rho0*dzt`` fixed in time, ``rho_dztr = 1/(rho_dzt + epsln)``
  (ocean_thickness.F90:1229);
* the vertical mass flux from continuity (ocean_advection_velocity.F90:600-627)
  with ``rho_dzt_tendency = mass_source = 0``.

Arrays use the reference's data-domain layout with a one-cell halo,
column-major in Fortran terms, which is a C-ordered tensor of shape
``(nk, nj+2, ni+2)`` here (i fastest).  Everything is FP64.

Generation runs on any torch device: the CPU for the oracle-sized parity cases
and the GPU for the full-size bench workloads.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Dict, Optional, Tuple

import torch

RADIUS = 6371.0e3  # constants.F90:72
OMEGA = 7.292e-5  # constants.F90:75
GRAV = 9.80  # ocean_parameters.F90:176
RHO0 = 1035.0  # ocean_parameters.F90:194
EPSLN = 1.0e-40  # constants.F90:123


@dataclass
class DomainSpec:
    """Shape and physical layout of one synthetic domain."""

    ni: int
    nj: int
    nk: int
    lon0: float = 0.0
    lon1: float = 60.0
    lat0: float = -40.0
    lat1: float = 40.0
    cyclic_x: bool = False
    cyclic_y: bool = False
    depth: float = 4000.0
    dz_top: float = 10.0
    dz_bot: float = 250.0
    # rectangular continent (i0, j0, width, height) in compute-domain cells, or None
    continent: Optional[Tuple[int, int, int, int]] = None
    # partial bottom: column depth uniform in [hmin, depth]; None = flat bottom
    hmin: Optional[float] = 2000.0
    # seeded ridge (+-amplitude) added to a flat bottom instead of random columns
    ridge_amp: float = 0.0
    min_depth: float = 50.0
    max_speed: float = 0.5  # m/s, scale of the streamfunction-derived flow
    wavelength_cells: float = 8.0
    overturning: float = 0.2  # overturning speed relative to max_speed (3-D, divergence-free)
    ntracers: int = 2
    seed: int = 0

    @property
    def nxd(self) -> int:
        return self.ni + 2

    @property
    def nyd(self) -> int:
        return self.nj + 2


def config_c0(seed: int = 0, ntracers: int = 2) -> DomainSpec:
    """Regional box 120x80x30, lon 0-60, lat -40..40, 20x15 continent."""
    return DomainSpec(ni=120, nj=80, nk=30, lon0=0.0, lon1=60.0, lat0=-40.0, lat1=40.0,
                      continent=(50, 33, 20, 15), hmin=2000.0, ntracers=ntracers, seed=seed)


def config_c1(seed: int = 1) -> DomainSpec:
    """Barotropic 360x300, 1 degree, lat -75..75, ridge bathymetry."""
    return DomainSpec(ni=360, nj=300, nk=1, lon0=0.0, lon1=360.0, lat0=-75.0, lat1=75.0,
                      cyclic_x=True, hmin=None, ridge_amp=1500.0, ntracers=0, seed=seed)


def config_c2(seed: int = 2, ntracers: int = 10) -> DomainSpec:
    """Global 0.25 degree 1440x1080x50, lat -80..80, cyclic in x, 10 tracers."""
    return DomainSpec(ni=1440, nj=1080, nk=50, lon0=0.0, lon1=360.0, lat0=-80.0, lat1=80.0,
                      cyclic_x=True, continent=(600, 400, 160, 120), hmin=2000.0,
                      ntracers=ntracers, seed=seed)


def config_c2_block(seed: int = 3, ntracers: int = 10) -> DomainSpec:
    """A 360x270x50 block of the 0.25 degree grid (lon 0-90, lat -40..27.5) with
    10 tracers: 1/16 of the global config, used for profiling captures."""
    return DomainSpec(ni=360, nj=270, nk=50, lon0=0.0, lon1=90.0, lat0=-40.0, lat1=27.5,
                      cyclic_x=False, continent=(150, 100, 40, 30), hmin=2000.0, ntracers=ntracers, seed=seed)


def config_c2_band(seed: int = 5, ntracers: int = 10) -> DomainSpec:
    """A 1440x360x50 band of the 0.25 degree global grid (lat -40..50, periodic
    in x), 10 tracers: one third of the global config's rows, for profiling
    captures that fill more than two waves of the precision-form kernel while
    holding about 6 GB on the device."""
    return DomainSpec(ni=1440, nj=360, nk=50, lon0=0.0, lon1=360.0, lat0=-40.0, lat1=50.0,
                      cyclic_x=True, continent=(600, 120, 160, 120), hmin=2000.0, ntracers=ntracers, seed=seed)


def config_c2_polar_block(seed: int = 4, ntracers: int = 10) -> DomainSpec:
    """A 360x270x50 block of the 0.25 degree grid reaching the global grid's
    poleward edge (lon 0-90, lat 12.5..80), periodic in x, 10 tracers: the
    metrics where the global config is most extreme (dxt = 4.8 km at 80 deg,
    the barotropic CFL limit about 24 s) at an oracle-checkable size."""
    return DomainSpec(ni=360, nj=270, nk=50, lon0=0.0, lon1=90.0, lat0=12.5, lat1=80.0,
                      cyclic_x=True, continent=(150, 100, 40, 30), hmin=2000.0, ntracers=ntracers, seed=seed)


def stretched_dz(nk: int, top: float, bot: float, total: float) -> torch.Tensor:
    """Level thicknesses growing from ``top`` to ``bot`` as a power law whose
    exponent is solved so that the levels sum to ``total``."""
    if nk == 1:
        return torch.tensor([total], dtype=torch.float64)
    s = torch.arange(nk, dtype=torch.float64) / (nk - 1)
    lo, hi = 0.01, 50.0
    for _ in range(200):
        p = 0.5 * (lo + hi)
        tot = float((top + (bot - top) * s ** p).sum())
        if tot > total:
            lo = p
        else:
            hi = p
    dz = top + (bot - top) * s ** (0.5 * (lo + hi))
    return dz * (total / float(dz.sum()))


def _periodic_fill(a: torch.Tensor, cx: bool, cy: bool) -> torch.Tensor:
    """Single-domain halo update of the last two dims (halo 1)."""
    if cx:
        a[..., 1:-1, 0] = a[..., 1:-1, -2]
        a[..., 1:-1, -1] = a[..., 1:-1, 1]
    if cy:
        a[..., 0, 1:-1] = a[..., -2, 1:-1]
        a[..., -1, 1:-1] = a[..., 1, 1:-1]
    if cx and cy:
        a[..., 0, 0] = a[..., -2, -2]
        a[..., 0, -1] = a[..., -2, 1]
        a[..., -1, 0] = a[..., 1, -2]
        a[..., -1, -1] = a[..., 1, 1]
    return a


def _smooth_field(g: torch.Generator, ny: int, nx: int, sigma_cells: float, device) -> torch.Tensor:
    """Seeded N(0,1) noise smoothed by a Gaussian of ``sigma_cells`` (FFT, periodic)."""
    noise = torch.randn((ny, nx), generator=g, dtype=torch.float64, device="cpu").to(device)
    ky = torch.fft.fftfreq(ny, dtype=torch.float64, device=device)[:, None]
    kx = torch.fft.fftfreq(nx, dtype=torch.float64, device=device)[None, :]
    filt = torch.exp(-2.0 * (math.pi * sigma_cells) ** 2 * (kx ** 2 + ky ** 2))
    out = torch.fft.ifft2(torch.fft.fft2(noise) * filt).real
    return out / out.std().clamp_min(1e-300)


def _band_field(g: torch.Generator, ny: int, nx: int, wavelength: float, device) -> torch.Tensor:
    """Seeded random field with a Gaussian spectrum peaked at ``wavelength`` cells."""
    noise = torch.randn((ny, nx), generator=g, dtype=torch.float64, device="cpu").to(device)
    ky = torch.fft.fftfreq(ny, dtype=torch.float64, device=device)[:, None]
    kx = torch.fft.fftfreq(nx, dtype=torch.float64, device=device)[None, :]
    kk = torch.sqrt(kx ** 2 + ky ** 2)
    k0 = 1.0 / wavelength
    filt = torch.exp(-((kk - k0) / (0.35 * k0)) ** 2)
    out = torch.fft.ifft2(torch.fft.fft2(noise) * filt).real
    return out / out.abs().max().clamp_min(1e-300)


@dataclass
class Domain:
    spec: DomainSpec
    f: Dict[str, torch.Tensor] = field(default_factory=dict)  # every array, FP64 (kmt int32)
    dzt: torch.Tensor = None  # nominal level thickness (nk)
    zw: torch.Tensor = None  # depth of level bottoms (nk)

    def __getitem__(self, k: str) -> torch.Tensor:
        return self.f[k]

    def to(self, device) -> "Domain":
        return Domain(self.spec, {k: v.to(device) for k, v in self.f.items()}, self.dzt, self.zw)

    @property
    def cells(self) -> int:
        s = self.spec
        return s.ni * s.nj * s.nk


def make_domain(spec: DomainSpec, device="cpu", with_barotropic: bool = True) -> Domain:
    """Build every input array of the path for ``spec`` on ``device``."""
    dev = torch.device(device)
    f64 = torch.float64
    g = torch.Generator(device="cpu")
    g.manual_seed(int(spec.seed) * 1000003 + 12345)
    ni, nj, nk, nxd, nyd = spec.ni, spec.nj, spec.nk, spec.nxd, spec.nyd
    d2r = math.pi / 180.0
    dlon = (spec.lon1 - spec.lon0) / ni
    dlat = (spec.lat1 - spec.lat0) / nj
    ii = torch.arange(nxd, dtype=f64, device=dev)
    jj = torch.arange(nyd, dtype=f64, device=dev)
    lon_t = spec.lon0 + (ii - 0.5) * dlon
    lat_t = spec.lat0 + (jj - 0.5) * dlat
    lat_u = lat_t + 0.5 * dlat
    phi_t = (lat_t * d2r)[:, None].expand(nyd, nxd)
    phi_u = (lat_u * d2r)[:, None].expand(nyd, nxd)
    F: Dict[str, torch.Tensor] = {}

    dxt = RADIUS * torch.cos(phi_t) * (dlon * d2r)
    dyt = torch.full((nyd, nxd), RADIUS * dlat * d2r, dtype=f64, device=dev)
    dxu = RADIUS * torch.cos(phi_u) * (dlon * d2r)
    dyu = dyt.clone()
    F["dxt"], F["dyt"], F["dxu"], F["dyu"] = dxt.contiguous(), dyt, dxu.contiguous(), dyu
    F["dxte"] = dxt.contiguous().clone()  # T-to-T distance across the east face (uniform longitude)
    F["dyte"] = dyt.clone()  # length of the east face
    F["dxtn"] = dxu.contiguous().clone()  # length of the north face
    F["dytn"] = dyt.clone()  # T-to-T distance across the north face
    F["dat"] = F["dxt"] * F["dyt"]
    F["datr"] = 1.0 / (F["dat"] + EPSLN)
    F["dau"] = F["dxu"] * F["dyu"]
    F["daur"] = 1.0 / (F["dau"] + EPSLN)
    F["dxur"] = 1.0 / (F["dxu"] + EPSLN)
    F["dyur"] = 1.0 / (F["dyu"] + EPSLN)
    F["dxter"] = 1.0 / (F["dxte"] + EPSLN)
    F["dytnr"] = 1.0 / (F["dytn"] + EPSLN)
    F["dte"] = 0.5 * F["dxt"]
    F["dtw"] = 0.5 * F["dxt"]
    F["dus"] = 0.5 * F["dyu"]
    F["dun"] = 0.5 * F["dyu"]
    F["f"] = (2.0 * OMEGA * torch.sin(phi_u)).contiguous()
    # the metrics' halos hold the periodic images, as after the grid's halo
    # updates (ocean_grids.F90:2083-2165)
    for name in ("dxt", "dyt", "dxu", "dyu", "dxte", "dyte", "dxtn", "dytn", "dat", "datr", "dau", "daur", "dxur",
                 "dyur", "dxter", "dytnr", "dte", "dtw", "dus", "dun", "f"):
        F[name] = _periodic_fill(F[name].contiguous().clone(), spec.cyclic_x, spec.cyclic_y)

    # vertical grid
    dz = stretched_dz(nk, spec.dz_top, spec.dz_bot, spec.depth)
    zw = torch.cumsum(dz, 0)
    zt = zw - 0.5 * dz
    dzd = dz.to(dev)

    # bathymetry on the compute domain
    if spec.ridge_amp > 0.0:
        ridge = _smooth_field(g, nj, ni, 10.0, dev)
        ridge = ridge / ridge.abs().max().clamp_min(1e-300)
        ht_c = (spec.depth + spec.ridge_amp * ridge).clamp_min(spec.min_depth)
    elif spec.hmin is not None:
        u = torch.rand((nj, ni), generator=g, dtype=f64).to(dev)
        ht_c = spec.hmin + (spec.depth - spec.hmin) * u
    else:
        ht_c = torch.full((nj, ni), spec.depth, dtype=f64, device=dev)
    if spec.continent is not None:
        i0, j0, w, h = spec.continent
        ht_c[j0:j0 + h, i0:i0 + w] = 0.0
    ht = torch.zeros((nyd, nxd), dtype=f64, device=dev)
    ht[1:-1, 1:-1] = ht_c
    _periodic_fill(ht, spec.cyclic_x, spec.cyclic_y)

    # kmt and partial bottom cells
    zw_d = zw.to(dev)
    kmt = torch.zeros((nyd, nxd), dtype=torch.int32, device=dev)
    wet = ht > 0.0
    kmt_f = torch.searchsorted(zw_d.contiguous(), ht.clamp_max(float(zw[-1])).reshape(-1).contiguous(), right=False)
    kmt_f = (kmt_f + 1).clamp(1, nk).reshape(nyd, nxd).to(torch.int32)
    kmt = torch.where(wet, kmt_f, kmt)
    kk = torch.arange(1, nk + 1, device=dev, dtype=torch.int32)[:, None, None]
    tmask = (kk <= kmt[None, :, :]).to(f64)
    dzt3 = dzd[:, None, None].expand(nk, nyd, nxd).clone()
    if spec.hmin is not None or spec.ridge_amp > 0.0:
        zw_above = torch.cat([torch.zeros(1, dtype=f64, device=dev), zw_d])  # zw(k-1), k=1..nk
        kb = (kmt.long() - 1).clamp_min(0)
        part = ht - zw_above[kb]
        part = torch.maximum(part, 0.2 * dzd[kb])
        bot = torch.zeros((nk, nyd, nxd), dtype=torch.bool, device=dev)
        bot.scatter_(0, kb[None], wet[None])
        dzt3 = torch.where(bot, part[None].expand_as(dzt3), dzt3)
    F["kmt"] = kmt
    F["ht"] = ht
    F["tmask"] = tmask.contiguous()
    F["tmasken_e"] = torch.zeros_like(tmask)
    F["tmasken_e"][:, :, :-1] = tmask[:, :, :-1] * tmask[:, :, 1:]
    F["tmasken_n"] = torch.zeros_like(tmask)
    F["tmasken_n"][:, :-1, :] = tmask[:, :-1, :] * tmask[:, 1:, :]
    umask = torch.zeros_like(tmask)
    umask[:, :-1, :-1] = tmask[:, :-1, :-1] * tmask[:, :-1, 1:] * tmask[:, 1:, :-1] * tmask[:, 1:, 1:]
    F["umask1"] = umask[0].contiguous()
    F["tmask1"] = tmask[0].contiguous()
    F["tmasken_e1"] = F["tmasken_e"][0].contiguous()
    F["tmasken_n1"] = F["tmasken_n"][0].contiguous()
    F["rho_dzt"] = (RHO0 * dzt3).contiguous()
    F["rho_dztr"] = 1.0 / (F["rho_dzt"] + EPSLN)

    # Flow: a per-level horizontal streamfunction (rotational part) plus x-z and
    # y-z overturning streamfunctions, all zero wherever they touch land or the
    # sea floor, so the discrete 3-D divergence vanishes cell by cell and the
    # vertical mass flux from continuity is zero at the bottom up to roundoff.
    psi = torch.zeros((nyd, nxd), dtype=f64, device=dev)
    psi[1:-1, 1:-1] = _band_field(g, nj, ni, spec.wavelength_cells, dev)
    _periodic_fill(psi, spec.cyclic_x, spec.cyclic_y)
    # speed scale of the rotational part: max |u| over the compute domain = max_speed
    u2 = torch.zeros_like(psi)
    v2 = torch.zeros_like(psi)
    u2[1:, :] = -(psi[1:, :] - psi[:-1, :]) / F["dyte"][1:, :]
    v2[:, 1:] = (psi[:, 1:] - psi[:, :-1]) / F["dxtn"][:, 1:]
    vmax = torch.maximum(u2[1:-1, 1:-1].abs().max(), v2[1:-1, 1:-1].abs().max()).clamp_min(1e-300)
    psi = psi * (spec.max_speed / vmax)
    # transport streamfunction (kg/s) at U points per level: rho0*dz_k*psi*umask
    Psi = (RHO0 * dzd)[:, None, None] * psi[None] * umask
    U = torch.zeros((nk, nyd, nxd), dtype=f64, device=dev)  # east-face transport (kg/s)
    V = torch.zeros((nk, nyd, nxd), dtype=f64, device=dev)  # north-face transport (kg/s)
    U[:, 1:, :] = -(Psi[:, 1:, :] - Psi[:, :-1, :])
    V[:, :, 1:] = Psi[:, :, 1:] - Psi[:, :, :-1]
    if spec.overturning > 0.0 and nk > 1:
        # phi_x at (east face, interface below level k), k = 1..nk-1 (0 at surface and bottom)
        zwi = zw_d[:-1]
        vert = torch.sin(math.pi * zwi / spec.depth)[:, None, None]
        amp = spec.overturning * spec.max_speed * spec.depth * RHO0 * float(F["dyte"][1:-1, 1:-1].mean()) / math.pi
        open_e = tmask[:-1, :, :-1] * tmask[:-1, :, 1:] * tmask[1:, :, :-1] * tmask[1:, :, 1:]
        open_n = tmask[:-1, :-1, :] * tmask[:-1, 1:, :] * tmask[1:, :-1, :] * tmask[1:, 1:, :]
        bx = torch.zeros((nyd, nxd), dtype=f64, device=dev)
        by = torch.zeros((nyd, nxd), dtype=f64, device=dev)
        bx[1:-1, 1:-1] = _band_field(g, nj, ni, 2.0 * spec.wavelength_cells, dev)
        by[1:-1, 1:-1] = _band_field(g, nj, ni, 2.0 * spec.wavelength_cells, dev)
        _periodic_fill(bx, spec.cyclic_x, spec.cyclic_y)
        _periodic_fill(by, spec.cyclic_x, spec.cyclic_y)
        phx = torch.zeros((nk + 1, nyd, nxd), dtype=f64, device=dev)  # interface index 0..nk
        phy = torch.zeros((nk + 1, nyd, nxd), dtype=f64, device=dev)
        phx[1:nk, :, :-1] = amp * vert * bx[None, :, :-1] * open_e
        phy[1:nk, :-1, :] = amp * vert * by[None, :-1, :] * open_n
        _periodic_fill(phx, spec.cyclic_x, spec.cyclic_y)
        _periodic_fill(phy, spec.cyclic_x, spec.cyclic_y)
        U = U + (phx[:-1] - phx[1:])
        V = V + (phy[:-1] - phy[1:])
    _periodic_fill(U, spec.cyclic_x, spec.cyclic_y)
    _periodic_fill(V, spec.cyclic_x, spec.cyclic_y)
    uh = U / F["dyte"][None]
    vh = V / F["dxtn"][None]
    F["uhrho_et"] = uh.contiguous()
    F["vhrho_nt"] = vh.contiguous()

    # continuity (ocean_advection_velocity.F90:600-627, BDX_ET/BDY_NT with halo 1)
    w = torch.zeros((nk + 1, nyd, nxd), dtype=f64, device=dev)
    w[0] = -(torch.zeros_like(psi))  # pme = river = 0
    for k in range(nk):
        bdx = torch.zeros_like(psi)
        bdx[:, 1:] = (F["dyte"][:, 1:] * uh[k, :, 1:] - F["dyte"][:, :-1] * uh[k, :, :-1]) * F["datr"][:, 1:]
        bdy = torch.zeros_like(psi)
        bdy[1:, :] = (F["dxtn"][1:, :] * vh[k, 1:, :] - F["dxtn"][:-1, :] * vh[k, :-1, :]) * F["datr"][1:, :]
        div = tmask[k] * (bdx + bdy)
        w[k + 1] = (0.0 + div + w[k]) * tmask[k]
    F["wrho_bt"] = w.contiguous()

    # tracers: T = 25 exp(-z/800) + N(0,0.1); S = 35 + 0.5 tanh(lat/20); passive U(0,1)
    ntr = spec.ntracers
    if ntr > 0:
        T = torch.zeros((ntr, nk, nyd, nxd), dtype=f64, device=dev)
        T[0] = 25.0 * torch.exp(-zt.to(dev) / 800.0)[:, None, None] + 0.1 * torch.randn(
            (nk, nyd, nxd), generator=g, dtype=f64).to(dev)
        if ntr > 1:
            T[1] = (35.0 + 0.5 * torch.tanh(lat_t / 20.0))[None, :, None].expand(nk, nyd, nxd)
        for n in range(2, ntr):
            T[n] = torch.rand((nk, nyd, nxd), generator=g, dtype=f64).to(dev)
        T = T * tmask[None]
        _periodic_fill(T, spec.cyclic_x, spec.cyclic_y)
        F["T"] = T.contiguous()

    if with_barotropic:
        eta = _smooth_field(g, nj, ni, 5.0, dev) * 0.05
        F["eta_t"] = torch.zeros((nyd, nxd), dtype=f64, device=dev)
        F["eta_t"][1:-1, 1:-1] = eta
        F["eta_t"] = _periodic_fill(F["eta_t"] * F["tmask1"], spec.cyclic_x, spec.cyclic_y)
        F["eta_t_bar"] = F["eta_t"].clone()
        tx = _smooth_field(g, nj, ni, 10.0, dev) * 0.1
        ty = _smooth_field(g, nj, ni, 10.0, dev) * 0.1
        F["forcing_u"] = torch.zeros((nyd, nxd), dtype=f64, device=dev)
        F["forcing_v"] = torch.zeros((nyd, nxd), dtype=f64, device=dev)
        F["forcing_u"][1:-1, 1:-1] = tx
        F["forcing_v"][1:-1, 1:-1] = ty
        F["forcing_u"] = _periodic_fill(F["forcing_u"] * F["umask1"], spec.cyclic_x, spec.cyclic_y)
        F["forcing_v"] = _periodic_fill(F["forcing_v"] * F["umask1"], spec.cyclic_x, spec.cyclic_y)
        hu = torch.zeros_like(ht)
        hu[:-1, :-1] = torch.minimum(torch.minimum(ht[:-1, :-1], ht[:-1, 1:]), torch.minimum(ht[1:, :-1], ht[1:, 1:]))
        F["thicku"] = _periodic_fill(hu * F["umask1"], spec.cyclic_x, spec.cyclic_y)
        he = torch.zeros_like(ht)
        he[:, :-1] = torch.minimum(ht[:, :-1], ht[:, 1:])
        hn = torch.zeros_like(ht)
        hn[:-1, :] = torch.minimum(ht[:-1, :], ht[1:, :])
        F["thicken_e"] = _periodic_fill(he * F["tmasken_e1"], spec.cyclic_x, spec.cyclic_y)
        F["thicken_n"] = _periodic_fill(hn * F["tmasken_n1"], spec.cyclic_x, spec.cyclic_y)
        z2 = torch.zeros((nyd, nxd), dtype=f64, device=dev)
        F["udrho_u"] = z2.clone()
        F["udrho_v"] = z2.clone()
        F["patm"] = z2.clone()
        F["pme"] = z2.clone()
        F["river"] = z2.clone()
        F["source"] = z2.clone()
        F["eta_smooth"] = z2.clone()
        F["conv_rho_ud_t"] = z2.clone()
        F["rho_g"] = torch.full((nyd, nxd), GRAV * RHO0, dtype=f64, device=dev)  # ocean_barotropic.F90:1265
    dom = Domain(spec, F, dz, zw)
    return dom


def barotropic_cfl_limit(dom: Domain) -> float:
    """Largest stable barotropic time step, as the gravity-wave check of
    ocean_barotropic.F90:1595-1662 computes it (cfl_grid_factor = 1, the
    limit truncated with int())."""
    kmt = dom["kmt"][1:-1, 1:-1]
    wet = kmt > 0
    zw = dom.zw.to(kmt.device)
    depth = zw[(kmt.long() - 1).clamp_min(0)]
    cg = torch.sqrt(GRAV * depth)
    dxt = dom["dxt"][1:-1, 1:-1]
    dyt = dom["dyt"][1:-1, 1:-1]
    gridsp = torch.sqrt(1.0 / (1.0 / (dxt * dxt) + 1.0 / (dyt * dyt)))
    dtcg = torch.where(wet, gridsp / cg, torch.full_like(cg, 1.0e6))
    return float(int(float(dtcg.min())))


def thickness_state(ni: int, nj: int, nk: int, cyclic_x: bool = False, cyclic_y: bool = False, seed: int = 0,
                    rho0: float = 1035.0) -> dict:
    """Seeded thickness fields of a partial-cell domain for update_ucell_thickness
    (ocean_thickness.F90:3507-3886), data-domain arrays [k][j][i] (numpy):
    T-cell dzt with partial bottom cells and a time-varying top cell, dzwt
    (levels 0..nk, half-cell distances), rho_dzt = rho0*dzt (perturbed, as a
    non-Boussinesq density would), depth_zt/zwt (cumulative), kmt; the U-cell
    kmu = min of the four surrounding kmt with umask(k) = (k <= kmu); tmasken
    of the east and north faces; eta_u; and the current U-cell and face
    fields the routine updates, filled with values it must overwrite or keep."""
    import numpy as np
    rng = np.random.default_rng(seed)
    nx, ny = ni + 2, nj + 2
    dz0 = 10.0 + 40.0 * np.arange(nk) / max(nk - 1, 1)
    kmt = rng.integers(0, nk + 1, size=(ny, nx))
    kmt[rng.random((ny, nx)) < 0.6] = nk
    dzt = np.zeros((nk, ny, nx))
    for k in range(nk):
        dzt[k] = dz0[k] * np.where(kmt - 1 == k, 0.3 + 0.7 * rng.random((ny, nx)), 1.0)
    dzt[0] += rng.normal(0.0, 0.3, size=(ny, nx))
    dzwt = np.zeros((nk + 1, ny, nx))
    dzwt[0] = 0.5 * dzt[0]
    for k in range(1, nk):
        dzwt[k] = 0.5 * (dzt[k - 1] + dzt[k])
    dzwt[nk] = 0.5 * dzt[nk - 1]
    rho_dzt = rho0 * dzt * (1.0 + 1e-3 * rng.standard_normal((nk, ny, nx)))
    depth_zwt = np.cumsum(dzt, axis=0)
    depth_zt = np.cumsum(dzwt[:nk], axis=0)
    kp = np.pad(kmt, 1, mode="edge")
    kmu = np.minimum(np.minimum(kmt, kp[1:-1, 2:]), np.minimum(kp[2:, 1:-1], kp[2:, 2:]))
    if cyclic_x:
        kmu[:, 0], kmu[:, -1] = kmu[:, -2], kmu[:, 1]
    if cyclic_y:
        kmu[0, :], kmu[-1, :] = kmu[-2, :], kmu[1, :]
    lev = np.arange(nk)[:, None, None]
    umask = (lev < kmu[None]).astype(np.float64)
    tmask = (lev < kmt[None]).astype(np.float64)
    tme = tmask * np.concatenate([tmask[:, :, 1:], tmask[:, :, -1:]], axis=2)
    tmn = tmask * np.concatenate([tmask[:, 1:, :], tmask[:, -1:, :]], axis=1)
    junk = lambda shape: rng.normal(5.0, 1.0, size=shape)
    return {"dzt": dzt, "dzwt": dzwt, "rho_dzt": rho_dzt, "depth_zt": depth_zt, "depth_zwt": depth_zwt,
            "kmt": kmt.astype(np.int32), "kmu": kmu.astype(np.int32), "umask": umask, "tmasken_e": tme,
            "tmasken_n": tmn, "eta_u": rng.normal(0.0, 0.5, size=(ny, nx)),
            "dzu": junk((nk, ny, nx)), "dzwu": junk((nk + 1, ny, nx)), "rho_dzu": junk((nk, ny, nx)),
            "rho_dzur": junk((nk, ny, nx)), "dzten_e": dzt * 0.9, "dzten_n": dzt * 0.8,
            "rho_dzten_e": rho_dzt * 0.9, "rho_dzten_n": rho_dzt * 0.8,
            "depth_zu": depth_zt.copy(), "depth_zwu": depth_zwt.copy()}
