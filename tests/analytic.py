"""Known answers from the mathematics of the advection equation and of the
barotropic momentum equation (at the end), shared by the oracle and GPU tests.

In a box with uniform metrics (dx, dy, dz) and a uniform velocity, the exact
solution translates the tracer by (u, v, w)*dt.  Cell averages commute with
translation, so cell averages that follow a polynomial P(i, j, k) of the cell
indices become P(i - cx, j - cy, k + cz) (k counts downward, w > 0 is upward).

- MDFL Sweby (ocean_tracer_advect.F90:3806-4066) is direction split into 1-D
  passes of the third-order DST3 scheme (d0 = (2-cfl)(1-cfl)/6,
  d1 = (1-cfl^2)/6): exact in space and time for polynomials of degree 3
  while the limiter is inactive (a smooth profile at moderate Courant numbers).
- Upwind (:2238-2294, :2792-2824) is the first-order DST scheme: exact for
  linear profiles.
- The centred 2nd/4th/6th-order and Quicker fluxes are spatial
  discretisations: on a quadratic their flux divergence is the exact
  derivative, so one forward step gives P - dt*(u, v, -w).grad P.

Cells away from the boundaries (whose halo rules are not those of a
polynomial) must match these to roundoff.  The expectations are derived from
the equation, not from a reading of the Fortran."""
import numpy as np

RHO0 = 1035.0

VELOCITIES = [(0.4, 0.0, 0.0), (0.0, -0.3, 0.0), (0.0, 0.0, 1e-3), (0.4, -0.3, 1e-3), (-0.2, 0.25, -2e-3)]


def cubic(x, y, z):
    return 5.0 + 0.3 * x + 0.01 * x * x + 0.002 * y * y + 1e-4 * z ** 3 + 1e-4 * x * y * z


def linear(x, y, z):
    return 1.0 + 0.2 * x - 0.15 * y + 0.05 * z


def quadratic(x, y, z):
    return 1.0 + 0.2 * x + 0.01 * x * x - 0.15 * y + 0.003 * y * y + 0.05 * z + 0.002 * z * z


def quadratic_grad(x, y, z):
    return 0.2 + 0.02 * x, -0.15 + 0.006 * y, 0.05 + 0.004 * z


PROFILES = {"cubic": cubic, "linear": linear, "quadratic": quadratic}


def indices(shape):
    nk, nyd, nxd = shape
    K, J, I = np.meshgrid(np.arange(nk, dtype=float), np.arange(nyd, dtype=float), np.arange(nxd, dtype=float),
                          indexing="ij")
    return I, J, K


def profile(kind, shape):
    I, J, K = indices(shape)
    return PROFILES[kind](I, J, K)


def expected(kind, shape, u, v, w, dt, spacing):
    """The known answer after one forward step of dt: a translated profile for
    the schemes exact in space and time (cubic: MDFL Sweby; linear: upwind),
    the forward-Euler step of the exact tendency for the quadratic."""
    dx, dy, dz = spacing
    I, J, K = indices(shape)
    cx, cy, cz = u * dt / dx, v * dt / dy, w * dt / dz
    if kind != "quadratic":
        return PROFILES[kind](I - cx, J - cy, K + cz)
    gx, gy, gz = quadratic_grad(I, J, K)
    return quadratic(I, J, K) - cx * gx - cy * gy + cz * gz


def make_box(kind, u, v, w, ni=30, nj=30, nk=30, dx=8000.0, dy=6000.0, dz=10.0):
    """A grid.Domain with uniform metrics and levels, every cell wet, uniform
    velocity (u, v, w) and one tracer = the profile `kind` on the whole data
    domain.  Returns the domain and (dx, dy, dz)."""
    import torch
    from mom5_gb300 import grid
    sp = grid.DomainSpec(ni=ni, nj=nj, nk=nk, lon0=0.0, lon1=0.1 * ni, lat0=-0.05 * nj, lat1=0.05 * nj,
                         continent=None, hmin=None, ntracers=1, seed=0)
    dom = grid.make_domain(sp)
    for k in ("dxt", "dxte", "dxtn", "dxu"):
        dom[k].fill_(dx)
    for k in ("dyt", "dyte", "dytn", "dyu"):
        dom[k].fill_(dy)
    dom["dat"].fill_(dx * dy)
    dom["datr"].fill_(1.0 / (dx * dy))
    dom["rho_dzt"].fill_(RHO0 * dz)
    dom["rho_dztr"].fill_(1.0 / (RHO0 * dz))
    dom["tmask"].fill_(1.0)
    dom.dzt = torch.full((nk,), dz, dtype=torch.float64)
    dom.zw = torch.cumsum(dom.dzt, 0)
    dom["uhrho_et"].fill_(u * RHO0 * dz)
    dom["vhrho_nt"].fill_(v * RHO0 * dz)
    dom["wrho_bt"].fill_(w * RHO0)
    dom["T"][0].copy_(torch.from_numpy(profile(kind, tuple(dom["T"][0].shape))))
    return dom, (dx, dy, dz)


# At Courant number 1 in every direction MDFL's limiter and DST3 terms vanish
# (d0 = d1 = 0, slope (1-cfl)/(1e-30+cfl) = 0): every pass is first-order
# upwind at Courant number 1 and moves any profile, a random one included,
# exactly one cell.  dx/0.4 = dy/0.3 = dz/5e-4 = 20000 s.
CFL1_DT = 20000.0
CFL1_VELOCITIES = [(0.4, 0.0, 0.0), (0.0, -0.3, 0.0), (0.0, 0.0, 5e-4), (0.4, 0.3, 5e-4), (-0.4, -0.3, -5e-4)]


def make_random_box(u, v, w, seed=5):
    """make_box with a uniform-random tracer; returns (domain, spacing, tracer)."""
    import torch
    dom, spacing = make_box("linear", u, v, w)
    T0 = np.random.default_rng(seed).uniform(0.0, 1.0, size=tuple(dom["T"][0].shape))
    dom["T"][0].copy_(torch.from_numpy(T0))
    return dom, spacing, T0


def shifted_one_cell(T0, u, v, w):
    """T0 moved one cell along each non-zero velocity component (k counts down)."""
    return np.roll(T0, shift=(-int(np.sign(w)), int(np.sign(v)), int(np.sign(u))), axis=(0, 1, 2))


def interior(a, margin=8):
    """Cells at least `margin` cells from every boundary."""
    nk, nyd, nxd = a.shape
    return a[margin:nk - margin, margin:nyd - margin, margin:nxd - margin]


def rel_err(got, want):
    g, e = interior(np.asarray(got)), interior(np.asarray(want))
    return np.abs(g - e).max() / np.abs(e).max()


# ---- the Sweby limiter's branches ----
#
# MDFL Sweby is the third-order DST scheme with Sweby's flux limiter: along the
# flow, the face value is T_up + psi*(T_dn - T_up) with
#   psi = max(0, min(1, d0 + d1*theta, (1 - c)/c*theta)),
#   d0 = (2 - c)(1 - c)/6, d1 = (1 - c^2)/6,
# theta the ratio of the difference upstream of the face to the difference
# across it, and c the Courant number.  On a profile whose differences along
# the flow form a geometric sequence (T = r^i, or T alternating, theta = -1)
# theta is the same at every face, so one psi holds everywhere and one step of
# the 1-D flux form gives the cell values directly.  The cases below put psi on
# each branch: the DST3 line, the slope bound (1 - c)/c*theta, the bound 1, and
# 0 (upwind) where theta < 0.

LIMITER_CASES = {
    # name: (profile ratio r or "alt", Courant number c, sign of the velocity, branch)
    "line": (3.0, 0.4, +1, "line"),
    "slope": (8.0, 0.6, +1, "slope"),
    "one": (0.2, 0.1, +1, "one"),
    "zero": ("alt", 0.4, +1, "zero"),
    "slope_negative_u": (1.0 / 8.0, 0.6, -1, "slope"),
    "one_negative_u": (5.0, 0.1, -1, "one"),
}


def limiter_psi(theta, c):
    d0, d1 = (2 - c) * (1 - c) / 6, (1 - c * c) / 6
    return max(0.0, min(1.0, d0 + d1 * theta, (1 - c) / c * theta)), d0 + d1 * theta, (1 - c) / c * theta


def limiter_profile(r, shape, axis):
    """T = r^i (or 1 + 0.1*(-1)^i) along `axis` of a (nk, nyd, nxd) array."""
    idx = np.arange(shape[axis], dtype=float)
    line = 1.0 + 0.1 * (-1.0) ** idx if r == "alt" else r ** idx
    view = [1, 1, 1]
    view[axis] = shape[axis]
    return np.broadcast_to(line.reshape(view), shape).copy()


def limiter_theta(r, sign):
    if r == "alt":
        return -1.0
    return 1.0 / r if sign > 0 else r


def limiter_expected(T, axis, c, sign, psi):
    """One step of the 1-D flux form with one psi at every face, along `axis`
    (i increasing); only cells away from the ends are meaningful."""
    Tp = np.roll(T, -1, axis)  # T(i+1)
    if sign > 0:
        F = T + psi * (Tp - T)  # face i+1/2, upstream cell i
        return T - c * (F - np.roll(F, 1, axis))
    F = Tp - psi * (Tp - T)  # face i+1/2, upstream cell i+1
    return T + c * (F - np.roll(F, 1, axis))


def make_limiter_box(case, axis, ni=30, nj=30, nk=None, dx=8000.0, dy=6000.0, dz=10.0, dt=2000.0):
    """make_box with flow along x (axis 2), y (axis 1) or z (axis 0: k counts
    down, so the case's sign is that of -w) at the case's Courant number and the
    case's profile along it; returns (domain, expected, psi)."""
    import torch
    r, c, sign, branch = LIMITER_CASES[case]
    nk = nk if nk is not None else (30 if axis == 0 else 12)
    spacing = (dz, dy, dx)[axis]
    vel = sign * c * spacing / dt
    u, v, w = (vel, 0.0, 0.0) if axis == 2 else (0.0, vel, 0.0) if axis == 1 else (0.0, 0.0, -vel)
    dom, _ = make_box("linear", u, v, w, ni=ni, nj=nj, nk=nk, dx=dx, dy=dy, dz=dz)
    shape = tuple(dom["T"][0].shape)
    T0 = limiter_profile(r, shape, axis)
    dom["T"][0].copy_(torch.from_numpy(T0))
    psi, line, slope = limiter_psi(limiter_theta(r, sign), c)
    chosen = {"line": line, "slope": slope, "one": 1.0, "zero": 0.0}[branch]
    assert psi == chosen, (case, psi, line, slope)  # the case sits on its branch
    return dom, limiter_expected(T0, axis, c, sign, psi), psi


def _away(a, margin, vertical):
    nk, nyd, nxd = a.shape
    km = margin if vertical else 0
    return a[km:nk - km, margin:nyd - margin, margin:nxd - margin]


def rel_err_side(got, want, margin=8, vertical=False):
    """max|got - want| / max|want| away from the side boundaries (and from the
    top and bottom when the flow is vertical)."""
    g, e = _away(np.asarray(got), margin, vertical), _away(np.asarray(want), margin, vertical)
    return float(np.abs(g - e).max() / np.abs(e).max())


def rel_err_cells(got, want, margin=8, vertical=False):
    """Largest per-cell relative difference, cells as in rel_err_side."""
    g, e = _away(np.asarray(got), margin, vertical), _away(np.asarray(want), margin, vertical)
    return float((np.abs(g - e) / np.abs(e)).max())


# ---- barotropic subcycle ----
#
# With no Coriolis force, no forcing, a flat bottom (depth H), every cell wet and
# a sea surface of uniform slope, the depth-integrated transport udrho
# (kg m^-1 s^-1) accelerates uniformly, d(udrho)/dt = -H rho0 g grad(eta),
# and its divergence vanishes, so eta does not change away from the walls.  The
# state after subcycle n is u0 + n*a*dtbt; the step's time average over the nts
# subcycles weights n equally (time stepping A, mean n = (nts+1)/2) or by
# nts-n+1 (time stepping B, mean n = (nts+2)/3).

GRAV = 9.8


def make_baro_box(sx, sy, u0, v0, ni=60, nj=50, dx=8000.0, dy=6000.0, depth=4000.0, f=0.0, periodic=False):
    """A one-level grid.Domain with uniform metrics, a uniform Coriolis
    parameter f (0 by default), no forcing, eta = 0.5 + sx*i + sy*j and uniform
    transports (u0, v0) at time level tau; walled, or periodic in both
    directions."""
    import torch
    from mom5_gb300 import grid
    sp = grid.DomainSpec(ni=ni, nj=nj, nk=1, lon0=0.0, lon1=0.1 * ni, lat0=-0.05 * nj, lat1=0.05 * nj,
                         continent=None, hmin=None, depth=depth, ntracers=0, seed=0, cyclic_x=periodic,
                         cyclic_y=periodic)
    dom = grid.make_domain(sp)
    for k, v in (("dxt", dx), ("dxte", dx), ("dxtn", dx), ("dxu", dx), ("dte", dx), ("dtw", dx),
                 ("dyt", dy), ("dyte", dy), ("dytn", dy), ("dyu", dy), ("dus", dy), ("dun", dy),
                 ("dxur", 1 / dx), ("dyur", 1 / dy), ("dxter", 1 / dx), ("dytnr", 1 / dy),
                 ("dat", dx * dy), ("datr", 1 / (dx * dy)), ("daur", 1 / (dx * dy)), ("f", f),
                 ("tmask1", 1.0), ("umask1", 1.0), ("tmasken_e1", 1.0), ("tmasken_n1", 1.0),
                 ("patm", 0.0), ("pme", 0.0), ("river", 0.0), ("source", 0.0), ("eta_smooth", 0.0),
                 ("forcing_u", 0.0), ("forcing_v", 0.0), ("thicku", depth), ("thicken_e", depth),
                 ("thicken_n", depth), ("rho_g", RHO0 * GRAV), ("udrho_u", u0), ("udrho_v", v0)):
        dom[k].fill_(v)
    J, I = np.meshgrid(np.arange(nj + 2, dtype=float), np.arange(ni + 2, dtype=float), indexing="ij")
    eta = torch.from_numpy(0.5 + sx * I + sy * J)
    dom["eta_t"].copy_(eta)
    dom["eta_t_bar"].copy_(eta)
    return dom, (dx, dy, depth)


def baro_expected(sx, sy, u0, v0, nts, dtbt, spacing, stepping_B):
    dx, dy, depth = spacing
    ax, ay = -depth * RHO0 * GRAV * sx / dx, -depth * RHO0 * GRAV * sy / dy
    nbar = (nts + 2) / 3.0 if stepping_B else (nts + 1) / 2.0
    return u0 + ax * dtbt * nbar, v0 + ay * dtbt * nbar


# With a flat sea surface and uniform transports on an f-plane (no forcing, no
# pressure gradient, no divergence) the transports only rotate: the inertial
# oscillation du/dt = f v, dv/dt = -f u.
# - B grid: the subcycle takes it Crank-Nicolson, u(n+1) - u(n) = dt f (v(n) +
#   v(n+1))/2 and likewise for v, which is a rotation by the angle theta with
#   cos(theta) = (1 - a^2)/(1 + a^2), sin(theta) = 2a/(1 + a^2), a = f dt/2:
#   the amplitude is kept exactly.
# - C grid: the Coriolis force is extrapolated by the third-order Adams-Bashforth
#   weights (23, -16, 5)/12 from the subcycles of the same step, u(n+1) = u(n) +
#   dt (23 C(n) - 16 C(n-1) + 5 C(n-2))/12 with C = f v for u and -f u for v,
#   the force of the step's initial state standing in for the subcycles before
#   the first (whose update is then forward Euler).
# The step returns the subcycles' average (weights 1, or nts-n+1 for time
# stepping B).

def baro_inertial_expected(f, u0, v0, nts, dtbt, stepping_B, cgrid=False):
    u, v = float(u0), float(v0)
    hist = [(f * v, -f * u)] * 2  # (C_u, C_v) standing in for the subcycles before the first
    a = 0.5 * f * dtbt
    c, s = (1 - a * a) / (1 + a * a), 2 * a / (1 + a * a)
    su = sv = sw = 0.0
    for n in range(1, nts + 1):
        if cgrid:
            hist.insert(0, (f * v, -f * u))
            cu = sum(w * h[0] for w, h in zip((23 / 12, -16 / 12, 5 / 12), hist))
            cv = sum(w * h[1] for w, h in zip((23 / 12, -16 / 12, 5 / 12), hist))
            u, v = u + dtbt * cu, v + dtbt * cv
        else:
            u, v = c * u + s * v, -s * u + c * v
        w = (nts - n + 1) if stepping_B else 1.0
        su, sv, sw = su + w * u, sv + w * v, sw + w
    return su / sw, sv / sw


def interior2(a, margin=15):
    nyd, nxd = a.shape
    return a[margin:nyd - margin, margin:nxd - margin]
