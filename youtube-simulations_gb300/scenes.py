"""Seeded synthetic scenes: the host-side setup of the reference, restated in numpy.

The reference builds its inputs once per scene on the host, in animation() before its time loop
(wave_billiard.c:654-881):
  * the domain mask ``xy_in`` from ``xy_in_billiard_single_domain``
    (sub_wave.c:5712-6259) evaluated at ``ij_to_xy`` (sub_wave.c:469-476);
  * the speed/damping tables from ``init_ior_2d``'s constant branch
    (sub_wave.c:12983-13002);
  * the initial pulse of ``add_circular_wave`` (wave_common.c:337-351).
This module restates those for the shapes the workloads use, with explicit seeds in
place of the reference's unseeded ``rand()``.  Arrays are flat [nx][ny] (j
contiguous), FP64 fields and int16 masks, as the reference's rows.
"""
import math

import numpy as np

from .params import BC_ABSORBING, BC_DIRICHLET, BC_PERIODIC, make_params

R_PI, R_DPI, R_PID = 3.141592654, 6.283185307, 1.570796327   # global_pdes.c:8-10
D_RECTANGLE, D_ELLIPSE, D_STADIUM, D_POLYGON, D_CIRCLES, D_CIRCLES_IN_RECT = 0, 1, 2, 8, 20, 201


def grid_xy(p):
    """ij_to_xy (sub_wave.c:469-476) for every cell: x[i], y[j]."""
    i = np.arange(p.nx, dtype=np.float64)
    j = np.arange(p.ny, dtype=np.float64)
    x = p.xmin + i * (p.xmax - p.xmin) / float(p.nx)
    y = p.ymin + j * (p.ymax - p.ymin) / float(p.ny)
    return x, y


def mask(p, domain, lam=1.8, npoly=6, apoly=0.0, circles=()):
    """xy_in_billiard_single_domain for the workload shapes (sub_wave.c:5712-6252)."""
    x1, y1 = grid_xy(p)
    x = x1[:, None] * np.ones((1, p.ny))
    y = np.ones((p.nx, 1)) * y1[None, :]
    if domain == D_RECTANGLE:
        m = (np.abs(x) < lam) & (np.abs(y) < 1.0)
    elif domain == D_ELLIPSE:
        m = x * x / (lam * lam) + y * y < 1.0
    elif domain == D_STADIUM:
        m = ((x > -0.5 * lam) & (x < 0.5 * lam) & (y > -1.0) & (y < 1.0))
        m |= np.sqrt((x + 0.5 * lam) * (x + 0.5 * lam) + y * y) < 1.0
        m |= np.sqrt((x - 0.5 * lam) * (x - 0.5 * lam) + y * y) < 1.0
    elif domain == D_POLYGON:
        omega = R_DPI / float(npoly)
        c = lam * math.cos(omega * 0.5)
        m = np.ones(x.shape, dtype=bool)
        for k in range(npoly):
            angle = apoly * R_PID + (k + 0.5) * omega
            m &= (x * math.cos(angle) + y * math.sin(angle)) < c
    elif domain in (D_CIRCLES, D_CIRCLES_IN_RECT):
        m = np.ones(x.shape, dtype=bool)
        for (xc, yc, r) in circles:
            m &= ~((x - xc) * (x - xc) + (y - yc) * (y - yc) < r * r)
        if domain == D_CIRCLES_IN_RECT:
            m &= ~((np.abs(x) >= lam) | (np.abs(y) >= p.ymax - p.xmax + lam))
    else:
        raise ValueError(f"domain {domain} not supported")
    return m.astype(np.int16).reshape(-1)


def tables(p, xy):
    """init_ior_2d constant branch (sub_wave.c:12983-13002): (tcc, tc, tgamma).
    Cells neither inside nor TWOSPEEDS keep 0, as the caller's zeroed arrays."""
    xy = np.asarray(xy).reshape(-1)
    n = xy.size
    tcc, tc, tg = np.zeros(n), np.zeros(n), np.zeros(n)
    inside = xy != 0
    tc[inside] = p.courant
    tcc[inside] = p.courant * p.courant
    tg[inside] = np.where(xy[inside] == 1, p.gamma, p.gammab)
    if p.twospeeds:
        out = ~inside
        tc[out] = p.courantb
        tcc[out] = p.courantb * p.courantb
        tg[out] = p.gammab
    return tcc, tc, tg


def pulse(p, xy, xc, yc, amp=1.0, variance=0.02 ** 2, wavelength=math.inf):
    """add_circular_wave (wave_common.c:337-351) onto a zero field: masked cells
    (or all cells when TWOSPEEDS) get amp*exp(-r^2/variance)*cos(-r/wavelength)."""
    x1, y1 = grid_xy(p)
    d2 = (x1[:, None] - xc) ** 2 + (y1[None, :] - yc) ** 2
    f = amp * np.exp(-d2 / variance)
    if math.isfinite(wavelength):
        f = f * np.cos(-np.sqrt(d2) / wavelength)
    xy2 = np.asarray(xy).reshape(p.nx, p.ny)
    if not p.twospeeds:
        f = np.where(xy2 != 0, f, 0.0)
    return np.ascontiguousarray(f.reshape(-1))


def seeded_point_inside(rng, p, xy, margin=0):
    """A uniformly drawn cell centre inside the mask (rejection sampling)."""
    xy2 = np.asarray(xy).reshape(p.nx, p.ny)
    x1, y1 = grid_xy(p)
    for _ in range(100000):
        i = int(rng.integers(margin + 1, p.nx - 1 - margin))
        j = int(rng.integers(margin + 1, p.ny - 1 - margin))
        if xy2[i, j] > 0:
            return i, j, float(x1[i]), float(y1[j])
    raise RuntimeError("no inside cell found")


def seeded_discs(rng, n, rmin=0.02, rmax=0.1, box=(-2.0, 2.0, -1.125, 1.125)):
    """n discs with radius U(rmin, rmax) and centres uniform in the box."""
    xs = rng.uniform(box[0], box[1], n)
    ys = rng.uniform(box[2], box[3], n)
    rs = rng.uniform(rmin, rmax, n)
    return [(float(a), float(b), float(c)) for a, b, c in zip(xs, ys, rs)]


class Scene:
    """One seeded scene: params plus FP64 host arrays."""

    def __init__(self, params, phi, psi, xy, tcc, tc, tgamma, nbc=None, meta=None):
        self.params, self.phi, self.psi, self.xy = params, phi, psi, xy
        self.tcc, self.tc, self.tgamma, self.nbc = tcc, tc, tgamma, nbc
        self.meta = meta or {}

    @property
    def cells(self):
        return self.params.nx * self.params.ny


def config1(seed=0, nx=1280, ny=720):
    """1280x720 ellipse (semi-axes 1.8, 1.0), Dirichlet, COURANT 0.1, GAMMA 0, one
    Gaussian pulse (amplitude 1, width 0.02) at a seeded point inside, psi = phi."""
    rng = np.random.default_rng(seed)
    p = make_params(nx, ny, b_cond=BC_DIRICHLET, courant=0.1, gamma=0.0)
    xy = mask(p, D_ELLIPSE, lam=1.8)
    tcc, tc, tg = tables(p, xy)
    _, _, xc, yc = seeded_point_inside(rng, p, xy)
    phi = pulse(p, xy, xc, yc)
    return Scene(p, phi, phi.copy(), xy, tcc, tc, tg, meta=dict(seed=seed, centre=(xc, yc)))


def config2(seed=0, nx=3840, ny=2160, ndiscs=64):
    """3840x2160, 64 seeded discs r~U(0.02,0.1) of refractive index 1.5 (TWOSPEEDS with
    COURANTB = COURANT/1.5), absorbing boundary, GAMMA = GAMMAB = 1e-4, point source of
    amplitude 0.05 and seeded period in [20, 60] updates, one Gaussian pulse."""
    rng = np.random.default_rng(seed)
    discs = seeded_discs(rng, ndiscs)
    period = float(rng.uniform(20.0, 60.0))
    p = make_params(nx, ny, b_cond=BC_ABSORBING, twospeeds=1, courant=0.1, courantb=0.1 / 1.5,
                    gamma=1e-4, gammab=1e-4)
    xy = mask(p, D_CIRCLES, circles=discs)
    tcc, tc, tg = tables(p, xy)
    si, sj, _, _ = seeded_point_inside(rng, p, xy, margin=2)
    p.src_on, p.src_i, p.src_j, p.src_amp, p.src_period = 1, si, sj, 0.05, period
    _, _, xc, yc = seeded_point_inside(rng, p, xy)
    phi = pulse(p, xy, xc, yc)
    return Scene(p, phi, phi.copy(), xy, tcc, tc, tg,
                 meta=dict(seed=seed, discs=discs, period=period, source=(si, sj), centre=(xc, yc)))


def batch_member(rng, smin=(256, 256), smax=(1280, 720), bconds=(BC_DIRICHLET, BC_PERIODIC),
                 courant=(0.05, 0.15)):
    """One instance of the uneven batch: size log-uniform between smin and smax cells
    with a seeded aspect, mask in {ellipse, stadium, polygon, disc array}, boundary
    drawn from bconds, COURANT uniform in `courant`, one Gaussian pulse."""
    cmin, cmax = smin[0] * smin[1], smax[0] * smax[1]
    cells = math.exp(rng.uniform(math.log(cmin), math.log(cmax)))
    aspect = math.exp(rng.uniform(math.log(1.0), math.log(16.0 / 9.0)))
    nx = int(round(math.sqrt(cells * aspect)))
    ny = int(round(cells / nx))
    nx, ny = max(nx, 16), max(ny, 16)
    bc = int(bconds[int(rng.integers(0, len(bconds)))])
    c = float(rng.uniform(*courant))
    p = make_params(nx, ny, b_cond=bc, courant=c)
    shape = int(rng.integers(0, 4))
    if shape == 0:
        xy = mask(p, D_ELLIPSE, lam=float(rng.uniform(1.2, 1.9)))
    elif shape == 1:
        xy = mask(p, D_STADIUM, lam=float(rng.uniform(0.6, 1.6)))
    elif shape == 2:
        xy = mask(p, D_POLYGON, lam=float(rng.uniform(0.8, 1.05)), npoly=int(rng.integers(3, 9)),
                  apoly=float(rng.uniform(0, 1)))
    else:
        xs = np.linspace(-1.6, 1.6, 5)
        ys = np.linspace(-0.8, 0.8, 3)
        r = float(rng.uniform(0.08, 0.18))
        xy = mask(p, D_CIRCLES, circles=[(a, b, r) for a in xs for b in ys])
    tcc, tc, tg = tables(p, xy)
    _, _, xc, yc = seeded_point_inside(rng, p, xy)
    phi = pulse(p, xy, xc, yc, variance=0.05 ** 2)
    return Scene(p, phi, phi.copy(), xy, tcc, tc, tg, meta=dict(shape=shape))


def sweep_member(rng, smin=128, smax=512):
    """One instance of the parameter-sweep batch: nx and ny log-uniform between smin and
    smax, a rectangle domain (the whole box) with 1-3 seeded circular obstacles of
    radius U(0.1, 0.3), absorbing boundary, GAMMA U(0, 1e-3), COURANT U(0.05, 0.2), one
    Gaussian pulse at a seeded point inside, psi = phi."""
    nx = int(round(math.exp(rng.uniform(math.log(smin), math.log(smax)))))
    ny = int(round(math.exp(rng.uniform(math.log(smin), math.log(smax)))))
    p = make_params(nx, ny, b_cond=BC_ABSORBING, courant=float(rng.uniform(0.05, 0.2)),
                    gamma=float(rng.uniform(0.0, 1e-3)))
    discs = seeded_discs(rng, int(rng.integers(1, 4)), 0.1, 0.3, box=(-1.6, 1.6, -0.8, 0.8))
    xy = mask(p, D_CIRCLES, circles=discs)
    _, _, xc, yc = seeded_point_inside(rng, p, xy, margin=2)
    phi = pulse(p, xy, xc, yc, variance=0.05 ** 2)
    return Scene(p, phi, phi.copy(), xy, None, None, None, meta=dict(discs=discs))

