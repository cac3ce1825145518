"""Scenario builders: the initial particle states of the ring-impact and plate-tension
set-ups, in the reference's own lattice construction, with either the reference's
constants or the workload constants of the GPU configurations.

Every builder returns a :class:`Scenario` -- per body the 13 input arrays of the
reference's particle (x, y, X, Y, m, rho, h, quad_weight, vx, vy, Sxx, Sxy, Syy),
the convex-hull contact boundary and boundary conditions, plus the simulation
constants and the ordered action list.  All arithmetic is IEEE binary64 in the same
order as the reference's set-up code, so the initial states are bit-identical to the
ones its scenario functions build (checked against the compiled reference).
"""
from __future__ import annotations

import math
import struct
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence

import numpy as np

from .actions import (
    UL_FEM_ACTIONS,
    RINGS_UL_WEAK_ACTIONS,
    TENSILE_UL_WEAK_ACTIONS,
    RINGS_COROT_ACTIONS,
    RINGS_GODUNOV_ACTIONS,
    RINGS_MONAGHAN_ACTIONS,
    RINGS_POTENTIAL_ACTIONS,
    ROTATION_COROT_ACTIONS,
    ROTATION_POTENTIAL_ACTIONS,
    TENSILE_COROT_ACTIONS,
    RINGS_TL_ACTIONS,
    TENSILE_TL_ACTIONS,
    TENSILE_TL_WEAK_ACTIONS,
)

M_1_PI = 0.31830988618379067154  # the C library's M_1_PI

IN_NAMES = ("x", "y", "X", "Y", "m", "rho", "h", "quad_weight", "vx", "vy", "Sxx", "Sxy", "Syy")
OUT_NAMES = ("x", "y", "vx", "vy", "rho", "Sxx", "Sxy", "Syy", "fcx", "fcy")

METHOD_UL, METHOD_TL, METHOD_TL_WEAK, METHOD_COROT, METHOD_POTENTIAL, METHOD_UL_WEAK = 1, 2, 3, 4, 5, 6
BC_PULL_TL = 1       # tensile.cpp:20-42 (total-Lagrangian bodies)
BC_VELOCITY_UL = 2   # tensile.cpp:44-66 (updated-Lagrangian bodies)
SHAPE_RKPM, SHAPE_ELEMENT = 0, 1


def cubic_spline(xi: float, yi: float, xj: float, yj: float, h: float):
    """Scalar 2-D cubic spline W, dW/dx, dW/dy (kernel.cpp:20-55), same operation order."""
    h1 = 1.0 / h
    xij = xi - xj
    yij = yi - yj
    rij = math.sqrt(xij * xij + yij * yij)
    fac = 10 * M_1_PI / 7.0 * h1 * h1
    q = rij * h1
    if q >= 2.0:
        return 0.0, 0.0, 0.0
    if q >= 1.0:
        w = fac * (0.25 * (2 - q) * (2 - q) * (2 - q))
        if rij > 1e-12:
            der = -0.75 * (2 - q) * (2 - q) * h1 / rij
            return w, xij * der * fac, yij * der * fac
        return w, 0.0, 0.0
    w = fac * (1 - 1.5 * q * q * (1 - 0.5 * q))
    if rij > 1e-12:
        der = -3.0 * q * (1 - 0.75 * q) * h1 / rij
        return w, xij * der * fac, yij * der * fac
    return w, 0.0, 0.0


@dataclass
class BC:
    kind: int
    v: float
    idx: np.ndarray


@dataclass
class Body:
    arrays: Dict[str, np.ndarray]
    hull: np.ndarray = field(default_factory=lambda: np.zeros(0, np.uint32))
    bcs: List[BC] = field(default_factory=list)
    ex: int = 0
    ey: int = 0
    # per-body constants overriding the scenario's (ensembles): keys of Scenario
    # (E, nu, rho0, dt, wdeltap, ...)
    params: Dict[str, float] = field(default_factory=dict)
    # METHOD_UL_WEAK: the stress points, the same 13 arrays as the particles;
    # METHOD_TL_WEAK with an explicit element map: the Gauss points as the set-up left them
    gp: Optional[Dict[str, np.ndarray]] = None
    # METHOD_TL_WEAK with ex = ey = 0: element map (n_elem x 4: ll, lr, tr, tl), Gauss order,
    # shape functions (SHAPE_RKPM or SHAPE_ELEMENT)
    quads: Optional[np.ndarray] = None
    order: int = 2
    shape: int = 0

    @property
    def n(self) -> int:
        return int(self.arrays["x"].shape[0])


@dataclass
class Scenario:
    method: int
    bodies: List[Body]
    actions: List[int]
    dt: float
    nu: float
    E: float
    rho0: float
    wdeltap: float = 0.0
    corr_exp: float = 0.0
    mghn_eps: float = 0.0
    alpha: float = 0.0
    beta: float = 0.0
    eta: float = 0.0
    xsph_eps: float = 0.0
    do_smooth: int = 0
    nbh_h: float = 0.0
    nbh_eps: float = 1e-6
    gp_h: float = 0.0
    gp_rho: float = 0.0
    contact: int = 0
    name: str = ""
    # contact groups per body (bodies touch only within their group); None: all in group 0,
    # or one group per body when bodies carry their own constants (ensembles of one body)
    groups: Optional[List[int]] = None

    @property
    def n_total(self) -> int:
        return sum(b.n for b in self.bodies)

    # physical_constants, simulation_data.cpp:32-47
    @property
    def G(self) -> float:
        return self.E / (2.0 * (1.0 + self.nu))

    @property
    def K(self) -> float:
        g = self.G
        return 2.0 * g * (1 + self.nu) / (3 * (1 - 2 * self.nu))

    @property
    def c0(self) -> float:
        return math.sqrt(self.K / self.rho0)


def _body_from_lists(xs, ys, X=None, Y=None) -> Dict[str, np.ndarray]:
    n = len(xs)
    a = {k: np.zeros(n, np.float64) for k in IN_NAMES}
    a["x"][:] = xs
    a["y"][:] = ys
    if X is not None:
        a["X"][:] = X
        a["Y"][:] = Y
    return a


def _ring_lattice(nbox: int, dx: float, ro: float, ri: float):
    """Lattice points of one annulus, in the reference's loop order (rings.cpp:40-56)."""
    px, py = _ring_lattice_np(nbox, dx, ro, ri)
    return list(zip(px.tolist(), py.tolist()))


def _ring_lattice_np(nbox: int, dx: float, ro: float, ri: float, edge_tol: float = 0.0):
    """Vectorised :func:`_ring_lattice`: the same IEEE operations elementwise
    (px = -ro + i*dx, dist = sqrt(px*px + py*py)), i-major order.

    edge_tol > 0 leaves out the lattice points within that relative distance of either
    circle.  The lattice always has points exactly on the outer circle ((+-ro, 0) among
    them, the points where two rings meet first); whether their rounded distance falls
    below ro depends on ro's last bits, so without a tolerance two nearly equal radii
    can give rings with different outlines."""
    i = np.arange(nbox, dtype=np.float64)
    p = -ro + i * dx
    PX, PY = np.meshgrid(p, p, indexing="ij")
    dist = np.sqrt(PX * PX + PY * PY)
    mask = (dist < ro * (1.0 - edge_tol)) & (dist >= ri * (1.0 + edge_tol))
    return PX[mask], PY[mask]


def convex_hull(x: np.ndarray, y: np.ndarray) -> np.ndarray:
    """Monotone-chain hull indices with collinear points kept (convex_hull.h:62-95).

    Ties in the (x, y) sort are impossible for distinct lattice points, so the order is
    the unique lexicographic one the reference's std::sort produces.
    """
    n = len(x)
    order = sorted(range(n), key=lambda i: (x[i], y[i]))
    pts = [(float(x[i]), float(y[i]), i) for i in order]

    def ccw(p1, p2, p3):
        return (p2[0] - p1[0]) * (p3[1] - p1[1]) - (p2[1] - p1[1]) * (p3[0] - p1[0])

    hull = [None] * n
    k = 0
    for i in range(n):
        while k >= 2 and ccw(hull[k - 2], hull[k - 1], pts[i]) < 0:
            k -= 1
        hull[k] = pts[i]
        k += 1
    t = k + 1
    for i in range(n - 2, -1, -1):
        while k >= t and ccw(hull[k - 2], hull[k - 1], pts[i]) < 0:
            k -= 1
        hull[k] = pts[i]
        k += 1
    return np.array([hull[i][2] for i in range(k - 1)], np.uint32)


def rings(
    nbox: int,
    *,
    ro: float = 0.04,
    ri: float = 0.03,
    spacing: Optional[float] = None,
    rho0: float = 1.0,
    E: float = 1e7,
    nu: float = 0.4,
    hdx: float = 1.7,
    speed: float = 180.0,
    dt: Optional[float] = 1e-6,
    cfl: float = 0.3,
    method: int = METHOD_UL,
    two_bodies: bool = False,
    alpha: float = 1.0,
    beta: float = 1.0,
    eta: float = 0.1,
    art_stress_eps: float = 0.3,
    stress_exponent: float = 4.0,
    xsph_eps: float = 0.5,
    nbh_eps: float = 1e-6,
    edge_tol: float = 0.0,
    exact_hull: bool = False,
    godunov: bool = False,
    name: str = "",
) -> Scenario:
    """Two rings on a square lattice, as rings_monaghan (rings.cpp:20-99),
    rings_monaghan_contact (:522-621), rings_tl_contact (:338-429) and the other
    families' ring set-ups build them.

    Defaults are the reference's constants; ``dt=None`` selects dt = cfl*h/c0.
    ``godunov`` selects the Godunov action list for UL (all correction constants zero).
    ``exact_hull`` runs the hull's orientation tests on the integer lattice indices
    instead of the rounded coordinates, so the points kept on straight hull edges do not
    depend on rounding (the reference tests the coordinates).
    """
    if spacing is None:
        spacing = ro + 0.001
    dx = 2 * ro / (nbox - 1)
    pts = _ring_lattice(nbox, dx, ro, ri)
    tl = method in (METHOD_TL, METHOD_COROT, METHOD_POTENTIAL)
    sc = Scenario(method=method, bodies=[], actions=[], dt=0.0, nu=nu, E=E, rho0=rho0, name=name)
    if dt is None:
        dt = cfl * (hdx * dx) / sc.c0
    sc.dt = dt

    def finish(a: Dict[str, np.ndarray], vx) -> None:
        a["rho"][:] = rho0
        a["h"][:] = hdx * dx
        a["m"][:] = dx * dx * rho0
        a["quad_weight"][:] = a["m"] / a["rho"]
        a["vx"][:] = vx

    px, py = _ring_lattice_np(nbox, dx, ro, ri, edge_tol)
    # hull candidates: only lattice points within 3 dx of the outer circle can be hull
    # vertices or lie on hull edges, and the monotone chain visits any subset in the
    # same relative order, so the hull of the subset is the hull of the ring
    cand = np.nonzero(np.sqrt(px * px + py * py) >= ro - 3 * dx)[0]
    if not two_bodies:
        xs = np.stack([px - spacing, px + spacing], axis=1).ravel()
        ys = np.stack([py, py], axis=1).ravel()
        a = _body_from_lists(xs, ys, xs if tl else None, ys if tl else None)
        vx = np.where(a["x"] < 0.0, speed, -speed)
        finish(a, vx)
        sc.bodies = [Body(a)]
    else:
        for sgn, v in ((-1.0, speed), (1.0, -speed)):
            xs = px + sgn * spacing
            ys = py.copy()
            a = _body_from_lists(xs, ys, xs if tl else None, ys if tl else None)
            finish(a, v)
            if exact_hull:
                li, lj = np.rint((px + ro) / dx), np.rint((py + ro) / dx)
                hull = cand[convex_hull(li[cand], lj[cand])].astype(np.uint32)
            else:
                hull = cand[convex_hull(xs[cand], ys[cand])].astype(np.uint32)
            sc.bodies.append(Body(a, hull=hull))
        sc.contact = 1

    if method == METHOD_UL and godunov:
        sc.actions = list(RINGS_GODUNOV_ACTIONS)
    elif method == METHOD_UL:
        _monaghan_constants(sc, dx, hdx, alpha, beta, eta, art_stress_eps, stress_exponent, xsph_eps)
    else:
        sc.actions = list({METHOD_TL: RINGS_TL_ACTIONS, METHOD_COROT: RINGS_COROT_ACTIONS,
                           METHOD_POTENTIAL: RINGS_POTENTIAL_ACTIONS}[method])
        sc.alpha, sc.beta, sc.eta = alpha, beta, eta
        sc.nbh_h = hdx * dx
    sc.nbh_eps = nbh_eps
    return sc


def _monaghan_constants(sc: Scenario, dx: float, hdx: float, alpha: float = 1.0, beta: float = 1.0,
                        eta: float = 0.1, art_stress_eps: float = 0.3, stress_exponent: float = 4.0,
                        xsph_eps: float = 0.5) -> None:
    """The Gray-Monaghan action list and correction constants of the reference's UL
    set-ups (rings.cpp:58-96): W(dx) for the artificial stress, exponent 4, eps 0.3,
    XSPH 0.5."""
    sc.actions = list(RINGS_MONAGHAN_ACTIONS)
    sc.alpha, sc.beta, sc.eta = alpha, beta, eta
    sc.wdeltap = cubic_spline(0, 0, dx, 0, hdx * dx)[0]
    sc.corr_exp = stress_exponent
    sc.mghn_eps = art_stress_eps
    sc.xsph_eps = xsph_eps


def rings_monaghan(nbox: int) -> Scenario:
    """The reference's rings_monaghan(nbox), rings.cpp:20-99."""
    return rings(nbox, name=f"rings_monaghan({nbox})")


def rings_monaghan_contact(nbox: int) -> Scenario:
    """The reference's rings_monaghan_contact(nbox), rings.cpp:522-621."""
    return rings(nbox, two_bodies=True, name=f"rings_monaghan_contact({nbox})")


def rings_tl_contact(nbox: int) -> Scenario:
    """The reference's rings_tl_contact(nbox), rings.cpp:338-429."""
    return rings(nbox, method=METHOD_TL, two_bodies=True, dt=1e-7, alpha=3.0, beta=3.0, eta=0.1,
                 name=f"rings_tl_contact({nbox})")


def rings_corot_contact(nbox: int) -> Scenario:
    """The reference's rings_corot_contact(nbox), rings.cpp:245-336."""
    return rings(nbox, method=METHOD_COROT, two_bodies=True, dt=1e-7, alpha=1.0, beta=1.0, eta=0.1,
                 name=f"rings_corot_contact({nbox})")


def rings_godunov(nbox: int) -> Scenario:
    """The reference's rings_godunov(nbox), rings.cpp:101-162: both rings in one body."""
    return rings(nbox, godunov=True, dt=1e-7, name=f"rings_godunov({nbox})")


def rings_godunov_contact(nbox: int) -> Scenario:
    """The reference's rings_godunov_contact(nbox), rings.cpp:164-243."""
    return rings(nbox, godunov=True, two_bodies=True, dt=1e-7, name=f"rings_godunov_contact({nbox})")


def rings_potential_contact(nbox: int) -> Scenario:
    """The reference's rings_potential_contact(nbox), rings.cpp:431-520: rings of radius
    1 m and 0.75 m, h = 1.3 dx."""
    return rings(nbox, ro=1.0, ri=0.75, hdx=1.3, method=METHOD_POTENTIAL, two_bodies=True, dt=1e-7, alpha=1.0,
                 beta=1.0, eta=0.1, name=f"rings_potential_contact({nbox})")


def disc(nbox: int, *, method: int, actions: Sequence[int], hdx: float, dt: float, ro: float = 1.0,
         rho0: float = 1.0, E: float = 1e7, nu: float = 0.4, omega_r: float = 50.0, alpha: float = 0.0,
         beta: float = 0.0, eta: float = 0.0, name: str = "") -> Scenario:
    """A disc spinning as a rigid body (v = omega x r, |v| = omega_r at r = ro), the
    rotation set-ups of rotation.cpp (lattice px = -ro + i*dx, disc dist < ro)."""
    dx = 2 * ro / (nbox - 1)
    px, py = _ring_lattice_np(nbox, dx, ro, 0.0)
    tl = method != METHOD_UL
    a = _body_from_lists(px, py, px if tl else None, py if tl else None)
    a["rho"][:] = rho0
    a["h"][:] = hdx * dx
    a["m"][:] = dx * dx * rho0
    a["quad_weight"][:] = a["m"] / a["rho"]
    a["vx"][:] = -a["y"] / ro * omega_r
    a["vy"][:] = +a["x"] / ro * omega_r
    sc = Scenario(method=method, bodies=[Body(a)], actions=list(actions), dt=dt, nu=nu, E=E, rho0=rho0, alpha=alpha,
                  beta=beta, eta=eta, name=name)
    if tl:
        sc.nbh_h = hdx * dx
    return sc


def rotation_monaghan(nbox: int) -> Scenario:
    """The reference's rotation_monaghan(nbox), rotation.cpp:274-351."""
    sc = disc(nbox, method=METHOD_UL, actions=RINGS_MONAGHAN_ACTIONS, hdx=1.7, dt=1e-5,
              name=f"rotation_monaghan({nbox})")
    _monaghan_constants(sc, 2.0 / (nbox - 1), 1.7)
    return sc


def rotation_tl(nbox: int) -> Scenario:
    """The reference's rotation_tl(nbox), rotation.cpp:142-210 (the reference notes that
    the total-Lagrangian disc fails as rotations grow)."""
    return disc(nbox, method=METHOD_TL, actions=TENSILE_TL_ACTIONS, hdx=1.7, dt=1e-6, alpha=3.0, beta=3.0, eta=0.1,
                name=f"rotation_tl({nbox})")


def rotation_godunov(nbox: int) -> Scenario:
    """The reference's rotation_godunov(nbox), rotation.cpp:20-76."""
    return disc(nbox, method=METHOD_UL, actions=RINGS_GODUNOV_ACTIONS, hdx=1.7, dt=1e-6,
                name=f"rotation_godunov({nbox})")


def rotation_corot(nbox: int) -> Scenario:
    """The reference's rotation_corot(nbox), rotation.cpp:78-140 (no artificial viscosity)."""
    return disc(nbox, method=METHOD_COROT, actions=ROTATION_COROT_ACTIONS, hdx=1.3, dt=2.5e-6, alpha=1.0, beta=1.0,
                eta=0.1, name=f"rotation_corot({nbox})")


def rotation_potential(nbox: int) -> Scenario:
    """The reference's rotation_potential(nbox), rotation.cpp:212-272 (no artificial viscosity)."""
    return disc(nbox, method=METHOD_POTENTIAL, actions=ROTATION_POTENTIAL_ACTIONS, hdx=1.7, dt=1e-6, alpha=1.0,
                beta=1.0, eta=0.1, name=f"rotation_potential({nbox})")


def workload_nbh_eps(dx: float) -> float:
    """Scale-aware neighbour epsilon: the reference's 1e-6 m^2 at dx = 1 mm, scaled with dx^2.

    The reference's absolute +1e-6 m^2 grows the search radius to ~20 dx at dx = 0.05 mm,
    overflowing its own MAX_NBH; scaling it keeps the radius sqrt(4 h^2 + dx^2)."""
    return 1e-6 * (dx / 1e-3) ** 2


def c1_rings(dx: float = 1e-3, two_bodies: bool = False, method: int = METHOD_UL, **kw) -> Scenario:
    """Ring impact with the workload constants: r_in 0.03 m, r_out 0.04 m, centres 0.09 m
    apart, E 1e7 Pa, nu 0.4, rho 1200 kg/m^3, +-10 m/s, h = 1.3 dx, dt = 0.3 h / c0."""
    nbox = int(round(0.08 / dx)) + 1
    params = dict(spacing=0.045, rho0=1200.0, E=1e7, nu=0.4, hdx=1.3, speed=10.0, dt=None, cfl=0.3,
                  alpha=1.0, beta=1.0, eta=0.1, art_stress_eps=0.3, stress_exponent=4.0, xsph_eps=0.5,
                  nbh_eps=workload_nbh_eps(2 * 0.04 / (nbox - 1)))
    if method == METHOD_TL:
        params.update(alpha=3.0, beta=3.0)
    params.update(kw)
    return rings(nbox, method=method, two_bodies=two_bodies, name=f"rings dx={dx}", **params)


def c2_rings_tl(dx: float = 5e-5, **kw) -> Scenario:
    """Ring impact, total-Lagrangian SPH with Randles-Libersky correction, two bodies with
    penalty contact (the rings_tl_contact structure) and the workload constants."""
    return c1_rings(dx=dx, two_bodies=True, method=METHOD_TL, **kw)


def tensile_plate(
    nx: int,
    ny: int,
    *,
    Lx: float,
    method: int = METHOD_TL,
    rho0: float = 1.0,
    E: float = 1e7,
    nu: float = 0.4,
    hdx: float = 1.0,
    pull: float = 10.0,
    dt: Optional[float] = 1e-6,
    cfl: float = 0.3,
    jitter: float = 0.0,
    seed: int = 0,
    alpha: float = 1.0,
    beta: float = 1.0,
    eta: float = 0.1,
    do_smooth: int = 1,
    nbh_eps: float = 1e-6,
    godunov: bool = False,
    bc_cols: int = 1,
    name: str = "",
) -> Scenario:
    """A rectangular plate pulled at both ends: tensile_tl (tensile.cpp:213-289) and
    tensile_tl_weak (:731-826) lattices (px = i*dx, py = j*dx; column i = 0 and
    i = nx-1 carry the pull), generalised to nx != ny and optional seeded jitter.
    Updated-Lagrangian plates (tensile_monaghan :363-450, tensile_godunov :68-135 with
    ``godunov``) carry the velocity conditions of tensile.cpp:44-66 and no reference
    coordinates; ``bc_cols`` lattice columns at each end are pulled (tensile_monaghan
    pulls three, tensile.cpp:392-398)."""
    dx = Lx / (nx - 1)
    I, J = np.meshgrid(np.arange(nx, dtype=np.float64), np.arange(ny, dtype=np.float64), indexing="ij")
    xs = (I * dx).ravel()
    ys = (J * dx).ravel()
    left = np.arange(bc_cols * ny, dtype=np.uint32)
    right = (np.uint32(nx - bc_cols) * np.uint32(ny) + np.arange(bc_cols * ny, dtype=np.uint32)).astype(np.uint32)
    if jitter > 0.0:
        rng = np.random.default_rng(seed)
        xs = xs + rng.uniform(-jitter, jitter, xs.shape) * dx
        ys = ys + rng.uniform(-jitter, jitter, ys.shape) * dx
    ul = method == METHOD_UL
    a = _body_from_lists(xs, ys, None if ul else xs, None if ul else ys)
    a["rho"][:] = rho0
    a["h"][:] = hdx * dx
    a["m"][:] = dx * dx * rho0
    a["quad_weight"][:] = a["m"] / a["rho"]
    kind = BC_VELOCITY_UL if ul else BC_PULL_TL
    body = Body(a, bcs=[BC(kind, -pull, left), BC(kind, pull, right)])
    sc = Scenario(method=method, bodies=[body], actions=[], dt=0.0, nu=nu, E=E, rho0=rho0, name=name)
    sc.dt = dt if dt is not None else cfl * (hdx * dx) / sc.c0
    sc.nbh_eps = nbh_eps
    if ul:
        if godunov:
            sc.actions = list(RINGS_GODUNOV_ACTIONS)
        else:
            _monaghan_constants(sc, dx, hdx, alpha, beta, eta)
        return sc
    sc.nbh_h = hdx * dx
    if method in (METHOD_TL, METHOD_COROT, METHOD_POTENTIAL):
        sc.actions = list({METHOD_TL: TENSILE_TL_ACTIONS, METHOD_COROT: TENSILE_COROT_ACTIONS,
                           METHOD_POTENTIAL: RINGS_POTENTIAL_ACTIONS}[method])
        sc.alpha, sc.beta, sc.eta = alpha, beta, eta
    else:
        sc.actions = list(TENSILE_TL_WEAK_ACTIONS)
        sc.do_smooth = do_smooth
        sc.gp_h = hdx * dx
        sc.gp_rho = rho0
        # element_map_rectangle(ex, ey) numbers nodes row by row with ex+1 nodes per
        # row (element.cpp:23-39); here rows run along the outer (x) index, so a row
        # holds the ny nodes of one lattice column
        body.ex, body.ey = ny - 1, nx - 1
    return sc


def tensile_tl(nbox: int) -> Scenario:
    """The reference's tensile_tl(nbox), tensile.cpp:213-289."""
    return tensile_plate(nbox, nbox, Lx=1.0, method=METHOD_TL, hdx=1.0, dt=1e-6, name=f"tensile_tl({nbox})")


def tensile_corot(nbox: int) -> Scenario:
    """The reference's tensile_corot(nbox), tensile.cpp:137-211."""
    return tensile_plate(nbox, nbox, Lx=1.0, method=METHOD_COROT, hdx=1.0, dt=1e-6, name=f"tensile_corot({nbox})")


def tensile_monaghan(nbox: int) -> Scenario:
    """The reference's tensile_monaghan(nbox), tensile.cpp:363-450."""
    return tensile_plate(nbox, nbox, Lx=1.0, method=METHOD_UL, hdx=1.3, dt=1e-6, bc_cols=3,
                         name=f"tensile_monaghan({nbox})")


def tensile_godunov(nbox: int) -> Scenario:
    """The reference's tensile_godunov(nbox), tensile.cpp:68-135."""
    return tensile_plate(nbox, nbox, Lx=1.0, method=METHOD_UL, hdx=1.7, dt=1e-6, godunov=True,
                         name=f"tensile_godunov({nbox})")


def tensile_potential(nbox: int) -> Scenario:
    """The reference's tensile_potential(nbox), tensile.cpp:291-361."""
    return tensile_plate(nbox, nbox, Lx=1.0, method=METHOD_POTENTIAL, hdx=1.0, dt=1e-6,
                         name=f"tensile_potential({nbox})")


def tensile_tl_weak(nbox: int) -> Scenario:
    """The reference's tensile_tl_weak(nbox), tensile.cpp:731-826."""
    return tensile_plate(nbox, nbox, Lx=1.0, method=METHOD_TL_WEAK, hdx=1.3, dt=1e-7, alpha=0.0, beta=0.0,
                         eta=0.0, name=f"tensile_tl_weak({nbox})")


def c3_plate(dx: float = 2e-5, Lx: float = 0.1, Ly: float = 0.02, seed: int = 20261203, **kw) -> Scenario:
    """Uniaxial tension of a steel plate with the weak-form RKPM structure: E 2e11 Pa,
    nu 0.3, rho 7850 kg/m^3, ends at +-1 m/s, +-1% dx seeded jitter, h = 1.3 dx."""
    nx = int(round(Lx / dx)) + 1
    ny = int(round(Ly / dx)) + 1
    params = dict(rho0=7850.0, E=2e11, nu=0.3, hdx=1.3, pull=1.0, dt=None, cfl=0.3, jitter=0.01, seed=seed,
                  alpha=0.0, beta=0.0, eta=0.0, nbh_eps=workload_nbh_eps(dx))
    params.update(kw)
    return tensile_plate(nx, ny, Lx=Lx, method=METHOD_TL_WEAK, name=f"plate dx={dx}", **params)


def c4_ensemble(n_instances: int = 512, seed: int = 20261203, dx_range=(2e-4, 1e-3), E_range=(5e6, 5e7),
                nu_range=(0.3, 0.45), speed_range=(5.0, 40.0), rho0: float = 1200.0) -> Scenario:
    """Batched ensemble of independent ring impacts, one body per instance, each with its
    own seeded dx ~ U[0.2, 1] mm, E ~ U[5e6, 5e7] Pa, nu ~ U[0.3, 0.45] and ring speed
    ~ U[5, 40] m/s (Gray-Monaghan SPH, the ring workload's other constants).  Instance k
    draws from numpy's PCG64 seeded with seed + k, so any subset is reproducible alone."""
    bodies = []
    first = None
    for k in range(n_instances):
        rng = np.random.default_rng(seed + k)
        dx = rng.uniform(*dx_range)
        E = rng.uniform(*E_range)
        nu = rng.uniform(*nu_range)
        speed = rng.uniform(*speed_range)
        sc = c1_rings(dx=dx, E=E, nu=nu, speed=speed, rho0=rho0)
        b = sc.bodies[0]
        b.params = {"E": sc.E, "nu": sc.nu, "rho0": sc.rho0, "dt": sc.dt, "wdeltap": sc.wdeltap, "dx": dx,
                    "speed": speed}
        bodies.append(b)
        if first is None:
            first = sc
    ens = Scenario(method=METHOD_UL, bodies=bodies, actions=list(first.actions), dt=first.dt, nu=first.nu, E=first.E,
                   rho0=rho0, wdeltap=first.wdeltap, corr_exp=first.corr_exp, mghn_eps=first.mghn_eps,
                   alpha=first.alpha, beta=first.beta, eta=first.eta, xsph_eps=first.xsph_eps,
                   nbh_eps=first.nbh_eps, name=f"ensemble of {n_instances} ring impacts")
    return ens


# ------------------------------------------------------------ UL weak form
def element_map_rectangle(ex: int, ey: int) -> np.ndarray:
    """element_map_rectangle (element.cpp:23-39): rows of (ll, lr, tr, tl) node
    indices, ex elements per row, nodes numbered row by row with ex+1 per row."""
    out = []
    nx = ex + 1
    inc = 0
    for i in range(ey):
        for _ in range(ex):
            out.append((inc, inc + 1, inc + nx + 1, inc + nx))
            inc += 1
        inc = (i + 1) * nx
    return np.array(out, dtype=np.int64).reshape(-1, 4)


def mesh_ring(nbox: int, rin: float, rout: float):
    """mesh_ring (benchmarks/utils.h:20-109): the lattice x = i dx - rout, y = j dx - rout
    reduced to the quads whose four corners all lie strictly inside the annulus
    (rin^2 < r^2 < rout^2), and to the nodes those quads use, renumbered in lattice
    order.  Returns the nodes' x, y and the remapped (ll, lr, tr, tl) elements."""
    dx = 2.0 * rout / (nbox - 1)
    I, J = np.meshgrid(np.arange(nbox, dtype=np.float64), np.arange(nbox, dtype=np.float64), indexing="ij")
    px = (I * dx - rout).ravel()
    py = (J * dx - rout).ravel()
    el = element_map_rectangle(nbox - 1, nbox - 1)
    r = px * px + py * py
    inside = (r < rout * rout) & (r > rin * rin)
    el = el[inside[el].all(axis=1)]
    used = np.zeros(len(px), bool)
    used[el.ravel()] = True
    new = np.cumsum(used) - 1
    return px[used], py[used], new[el]


def _gauss_centres(x: np.ndarray, y: np.ndarray, el: np.ndarray):
    """The one-point Gauss rule of gauss_int(elements, 1) (gauss_integration.h:47-123):
    the shape functions at the element centre are all 0.25 exactly, so each stress point
    is 0.25 x_ll + 0.25 x_lr + 0.25 x_tr + 0.25 x_tl, summed in that order."""
    gx = ((x[el[:, 0]] * 0.25 + x[el[:, 1]] * 0.25) + x[el[:, 2]] * 0.25) + x[el[:, 3]] * 0.25
    gy = ((y[el[:, 0]] * 0.25 + y[el[:, 1]] * 0.25) + y[el[:, 2]] * 0.25) + y[el[:, 3]] * 0.25
    return gx, gy


def _ul_weak_body(x, y, X, Y, gx, gy, GX, GY, dx, hdx, rho0, vx=0.0, vy=0.0) -> Body:
    a = _body_from_lists(x, y, X, Y)
    g = _body_from_lists(gx, gy, GX, GY)
    for d in (a, g):
        d["rho"][:] = rho0
        d["h"][:] = hdx * dx
        d["m"][:] = dx * dx * rho0
        d["quad_weight"][:] = d["m"] / d["rho"]
    a["vx"][:] = vx
    a["vy"][:] = vy
    b = Body(a)
    b.gp = g
    return b


def _ul_weak_scenario(bodies, actions, dt, dx, name, contact=0, nu=0.4, E=1e7, rho0=1.0) -> Scenario:
    # correction_constants(.., 0, true): velocity smoothing on, the rest zero;
    # candidates by find_neighbors(.., 1.5*dx, distance_manhattan)
    sc = Scenario(method=METHOD_UL_WEAK, bodies=bodies, actions=list(actions), dt=dt, nu=nu, E=E, rho0=rho0,
                  do_smooth=1, contact=contact, name=name)
    sc.nbh_h = 1.5 * dx
    return sc


def tensile_ul_weak(nbox: int) -> Scenario:
    """The reference's tensile_ul_weak(nbox), tensile.cpp:626-729: the plate lattice with
    one stress point per cell centre, velocity conditions on the end columns."""
    dx = 1.0 / (nbox - 1)
    I, J = np.meshgrid(np.arange(nbox, dtype=np.float64), np.arange(nbox, dtype=np.float64), indexing="ij")
    x, y = (I * dx).ravel(), (J * dx).ravel()
    I, J = np.meshgrid(np.arange(nbox - 1, dtype=np.float64), np.arange(nbox - 1, dtype=np.float64), indexing="ij")
    gx, gy = (I * dx + dx / 2).ravel(), (J * dx + dx / 2).ravel()
    b = _ul_weak_body(x, y, None, None, gx, gy, None, None, dx, 1.0, 1.0)
    left = np.arange(nbox, dtype=np.uint32)
    right = (np.uint32(nbox - 1) * np.uint32(nbox) + left).astype(np.uint32)
    b.bcs = [BC(BC_VELOCITY_UL, -10.0, left), BC(BC_VELOCITY_UL, 10.0, right)]
    return _ul_weak_scenario([b], TENSILE_UL_WEAK_ACTIONS, 1e-6, dx, f"tensile_ul_weak({nbox})")


def rotation_ul_weak(nbox: int) -> Scenario:
    """The reference's rotation_ul_weak(nbox), rotation.cpp:466-535: mesh_ring(nbox, 0, 1)
    with one stress point per quad, spinning at 50 m/s rim speed."""
    ro = 1.0
    dx = 2 * ro / (nbox - 1)
    x, y, el = mesh_ring(nbox, 0.0, ro)
    gx, gy = _gauss_centres(x, y, el)
    b = _ul_weak_body(x, y, x, y, gx, gy, gx, gy, dx, 1.0, 1.0, vx=-y / ro * 50, vy=+x / ro * 50)
    return _ul_weak_scenario([b], RINGS_UL_WEAK_ACTIONS, 1e-6, dx, f"rotation_ul_weak({nbox})")


def rings_ul_weak_contact(nbox: int) -> Scenario:
    """The reference's rings_ul_weak_contact(nbox), rings.cpp:817-934: two meshed rings
    (mesh_ring, r 0.03-0.04 m) at +-(ro + 1 mm), one stress point per quad, 180 m/s
    each, penalty contact on their hulls.  The shift applies to x only: X keeps the
    unshifted positions, as the reference's does."""
    ri, ro = 0.03, 0.04
    spacing = ro + 0.001
    dx = 2 * ro / (nbox - 1)
    x, y, el = mesh_ring(nbox, ri, ro)
    gx, gy = _gauss_centres(x, y, el)
    bodies = []
    for sgn, v in ((-1.0, 180.0), (1.0, -180.0)):
        xs = x - spacing if sgn < 0 else x + spacing
        gxs = gx - spacing if sgn < 0 else gx + spacing
        b = _ul_weak_body(xs, y, x, y, gxs, gy, gx, gy, dx, 1.0, 1.0, vx=v)
        b.hull = convex_hull(xs, y)
        bodies.append(b)
    return _ul_weak_scenario(bodies, RINGS_UL_WEAK_ACTIONS, 1e-7, dx, f"rings_ul_weak_contact({nbox})", contact=1)


def gauss_points(X: np.ndarray, Y: np.ndarray, el: np.ndarray, order: int = 2):
    """update_gauss_points (gauss_integration.h:47-123) on the nodes' reference positions:
    per element (rows of ``el``) the order x order points of the tensor rule
    (get_weight_pos_2d, gauss_integration.cpp:144-157: abscissa i of xi, j of eta, point
    i*order + j), placed by the bilinear functions (transpose(m_node) * N, summed over
    the nodes in order) with weight w_i w_j J, J = -det(x_xi) accumulated node by node.
    Returns the points' x, y and weights, element-major."""
    p1, w1 = {1: ([0.0], [2.0]), 2: ([0.577350269189626, -0.577350269189626], [1.0, 1.0])}[order]
    mx, my = X[el], Y[el]
    par_x, par_y = (-1.0, 1.0, 1.0, -1.0), (-1.0, -1.0, 1.0, 1.0)
    npe = order * order
    gx = np.empty((len(el), npe))
    gy = np.empty_like(gx)
    qw = np.empty_like(gx)
    for k in range(npe):
        xi, eta, lw = p1[k // order], p1[k % order], w1[k // order] * w1[k % order]
        N = [0.25 * (1 + par_x[I] * xi) * (1 + par_y[I] * eta) for I in range(4)]
        gx[:, k] = mx[:, 0] * N[0] + mx[:, 1] * N[1] + mx[:, 2] * N[2] + mx[:, 3] * N[3]
        gy[:, k] = my[:, 0] * N[0] + my[:, 1] * N[1] + my[:, 2] * N[2] + my[:, 3] * N[3]
        a00 = a01 = a10 = a11 = 0.0
        for I in range(4):
            a00 = a00 + 0.25 * mx[:, I] * par_x[I] * (1 + par_y[I] * eta)
            a10 = a10 + 0.25 * mx[:, I] * par_y[I] * (1 + par_x[I] * xi)
            a01 = a01 + 0.25 * my[:, I] * par_x[I] * (1 + par_y[I] * eta)
            a11 = a11 + 0.25 * my[:, I] * par_y[I] * (1 + par_x[I] * xi)
        qw[:, k] = lw * -(a00 * a11 - a10 * a01)
    return gx.ravel(), gy.ravel(), qw.ravel()


def _tl_element_body(x, y, X, Y, el, *, dx, rho0, fem, hdx=1.0, vx=0.0, vy=0.0, gshift=0.0) -> Body:
    """A weak TL body on an explicit element map with 2x2 Gauss points: fem nodes carry
    unit quad weights and no density or h (the *_fem set-ups), RKPM particles
    rho0, h = hdx dx and quad weight m / rho; the Gauss points take rho0 (and h = hdx dx
    with RKPM) and sit where update_gauss_points put them, shifted by ``gshift``."""
    a = _body_from_lists(x, y, X, Y)
    a["m"][:] = dx * dx * rho0
    if fem:
        a["quad_weight"][:] = 1.0
    else:
        a["rho"][:] = rho0
        a["h"][:] = hdx * dx
        a["quad_weight"][:] = a["m"] / a["rho"]
    a["vx"][:] = vx
    a["vy"][:] = vy
    GX, GY, qw = gauss_points(a["X"], a["Y"], el, 2)
    g = _body_from_lists(GX + gshift if gshift else GX, GY, GX, GY)
    g["rho"][:] = rho0
    g["quad_weight"][:] = qw
    if not fem:
        g["h"][:] = hdx * dx
    return Body(a, gp=g, quads=np.ascontiguousarray(el, np.uint32), order=2,
                shape=SHAPE_ELEMENT if fem else SHAPE_RKPM)


def _tl_element_scenario(bodies, dt, dx, fem, name, contact=0, hdx=1.0) -> Scenario:
    # the *_fem set-ups take correction_constants() (all zero), the RKPM ones
    # correction_constants(.., 0, true) (velocity smoothing) and neighbourhoods of hdx dx
    sc = Scenario(method=METHOD_TL_WEAK, bodies=bodies, actions=list(TENSILE_TL_WEAK_ACTIONS), dt=dt, nu=0.4, E=1e7,
                  rho0=1.0, do_smooth=0 if fem else 1, contact=contact, name=name)
    sc.nbh_h = 0.0 if fem else hdx * dx
    return sc


def tensile_tl_fem(nbox: int) -> Scenario:
    """The reference's tensile_tl_fem(nbox), tensile.cpp:539-624: the plate lattice as
    bilinear elements (element_map_rectangle), 2x2 Gauss points, the pull conditions."""
    dx = 1.0 / (nbox - 1)
    I, J = np.meshgrid(np.arange(nbox, dtype=np.float64), np.arange(nbox, dtype=np.float64), indexing="ij")
    x, y = (I * dx).ravel(), (J * dx).ravel()
    b = _tl_element_body(x, y, x, y, element_map_rectangle(nbox - 1, nbox - 1), dx=dx, rho0=1.0, fem=True)
    left = np.arange(nbox, dtype=np.uint32)
    right = (np.uint32(nbox - 1) * np.uint32(nbox) + left).astype(np.uint32)
    b.bcs = [BC(BC_PULL_TL, -10.0, left), BC(BC_PULL_TL, 10.0, right)]
    return _tl_element_scenario([b], 1e-6, dx, True, f"tensile_tl_fem({nbox})")


def _rotation_tl_element(nbox: int, fem: bool, name: str) -> Scenario:
    ro = 1.0
    dx = 2 * ro / (nbox - 1)
    x, y, el = mesh_ring(nbox, 0.0, ro)
    b = _tl_element_body(x, y, x, y, el, dx=dx, rho0=1.0, fem=fem, vx=-y / ro * 50, vy=+x / ro * 50)
    return _tl_element_scenario([b], 1e-6, dx, fem, name)


def rotation_tl_fem(nbox: int) -> Scenario:
    """The reference's rotation_tl_fem(nbox), rotation.cpp:408-459: mesh_ring(nbox, 0, 1)
    as bilinear elements with 2x2 Gauss points, spinning at 50 m/s rim speed."""
    return _rotation_tl_element(nbox, True, f"rotation_tl_fem({nbox})")


def rotation_tl_weak(nbox: int) -> Scenario:
    """The reference's rotation_tl_weak(nbox), rotation.cpp:537-605: the same disc mesh
    with RKPM on neighbourhoods of dx and velocity smoothing."""
    return _rotation_tl_element(nbox, False, f"rotation_tl_weak({nbox})")


def _rings_tl_element(nbox: int, fem: bool, name: str) -> Scenario:
    ri, ro = 0.03, 0.04
    spacing = ro + 0.001
    dx = 2 * ro / (nbox - 1)
    x, y, el = mesh_ring(nbox, ri, ro)
    bodies = []
    for sgn, v in ((-1.0, 180.0), (1.0, -180.0)):
        xs = x - spacing if sgn < 0 else x + spacing
        b = _tl_element_body(xs, y, x, y, el, dx=dx, rho0=1.0, fem=fem, vx=v, gshift=0.0 if fem else sgn * spacing)
        b.hull = convex_hull(xs, y)
        bodies.append(b)
    return _tl_element_scenario(bodies, 1e-7, dx, fem, name, contact=1)


def rings_tl_fem_contact(nbox: int) -> Scenario:
    """The reference's rings_tl_fem_contact(nbox), rings.cpp:720-815: two meshed rings
    (r 0.03-0.04 m) at +-(ro + 1 mm), 180 m/s each, bilinear elements with 2x2 Gauss
    points, penalty contact on their hulls.  The particles' x is shifted, X and the
    Gauss points are not (the set-up moves only the particles)."""
    return _rings_tl_element(nbox, True, f"rings_tl_fem_contact({nbox})")


def rings_tl_weak_contact(nbox: int) -> Scenario:
    """The reference's rings_tl_weak_contact(nbox), rings.cpp:936-1051: the same rings
    with RKPM on neighbourhoods of dx; particles and Gauss points both move with their
    ring, their reference positions do not."""
    return _rings_tl_element(nbox, False, f"rings_tl_weak_contact({nbox})")


def _ul_element_body(x, y, X, Y, el, *, dx, rho0, vx=0.0, vy=0.0) -> Body:
    """A weak UL body on an explicit element map (the *_ul_fem set-ups): nodes with
    unit quad weights and no density or h, 2x2 stress points of density rho0.  The
    stress points are recorded as the first update_gauss_points of the step loop leaves
    them: placed on the nodes' current positions (it places them again at every
    derivative evaluation, so their set-up positions are no input)."""
    a = _body_from_lists(x, y, X, Y)
    a["m"][:] = dx * dx * rho0
    a["quad_weight"][:] = 1.0
    a["vx"][:] = vx
    a["vy"][:] = vy
    gx, gy, qw = gauss_points(a["x"], a["y"], el, 2)
    g = _body_from_lists(gx, gy, gx, gy)
    g["rho"][:] = rho0
    g["quad_weight"][:] = qw
    return Body(a, ex=1, gp=g, quads=np.ascontiguousarray(el, np.uint32), order=2, shape=SHAPE_ELEMENT)


def _ul_element_scenario(bodies, dt, name, contact=0) -> Scenario:
    # correction_constants() (all zero); no neighbour search
    return Scenario(method=METHOD_UL_WEAK, bodies=bodies, actions=list(UL_FEM_ACTIONS), dt=dt, nu=0.4, E=1e7, rho0=1.0,
                    contact=contact, name=name)


def tensile_ul_fem(nbox: int) -> Scenario:
    """The reference's tensile_ul_fem(nbox), tensile.cpp:452-537: the plate lattice as
    bilinear elements, the velocity conditions on the end columns, its hull set."""
    dx = 1.0 / (nbox - 1)
    I, J = np.meshgrid(np.arange(nbox, dtype=np.float64), np.arange(nbox, dtype=np.float64), indexing="ij")
    x, y = (I * dx).ravel(), (J * dx).ravel()
    b = _ul_element_body(x, y, x, y, element_map_rectangle(nbox - 1, nbox - 1), dx=dx, rho0=1.0)
    left = np.arange(nbox, dtype=np.uint32)
    right = (np.uint32(nbox - 1) * np.uint32(nbox) + left).astype(np.uint32)
    b.bcs = [BC(BC_VELOCITY_UL, -10.0, left), BC(BC_VELOCITY_UL, 10.0, right)]
    b.hull = convex_hull(x, y)
    return _ul_element_scenario([b], 1e-6, f"tensile_ul_fem({nbox})")


def rotation_ul_fem(nbox: int) -> Scenario:
    """The reference's rotation_ul_fem(nbox), rotation.cpp:353-405: mesh_ring(nbox, 0, 1)
    as bilinear elements, spinning at 50 m/s rim speed, dt 1e-5."""
    ro = 1.0
    dx = 2 * ro / (nbox - 1)
    x, y, el = mesh_ring(nbox, 0.0, ro)
    b = _ul_element_body(x, y, x, y, el, dx=dx, rho0=1.0, vx=-y / ro * 50, vy=+x / ro * 50)
    return _ul_element_scenario([b], 1e-5, f"rotation_ul_fem({nbox})")


def rings_ul_fem_contact(nbox: int) -> Scenario:
    """The reference's rings_ul_fem_contact(nbox), rings.cpp:623-718: two meshed rings
    (r 0.03-0.04 m) at +-(ro + 1 mm), 180 m/s each, bilinear elements, penalty contact
    on their hulls; X keeps the unshifted positions."""
    ri, ro = 0.03, 0.04
    spacing = ro + 0.001
    dx = 2 * ro / (nbox - 1)
    x, y, el = mesh_ring(nbox, ri, ro)
    bodies = []
    for sgn, v in ((-1.0, 180.0), (1.0, -180.0)):
        xs = x - spacing if sgn < 0 else x + spacing
        b = _ul_element_body(xs, y, x, y, el, dx=dx, rho0=1.0, vx=v)
        b.hull = convex_hull(xs, y)
        bodies.append(b)
    return _ul_element_scenario(bodies, 1e-7, f"rings_ul_fem_contact({nbox})", contact=1)


# ------------------------------------------------- workloads of the other families
def family_rings(family: str, dx: float = 5e-5) -> Scenario:
    """The ring-impact workload (two bodies with penalty contact, the constants of
    :func:`c1_rings`) run by another SPH family: "corot" (corotational, viscosity
    1/1/0.1 as rings_corot_contact), "potential" (elastic potential, the same
    viscosity) or "godunov" (Godunov UL, no correction terms)."""
    if family == "corot":
        return c1_rings(dx=dx, two_bodies=True, method=METHOD_COROT, alpha=1.0, beta=1.0, eta=0.1)
    if family == "potential":
        return c1_rings(dx=dx, two_bodies=True, method=METHOD_POTENTIAL, alpha=1.0, beta=1.0, eta=0.1)
    if family == "godunov":
        return c1_rings(dx=dx, two_bodies=True, method=METHOD_UL, godunov=True)
    raise ValueError(family)


def plate_ul_weak(dx: float = 5e-5, Lx: float = 0.1, Ly: float = 0.02, seed: int = 20261203,
                  jitter: float = 0.01) -> Scenario:
    """Uniaxial tension of the steel plate of :func:`c3_plate` with the weak UL form
    (tensile_ul_weak structure): particles on the jittered lattice, one stress point per
    cell centre, velocity conditions +-1 m/s on the end columns, h = dx, candidates by
    the 1.5 dx Manhattan search, dt = 0.3 dx / c0, smoothing on."""
    nx = int(round(Lx / dx)) + 1
    ny = int(round(Ly / dx)) + 1
    I, J = np.meshgrid(np.arange(nx, dtype=np.float64), np.arange(ny, dtype=np.float64), indexing="ij")
    x, y = (I * dx).ravel(), (J * dx).ravel()
    if jitter > 0.0:
        rng = np.random.default_rng(seed)
        x = x + rng.uniform(-jitter, jitter, x.shape) * dx
        y = y + rng.uniform(-jitter, jitter, y.shape) * dx
    I, J = np.meshgrid(np.arange(nx - 1, dtype=np.float64), np.arange(ny - 1, dtype=np.float64), indexing="ij")
    gx, gy = (I * dx + dx / 2).ravel(), (J * dx + dx / 2).ravel()
    rho0, E, nu = 7850.0, 2e11, 0.3
    b = _ul_weak_body(x, y, None, None, gx, gy, None, None, dx, 1.0, rho0)
    left = np.arange(ny, dtype=np.uint32)
    right = (np.uint32(nx - 1) * np.uint32(ny) + left).astype(np.uint32)
    b.bcs = [BC(BC_VELOCITY_UL, -1.0, left), BC(BC_VELOCITY_UL, 1.0, right)]
    sc = _ul_weak_scenario([b], TENSILE_UL_WEAK_ACTIONS, 0.0, dx, f"plate dx={dx} (weak UL)", nu=nu, E=E, rho0=rho0)
    sc.dt = 0.3 * dx / sc.c0
    return sc


FAMILY_RING_SETUPS = {"corot": "rings_corot_contact", "godunov": "rings_godunov_contact",
                      "potential": "rings_potential_contact", "ulweak": "rings_ul_weak_contact",
                      "tlweak": "rings_tl_weak_contact", "tlfem": "rings_tl_fem_contact",
                      "ulfem": "rings_ul_fem_contact"}


def family_ensemble(family: str, instances: int = 256, nbox: int = 81, seed: int = 20261203,
                    E_range=(0.8e7, 1.2e7)) -> Scenario:
    """An ensemble of independent two-ring impacts of one SPH family, each the
    reference's own set-up (rings_corot_contact, rings_godunov_contact,
    rings_potential_contact, rings_ul_weak_contact, rings_tl_weak_contact,
    rings_tl_fem_contact or rings_ul_fem_contact at nbox) with its own seeded
    Young's modulus E ~ U[E_range]; the two rings of an instance form one contact group.
    (The reference's potential and Godunov rings do not stay finite at much finer
    lattices, so the ensemble, not one large lattice, gives the size.)"""
    make = globals()[FAMILY_RING_SETUPS[family]]
    base = make(nbox)
    bodies, groups = [], []
    for k in range(instances):
        E = float(np.random.default_rng(seed + k).uniform(*E_range))
        for b in base.bodies:
            nb = Body({f: a.copy() for f, a in b.arrays.items()}, hull=b.hull.copy(), bcs=list(b.bcs), ex=b.ex,
                      ey=b.ey, params={"E": E})
            if b.gp is not None:
                nb.gp = {f: a.copy() for f, a in b.gp.items()}
            nb.quads, nb.order, nb.shape = b.quads, b.order, b.shape
            bodies.append(nb)
            groups.append(k)
    sc = Scenario(method=base.method, bodies=bodies, actions=list(base.actions), dt=base.dt, nu=base.nu, E=base.E,
                  rho0=base.rho0, wdeltap=base.wdeltap, corr_exp=base.corr_exp, mghn_eps=base.mghn_eps,
                  alpha=base.alpha, beta=base.beta, eta=base.eta, xsph_eps=base.xsph_eps, do_smooth=base.do_smooth,
                  nbh_h=base.nbh_h, nbh_eps=base.nbh_eps, contact=base.contact, groups=groups,
                  name=f"ensemble of {instances} x {base.name}")
    return sc


# ---------------------------------------------------------------- case files
def write_case(path: str, sc: Scenario, nsteps: int, dump_every: int = 0) -> None:
    """Write the binary case file read by the oracle (oracle/mfcase.h)."""
    out = bytearray(b"MFCASE1\0")
    u32 = lambda v: out.extend(struct.pack("<I", int(v)))
    f64 = lambda v: out.extend(struct.pack("<d", float(v)))
    u32(sc.method); u32(len(sc.bodies)); u32(nsteps); u32(dump_every); u32(sc.contact)
    u32(len(sc.actions))
    for a in sc.actions:
        u32(a)
    f64(sc.dt)
    for v in (sc.nu, sc.E, sc.rho0, sc.wdeltap, sc.corr_exp, sc.mghn_eps, sc.alpha, sc.beta, sc.eta, sc.xsph_eps):
        f64(v)
    u32(sc.do_smooth)
    for v in (sc.nbh_h, sc.nbh_eps, sc.gp_h, sc.gp_rho):
        f64(v)
    for b in sc.bodies:
        u32(b.n)
        for k in IN_NAMES:
            out.extend(np.ascontiguousarray(b.arrays[k], np.float64).tobytes())
        u32(len(b.hull))
        out.extend(np.ascontiguousarray(b.hull, np.uint32).tobytes())
        u32(len(b.bcs))
        for bc in b.bcs:
            u32(bc.kind); f64(bc.v); u32(len(bc.idx))
            out.extend(np.ascontiguousarray(bc.idx, np.uint32).tobytes())
        u32(b.ex); u32(b.ey)
        # an element map follows for TL_WEAK bodies without a rectangle and for UL_WEAK
        # bodies with ex = 1 (a gauss_int in place of the ellipse)
        explicit = (sc.method == METHOD_TL_WEAK and b.ex == 0) or (sc.method == METHOD_UL_WEAK and b.ex == 1)
        if explicit:
            q = np.ascontiguousarray(b.quads, np.uint32).reshape(-1, 4)
            u32(len(q)); u32(b.order); u32(b.shape)
            out.extend(q.tobytes())
        if sc.method == METHOD_UL_WEAK or explicit:
            ng = len(b.gp["x"])
            u32(ng)
            for k in IN_NAMES:
                out.extend(np.ascontiguousarray(b.gp[k], np.float64).tobytes())
    with open(path, "wb") as f:
        f.write(bytes(out))


def read_case(path: str) -> Scenario:
    """Read a case file back (inverse of :func:`write_case`)."""
    buf = open(path, "rb").read()
    assert buf[:7] == b"MFCASE1"
    off = 8

    def u32():
        nonlocal off
        v = struct.unpack_from("<I", buf, off)[0]
        off += 4
        return v

    def f64():
        nonlocal off
        v = struct.unpack_from("<d", buf, off)[0]
        off += 8
        return v

    def arr(dt, n):
        nonlocal off
        a = np.frombuffer(buf, dt, n, off).copy()
        off += n * np.dtype(dt).itemsize
        return a

    method, nb, nsteps, dump_every, contact = u32(), u32(), u32(), u32(), u32()
    actions = list(arr(np.uint32, u32()))
    dt = f64()
    vals = [f64() for _ in range(10)]
    do_smooth = u32()
    nbh_h, nbh_eps, gp_h, gp_rho = f64(), f64(), f64(), f64()
    bodies = []
    for _ in range(nb):
        n = u32()
        a = {k: arr(np.float64, n) for k in IN_NAMES}
        hull = arr(np.uint32, u32())
        bcs = []
        for _ in range(u32()):
            kind = u32(); v = f64(); idx = arr(np.uint32, u32())
            bcs.append(BC(kind, v, idx))
        ex, ey = u32(), u32()
        body = Body(a, hull, bcs, ex, ey)
        explicit = (method == METHOD_TL_WEAK and ex == 0) or (method == METHOD_UL_WEAK and ex == 1)
        if explicit:
            ne = u32()
            body.order, body.shape = u32(), u32()
            body.quads = arr(np.uint32, 4 * ne).reshape(-1, 4)
        if method == METHOD_UL_WEAK or explicit:
            ng = u32()
            body.gp = {k: arr(np.float64, ng) for k in IN_NAMES}
        bodies.append(body)
    sc = Scenario(method=method, bodies=bodies, actions=[int(a) for a in actions], dt=dt, nu=vals[0], E=vals[1],
                  rho0=vals[2], wdeltap=vals[3], corr_exp=vals[4], mghn_eps=vals[5], alpha=vals[6], beta=vals[7],
                  eta=vals[8], xsph_eps=vals[9], do_smooth=do_smooth, nbh_h=nbh_h, nbh_eps=nbh_eps, gp_h=gp_h,
                  gp_rho=gp_rho, contact=contact)
    return sc


@dataclass
class Result:
    dumps: List[dict]          # [{"step", "time", "bodies": [ {name: array} ]}]
    neighbors: List[List[np.ndarray]]
    seconds: float
    ok: bool


def read_result(path: str) -> Result:
    """Parse a result file written by the oracle or the reference harness."""
    buf = open(path, "rb").read()
    assert buf[:6] == b"MFOUT1", "bad result file"
    off = 8
    nb = struct.unpack_from("<I", buf, off)[0]
    off += 4
    ns = list(struct.unpack_from(f"<{nb}I", buf, off))
    off += 4 * nb
    dumps, nbh, secs, ok = [], [], 0.0, False
    while off < len(buf):
        tag = struct.unpack_from("<I", buf, off)[0]
        off += 4
        if tag == 0:
            ok = True
            break
        if tag == 1:
            step = struct.unpack_from("<I", buf, off)[0]
            t = struct.unpack_from("<d", buf, off + 4)[0]
            off += 12
            bodies = []
            for n in ns:
                d = {}
                for k in OUT_NAMES:
                    d[k] = np.frombuffer(buf, np.float64, n, off).copy()
                    off += 8 * n
                bodies.append(d)
            dumps.append({"step": step, "time": t, "bodies": bodies})
        elif tag == 2:
            for _ in range(nb):
                n = struct.unpack_from("<I", buf, off)[0]
                off += 4
                counts = np.frombuffer(buf, np.uint32, n, off).copy()
                off += 4 * n
                tot = int(counts.sum())
                flat = np.frombuffer(buf, np.uint32, tot, off).copy()
                off += 4 * tot
                starts = np.concatenate([[0], np.cumsum(counts, dtype=np.int64)]).astype(np.int64)
                nbh.append([flat[int(starts[i]):int(starts[i + 1])] for i in range(n)])
        elif tag == 3:
            secs = struct.unpack_from("<d", buf, off)[0]
            off += 8
        elif tag == 9:
            break
        else:
            raise ValueError(f"bad record tag {tag}")
    return Result(dumps, nbh, secs, ok)
