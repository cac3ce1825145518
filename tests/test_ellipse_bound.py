"""The error bound of the mixed weak UL form's FP32 neighbour ellipse.

`k_uw_nbh32` (mf_ulweak.cu) computes a row's ellipse (covariance, eigen-decomposition,
per-candidate test) in FP32 from float-float positions and hands the row to the FP64
ellipse whenever a decision falls within twice its derived error bound, so that the
selected neighbours are the FP64 form's (nbh_ellipse, neighbor_ellipse.h:29-127, in the
fast form: the unit eigenvector as (cos phi, sin phi), reciprocal semi-axes).  This
restates both paths in numpy -- the FP32 one in float32 arithmetic, step by step -- and
checks on random neighbourhoods that wherever the FP32 path is sure, its selection
equals FP64's: point clouds and rotated, stretched, jittered lattices, 12 to 49
candidates, spacings from 0.1 mm to 10 m, positions far from the origin, half of the
rows with one candidate moved to within 1e-9 .. 1e-4 of the FP64 ellipse.  (On such
cases a margin of 1 % of the kernel's still gave a wrong sure row now and then, none
at 10 %: the derived bound holds with room.)"""
import numpy as np

F = np.float32
U = F(2.0 ** -24)
K2 = F(F(1.6651) * F(1.6651))


def split(x):
    hi = x.astype(np.float32)
    return hi, (x - hi.astype(np.float64)).astype(np.float32)


def fp64_select(dx, dy):
    """The fast FP64 form's selection (rows x candidates); dx, dy = query - candidate."""
    n = dx.shape[1]
    A00 = (dx * dx).sum(1) / n
    A01 = (dx * dy).sum(1) / n
    A11 = (dy * dy).sum(1) / n
    axis = np.abs(A01) < 1e-9
    T = A00 + A11
    det = A00 * A11 - A01 * A01
    root = np.sqrt(np.maximum(T * T / 4 - det, 0.0))
    l1, l2 = T / 2 - root, T / 2 + root
    vx, vy = l1 - A11, A01
    inv = 1 / np.sqrt(vx * vx + vy * vy)
    cs = np.where(axis, 1.0, vx * inv)[:, None]
    sn = np.where(axis, 0.0, vy * inv)[:, None]
    D0 = np.where(axis, A00, l1)[:, None]
    D1 = np.where(axis, A11, l2)[:, None]
    ia, ib = 1 / (1.6651 * np.sqrt(D0)), 1 / (1.6651 * np.sqrt(D1))
    xc, yc = -dx, -dy
    left, right = (cs * xc + sn * yc) * ia, (sn * xc - cs * yc) * ib
    return left * left + right * right <= 1


def fp32_select(qx, qy, cx, cy, margin=1.0):
    """The FP32 path of k_uw_nbh32: per row (sure, selection); `margin` scales the
    kernel's margin (twice the bound) for the sensitivity check."""
    qxh, qxl = split(qx)
    qyh, qyl = split(qy)
    cxh, cxl = split(cx)
    cyh, cyl = split(cy)
    dx = (qxh[:, None] - cxh) + (qxl[:, None] - cxl)
    dy = (qyh[:, None] - cyh) + (qyl[:, None] - cyl)
    rows, n = dx.shape
    Hxx = np.zeros(rows, F)
    Hxy = np.zeros(rows, F)
    Hyy = np.zeros(rows, F)
    for k in range(n):  # sequential FP32 sums, as the kernel
        Hxx = Hxx + dx[:, k] * dx[:, k]
        Hxy = Hxy + dx[:, k] * dy[:, k]
        Hyy = Hyy + dy[:, k] * dy[:, k]
    nf = F(n)
    A00, A01, A11 = Hxx / nf, Hxy / nf, Hyy / nf
    T = A00 + A11
    e = (nf + F(8)) * U * T
    a01 = np.abs(A01.astype(np.float64))
    branch = (a01 + e < 1e-9) | (a01 - e >= 1e-9)
    axis = a01 < 1e-9
    # rows FP32 cannot place: A01 summed in FP64
    ddx = qx[:, None] - cx
    ddy = qy[:, None] - cy
    a01d = np.abs((ddx * ddy).sum(1) / n)
    undecided = ~branch
    branch = np.where(undecided, np.abs(a01d - 1e-9) > 1e-15 + 1e-14 * T.astype(np.float64), branch)
    axis = np.where(undecided, a01d < 1e-9, axis)
    sure = (T > 0) & branch
    d = F(0.5) * (A00 - A11)
    r = np.sqrt(d * d + A01 * A01)
    l1, l2 = F(0.5) * T - r, F(0.5) * T + r
    vx = np.where(d >= 0, A01, d - r)
    vy = np.where(d >= 0, -(d + r), A01)
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = F(1) / np.sqrt(vx * vx + vy * vy)
        cond = T / l1
        cs = np.where(axis, F(1), vx * inv)
        sn = np.where(axis, F(0), vy * inv)
        ia2 = np.where(axis, F(1) / (K2 * A00), F(1) / (K2 * l1))
        ib2 = np.where(axis, F(1) / (K2 * A11), F(1) / (K2 * l2))
    bound = np.where(axis, nf + F(19), (F(3) * nf + F(48)) * cond)
    sure &= np.where(axis, (A00 > 0) & (A11 > 0), (l1 > 0) & (cond < F(1e4)))
    m = F(2) * bound * U * F(margin)
    left = cs[:, None] * dx + sn[:, None] * dy
    right = sn[:, None] * dx - cs[:, None] * dy
    s = left * left * ia2[:, None] + right * right * ib2[:, None]
    lo, hi = (F(1) - m)[:, None], (F(1) + m)[:, None]
    sure &= ((s < lo) | (s > hi)).all(1)
    return sure, s <= 1


def neighbourhoods(rng, rows, n, spacing, kind):
    """Query points and n candidates per row around them (float64)."""
    far = rng.uniform(-100, 100, size=(rows, 2)) * spacing * rng.choice([1.0, 1e3], size=(rows, 1))
    if kind == "cloud":
        off = rng.uniform(-3, 3, size=(rows, n, 2))
    else:  # a lattice patch, stretched, rotated and jittered
        g = np.stack(np.meshgrid(np.arange(-3, 4), np.arange(-3, 4)), -1).reshape(-1, 2).astype(float)
        pick = np.stack([rng.permutation(len(g))[:n] for _ in range(rows)])
        off = g[pick] * rng.uniform(1.0, 2.5, size=(rows, 1, 2))
        th = rng.uniform(0, 2 * np.pi, size=(rows, 1))
        c, s_ = np.cos(th), np.sin(th)
        off = np.stack([c * off[..., 0] - s_ * off[..., 1], s_ * off[..., 0] + c * off[..., 1]], -1)
        off += rng.normal(scale=rng.choice([0.0, 1e-6, 1e-2]), size=off.shape)
    q = far + rng.uniform(-0.5, 0.5, size=(rows, 2)) * spacing
    cand = far[:, None, :] + off * spacing
    return q[:, 0], q[:, 1], cand[..., 0], cand[..., 1]


def quadratic_form(dx, dy):
    """FP64 ellipse metric per row: s(p) = left^2 + right^2 as a function of the
    offset p - query (the fast form's expressions, vectorised)."""
    n = dx.shape[1]
    A00 = (dx * dx).sum(1) / n
    A01 = (dx * dy).sum(1) / n
    A11 = (dy * dy).sum(1) / n
    axis = np.abs(A01) < 1e-9
    T = A00 + A11
    root = np.sqrt(np.maximum(T * T / 4 - (A00 * A11 - A01 * A01), 0.0))
    l1, l2 = T / 2 - root, T / 2 + root
    vx, vy = l1 - A11, A01
    inv = 1 / np.sqrt(vx * vx + vy * vy)
    cs, sn = np.where(axis, 1.0, vx * inv), np.where(axis, 0.0, vy * inv)
    a2 = 1.6651 ** 2 * np.where(axis, A00, l1)
    b2 = 1.6651 ** 2 * np.where(axis, A11, l2)
    return lambda ux, uy: (cs * ux + sn * uy) ** 2 / a2 + (sn * ux - cs * uy) ** 2 / b2


def on_boundary(rng, qx, qy, cx, cy):
    """Moves one candidate per row onto the FP64 ellipse, s = 1 + delta with |delta|
    log-uniform in [1e-9, 1e-4] (a few fixed-point passes: the move changes the
    covariance slightly)."""
    rows, n = cx.shape
    k = rng.integers(0, n, rows)
    r = np.arange(rows)
    ang = rng.uniform(0, 2 * np.pi, rows)
    ux, uy = np.cos(ang), np.sin(ang)
    delta = rng.choice([-1.0, 1.0], rows) * 10.0 ** rng.uniform(-9, -4, rows)
    cx, cy = cx.copy(), cy.copy()
    for _ in range(6):
        Q = quadratic_form(qx[:, None] - cx, qy[:, None] - cy)(ux, uy)
        t = np.sqrt((1 + delta) / Q)
        cx[r, k] = qx + t * ux
        cy[r, k] = qy + t * uy
    return cx, cy


def cases(seed):
    rng = np.random.default_rng(seed)
    for kind in ("cloud", "lattice"):
        for n in (12, 20, 33, 49):
            for spacing in (1e-4, 1e-3, 5e-2, 1.0, 10.0):
                qx, qy, cx, cy = neighbourhoods(rng, 120, n, spacing, kind)
                if rng.random() < 0.5:  # a candidate within 1e-9 .. 1e-4 of the ellipse
                    cx, cy = on_boundary(rng, qx, qy, cx, cy)
                yield (kind, n, spacing), qx, qy, cx, cy


def test_fp32_ellipse_sure_rows_select_as_fp64():
    tested = sure_rows = 0
    for case, qx, qy, cx, cy in cases(20261204):
        sure, sel32 = fp32_select(qx, qy, cx, cy)
        sel64 = fp64_select(qx[:, None] - cx, qy[:, None] - cy)
        bad = sure & (sel32 != sel64).any(1)
        assert not bad.any(), (case, np.flatnonzero(bad)[:5])
        tested += len(qx)
        sure_rows += int(sure.sum())
    # the FP32 path decides most rows itself, so the check is not vacuous
    assert sure_rows > 0.5 * tested, (sure_rows, tested)


def test_check_is_sensitive_to_the_margin():
    """Without the margin the same cases give wrong sure rows: the near-boundary
    candidates do probe the bound."""
    bad = 0
    for _, qx, qy, cx, cy in cases(20261204):
        sure, sel32 = fp32_select(qx, qy, cx, cy, margin=0.0)
        bad += int((sure & (sel32 != fp64_select(qx[:, None] - cx, qy[:, None] - cy)).any(1)).sum())
    assert bad > 0


def test_fp64_branch_sum_places_symmetric_coarse_rows():
    """At coarse spacing a symmetric neighbourhood (A01 ~ 0) has an FP32 A01 error
    above the reference's absolute 1e-9 threshold; the FP64 A01 sum places it."""
    g = np.stack(np.meshgrid(np.arange(-3, 4), np.arange(-3, 4)), -1).reshape(-1, 2).astype(float)
    spacing = 0.05  # the spinning disc's lattice (radius 1 m, nbox 41)
    cx = (0.3 + g[:, 0] * spacing)[None, :]
    cy = (-0.7 + g[:, 1] * spacing)[None, :]
    sure, sel32 = fp32_select(np.array([0.3]), np.array([-0.7]), cx, cy)
    assert sure[0]
    assert np.array_equal(sel32, fp64_select(0.3 - cx, -0.7 - cy))
