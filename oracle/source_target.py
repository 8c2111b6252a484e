"""Oracle (test infrastructure only): numpy restatement of the reference's
translational products from forces on source blobs to velocities of target
blobs with per-blob radii, and of the single-radius free-surface product.

* pair block with radii a (target) and b (source), separation r = x_t - x_s
  (Rotne-Prager-Yamakawa for unequal spheres):
    r > a + b            C1 = (1 + (a^2+b^2)/(3 r^2)) / r,  C2 = (1 - (a^2+b^2)/r^2) / r^3
    |b - a| < r <= a + b C1 = (4/3)/(ab) [(a+b)/2 - ((b-a)^2 + 3 r^2)^2/(32 r^3)],
                         C2 = ((b-a)^2 - r^2)^2 / (8 r^5 ab)
    otherwise            C1 = (4/3)/max(a, b), C2 = 0
  M = C1 I + C2 r r^T, velocities (1/(8 pi eta)) sum_s M f_s
  (mobility/mobility_numba.py:1480-1572, 1941-2030);
* wall (mobility_numba.py:1573-1653 with the wrapper mobility/mobility.py:551-590):
  heights shifted to max(z, radius) on both sides, forces and velocities
  damped by z/radius below the radius, and the image system subtracted,
  M -= W diag(1, 1, -1) with, for the image vector r = (dx, dy, z_t + z_s),
  h = z_t, s = z_s, S = a^2 + b^2, ca = 2a^2/3, cb = 2b^2/3, cab = ca b^2,
  W = al I + be e e^T + ga r e^T + de e r^T + ep r r^T:
    al = (1 + S/(3r^2))/r + 2hs/r^3 - 3R(ca s + cb h)/r^5 + cab(5R^2/r^7 - 1/r^5)
    be = -2/r - (ca + cb)/r^3 - 2 cab/r^5
    ga = -2h/r^3 + 3(ca R - ca s - cb h)/r^5 + 10 cab R/r^7
    de = -2s/r^3 + 3(cb R - ca s - cb h)/r^5 + 10 cab R/r^7
    ep = (1 - S/r^2)/r^3 - 6hs/r^5 + 15R(ca s + cb h)/r^7 + cab(5/r^7 - 35R^2/r^9)
  (a regrouping of the reference's term-by-term image expressions; R = z_t + z_s);
* free surface (mobility_numba.py:1941-2093): M += M_pair(dx, dy, z_t + z_s) diag(1, 1, -1);
* single-radius free surface (mobility_numba.py:1770-1938, mobility.py:1390-1406):
  the same with a = b and the self block 4/3 / (8 pi eta a).
Pseudo-periodic images: minimum image plus the neighbouring boxes in each
periodic direction; the image separation always uses the unshifted z_t + z_s.
Pinned to tests/golden/source_target.npz.
"""
import numpy as np

SIGMA = np.array([1.0, 1.0, -1.0])


def _images(d, L):
    """Minimum image of d (..., 3) (truncation toward zero, as the reference)
    and the list of box shifts to add."""
    d = d.copy()
    shifts = [np.zeros(3)]
    for c in range(3):
        if L[c] > 0:
            q = d[..., c] / L[c] + 0.5 * np.sign(d[..., c])
            d[..., c] -= np.trunc(q) * L[c]
            shifts = [s + k * L[c] * np.eye(3)[c] for s in shifts for k in (-1, 0, 1)]
    return d, shifts


def pair_coefficients(r2, a, b):
    """(C1, C2) of the unequal-sphere pair block for squared separations r2."""
    r = np.sqrt(r2)
    S = a * a + b * b
    far = r > a + b
    mid = (~far) & (r > np.abs(b - a))
    with np.errstate(divide="ignore", invalid="ignore"):
        C1 = np.where(far, (1 + S / (3 * r2)) / r, 0.0)
        C2 = np.where(far, (1 - S / r2) / (r2 * r), 0.0)
        r3 = r2 * r
        C1m = (4.0 / 3.0) / (a * b) * ((a + b) / 2 - ((b - a) ** 2 + 3 * r2) ** 2 / (32 * r3))
        C2m = ((b - a) ** 2 - r2) ** 2 / (8 * r3 * r2 * a * b)
    C1 = np.where(mid, C1m, C1)
    C2 = np.where(mid, C2m, C2)
    inner = (~far) & (~mid)
    C1 = np.where(inner, (4.0 / 3.0) / np.maximum(a, b), C1)
    return C1, C2


def _pair_apply(dv, a, b, f):
    """sum_s (C1 f + C2 d (d.f)) for separations dv (nt, ns, 3)."""
    C1, C2 = pair_coefficients((dv * dv).sum(-1), a, b)
    return C1[..., None] * f + C2[..., None] * dv * (dv * f).sum(-1)[..., None]


def _wall_apply(rv, h, s, a, b, g):
    """W g for image vectors rv (nt, ns, 3), target heights h, source heights s."""
    r2 = (rv * rv).sum(-1)
    r = np.sqrt(r2)
    R = rv[..., 2]
    S = a * a + b * b
    ca, cb = 2 * a * a / 3, 2 * b * b / 3
    cab = ca * b * b
    r3, r5 = r2 * r, r2 * r2 * r
    r7, r9 = r5 * r2, r5 * r2 * r2
    q = ca * s + cb * h
    al = (1 + S / (3 * r2)) / r + 2 * h * s / r3 - 3 * R * q / r5 + cab * (5 * R * R / r7 - 1 / r5)
    be = -2 / r - (ca + cb) / r3 - 2 * cab / r5
    ga = -2 * h / r3 + 3 * (ca * R - q) / r5 + 10 * cab * R / r7
    de = -2 * s / r3 + 3 * (cb * R - q) / r5 + 10 * cab * R / r7
    ep = (1 - S / r2) / r3 - 6 * h * s / r5 + 15 * R * q / r7 + cab * (5 / r7 - 35 * R * R / r9)
    gz = g[..., 2]
    rg = (rv * g).sum(-1)
    e = np.array([0.0, 0.0, 1.0])
    return (al[..., None] * g + (be * gz + de * rg)[..., None] * e + (ga * gz + ep * rg)[..., None] * rv)


def source_target(geometry, source, target, force, radius_source, radius_target, eta, periodic_length=None):
    """Velocities (nt*3,) of targets from forces on sources; geometry 'wall',
    'no_wall' or 'free_surface'."""
    src = np.asarray(source, dtype=np.float64).reshape(-1, 3).copy()
    trg = np.asarray(target, dtype=np.float64).reshape(-1, 3).copy()
    f = np.asarray(force, dtype=np.float64).reshape(-1, 3).copy()
    rs = np.asarray(radius_source, dtype=np.float64).reshape(-1)
    rt = np.asarray(radius_target, dtype=np.float64).reshape(-1)
    L = np.zeros(3) if periodic_length is None else np.asarray(periodic_length, dtype=np.float64)
    damp_t = np.ones(trg.shape[0])
    if geometry == "wall":
        damp_s = np.where(src[:, 2] < rs, src[:, 2] / rs, 1.0)
        damp_t = np.where(trg[:, 2] < rt, trg[:, 2] / rt, 1.0)
        f = f * damp_s[:, None]
        src[:, 2] = np.where(src[:, 2] > rs, src[:, 2], rs)
        trg[:, 2] = np.where(trg[:, 2] > rt, trg[:, 2], rt)
    d0, shifts = _images(trg[:, None, :] - src[None, :, :], L)
    a = rt[:, None]
    b = rs[None, :]
    fb = np.broadcast_to(f[None, :, :], d0.shape)
    h = np.broadcast_to(trg[:, None, 2], d0.shape[:2])
    s = np.broadcast_to(src[None, :, 2], d0.shape[:2])
    u = np.zeros((trg.shape[0], 3))
    for sh in shifts:
        d = d0 + sh
        m = _pair_apply(d, a, b, fb)
        if geometry != "no_wall":
            img = d.copy()
            img[..., 2] = h + s
            if geometry == "wall":
                m = m - _wall_apply(img, h, s, a, b, fb * SIGMA)
            else:
                m = m + _pair_apply(img, a, b, fb * SIGMA)
        u += m.sum(axis=1)
    u = u / (8 * np.pi * eta)
    return (u * damp_t[:, None]).reshape(-1)


def free_surface(r_vectors, force, eta, a, periodic_length=None):
    """Single-radius free-surface product (n*3,): pair blocks in units of a,
    RPY for r > 2a and the overlap form below, the 4/3 self block, plus the
    image block at (dx, dy, z_i + z_j) times diag(1, 1, -1)."""
    r = np.asarray(r_vectors, dtype=np.float64).reshape(-1, 3) / a
    f = np.asarray(force, dtype=np.float64).reshape(-1, 3)
    L = (np.zeros(3) if periodic_length is None else np.asarray(periodic_length, dtype=np.float64)) / a
    n = r.shape[0]
    d0, shifts = _images(r[:, None, :] - r[None, :, :], L)
    zsum = r[:, None, 2] + r[None, :, 2]
    fb = np.broadcast_to(f[None, :, :], d0.shape)
    u = np.zeros((n, 3))

    def rpy(dv, g, exclude_self):
        r2 = (dv * dv).sum(-1)
        rr = np.sqrt(r2)
        with np.errstate(divide="ignore", invalid="ignore"):
            far = rr > 2
            c1 = np.where(far, (1 + 2 / (3 * r2)) / rr, (4.0 / 3.0) * (1 - 0.28125 * rr))
            c2 = np.where(far, (1 - 2 / r2) / (r2 * rr), (4.0 / 3.0) * 0.09375 / rr)
            m = c1[..., None] * g + c2[..., None] * dv * (dv * g).sum(-1)[..., None]
        if exclude_self:
            idx = np.arange(n)
            m[idx, idx] = (4.0 / 3.0) * g[idx, idx]
        return m

    for sh in shifts:
        d = d0 + sh
        central = not sh.any()
        m = rpy(d, fb, central)
        img = d.copy()
        img[..., 2] = zsum
        m = m + rpy(img, fb * SIGMA, False)
        u += m.sum(axis=1)
    return (u / (8 * np.pi * eta * a)).reshape(-1)
