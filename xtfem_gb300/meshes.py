"""Generated C3D8 meshes of the reference's workloads whose mesh files are
not shipped with it: the single-edge-notched tension (SENT) plate.

The shipped rods come from the host generator (``Problem.rod``); these are
built here and handed over with ``Problem.from_mesh``.  Connectivity uses the
node order of the reference's C3D8 shape functions (src/procs.f90:1366-1389:
local node n sits at the natural coordinates of its sign row, xi along x,
eta along y, zeta along z), so every Jacobian is positive.
"""
from __future__ import annotations

import numpy as np

# natural coordinates of the 8 local nodes (src/procs.f90:1366-1373)
_SIGN = np.array([[-1, -1, 1], [-1, -1, -1], [-1, 1, -1], [-1, 1, 1],
                  [1, -1, 1], [1, -1, -1], [1, 1, -1], [1, 1, 1]])


def _graded(a, b, n, ratio, toward_b):
    """n + 1 coordinates on [a, b], spacings in geometric progression of the
    given ratio (>= 1), finest at b when toward_b, else at a."""
    w = ratio ** np.arange(n, dtype=float)
    w = w[::-1] if toward_b else w
    x = a + (b - a) * np.concatenate([[0.0], np.cumsum(w) / w.sum()])
    x[-1] = b
    return x


def sent_plate(nx=48, ny=96, nz=2, W=1.0, H=2.0, t=0.1, notch=0.3, ratio=1.05):
    """Single-edge-notched tension plate W x H x t with an edge notch of
    length notch*W at mid-height, made by removing one row of elements (the
    row just below y = H/2, from x = 0 to the notch tip).  The grid is graded
    toward the notch tip in x and toward the mid-height in y (spacing ratio
    `ratio` between neighbours), nz elements through the thickness.  Returns
    (xyz (nn x 3), conn (ne x 8, 1-based)) with no unattached node."""
    a = notch * W
    nxl = max(1, int(round(nx * notch)))
    xs = np.concatenate([_graded(0.0, a, nxl, ratio, True),
                         _graded(a, W, nx - nxl, ratio, False)[1:]])
    nyh = ny // 2
    ys = np.concatenate([_graded(0.0, H / 2, nyh, ratio, True),
                         _graded(H / 2, H, ny - nyh, ratio, False)[1:]])
    zs = np.linspace(0.0, t, nz + 1)
    # nodes numbered with the long side (y) outermost, then x, then z: the
    # matrix bandwidth is one x-z layer, as for the shipped rods, which the
    # level-of-fill-limited ILUT needs
    nxn, nzn = len(xs), len(zs)
    Y, X, Z = np.meshgrid(ys, xs, zs, indexing="ij")
    xyz = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)

    def node(i, j, k):
        return (j * nxn + i) * nzn + k + 1

    conn = []
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                if j == nyh - 1 and xs[i + 1] <= a + 1e-12:
                    continue  # the notch: one row of elements removed
                conn.append([node(i + (sx > 0), j + (sy > 0), k + (sz > 0)) for sx, sy, sz in _SIGN])
    return xyz, np.array(conn, np.int32)


def holed_panel(ntheta=64, nr=12, nz=1, W=1.0, t=0.05, radius=0.1, ratio=1.1, order="rings"):
    """Square panel W x W x t with a central circular hole of radius
    radius*W, one O-grid: ntheta elements around the hole (a multiple of 4,
    the square's corners at 45, 135, 225 and 315 degrees), nr elements from
    the hole to the outer edge (graded toward the hole, spacing ratio
    `ratio`), nz through the thickness.  Node (ring j, angle i) sits on the
    segment from the hole point at angle theta_i to the point where that ray
    meets the square.  Returns (xyz (nn x 3), conn (ne x 8, 1-based)).

    order="rings" numbers the rings outermost (bandwidth one ring);
    order="rays" numbers the rays outermost (bandwidth one ray), which
    leaves the ILUT(1e-4, 20) factor's triangular solves far more parallel
    and converges faster.  On a 96 x 24 panel: 1,139 dependent node-group
    levels against 4,704, and 939 GMRES(200) iterations to 1e-9 against
    1,370.  The geometry and elements are the same either way."""
    if ntheta % 4:
        raise ValueError("ntheta must be a multiple of 4")
    if order not in ("rings", "rays"):
        raise ValueError("order is 'rings' or 'rays'")
    c = 0.5 * W
    th = 2 * np.pi * np.arange(ntheta) / ntheta + np.pi / 4
    cs, sn = np.cos(th), np.sin(th)
    inner = np.stack([c + radius * W * cs, c + radius * W * sn], 1)
    scale = 0.5 * W / np.maximum(np.abs(cs), np.abs(sn))
    outer = np.stack([c + scale * cs, c + scale * sn], 1)
    # the square's edges exactly (the ray meets x or y = 0 or W)
    outer = np.where(np.abs(outer - 0.0) < 1e-12, 0.0, outer)
    outer = np.where(np.abs(outer - W) < 1e-12, W, outer)
    s = _graded(0.0, 1.0, nr, ratio, False)  # finest at the hole
    zs = np.linspace(0.0, t, nz + 1)
    nzn = nz + 1
    xyz = np.zeros(((nr + 1) * ntheta * nzn, 3))
    for j in range(nr + 1):
        P = inner + s[j] * (outer - inner)
        for i in range(ntheta):
            for k in range(nzn):
                xyz[(j * ntheta + i) * nzn + k] = (P[i, 0], P[i, 1], zs[k])

    def node(j, i, k):
        return (j * ntheta + (i % ntheta)) * nzn + k + 1

    # local xi along the ray (outward), eta around the hole (counterclockwise),
    # zeta through the thickness: a right-handed element
    conn = np.array([[node(j + (sx > 0), i + (sy > 0), k + (sz > 0)) for sx, sy, sz in _SIGN]
                     for k in range(nz) for j in range(nr) for i in range(ntheta)], np.int32)
    if order == "rays":
        # new number of node (ring j, angle i, layer k): (i (nr+1) + j) nzn + k
        jj, ii, kk = np.meshgrid(np.arange(nr + 1), np.arange(ntheta), np.arange(nzn),
                                 indexing="ij")
        new = ((ii * (nr + 1) + jj) * nzn + kk).ravel()  # indexed by the ring-order number
        xyz_r = np.empty_like(xyz)
        xyz_r[new] = xyz
        return xyz_r, (new[conn - 1] + 1).astype(np.int32)
    return xyz, conn
