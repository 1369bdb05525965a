"""The reference's finite-element set-up of the mechanical slab, restated in
numpy: the structured rod mesh of inp/prismaticrod-*.inp, the C3D8 element
stiffness and consistent mass over the 2x2x2 Gauss rule, the per-Gauss-point
strain rows, triplet assembly into CSR, the 1-0 boundary conditions and the
face traction.

TEST INFRASTRUCTURE ONLY: it builds the inputs of the CPU baseline (the
reference arm of bench.py) without the GPU library, and the tests check it
against the library's host assembly.

Reference statements restated:
  src/procs.f90:537          Gauss abscissa 0.577350269189626 (1/sqrt(3))
  src/procs.f90:1366-1389    trilinear shape functions and their signs
  src/elesubs.f90:2-57       element stiffness B^T D B and consistent mass,
                             Gauss points xi outermost
  src/spmtx.f90:359-454      triplets to CSR (duplicates summed, sorted
                             columns, zeros removed)
  src/spmtx.f90:268-307      csrapplybc: fixed rows and columns cleared,
                             unit diagonal, zeros removed
  src/main3d.f90:482-530     clamped face, traction shared over the loaded
                             face's element-node incidences
The mesh files hold single-precision coordinates printed with nine
significant digits; the generator reproduces that rounding.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import scipy.sparse as sp

GAUSS = 0.577350269189626
SIGN = np.array([[-1, -1, 1], [-1, -1, -1], [-1, 1, -1], [-1, 1, 1],
                 [1, -1, 1], [1, -1, -1], [1, 1, -1], [1, 1, 1]], float)


@dataclass
class Csr:
    """1-based CSR, the layout of the reference's ki/kj/kv arrays."""
    ia: np.ndarray
    ja: np.ndarray
    a: np.ndarray

    @property
    def n(self):
        return len(self.ia) - 1


def rod_mesh(nx, ny, nz, lx=3.0, ly=1.0, lz=1.0):
    """Nodes (nn x 3) and 1-based connectivity (ne x 8) of the rod meshes
    inp/prismaticrod-*.inp: x descends outermost, then z, then y."""
    py, pz, px = ny + 1, nz + 1, nx + 1

    def coord(v):
        return np.array([float("%.9g" % float(np.float32(x))) for x in v])

    ix, iz, iy = np.meshgrid(np.arange(px), np.arange(pz), np.arange(py), indexing="ij")
    xs = coord(lx - lx * np.arange(px) / nx)
    ys = coord(ly - ly * np.arange(py) / ny)
    zs = coord(lz - lz * np.arange(pz) / nz)
    xyz = np.stack([xs[ix.ravel()], ys[iy.ravel()], zs[iz.ravel()]], 1)

    def node(a, b, c):
        return a * py * pz + c * py + b + 1

    ex, ez, ey = (g.ravel() for g in np.meshgrid(np.arange(nx), np.arange(nz), np.arange(ny),
                                                 indexing="ij"))
    conn = np.stack([node(ex + 1, ey, ez), node(ex + 1, ey + 1, ez),
                     node(ex + 1, ey + 1, ez + 1), node(ex + 1, ey, ez + 1),
                     node(ex, ey, ez), node(ex, ey + 1, ez), node(ex, ey + 1, ez + 1),
                     node(ex, ey, ez + 1)], 1).astype(np.int32)
    return xyz, conn


def _shape(l):
    """Shape values and natural derivatives at Gauss point l (xi outermost),
    each product evaluated left to right as written in the reference."""
    g = (-GAUSS, GAUSS)
    xi, eta, zeta = g[(l >> 2) & 1], g[(l >> 1) & 1], g[l & 1]
    N, dn = [], []
    for i in range(8):
        sx, sy, sz = SIGN[i]
        N.append(0.125 * (1.0 + sx * xi) * (1.0 + sy * eta) * (1.0 + sz * zeta))
        dn.append((0.125 * sx * (1.0 + sy * eta) * (1.0 + sz * zeta),
                   0.125 * sy * (1.0 + sx * xi) * (1.0 + sz * zeta),
                   0.125 * sz * (1.0 + sx * xi) * (1.0 + sy * eta)))
    return N, dn


def gauss_point(xe, l):
    """Global shape derivatives dNdx (ne, 8, 3), shape values N (8) and the
    Jacobian determinant (ne) at Gauss point l for elements with nodal
    coordinates xe (ne, 8, 3): jac(a, m) = sum_i dN_i/dxi_a x_i^m, its
    determinant by the rule of Sarrus and its inverse by cofactors, every
    sum taken in index order (vectorised over the elements only)."""
    N, dn = _shape(l)
    J = [[None] * 3 for _ in range(3)]
    for a in range(3):
        for m in range(3):
            s = np.zeros(len(xe))
            for i in range(8):
                s = s + dn[i][a] * xe[:, i, m]
            J[a][m] = s
    det = (J[0][0] * J[1][1] * J[2][2] + J[0][1] * J[1][2] * J[2][0] + J[0][2] * J[1][0] * J[2][1]
           - J[0][0] * J[1][2] * J[2][1] - J[0][1] * J[1][0] * J[2][2] - J[0][2] * J[1][1] * J[2][0])
    inv = [[(J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det,
            (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det,
            (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det],
           [(J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det,
            (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det,
            (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det],
           [(J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det,
            (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det,
            (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det]]
    dNdx = np.zeros((len(xe), 8, 3))
    for i in range(8):
        for m in range(3):
            s = np.zeros(len(xe))
            for a in range(3):
                s = s + inv[m][a] * dn[i][a]
            dNdx[:, i, m] = s
    return dNdx, N, det


def elastic_matrix(E, nu):
    """src/elesubs.f90:374-401, isotropic (symmetric 6 x 6)."""
    c = E / ((1.0 + nu) * (1.0 - 2.0 * nu))
    D = np.zeros((6, 6))
    for i in range(3):
        for j in range(3):
            D[i, j] = c * ((1.0 - nu) if i == j else nu)
    for i in range(3, 6):
        D[i, i] = c * (0.5 - nu)
    return D


def strain_matrix(dNdx):
    """B (ne, 6, 24), strain order (xx, yy, zz, xy, yz, zx) of the
    reference's kernel."""
    ne = dNdx.shape[0]
    B = np.zeros((ne, 6, 24))
    nx, ny, nz = dNdx[:, :, 0], dNdx[:, :, 1], dNdx[:, :, 2]
    B[:, 0, 0::3], B[:, 1, 1::3], B[:, 2, 2::3] = nx, ny, nz
    B[:, 3, 0::3], B[:, 3, 1::3] = ny, nx
    B[:, 4, 1::3], B[:, 4, 2::3] = nz, ny
    B[:, 5, 0::3], B[:, 5, 2::3] = nz, nx
    return B


def element_matrices(xe, D, rho):
    """ke, me (ne, 24, 24) and the strain rows (ne, 8 points, 8 nodes, 3):
    per Gauss point l in order, ke += (B^T (D B)) det and
    me[3i+c, 3j+c] += rho N_i N_j det, each dot product summed in index
    order."""
    ne = len(xe)
    ke = np.zeros((ne, 24, 24))
    me = np.zeros((ne, 24, 24))
    rows = np.zeros((ne, 8, 8, 3))
    for l in range(8):
        dNdx, N, det = gauss_point(xe, l)
        rows[:, l] = dNdx
        B = strain_matrix(dNdx)
        DB = np.zeros((ne, 6, 24))
        for r in range(6):
            s = np.zeros((ne, 24))
            for k in range(6):
                s = s + D[r, k] * B[:, k, :]
            DB[:, r, :] = s
        s = np.zeros((ne, 24, 24))
        for k in range(6):
            s = s + B[:, k, :, None] * DB[:, k, None, :]
        ke += s * det[:, None, None]
        for i in range(8):
            for j in range(8):
                v = rho * N[i] * N[j] * det
                for c in range(3):
                    me[:, 3 * i + c, 3 * j + c] += v
    return ke, me, rows


def to_csr(rows, cols, vals, n):
    """Triplets (0-based) to 1-based CSR as tricsr does: entries ordered by
    row, then column, ties in input order; duplicates summed in that order;
    zeros removed."""
    order = np.lexsort((cols, rows))  # stable: ties keep the input order
    r, c, v = rows[order], cols[order], vals[order]
    new = np.ones(len(r), bool)
    new[1:] = (r[1:] != r[:-1]) | (c[1:] != c[:-1])
    start = np.flatnonzero(new)
    count = np.diff(np.append(start, len(r)))
    acc = v[start].copy()
    for t in range(1, int(count.max()) if len(count) else 1):
        sel = count > t
        acc[sel] = acc[sel] + v[start[sel] + t]
    ur, uc = r[start], c[start]
    keep = acc != 0.0
    ur, uc, acc = ur[keep], uc[keep], acc[keep]
    ia = np.concatenate([[1], 1 + np.cumsum(np.bincount(ur, minlength=n))]).astype(np.int32)
    return Csr(ia, (uc + 1).astype(np.int32), acc)


def assemble(xyz, conn, E=2.0e5, nu=0.3, rho=7.8e-9, chunk=4096):
    """K and M (1-based CSR over 3 nn DOFs, DOF 3 (node - 1) + c; element
    triplets row-major, src/spmtx.f90:85-97) and the strain rows Nx, Ny, Nz
    (8 per Gauss point, 8 points per element)."""
    nn, ne = len(xyz), len(conn)
    D = elastic_matrix(E, nu)
    dofs = (3 * (conn[:, :, None] - 1) + np.arange(3)).reshape(ne, 24)
    kv = np.empty((ne, 24, 24))
    mv = np.empty((ne, 24, 24))
    srows = np.empty((ne, 8, 8, 3))
    for b in range(0, ne, chunk):
        sl = slice(b, min(ne, b + chunk))
        kv[sl], mv[sl], srows[sl] = element_matrices(xyz[conn[sl] - 1], D, rho)
    rows = np.repeat(dofs, 24, axis=1).ravel()
    cols = np.tile(dofs, (1, 24)).ravel()
    K = to_csr(rows, cols, kv.ravel(), 3 * nn)
    M = to_csr(rows, cols, mv.ravel(), 3 * nn)
    Nx = np.ascontiguousarray(srows[..., 0]).ravel()
    Ny = np.ascontiguousarray(srows[..., 1]).ravel()
    Nz = np.ascontiguousarray(srows[..., 2]).ravel()
    return K, M, (Nx, Ny, Nz)


def applybc(A: Csr, bc):
    """csrapplybc: entries in a fixed row or column cleared, the diagonal of
    a fixed row set to one, then zeros removed."""
    n = A.n
    rows = np.repeat(np.arange(n), np.diff(A.ia))
    cols = A.ja - 1
    a = A.a.copy()
    hit = (bc[rows] != 0) | (bc[cols] != 0)
    a[hit] = np.where(rows[hit] == cols[hit], 1.0, 0.0)
    keep = a != 0.0
    counts = np.bincount(rows[keep], minlength=n)
    ia = np.concatenate([[1], 1 + np.cumsum(counts)]).astype(np.int32)
    return Csr(ia, A.ja[keep].copy(), a[keep])


def face_mask(xyz, axis, value):
    """All three DOFs of the nodes with x[axis] == value."""
    return np.repeat(xyz[:, axis] == value, 3).astype(np.int32)


def traction(xyz, conn, axis, value, comp, amplitude, area):
    """The load vector rext: amplitude * area shared over the loaded face's
    element-node incidences, on DOF component comp."""
    nn = len(xyz)
    share = np.bincount((conn - 1).ravel(), minlength=nn).astype(float)
    face = xyz[:, axis] == value
    fnode = amplitude * area / share[face].sum()
    rext = np.zeros(3 * nn)
    inc = (conn - 1).ravel()
    inc = inc[face[inc]]
    np.add.at(rext, 3 * inc + comp, fnode)
    return rext
