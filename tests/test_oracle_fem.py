"""The numpy restatement of the finite-element set-up (oracle/fem.py, the
inputs of the CPU baseline) against the reference's shipped meshes and the
library's host assembly: the rod meshes equal inp/prismaticrod-*.inp (their
digests), and K, M, the strain rows and the boundary conditions equal the
host C++ bit for bit (both keep the reference's summation order)."""
import hashlib
import json

import numpy as np
import pytest

from conftest import GOLDEN, clamp_mask
from oracle import fem


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("name", ["prismaticrod-325-192.inp", "prismaticrod-2025-1536.inp",
                                  "prismaticrod-3751-3000.inp", "prismaticrod-26901-24000.inp"])
def test_rod_mesh_equals_shipped_mesh(name):
    ref = json.loads((GOLDEN / "rod_meshes.json").read_text())[name]
    nx, ny, nz, lx, ly, lz = ref["generator"]
    xyz, conn = fem.rod_mesh(nx, ny, nz, lx, ly, lz)
    assert (len(xyz), len(conn)) == (ref["nn"], ref["ne"])
    assert digest(xyz.astype("<f8")) == ref["xyz_sha256"]
    assert digest(conn.astype("<i4")) == ref["conn_sha256"]


@pytest.mark.parametrize("size", [(12, 4, 4), (24, 8, 8)])
def test_assembly_equals_host_assembly(xt, size):
    nx, ny, nz = size
    xyz, conn = fem.rod_mesh(nx, ny, nz)
    K, M, (Nx, Ny, Nz) = fem.assemble(xyz, conn, 2.0e5, 0.3, 7.8e-9)
    pr = xt.Problem.rod(nx, ny, nz, 3.0, 1.0, 1.0, 2.0e5, 0.3, 7.8e-9)
    try:
        for a, b in [(K, pr.K()), (M, pr.M())]:
            assert np.array_equal(a.ia, b.ia) and np.array_equal(a.ja, b.ja)
            assert np.array_equal(a.a, b.a)
        for a, b in zip((Nx, Ny, Nz), pr.strain_rows()):
            assert np.array_equal(a, b)
        bc = clamp_mask(xyz)
        Kb = fem.applybc(K, bc)
        pr.apply_bc(bc)
        K2 = pr.K()
        assert np.array_equal(Kb.ia, K2.ia) and np.array_equal(Kb.ja, K2.ja)
        assert np.array_equal(Kb.a, K2.a)
    finally:
        pr.close()


def test_traction_shares_the_face_load():
    xyz, conn = fem.rod_mesh(12, 4, 4)
    rext = fem.traction(xyz, conn, 0, 3.0, 0, 100.0, 1.0)
    assert np.isclose(rext.sum(), 100.0)
    face = np.repeat(xyz[:, 0] == 3.0, 3)
    assert np.all(rext[~face] == 0.0) and np.all(rext[1::3] == 0.0)
    # corner nodes carry one incidence, edge nodes two, interior nodes four
    f = rext[0::3][xyz[:, 0] == 3.0]
    assert set(np.round(f / f.min()).astype(int)) == {1, 2, 4}
