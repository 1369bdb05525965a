"""Golden fixtures from the reference's shipped rod meshes.

Reads the reference's inp/prismaticrod-*.inp files (plain text: node count,
"id x y z" lines, element count, "id n1..n8" lines) with a parser of its own
and writes, per mesh, the sizes and SHA-256 digests of the coordinates
(float64, as parsed) and the connectivity (int32), plus the full arrays of
the 325-node mesh.  The tests compare the product's rod generator with
these, so the generated meshes are pinned to the reference's files without
the reference being present at test time.

Usage: python tests/golden/make_golden.py REFERENCE_ROOT

REFERENCE_ROOT is the directory of the reference checkout that holds inp/.
"""
import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
# mesh file -> rod generator arguments (nx, ny, nz elements; lx, ly, lz)
MESHES = {
    "prismaticrod-325-192.inp": [12, 4, 4, 3.0, 1.0, 1.0],
    "prismaticrod-2025-1536.inp": [24, 8, 8, 3.0, 1.0, 1.0],
    "prismaticrod-3751-3000.inp": [30, 10, 10, 3.0, 1.0, 1.0],
    "prismaticrod-26901-24000.inp": [60, 20, 20, 3.0, 1.0, 1.0],
}


def parse(path):
    tok = path.read_text().split("\n")
    nn = int(tok[0].split()[0])
    xyz = np.array([[float(v) for v in tok[1 + i].split()[1:4]] for i in range(nn)])
    ne = int(tok[1 + nn].split()[0])
    conn = np.array([[int(v) for v in tok[2 + nn + e].split()[1:9]] for e in range(ne)],
                    dtype=np.int32)
    return xyz, conn


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main(root):
    out = {}
    for name, args in MESHES.items():
        xyz, conn = parse(Path(root) / "inp" / name)
        out[name] = {"generator": args, "nn": len(xyz), "ne": len(conn),
                     "xyz_sha256": digest(xyz.astype("<f8")),
                     "conn_sha256": digest(conn.astype("<i4"))}
        if name == "prismaticrod-325-192.inp":
            np.savez_compressed(HERE / "rod_c1_mesh.npz", xyz=xyz, conn=conn)
    (HERE / "rod_meshes.json").write_text(json.dumps(out, indent=1) + "\n")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py REFERENCE_ROOT")
    main(sys.argv[1])
