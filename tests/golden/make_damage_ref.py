"""Golden vectors of the reference's own damage kernel.

Runs kokkos_host_ from the reference's src/kokkos_host.cpp and
src/kokkos_kernel.h, compiled unchanged against the host-only Kokkos
stand-in (oracle/Makefile target `ref`, output oracle/_ref/libxtref.so), on
seeded inputs over 32 elements of the 4x4x12 rod (the 16 at the clamp and
16 drawn by the seed; node ids refer to the whole rod), two calls in a row
per case, and writes inputs and the state after each call to
tests/golden/damage_ref.npz.  The cases:

  elastic   small displacement field: every step elastic;
  plastic   plastic cycling with the stored energy starting at zero;
  growth    the same field with the stored energy seeded just below the
            damage threshold, so damage grows on both calls.

Each point has its own E and nu.  The fixture lets the oracle's damage
statement and the GPU kernel be checked against the reference's kernel on
machines without the reference checkout.

Usage: python tests/golden/make_damage_ref.py   (after make -C oracle ref)
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from oracle import oracle as orc  # noqa: E402

NIP = 512
CASES = {"elastic": (1e-5, 0.0, 0.0), "plastic": (4e-4, 0.0, 0.5), "growth": (4e-4, 31.7, 1.0)}


def rod_inputs():
    """Mesh and strain rows of the 4x4x12 rod.  They come from the
    library's rod generator (equal to the reference's
    inp/prismaticrod-325-192.inp, tests/test_host.py) and are stored in the
    fixture as inputs, so the fixture does not depend on them later."""
    import xtfem_gb300 as xt

    pr = xt.Problem.rod(12, 4, 4, 3.0, 1.0, 1.0, 2.0e5, 0.3, 7.8e-9)
    xyz, conn = pr.mesh()
    Nx, Ny, Nz = pr.strain_rows()
    pr.close()
    return xyz, conn, Nx, Ny, Nz


def main():
    if orc.ref_lib() is None:
        sys.exit("oracle/_ref/libxtref.so is not built: run make -C oracle ref")
    xyz, conn, Nx, Ny, Nz = rod_inputs()
    nn, ne = len(xyz), len(conn)
    rng = np.random.default_rng(2024)
    clamp = [e for e in range(ne) if np.all(xyz[conn[e] - 1, 0] <= 0.25 + 1e-12)]
    rest = [e for e in range(ne) if e not in clamp]
    elems = np.array(sorted(clamp + list(rng.choice(rest, 16, replace=False))))
    gps = (elems[:, None] * 8 + np.arange(8)).ravel()
    rows = (gps[:, None] * 8 + np.arange(8)).ravel()
    out = {"elems": elems, "nn": np.array(nn), "nip": np.array(NIP),
           "nodes": np.repeat(conn[elems], 8, axis=0).ravel().astype(np.int32),
           "Nx": Nx[rows], "Ny": Ny[rows], "Nz": Nz[rows]}
    ngp = len(gps)
    for name, (amp, ws0, t1) in CASES.items():
        out[f"{name}_Nt"] = orc.nt_table(NIP, np.array([t1, t1 + 0.25, t1 + 0.5]), 2 * np.pi * 20)
        out[f"{name}_sol"] = rng.standard_normal(6 * 3 * nn) * amp
        out[f"{name}_ym"] = rng.uniform(1.9e5, 2.1e5, ngp)
        out[f"{name}_nu"] = rng.uniform(0.28, 0.32, ngp)
        st = {k: np.zeros(ngp * 6) for k in orc.STATE_KEYS[:4]}
        st.update({k: np.zeros(ngp) for k in orc.STATE_KEYS[4:]})
        st["ws"][:] = ws0
        for k in orc.STATE_KEYS:
            out[f"{name}_in_{k}"] = st[k].copy()
        for call in (1, 2):
            orc.ref_damage(len(elems), nn, NIP, out["nodes"], out["Nx"], out["Ny"], out["Nz"],
                           out[f"{name}_Nt"], out[f"{name}_sol"], out[f"{name}_ym"],
                           out[f"{name}_nu"], st)
            for k in orc.STATE_KEYS:
                out[f"{name}_out{call}_{k}"] = st[k].copy()
        print(name, "max D", st["D"].max(), "max p", st["p"].max())
    np.savez_compressed(HERE / "damage_ref.npz", **out)


if __name__ == "__main__":
    main()
