"""The workloads C1-C5 as configuration files (xtfem_gb300/configs/*.json).

The reference hard-codes its run parameters in its main program
(src/main3d.f90:151-202: material, damage threshold, temporal basis, slab
length, damage resolution, load, GMRES settings) and picks the mesh in its
makefile.  Here each workload is one JSON file holding the mesh (a shipped
rod or a generator with its sizes), the material, the boundary faces by
axis and coordinate, the seeded load, the slab and solver parameters and,
for the coupled panel, the thermal loop and the coupling.  `load` builds
the host-side objects; a caller creates the solvers on the GPU from them:

    w = workloads.load("c2")
    slab = SlabSolver(w.problem, w.slab)
"""
from __future__ import annotations

import json
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

CONFIGS = Path(__file__).resolve().parent / "configs"


def amplitude(seed, lo=50.0, hi=150.0):
    """The seeded load amplitude, U(lo, hi) from numpy's default generator."""
    return float(np.random.default_rng(seed).uniform(lo, hi))


@dataclass
class Workload:
    name: str
    description: str
    raw: dict
    problem: object = None      # Problem (host mesh, K, M)
    slab: object = None         # SlabConfig
    thermal: object = None      # ThermalConfig (coupled workloads)
    coupling: dict = field(default_factory=dict)
    slabs: int = 0
    rods: list = field(default_factory=list)  # (n, amplitude) per rod of a batch

    def close(self):
        if self.problem is not None:
            self.problem.close()
            self.problem = None


def read(name):
    """The configuration dict of a workload ("c1".."c5", or a path)."""
    p = Path(name)
    if not p.suffix:
        p = CONFIGS / f"{str(name).lower()}.json"
    return json.loads(p.read_text())


def _mesh(m):
    from .meshes import holed_panel, sent_plate

    if m["kind"] == "sent":
        return sent_plate(m["nx"], m["ny"], m["nz"], W=m["W"], H=m["H"], t=m["t"],
                          notch=m["notch"], ratio=m["ratio"])
    if m["kind"] == "panel":
        return holed_panel(m["ntheta"], m["nr"], m["nz"], W=m["W"], t=m["t"],
                           radius=m["radius"], ratio=m["ratio"], order=m.get("order", "rings"))
    raise ValueError(f"unknown mesh kind {m['kind']!r}")


def load(name, mesh=None):
    """Build a workload's host-side objects.  mesh: entries that replace
    those of the file's mesh block (a smaller case of the same workload)."""
    from . import api as xt

    c = read(name)
    w = Workload(c["name"], c["description"], c, slabs=int(c.get("slabs", 0)))
    mat = c["material"]
    if "batch" in c:
        # sizes, then amplitudes, from one generator
        b, ld = c["batch"], c["load"]
        rng = np.random.default_rng(b["seed"])
        ns = rng.integers(b["n_range"][0], b["n_range"][1] + 1, b["count"])
        amps = rng.uniform(*ld["amplitude_range"], b["count"])
        w.rods = [(int(n), float(a)) for n, a in zip(ns, amps)]
        return w
    m = dict(c["mesh"], **(mesh or {}))
    if m["kind"] == "rod":
        w.problem = xt.Problem.rod(m["nx"], m["ny"], m["nz"], m["lx"], m["ly"], m["lz"],
                                   mat["E"], mat["nu"], mat["rho"])
    else:
        xyz, conn = _mesh(m)
        w.problem = xt.Problem.from_mesh(xyz, conn, mat["E"], mat["nu"], mat["rho"])
    ld = c["load"]
    w.slab = xt.SlabConfig.make(**c["slab"], area=ld["area"],
                                amplitude=amplitude(ld["seed"], *ld["amplitude_range"]))
    if "thermal" in c:
        t = dict(c["thermal"])
        q0 = t.pop("q0_range")
        w.thermal = xt.ThermalConfig.make(**t, q0=amplitude(ld["seed"], *q0))
        w.coupling = dict(c["coupling"])
    return w
