#!/usr/bin/env python3
"""Benchmark: time-slab solves per second on one GB300.

Workload (the configuration the headline metric is quoted on): prismatic rod
of 20 x 20 x 60 C3D8 elements (26,901 nodes, 24,000 elements, 80,703 spatial
DOFs, 484,218 space-time DOFs), E = 200 GPa, nu = 0.3, rho = 7800 kg/m^3
(N-mm-tonne-s units), base clamped, axial sinusoidal traction of seeded
amplitude U(50, 150) MPa at 20 Hz, slabs of 10 load cycles (dt = 0.5 s) with
25,600 damage points per slab (256 per cycle).  One step = one time slab:
load and jump terms, ILUT(1e-4, 20)-preconditioned GMRES to a true FP64
relative residual of 1e-8 (FP32 operator, factor and basis inside FP64
iterative refinement), the per-Gauss-point damage update of all 192,000
points and the element-deletion test.  Synthetic data: the mesh is generated
(identical to the reference's inp/prismaticrod-26901-24000.inp) and the
amplitude is drawn from numpy's default_rng(seed).

Prints one JSON line.  --impl reference times the reference's CPU
implementation of the same slab (the oracle's C restatement of
kronpgmres/kronlusol/amux/lusol and the damage kernel) on the host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOAD = dict(nx=60, ny=20, nz=20, lx=3.0, ly=1.0, lz=1.0, E=2.0e5, nu=0.3, rho=7.8e-9,
                freq=20.0, dt0=0.005, n1=100, n2=10, nipc=256, lfil=20, droptol=1e-4, im=200,
                tol=1e-8, inner_tol=1e-5, Dc=0.99, seed=0, precision=2, overlap=1)
METRIC = "time-slab solves/s to rel.res 1e-8, mixed-prec batched vs FP64 GMRES, 1 GB300"
UNIT = "slab-solves/s"
DTYPE_NAMES = {0: "fp64", 1: "fp32 operator/factor/basis, fp64 residual+refinement+damage",
               2: "fp32 ilu factor and apply; double-float (fp32 pair) operator and Krylov basis; "
                  "fp64 true residual, refinement and damage"}
PRECISION_NAMES = {0: "fp64 gmres", 1: "fp32 gmres inside fp64 refinement",
                   2: "flexible gmres: double-float operator+basis, fp32 ilu, fp64 refinement"}


def amplitude(seed):
    return float(np.random.default_rng(seed).uniform(50.0, 150.0))


def make_config(xt, precision, seed):
    w = WORKLOAD
    return xt.SlabConfig.make(clamp_axis=0, clamp_value=0.0, load_axis=0, load_value=w["lx"],
                              load_comp=0, amplitude=amplitude(seed), area=w["ly"] * w["lz"],
                              freq=w["freq"], dt0=w["dt0"], n1=w["n1"], n2=w["n2"],
                              nipc=w["nipc"], lfil=w["lfil"], droptol=w["droptol"], im=w["im"],
                              tol=w["tol"], maxits=4000, precision=precision,
                              inner_tol=w["inner_tol"], Dc=w["Dc"], damage=1, group=3,
                              overlap=w["overlap"])


def make_problem(xt):
    w = WORKLOAD
    return xt.Problem.rod(w["nx"], w["ny"], w["nz"], w["lx"], w["ly"], w["lz"], w["E"], w["nu"],
                          w["rho"])


# ----------------------------------------------------------------- clocks
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ------------------------------------------------------------ byte counts
def algorithmic_bytes(problem, ilu_nnz, p, q=6, merged=True):
    nn, ne, nnz_k, nnz_m = problem.sizes()
    if merged:  # K and M share one pattern: one index array, two value arrays
        kron32 = nnz_k * (2 * 4 + 4) + (p + 1) * 4 + 2 * p * q * 4
        kron64 = nnz_k * (2 * 8 + 4) + (p + 1) * 4 + 2 * p * q * 8
    else:
        kron32 = (nnz_k + nnz_m) * (4 + 4) + 2 * (p + 1) * 4 + 2 * p * q * 4
        kron64 = (nnz_k + nnz_m) * (8 + 4) + 2 * (p + 1) * 4 + 2 * p * q * 8
    ilu32 = ilu_nnz * (4 + 4) + 2 * (p + 1) * 4 + p * 4 + 2 * p * q * 4
    ilu64 = ilu_nnz * (8 + 4) + 2 * (p + 1) * 4 + p * 8 + 2 * p * q * 8
    ngp = 8 * ne
    damage = ngp * (29 * 8 * 2 + 8 * 4 + 24 * 8 + 2 * 8) + p * q * 8
    # double-float SpMM: hi/lo values (8 B), FP32 input, double-float output
    if merged:
        krondf = nnz_k * (2 * 8 + 4) + (p + 1) * 4 + p * q * (4 + 8)
    else:
        krondf = (nnz_k + nnz_m) * (8 + 4) + 2 * (p + 1) * 4 + p * q * (4 + 8)
    # a CGS2 step's bytes depend on the step index; its class reports time only
    return {0: kron64, 1: kron32, 2: ilu64, 3: ilu32, 4: damage, 5: None, 6: None, 7: krondf}


# DRAM bytes per launch of the kernel classes, from one ncu capture each on
# this workload (profiles/): dram__bytes_read.sum + dram__bytes_write.sum.
# ilu_apply_fp32 = its forward and backward sweep kernels (the 6 us
# right-hand-side pre-pass is not included; the six thread blocks of a sweep
# read its blob, DRAM serves it once).  kron_spmm_df = the node-block
# kernel, which reads K as 3 x 3 blocks and M as one scalar per block (its
# algorithmic bytes are counted for the CSR operands, as for the others).
NCU_TRAFFIC = {1: 65_922_560 + 519_168, 3: 23_080_960 + 22_542_336,
               4: 99_808_256 + 41_192_960, 7: 57_748_992 + 28_160}

ROOFLINE_NOTES = {
    3: "level-scheduled triangular sweeps: 764 + 743 dependent levels, each sweep on six SMs, one "
       "per temporal block; bound by per-level shared-memory latency and barriers, not by HBM "
       "(DRAM at 0.5 % of peak under ncu); roofline_streaming gives the HBM-bound kernel",
}


def streaming_roofline(prof, nbytes, hbm):
    """HBM roofline of the operator apply of the timed solve (the
    double-float SpMM when it ran, else the FP32 or FP64 one)."""
    for c in (7, 1, 0):
        cnt, tot = prof[c]
        if cnt:
            gbs = nbytes[c] / (tot / cnt / 1e3) / 1e9
            return {"kernel": CLASS_NAMES[c], "achieved": round(gbs, 1), "peak": hbm, "unit": "GB/s",
                    "frac": round(gbs / hbm, 4), "traffic": NCU_TRAFFIC.get(c)}
    return None


CLASS_NAMES = {0: "kron_spmm_fp64", 1: "kron_spmm_fp32", 2: "ilu_apply_fp64",
               3: "ilu_apply_fp32", 4: "damage_update", 5: "cgs2_step_df", 6: "cgs2_step_fp32",
               7: "kron_spmm_df"}


# -------------------------------------------------------------- GPU arm
def run_gpu(args, rank, world):
    import xtfem_gb300 as xt

    xt.lib().xt_init(int(os.environ.get("LOCAL_RANK", "0")))
    prob = make_problem(xt)
    cfg = make_config(xt, precision=WORKLOAD["precision"], seed=WORKLOAD["seed"] + rank)
    slab = xt.SlabSolver(prob, cfg)
    p = slab.p
    K = prob.K()
    Mh = prob.M()
    merged = bool(np.array_equal(K.ia, Mh.ia) and np.array_equal(K.ja, Mh.ja))
    alu, jlu, ju = xt.ilut(K, WORKLOAD["lfil"], WORKLOAD["droptol"])
    ilu_nnz = len(alu) - p - 1
    info = []
    for _ in range(args.warmup):
        info.append(slab.step())
    dist_barrier(world)
    launches0 = xt.lib().xt_launch_count()
    xt.profile(True)
    xt.lib().xt_sync()
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        t_host0 = time.perf_counter()
        xt.lib().xt_mark(0)
        steps = [slab.step() for _ in range(args.steps)]
        slab.drain()  # the last slab's damage update belongs to the timed work
        xt.lib().xt_mark(1)
        ms = xt.lib().xt_elapsed_ms(0, 1)
        t_host = (time.perf_counter() - t_host0) * 1e3
    launches = xt.lib().xt_launch_count() - launches0
    prof = {c: xt.profile_read(c) for c in CLASS_NAMES}
    xt.profile(False)
    ms_max = dist_max(ms, world)
    value = args.steps * world / (ms_max / 1e3)

    # roofline of the dominant kernel class
    hbm, peak_kind = peaks()
    nbytes = algorithmic_bytes(prob, ilu_nnz, p, merged=merged)
    dom = max((c for c in prof if nbytes[c]), key=lambda c: prof[c][1])
    cnt, tot = prof[dom]
    avg_ms = tot / max(cnt, 1)
    achieved = nbytes[dom] / (avg_ms / 1e3) / 1e9 if cnt else 0.0
    kernels = {CLASS_NAMES[c]: {"launches": prof[c][0], "total_ms": round(prof[c][1], 3),
                                "avg_us": round(1e3 * prof[c][1] / max(prof[c][0], 1), 2),
                                "bytes_per_launch": nbytes[c],
                                "gbs": round(nbytes[c] / (prof[c][1] / max(prof[c][0], 1) / 1e3)
                                             / 1e9, 1) if prof[c][0] and nbytes[c] else None}
               for c in prof}
    its = [s["its"] for s in steps]
    res = [s["relres"] for s in steps]
    out = {
        "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_max / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": DTYPE_NAMES[WORKLOAD["precision"]],
        "data": "synthetic (generated rod mesh, seeded load amplitude)",
        "config": {"workload": "C2 prismatic rod 20x20x60 C3D8, 80,703 DOF x 6 temporal blocks",
                   "nip": WORKLOAD["nipc"] * WORKLOAD["n1"], "ilut": [WORKLOAD["droptol"],
                                                                      WORKLOAD["lfil"]],
                   "gmres_restart": WORKLOAD["im"], "tol": WORKLOAD["tol"],
                   "precision": PRECISION_NAMES[WORKLOAD["precision"]],
                   "amplitude_mpa": cfg.amplitude,
                   "l2": "inputs larger than L2 (operator+factor+basis >> 129 MB)",
                   "parallelism": f"replicas x{world}"},
        "iterations_per_slab": float(np.mean(its)), "relres_max": float(np.max(res)),
        "host_ms_per_step": round(t_host / args.steps, 3),
        "roofline": {"bound": "hbm", "kernel": CLASS_NAMES[dom], "achieved": round(achieved, 1),
                     "peak": hbm, "peak_kind": peak_kind, "unit": "GB/s",
                     "frac": round(achieved / hbm, 4), "traffic": NCU_TRAFFIC.get(dom),
                     "note": ROOFLINE_NOTES.get(dom)},
        "roofline_streaming": streaming_roofline(prof, nbytes, hbm),
        "kernels": kernels,
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
    }
    if rank == 0 and args.specimens > 1:
        out["batched"] = run_batched(xt, args, args.specimens)
    if rank == 0 and args.rods > 0:
        out["rod_batch"] = run_rod_batch(xt, args.rods, WORKLOAD["seed"])
    if rank == 0 and not args.skip_fp64:
        out["fp64_gpu"] = run_fp64_reference_point(xt, args)
    if rank == 0 and not args.skip_e2e:
        out["e2e"] = run_e2e(xt, args, world)
    if rank == 0 and not args.skip_cpu:
        out["cpu_baseline"] = cpu_baseline(its=float(np.mean(its)), sample_its=args.cpu_its,
                                           threads=os.cpu_count() or 1, for_arm=False)
    if rank == 0 and not args.skip_variants:
        out["variants"] = run_variants(xt, args)
    if rank == 0:
        out["refactor_host"] = refactor_host(xt)
    slab.close()
    prob.close()
    return out


def refactor_host(xt, nfail=24):
    """Host side of a deletion event on the C2 rod (host code only, after
    the GPU measurements): the deletion surgery of nfail seeded elements
    (K -= their element matrices, disconnected nodes fixed, boundary
    conditions re-applied) and the ILUT refactor of the new K, which the
    library pipelines over the host threads (serial-order ILUT timed beside
    it).  Wall clock; the factor's re-upload to the device is not included."""
    try:
        pr = make_problem(xt)
        xyz, conn = pr.mesh()
        bc = np.repeat((xyz[:, 0] == 0.0).astype(np.int32), 3)
        pr.apply_bc(bc)
        nef = np.sort(np.random.default_rng(WORKLOAD["seed"]).choice(len(conn), nfail,
                                                                      replace=False) + 1)
        t0 = time.perf_counter()
        pr.delete(nef.astype(np.int32), bc)
        t1 = time.perf_counter()
        K = pr.K()
        t2 = time.perf_counter()
        xt.ilut(K, WORKLOAD["lfil"], WORKLOAD["droptol"])
        t3 = time.perf_counter()
        prev = os.environ.get("XTFEM_ILUT_THREADS")
        os.environ["XTFEM_ILUT_THREADS"] = "1"
        try:
            t4 = time.perf_counter()
            xt.ilut(K, WORKLOAD["lfil"], WORKLOAD["droptol"])
            t5 = time.perf_counter()
        finally:
            if prev is None:
                del os.environ["XTFEM_ILUT_THREADS"]
            else:
                os.environ["XTFEM_ILUT_THREADS"] = prev
        pr.close()
        return {"deleted_elements": nfail, "surgery_ms": round((t1 - t0) * 1e3, 1),
                "ilut_ms": round((t3 - t2) * 1e3, 1),
                "ilut_ms_one_thread": round((t5 - t4) * 1e3, 1),
                "host_threads": os.cpu_count() or 1,
                "timer": "host wall clock", "scope": "deletion surgery + ILUT(1e-4, 20) of "
                "the C2 K; the device re-upload of the factor is not included"}
    except Exception as e:  # a failure here must not cost the measurements above
        return {"error": f"{type(e).__name__}: {e}"}


def rod_system(xt, n, amp, dt=0.5, freq=20.0):
    """Space-time system and first-slab load of the n x n x 3n rod (clamped
    at x = 0, axial traction amp MPa on x = 3 shared by the face's nodes),
    ILUT(1e-4, 20) factor attached."""
    pr = xt.Problem.rod(3 * n, n, n, 3.0, 1.0, 1.0, WORKLOAD["E"], WORKLOAD["nu"], WORKLOAD["rho"])
    xyz, _ = pr.mesh()
    bc = np.repeat((xyz[:, 0] == 0.0).astype(np.int32), 3)
    pr.apply_bc(bc)
    K, M = pr.K(), pr.M()
    alu, jlu, ju = xt.ilut(K, WORKLOAD["lfil"], WORKLOAD["droptol"])
    w = 2 * np.pi * freq
    k, m, kt, mt, _, _ = xt.stcoeff_m(0.0, dt, w)
    face = np.isclose(xyz[:, 0], 3.0)
    rext = np.zeros(K.n)
    rext[3 * np.flatnonzero(face)] = amp / face.sum()
    fextc, _ = xt.getfextc_m(0.0, w, dt)
    rhs = np.concatenate([f * rext for f in fextc])
    rhs[np.tile(bc, 6) == 1] = 0.0
    s = xt.SpaceTimeSystem(K, M)
    s.set_ilu(alu, jlu, ju, group=3)
    s.set_temporal(k + kt, m + mt)
    pr.close()
    return s, rhs


def run_rod_batch(xt, count, seed):
    """The many-rod workload: `count` rods of n x n x 3n elements, n drawn
    uniformly from 4..10 and the load amplitude from U(50, 150) MPa with
    numpy's default_rng(seed); one slab solve each (flexible GMRES with the
    batch's tuned restart length, FP32 ILU, true residual <= 1e-8) through
    xt_batch_solve, against the same systems solved one after another.
    Host wall clock with the device synchronised at both ends; the tuning
    call (one batch solve per candidate restart length) is untimed."""
    rng = np.random.default_rng(seed)
    ns = rng.integers(4, 11, count)
    amps = rng.uniform(50.0, 150.0, count)
    cases = [rod_system(xt, int(n), float(a)) for n, a in zip(ns, amps)]
    systems = [c[0] for c in cases]
    rhs = [c[1] for c in cases]
    batch = xt.SystemBatch(systems)
    kw = dict(im=0, tol=WORKLOAD["tol"], precision=2)  # tuned restart length
    batch.solve(rhs, **kw)  # tunes, then solves (untimed)
    kw["im"] = batch.restart
    xt.lib().xt_sync()
    t0 = time.perf_counter()
    _, stats, _ = batch.solve(rhs, **kw)
    xt.lib().xt_sync()
    t_batch = time.perf_counter() - t0
    t0 = time.perf_counter()
    for s, r in zip(systems, rhs):
        s.solve(r, **kw)
    xt.lib().xt_sync()
    t_seq = time.perf_counter() - t0
    batch.close()
    dofs = int(sum(s.p * s.q for s in systems))
    for s in systems:
        s.close()
    return {"rods": count, "value": round(count / t_batch, 2), "unit": "rod-slab-solves/s",
            "ms_all": round(t_batch * 1e3, 2), "one_after_another_ms": round(t_seq * 1e3, 2),
            "restart": kw["im"],
            "iterations_mean": round(float(np.mean([st["its"] for st in stats])), 1),
            "relres_max": float(max(st["relres"] for st in stats)),
            "space_time_dofs": dofs, "n_values": ns.tolist(),
            "timer": "host wall clock, device synchronised at both ends",
            "workload": f"{count} rods n x n x 3n, n ~ U{{4..10}}, amplitude U(50,150) MPa, seed {seed}"}


def run_batched(xt, args, specimens):
    """Independent specimens of the same workload, each with its own load
    amplitude (seeds 0..B-1), solved concurrently: one host thread and one
    CUDA stream per specimen.  A slab's ILU sweeps occupy one SM, so
    independent specimens fill the others.  Returns aggregate slab-solves/s
    over B specimens (host wall clock around the timed steps, device
    synchronised at both ends)."""
    import concurrent.futures as cf

    B = specimens
    probs = [make_problem(xt) for _ in range(B)]
    cfgs = [make_config(xt, precision=WORKLOAD["precision"], seed=WORKLOAD["seed"] + b)
            for b in range(B)]
    with cf.ThreadPoolExecutor(B) as ex:  # host ILUT of every specimen in parallel
        slabs = list(ex.map(lambda b: xt.SlabSolver(probs[b], cfgs[b]), range(B)))
    start = threading.Barrier(B + 1)
    done = threading.Barrier(B + 1)
    its = [[] for _ in range(B)]
    res = [[] for _ in range(B)]
    errs = []

    def worker(b):
        try:
            for _ in range(args.warmup):
                slabs[b].step()
            slabs[b].drain()
            start.wait()
            for _ in range(args.steps):
                st = slabs[b].step()
                its[b].append(st["its"])
                res[b].append(st["relres"])
            slabs[b].drain()
        except Exception as e:  # reported after the join
            errs.append(repr(e))
            start.abort()
        finally:
            try:
                done.wait()
            except threading.BrokenBarrierError:
                pass

    threads = [threading.Thread(target=worker, args=(b,)) for b in range(B)]
    for t in threads:
        t.start()
    try:
        start.wait()
    except threading.BrokenBarrierError:
        pass
    xt.lib().xt_sync()
    if args.batched_profile:
        xt.profile(True)
    t0 = time.perf_counter()
    try:
        done.wait()
    except threading.BrokenBarrierError:
        pass
    xt.lib().xt_sync()
    sec = time.perf_counter() - t0
    prof = {}
    if args.batched_profile:
        prof = {CLASS_NAMES[c]: dict(zip(("launches", "total_ms"), xt.profile_read(c)))
                for c in CLASS_NAMES}
        xt.profile(False)
    for t in threads:
        t.join()
    for sl in slabs:
        sl.close()
    for pr in probs:
        pr.close()
    if errs:
        raise RuntimeError("batched run failed: " + errs[0])
    return {"specimens": B, "value": round(B * args.steps / sec, 4), "unit": UNIT,
            "ms_per_step_all": round(sec * 1e3 / args.steps, 1),
            "iterations_per_slab": float(np.mean(its)), "relres_max": float(np.max(res)),
            "timer": "host wall clock, device synchronised at both ends",
            "workload": f"{B} independent C2 rods (load amplitudes of seeds 0..{B - 1})",
            **({"kernels": prof} if prof else {})}


def run_fp64_reference_point(xt, args):
    """The plain FP64 GPU GMRES on the same workload (the 3x denominator)."""
    prob = make_problem(xt)
    slab = xt.SlabSolver(prob, make_config(xt, precision=0, seed=WORKLOAD["seed"]))
    slab.step()
    xt.lib().xt_sync()
    n = max(1, min(args.steps, 3))
    xt.lib().xt_mark(2)
    st = [slab.step() for _ in range(n)]
    slab.drain()
    xt.lib().xt_mark(3)
    ms = xt.lib().xt_elapsed_ms(2, 3)
    slab.close()
    prob.close()
    return {"value": round(n / (ms / 1e3), 4), "unit": UNIT, "steps": n,
            "iterations_per_slab": float(np.mean([s["its"] for s in st]))}


def run_variants(xt, args):
    """The C2 slab two more ways, timed like fp64_gpu (CUDA events around
    n slabs after one untimed slab): without the damage update (the solve,
    load and jump terms only; sequential loop), and with the damage update
    at a reduced temporal resolution (16 points per load cycle, 1,600 per
    slab instead of 25,600; overlapped loop as the headline)."""
    out = {}
    variants = (("no_damage", {"damage": 0, "overlap": 0}),
                ("reduced_nip", {"nipc": 16}))
    for name, change in variants:
        try:
            prob = make_problem(xt)
            cfg = make_config(xt, precision=WORKLOAD["precision"], seed=WORKLOAD["seed"])
            for k, v in change.items():
                setattr(cfg, k, v)
            slab = xt.SlabSolver(prob, cfg)
            slab.step()
            xt.lib().xt_sync()
            n = max(1, min(args.steps, 3))
            xt.lib().xt_mark(4)
            st = [slab.step() for _ in range(n)]
            slab.drain()
            xt.lib().xt_mark(5)
            ms = xt.lib().xt_elapsed_ms(4, 5)
            slab.close()
            prob.close()
            out[name] = {"value": round(n / (ms / 1e3), 4), "unit": UNIT, "steps": n,
                         "nip": cfg.nipc * cfg.n1, "damage": int(cfg.damage),
                         "iterations_per_slab": float(np.mean([s["its"] for s in st])),
                         "relres_max": float(max(s["relres"] for s in st))}
        except Exception as e:  # a failure here must not cost the headline line
            out[name] = {"error": f"{type(e).__name__}: {e}"}
    return out


def run_e2e(xt, args, world):
    """Same slabs through the public API with host buffers: the load blocks
    go host->device and the slab displacement and damage come back, every
    step, inside the timed region."""
    prob = make_problem(xt)
    cfg = make_config(xt, precision=WORKLOAD["precision"], seed=WORKLOAD["seed"])
    slab = xt.SlabSolver(prob, cfg)
    p = slab.p
    xyz, conn = prob.mesh()
    nn = len(xyz)
    share = np.bincount(conn.ravel() - 1, minlength=nn).astype(float)
    face = xyz[:, 0] == WORKLOAD["lx"]
    fnode = cfg.amplitude * cfg.area / share[face].sum()
    rext = np.zeros(p)
    np.add.at(rext, 3 * (conn.ravel()[face[conn.ravel() - 1]] - 1), fnode)
    w = 2 * np.pi * WORKLOAD["freq"]
    dt = WORKLOAD["dt0"] * WORKLOAD["n1"]
    disp = np.zeros(p * 6)
    D = np.zeros(slab.ngp)

    def step(k):
        t1 = k * dt
        fextc, _ = xt.getfextc_m(t1, w, dt)
        fext = np.concatenate([f * rext for f in fextc])
        return slab.step_host(fext, disp, D)

    k = 0
    for _ in range(args.warmup):
        step(k)
        k += 1
    xt.lib().xt_sync()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step(k)
        k += 1
    slab.drain()
    xt.lib().xt_sync()
    sec = time.perf_counter() - t0
    slab.close()
    prob.close()
    return {"value": round(args.steps / sec, 4), "unit": UNIT,
            "h2d_bytes_per_step": int(p * 6 * 8), "d2h_bytes_per_step": int(p * 6 * 8 + D.nbytes),
            "timer": "host wall clock around synchronized steps"}


# -------------------------------------------------------- CPU baseline
def cpu_baseline(its, sample_its, threads, for_arm):
    """The reference's CPU path (oracle restatement) on a bounded sample of
    the same slab: sample_its GMRES iterations and the damage update of a
    slice of the Gauss points (OpenMP over points, as src/cpu_damage.f90),
    scaled to one full slab.  GMRES is timed twice: in the reference's serial
    order (kronpgmres has no threading) and on all the host threads (OpenMP
    over the rows of each amux pass and vector update and over the q
    independent lusol calls); the threaded one gives the value."""
    import xtfem_gb300 as xt
    from oracle import oracle as orc

    prob = make_problem(xt)
    xyz, conn = prob.mesh()
    nn, ne = len(xyz), len(conn)
    p = 3 * nn
    bc = np.zeros(p, np.int32)
    bc[np.repeat(xyz[:, 0] == 0.0, 3)] = 1
    prob.apply_bc(bc)
    K, M = prob.K(), prob.M()
    (alu, jlu, ju), ierr = orc.ilut(K, WORKLOAD["lfil"], WORKLOAD["droptol"])
    w = 2 * np.pi * WORKLOAD["freq"]
    dt = WORKLOAD["dt0"] * WORKLOAD["n1"]
    k, m, kt, mt, k1, m1 = xt.stcoeff_m(0.0, dt, w)
    share = np.bincount(conn.ravel() - 1, minlength=nn).astype(float)
    face = xyz[:, 0] == WORKLOAD["lx"]
    rext = np.zeros(p)
    np.add.at(rext, 3 * (conn.ravel()[face[conn.ravel() - 1]] - 1),
              amplitude(WORKLOAD["seed"]) / share[face].sum())
    fextc, _ = xt.getfextc_m(0.0, w, dt)
    rhs = np.concatenate([f * rext for f in fextc])
    def gmres_sample(nt):
        # one restart cycle of sample_its steps (maxits is only tested at the
        # end of a cycle in kronpgmres); shorter cycles make the
        # orthogonalisation cheaper than in GMRES(im), so the scaled baseline
        # errs on the fast side
        orc.set_threads(nt)
        try:
            t0 = time.perf_counter()
            _, _, done, _ = orc.kronpgmres(k + kt, m + mt, K, M, alu, jlu, ju, rhs,
                                           im=sample_its, eps=1e-30, maxits=sample_its)
            return (time.perf_counter() - t0) / max(done, 1), done
        finally:
            orc.set_threads(1)

    t_serial, done = gmres_sample(1)
    t_iter, _ = gmres_sample(threads) if threads > 1 else (t_serial, done)
    # damage: a slice of the points over the full slab resolution
    nip = WORKLOAD["nipc"] * WORKLOAD["n1"]
    ne_s = max(1, min(ne, 8 * threads))
    Nx, Ny, Nz = prob.strain_rows()
    sol = np.random.default_rng(0).standard_normal(p * 6) * 1e-4
    nodes = np.repeat(conn[:ne_s], 8, axis=0).ravel().astype(np.int32)
    Nt = xt.nt_table(nip, np.array([0.0, dt / 2, dt]), w)
    ngs = 8 * ne_s
    st = {kk: np.zeros(ngs * 6) for kk in ["eps_old", "eps_pl", "sig_eff", "sig_back"]}
    st.update({kk: np.zeros(ngs) for kk in ["p", "D", "ws", "del_po", "sig_d"]})
    t0 = time.perf_counter()
    orc.damage(ne_s, nn, nip, nodes, Nx[: ngs * 8], Ny[: ngs * 8], Nz[: ngs * 8], Nt, sol,
               np.full(ngs, WORKLOAD["E"]), np.full(ngs, WORKLOAD["nu"]), st, nthreads=threads)
    t_dmg = (time.perf_counter() - t0) * (ne / ne_s)
    t_slab = t_iter * its + t_dmg
    prob.close()
    return {"value": round(1.0 / t_slab, 6), "unit": UNIT, "cores": threads,
            "kind": "port",
            "sample": (f"{done} GMRES iterations (one cycle) on {threads} threads "
                       f"({t_iter * 1e3:.1f} ms each; {t_serial * 1e3:.1f} ms in the reference's "
                       f"serial order), scaled to {its:.0f} per slab + damage of "
                       f"{ngs} of {8 * ne} Gauss points x {nip} steps on {threads} threads "
                       f"(scaled to all points)"),
            "seconds_per_slab": round(t_slab, 3), "gmres_s_per_iter": round(t_iter, 5),
            "gmres_s_per_iter_serial": round(t_serial, 5),
            "value_serial_gmres": round(1.0 / (t_serial * its + t_dmg), 6),
            "damage_s_per_slab": round(t_dmg, 3)}


def run_reference(args, rank, world):
    if rank != 0:
        return None
    threads = os.cpu_count() or 1
    vals = []
    for _ in range(args.warmup if args.warmup < 1 else 1):
        pass
    t0 = time.perf_counter()
    its_guess = float(args.ref_its)
    for _ in range(args.steps):
        b = cpu_baseline(its=its_guess, sample_its=args.cpu_its, threads=threads, for_arm=True)
        vals.append(b)
    sec = time.perf_counter() - t0
    v = float(np.median([b["value"] for b in vals]))
    cfg = {"workload": "C2 prismatic rod 20x20x60 C3D8, 80,703 DOF x 6 temporal blocks",
           "nip": WORKLOAD["nipc"] * WORKLOAD["n1"], "ilut": [WORKLOAD["droptol"],
                                                              WORKLOAD["lfil"]],
           "gmres_restart": WORKLOAD["im"], "tol": WORKLOAD["tol"],
           "iterations_per_slab_assumed": its_guess}
    return {"impl": "reference", "metric": METRIC, "value": round(v, 6), "unit": UNIT,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1e3 / v, 1), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp64", "data": "synthetic", "config": cfg,
            "cpu_baseline": {"value": round(v, 6), "unit": UNIT, "cores": threads,
                             "kind": "port", "sample": vals[0]["sample"],
                             "value_serial_gmres": float(np.median(
                                 [b["value_serial_gmres"] for b in vals]))},
            "e2e": {"value": round(v, 6), "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "wall_s": round(sec, 1)}


# ------------------------------------------------------------ harness
def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=world)
    return rank, world


def dist_barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def dist_max(v, world):
    if world > 1:
        import torch
        import torch.distributed as dist

        t = torch.tensor([float(v)])
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())
    return float(v)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-its", type=int, default=40)
    ap.add_argument("--ref-its", type=float, default=182.0)
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-variants", action="store_true",
                    help="skip the no-damage and reduced-nip slab lines")
    ap.add_argument("--inner-tol", type=float, default=None)
    ap.add_argument("--im", type=int, default=None)
    ap.add_argument("--specimens", type=int, default=8,
                    help="also time this many independent specimens solved concurrently "
                         "(the batched line); 1 = off")
    ap.add_argument("--rods", type=int, default=64,
                    help="also time a batch of this many uneven rods (xt_batch_solve); 0 = off")
    ap.add_argument("--batched-profile", action="store_true",
                    help="per-class CUDA-event times inside the batched run")
    ap.add_argument("--overlap", type=int, default=None,
                    help="1 = each slab's damage update overlaps the next slab's solve")
    ap.add_argument("--precision", type=int, default=None,
                    help="inner solve: 1 = FP32 GMRES in FP64 refinement, 2 = flexible GMRES "
                         "(FP64 operator and basis, FP32 factor)")
    args = ap.parse_args()
    if args.inner_tol is not None:
        WORKLOAD["inner_tol"] = args.inner_tol
    if args.im is not None:
        WORKLOAD["im"] = args.im
    if args.precision is not None:
        WORKLOAD["precision"] = args.precision
    if args.overlap is not None:
        WORKLOAD["overlap"] = args.overlap
    rank, world = dist_setup()
    if args.impl == "reference":
        out = run_reference(args, rank, world)
    else:
        out = run_gpu(args, rank, world)
    if rank == 0 and out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
