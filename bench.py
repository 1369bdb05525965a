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
                tol=1e-8, inner_tol=1e-5, Dc=0.99, seed=0, precision=2, overlap=1, gs_passes=1)
METRIC = "time-slab solves/s to rel.res 1e-8, mixed-prec batched vs FP64 GMRES, 1 GB300"
UNIT = "slab-solves/s"
DTYPE_NAMES = {0: "fp64", 1: "fp32 operator/factor/basis, fp64 residual+refinement+damage",
               3: "bf16-stored K and M with fp32 accumulation in the preconditioner, fp32 "
                  "factor; double-float operator and basis; fp64 residual, refinement and damage",
               2: "fp32 ilu factor and apply; double-float (fp32 pair) operator and Krylov basis; "
                  "fp64 true residual, refinement and damage"}
PRECISION_NAMES = {0: "fp64 gmres", 1: "fp32 gmres inside fp64 refinement",
                   2: "flexible gmres: double-float operator+basis, fp32 ilu, fp64 refinement",
                   3: "flexible gmres preconditioned by fp32 gmres on bf16-stored K and M, "
                      "fp64 refinement"}


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
                              overlap=w["overlap"], gs_passes=w["gs_passes"])


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
NCU_TRAFFIC = {1: 65_922_560 + 519_168, 3: 26_072_064 + 26_405_888,
               4: 99_808_256 + 41_192_960, 7: 57_748_992 + 28_160}

ROOFLINE_NOTES = {
    3: "level-scheduled triangular sweeps: 764 + 743 dependent levels, each sweep on six SMs, one "
       "per temporal block; bound by per-level latency (shared-memory window reads, shuffles, the "
       "level barrier), not by HBM (DRAM at about 1 % of peak under ncu); roofline_streaming gives "
       "the HBM-bound kernel",
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
    xt.lib().xt_sync()
    # The timed region runs without per-kernel events: a CUDA event pair
    # around every ILU apply, operator and Gram-Schmidt step costs about 6 %
    # of the slab rate on C2.  The per-kernel times come from a second timed
    # pass of the same slab loop with those events on (profile_steps slabs).
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        t_host0 = time.perf_counter()
        xt.lib().xt_mark(0)
        steps = [slab.step() for _ in range(args.steps)]
        slab.drain()  # the last slab's damage update belongs to the timed work
        xt.lib().xt_mark(1)
        ms = xt.lib().xt_elapsed_ms(0, 1)
        t_host = (time.perf_counter() - t_host0) * 1e3
    launches = xt.lib().xt_launch_count() - launches0
    ms_max = dist_max(ms, world)
    value = args.steps * world / (ms_max / 1e3)
    profile_steps = max(1, min(args.steps, 5))
    xt.profile(True)
    xt.lib().xt_mark(2)
    psteps = [slab.step() for _ in range(profile_steps)]
    slab.drain()
    xt.lib().xt_mark(3)
    ms_prof = xt.lib().xt_elapsed_ms(2, 3)
    prof = {c: xt.profile_read(c) for c in CLASS_NAMES}
    orth_bytes = {c: xt.profile_bytes(c) for c in (5, 6)}
    xt.profile(False)

    # roofline of the dominant kernel class
    hbm, peak_kind = peaks()
    nbytes = algorithmic_bytes(prob, ilu_nnz, p, merged=merged)
    for c in (5, 6):  # Gram-Schmidt steps: mean of the recorded per-step bytes
        if prof[c][0]:
            nbytes[c] = int(orth_bytes[c] / prof[c][0])
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
    # damage update: FP64 work of its exact steps against the FP64 pipe.
    # An exact step restates src/kokkos_kernel.h:56-180 in FP64: the
    # displacement interpolation (144 multiply-adds), the strain (144
    # flops), the elastic matrix, the predictor and the equivalent stress
    # (about 180 flops): 610 flops counted from the kernel source, more when
    # the plastic corrector runs.  Screened steps are FP32.
    exact = float(np.mean([s["exact_steps"] for s in psteps]))
    screened = float(np.mean([s["screened_steps"] for s in psteps]))
    dcnt, dms = prof[4]
    fp64_gflops = exact * 610.0 / (dms / max(dcnt, 1) / 1e3) / 1e9 if dcnt else 0.0
    out = {
        "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_max / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": DTYPE_NAMES[WORKLOAD["precision"]],
        "data": "synthetic (generated rod mesh, seeded load amplitude)",
        "config": dict(workload_config(cfg.amplitude), parallelism=f"replicas x{world}"),
        "precision": PRECISION_NAMES[WORKLOAD["precision"]],
        "iterations_per_slab": float(np.mean(its)), "relres_max": float(np.max(res)),
        "host_ms_per_step": round(t_host / args.steps, 3),
        "roofline": {"bound": "hbm", "kernel": CLASS_NAMES[dom], "achieved": round(achieved, 1),
                     "peak": hbm, "peak_kind": peak_kind, "unit": "GB/s",
                     "frac": round(achieved / hbm, 4), "traffic": NCU_TRAFFIC.get(dom),
                     "note": ROOFLINE_NOTES.get(dom)},
        "roofline_streaming": streaming_roofline(prof, nbytes, hbm),
        "kernels": kernels,
        "kernel_timing": {"pass": "profiled", "slabs": profile_steps,
                          "ms_per_step": round(ms_prof / profile_steps, 3),
                          "note": "per-kernel CUDA events on the library stream in a second "
                                  "timed pass of the same slab loop right after the timed "
                                  "region; value and ms_per_step come from the timed region, "
                                  "which runs without them (they cost about 6 % of the rate)"},
        "damage_pipes": {"exact_steps_per_slab": exact, "screened_steps_per_slab": screened,
                         "fp64_flops_per_exact_step": 610,
                         "fp64_achieved_gflops": round(fp64_gflops, 3),
                         "fp64_peak_gflops": 1250.0, "fp64_peak_kind": "nominal (no measured "
                         "FP64 peak on this pool)",
                         "fp64_frac": round(fp64_gflops / 1250.0, 7),
                         "note": "the update's time is set by the few points whose steps are "
                                 "plastic (C2: the four clamped corners), each a serial FP64 "
                                 "chain; every other step is proven elastic by the FP32 screen"},
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
        out["cpu_baseline"] = cpu_baseline(threads=os.cpu_count() or 1)
    if rank == 0 and not args.skip_variants:
        out["variants"] = run_variants(xt, args)
    if rank == 0:
        out["refactor_host"] = refactor_host(xt)
    slab.close()
    prob.close()
    return out


def refactor_host(xt, nfail=24):
    """A deletion event on the C2 rod (after the GPU measurements): the
    deletion surgery of nfail seeded elements (K -= their element matrices,
    disconnected nodes fixed, boundary conditions re-applied) and the ILUT
    refactor of the new K on the host, which the library pipelines over the
    host threads (serial-order ILUT timed beside it); then the device side:
    the new operator's upload (K, M and their node blocks) and the new
    factor's (upload, level schedule, and the register-sweep layout its
    first FP32 apply builds, net of a steady apply).  Host wall clock, the
    device synchronised."""
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
        alu, jlu, ju = xt.ilut(K, WORKLOAD["lfil"], WORKLOAD["droptol"])
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
        M = pr.M()
        pr.close()
        ones, eye = np.ones(K.n * 6), np.eye(6)
        xt.lib().xt_sync()
        t6 = time.perf_counter()
        sysm = xt.SpaceTimeSystem(K, M)
        xt.lib().xt_sync()
        t7 = time.perf_counter()
        sysm.set_ilu(alu, jlu, ju, group=3)
        sysm.lusol(eye, ones, fp32=True)  # builds the register-sweep layout
        t8 = time.perf_counter()
        sysm.lusol(eye, ones, fp32=True)  # a steady apply, with the same host copies
        t9 = time.perf_counter()
        sysm.close()
        return {"deleted_elements": nfail, "surgery_ms": round((t1 - t0) * 1e3, 1),
                "ilut_ms": round((t3 - t2) * 1e3, 1),
                "ilut_ms_one_thread": round((t5 - t4) * 1e3, 1),
                "operator_upload_ms": round((t7 - t6) * 1e3, 1),
                "factor_setup_ms": round(((t8 - t7) - (t9 - t8)) * 1e3, 1),
                "host_threads": os.cpu_count() or 1,
                "timer": "host wall clock, device synchronised",
                "scope": "deletion surgery + full ILUT(1e-4, 20) of the C2 K on the host; the "
                "new K and M uploaded with their node blocks; the factor uploaded, scheduled "
                "and laid out for the register sweep (net of a steady apply)"}
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
    batch's tuned restart length, ILU lanes per row and Gram-Schmidt
    passes, FP32 ILU, true residual <= 1e-8) through
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
    shares = batch.ilu_shares
    passes = batch.gs_passes
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
            "restart": kw["im"], "ilu_lanes_per_row": shares, "gram_schmidt_passes": passes,
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
    """The plain FP64 GPU GMRES on the same workload (the 3x denominator),
    CUDA events around up to 6 slabs after one untimed slab (about 2 s
    each)."""
    prob = make_problem(xt)
    slab = xt.SlabSolver(prob, make_config(xt, precision=0, seed=WORKLOAD["seed"]))
    slab.step()
    xt.lib().xt_sync()
    n = max(1, min(args.steps, 6))
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
    """The C2 slab more ways, timed like fp64_gpu (CUDA events around n
    slabs after one untimed slab): without the damage update (the solve,
    load and jump terms only; sequential loop); with the damage update at a
    reduced temporal resolution (16 points per load cycle, 1,600 per slab
    instead of 25,600; overlapped loop as the headline); and with the
    block-Jacobi ILUT of 4 and 8 row blocks in place of the ILUT of K (a
    different preconditioner from the reference's: more iterations, each
    block's triangular solves on SMs of their own)."""
    out = {}
    variants = (("no_damage", {"damage": 0, "overlap": 0}),
                ("reduced_nip", {"nipc": 16}),
                ("ilu_blocks_4", {"ilu_blocks": 4}),
                ("ilu_blocks_8", {"ilu_blocks": 8}))
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
                         "ilu_blocks": max(1, int(cfg.ilu_blocks)),
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
def workload_config(amp):
    """The workload definition both arms report as `config`."""
    return {"workload": "C2 prismatic rod 20x20x60 C3D8, 80,703 DOF x 6 temporal blocks",
            "nip": WORKLOAD["nipc"] * WORKLOAD["n1"],
            "ilut": [WORKLOAD["droptol"], WORKLOAD["lfil"]],
            "gmres_restart": WORKLOAD["im"], "gram_schmidt_passes": WORKLOAD["gs_passes"],
            "tol": WORKLOAD["tol"], "amplitude_mpa": amp,
            "l2": "inputs larger than L2 (operator+factor+basis >> 129 MB)",
            "parallelism": "replicas x1"}


class CpuSlab:
    """The reference's CPU path for the C2 slab loop, on the oracle (the C
    restatement of src/kronecker.f90, src/ilut.f and the damage kernel,
    src/kokkos_kernel.h): its inputs come from oracle/fem.py (the mesh,
    K, M, strain rows, boundary conditions and load restated in numpy) and
    the oracle's quadrature of the temporal integrals, so the GPU library is
    not loaded.

    One step is one slab of src/main3d.f90:609-937 in full except for the
    damage update, which runs on a stratified sample of the Gauss points
    over the slab's full 25,600 steps: stratum A is every point of the
    clamped layer (400 elements; it holds every plastic point of the slab,
    the four clamped corners), stratum B a seeded 1/sample_every of the
    other elements.  The update's full-slab time is tA + tB * (points of B
    in the rod / points of B sampled).  GMRES runs to the reference's
    convergence test (|rs| <= 1e-8 ||r0||, GMRES(200)) on the slab's real
    right-hand side, OpenMP over the rows of every amux pass and vector
    update and over the q independent lusol calls (bit-identical to the
    serial order); the damage update is OpenMP over the points, as
    src/cpu_damage.f90."""

    def __init__(self, threads, seed=0, sample_every=64):
        from oracle import fem
        from oracle import oracle as orc

        self.orc, self.threads = orc, threads
        w = WORKLOAD
        t0 = time.perf_counter()
        xyz, conn = fem.rod_mesh(w["nx"], w["ny"], w["nz"], w["lx"], w["ly"], w["lz"])
        K, M, (Nx, Ny, Nz) = fem.assemble(xyz, conn, w["E"], w["nu"], w["rho"])
        self.bc = fem.face_mask(xyz, 0, 0.0)
        self.K, self.M = fem.applybc(K, self.bc), fem.applybc(M, self.bc)
        self.amp = amplitude(seed)
        self.rext = fem.traction(xyz, conn, 0, w["lx"], 0, self.amp, w["ly"] * w["lz"])
        self.t_setup = time.perf_counter() - t0
        t0 = time.perf_counter()
        (self.alu, self.jlu, self.ju), ierr = orc.ilut(self.K, w["lfil"], w["droptol"])
        self.t_ilut = time.perf_counter() - t0
        if ierr != 0:
            raise RuntimeError(f"oracle ILUT ierr {ierr}")
        self.nn, self.ne, self.p = len(xyz), len(conn), 3 * len(xyz)
        xmin = xyz[conn - 1, 0].max(1)
        layer = np.flatnonzero(xmin <= w["lx"] / w["nx"] + 1e-9)
        rest = np.setdiff1d(np.arange(self.ne), layer)
        pick = np.sort(np.random.default_rng(seed).choice(rest, len(rest) // sample_every,
                                                          replace=False))
        self.strata = []
        for elems, weight in ((layer, 1.0), (pick, len(rest) / len(pick))):
            gps = (elems[:, None] * 8 + np.arange(8)).ravel()
            rows = (gps[:, None] * 8 + np.arange(8)).ravel()
            st = {k: np.zeros(len(gps) * 6) for k in orc.STATE_KEYS[:4]}
            st.update({k: np.zeros(len(gps)) for k in orc.STATE_KEYS[4:]})
            self.strata.append(dict(
                ne=len(elems), weight=weight, state=st,
                nodes=np.repeat(conn[elems], 8, axis=0).ravel().astype(np.int32),
                Nx=Nx[rows], Ny=Ny[rows], Nz=Nz[rows], ym=np.full(len(gps), w["E"]),
                nu=np.full(len(gps), w["nu"])))
        self.npts = 8 * (len(layer) + len(pick))
        self.disp = np.zeros(6 * self.p)
        self.bc6 = np.tile(self.bc, 6) == 1
        self.w = 2 * np.pi * w["freq"]
        self.dt = w["dt0"] * w["n1"]
        self.nip = w["nipc"] * w["n1"]
        self.tc = np.zeros(3)

    def step(self):
        orc = self.orc
        t_start = time.perf_counter()
        self.tc = self.tc[2] + np.arange(3) * self.dt / 2.0
        ck, cm, ckt, cmt, ck1, cm1 = orc.stcoeff_m_quad(self.tc[0], self.dt, self.w)
        fextc = orc.getfextc_m_quad(self.tc[0], self.w, self.dt)
        orc.set_threads(self.threads)
        try:
            f = np.concatenate([c * self.rext for c in fextc])
            f = orc.kronspgemv(ck1, cm1, 1.0, 1.0, self.K, self.M, self.disp, f)
            f[self.bc6] = 0.0
            disp, ierr, its, _ = orc.kronpgmres(ck + ckt, cm + cmt, self.K, self.M, self.alu,
                                                self.jlu, self.ju, f, im=WORKLOAD["im"],
                                                eps=WORKLOAD["tol"], maxits=4000)
        finally:
            orc.set_threads(1)
        if ierr != 0:
            raise RuntimeError(f"oracle GMRES ierr {ierr}")
        disp[self.bc6] = 0.0
        self.disp = disp
        t_solve = time.perf_counter() - t_start
        Nt = orc.nt_table(self.nip, self.tc, self.w)
        t_dmg = 0.0
        plastic = 0
        maxD = 0.0
        for s in self.strata:
            t0 = time.perf_counter()
            orc.damage(s["ne"], self.nn, self.nip, s["nodes"], s["Nx"], s["Ny"], s["Nz"], Nt,
                       disp, s["ym"], s["nu"], s["state"], nthreads=self.threads)
            t_dmg += (time.perf_counter() - t0) * s["weight"]
            plastic += int(np.count_nonzero(s["state"]["p"]))
            maxD = max(maxD, float(s["state"]["D"].max()))
        deletion = maxD >= WORKLOAD["Dc"]  # the deletion test over the sampled points
        return {"wall_s": time.perf_counter() - t_start, "slab_s": t_solve + t_dmg,
                "solve_s": t_solve, "damage_s": t_dmg, "its": its, "plastic_points": plastic,
                "deletion": bool(deletion)}

    def sample_text(self):
        a, b = self.strata
        return (f"each step one full C2 slab on {self.threads} host threads: oracle jump "
                f"term, GMRES(200) to the reference's test |rs| <= 1e-8 ||r0|| on the slab's "
                f"right-hand side, damage update over the full {self.nip} steps on a "
                f"stratified sample of {self.npts} of {8 * self.ne} Gauss points (all "
                f"{8 * a['ne']} points of the clamped layer, which hold every plastic point, "
                f"+ a seeded 1/{round(b['weight'])} of the other elements, time scaled by "
                f"stratum to all points); inputs from oracle/fem.py and the oracle's quadrature "
                f"(built without the GPU library)")


def cpu_baseline(threads, steps=1):
    """cpu_baseline of the GPU arm: `steps` slabs of CpuSlab on the host's
    cores, median projected slab time."""
    slab = CpuSlab(threads)
    recs = [slab.step() for _ in range(steps)]
    t = float(np.median([r["slab_s"] for r in recs]))
    return {"value": round(1.0 / t, 6), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": slab.sample_text(), "seconds_per_slab": round(t, 3),
            "solve_s": round(float(np.median([r["solve_s"] for r in recs])), 3),
            "damage_s_per_slab": round(float(np.median([r["damage_s"] for r in recs])), 3),
            "iterations_per_slab": float(np.mean([r["its"] for r in recs])),
            "plastic_points": recs[-1]["plastic_points"], "slabs": steps}


def run_reference(args, rank, world):
    """The reference arm: CpuSlab steps timed on rank 0 (other ranks exit
    without work).  ms_per_step is the measured wall time of a step (the
    work actually run); value is the projected full-slab rate of those
    steps (the damage update scaled from its sample by stratum)."""
    if rank != 0:
        return None
    threads = os.cpu_count() or 1
    t_run = time.perf_counter()
    slab = CpuSlab(threads)
    for _ in range(args.warmup):
        slab.step()
    recs = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        recs.append(slab.step())
    sec = time.perf_counter() - t0
    t_slab = float(np.median([r["slab_s"] for r in recs]))
    v = 1.0 / t_slab
    return {"impl": "reference", "metric": METRIC, "value": round(v, 6), "unit": UNIT,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(sec * 1e3 / args.steps, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp64", "data": "synthetic",
            "config": workload_config(slab.amp),
            "precision": "fp64 gmres (the reference's kronpgmres), fp64 damage",
            "cpu_baseline": {"value": round(v, 6), "unit": UNIT, "cores": threads,
                             "kind": "port", "sample": slab.sample_text()},
            "e2e": {"value": round(v, 6), "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "value_measured_steps": round(args.steps / sec, 6),
            "projected_slab_s": round(t_slab, 3),
            "solve_s": round(float(np.median([r["solve_s"] for r in recs])), 3),
            "damage_s_per_slab": round(float(np.median([r["damage_s"] for r in recs])), 3),
            "iterations_per_slab": float(np.mean([r["its"] for r in recs])),
            "plastic_points": recs[-1]["plastic_points"],
            "setup_s": {"mesh_assembly": round(slab.t_setup, 2), "ilut": round(slab.t_ilut, 2)},
            "wall_s": round(time.perf_counter() - t_run, 1)}


# ------------------------------------------------- other workloads (side runs)
def run_workload(args):
    """--workload c3|c5 (or any workload file): args.steps slabs of that
    workload's device slab loop at its full size, sequential (each slab's
    damage update before the next solve), host wall clock per slab with the
    device synchronised.  --predamage D seeds every Gauss point's damage at
    D and its stored energy just below the damage threshold (a specimen
    near the end of its fatigue life), so that elements reach Dc = 0.99
    within a few slabs.  Prints one JSON line with a record per slab.  Not
    the headline: bench.py without --workload measures C2."""
    import xtfem_gb300 as xt
    from xtfem_gb300 import workloads

    xt.lib().xt_init(int(os.environ.get("LOCAL_RANK", "0")))
    t0 = time.perf_counter()
    w = workloads.load(args.workload)
    cfg = w.slab
    if args.precision is not None:
        cfg.precision = args.precision
    cfg.overlap = 0
    nn, ne, nnz_k, _ = w.problem.sizes()
    s = xt.SlabSolver(w.problem, cfg)
    th = None
    if w.thermal is not None:
        w.thermal.precision = cfg.precision
        th = xt.ThermalSolver(w.problem, w.thermal)
        s.couple(th, **w.coupling)
    if args.predamage is not None:
        s.set_state(D=np.full(s.ngp, args.predamage), ws=np.full(s.ngp, 31.7))
    setup = time.perf_counter() - t0
    rows = []
    for _ in range(args.steps):
        xt.lib().xt_sync()
        t1 = time.perf_counter()
        st = s.step()
        xt.lib().xt_sync()
        rows.append({"slab": int(st["slab"]), "seconds": round(time.perf_counter() - t1, 3),
                     "its": int(st["its"]), "outer": int(st["outer"]),
                     "relres": float(st["relres"]), "ierr": int(st["ierr"]),
                     "deleted": int(st["deleted"]), "failed": int(st["nfailed"]),
                     "maxD": float(st["maxD"])})
    state = s.state()
    s.close()
    if th is not None:
        th.close()
    name = w.name
    w.close()
    return {"workload": name, "description": w.description, "nodes": nn, "elements": ne,
            "spatial_dofs": 3 * nn, "nnz_k": nnz_k, "precision": PRECISION_NAMES[cfg.precision],
            "predamage": args.predamage, "setup_s": round(setup, 2), "slabs": rows,
            "slab_s_mean": round(float(np.mean([r["seconds"] for r in rows])), 3),
            "deleted_elements": [int(e) for e in np.flatnonzero(state["elesta"] == 0) + 1],
            "timer": "host wall clock per slab, device synchronised"}


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
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-variants", action="store_true",
                    help="skip the no-damage and reduced-nip slab lines")
    ap.add_argument("--workload", default=None,
                    help="side run of another workload file (c3, c5, ...): --steps slabs at "
                         "full size, one JSON line with a record per slab")
    ap.add_argument("--predamage", type=float, default=None,
                    help="with --workload: seed D at this value and the stored energy just "
                         "below the damage threshold")
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
    if args.workload:
        out = run_workload(args) if rank == 0 else None
    elif args.impl == "reference":
        out = run_reference(args, rank, world)
    else:
        out = run_gpu(args, rank, world)
    if rank == 0 and out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
