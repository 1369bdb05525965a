"""Build the GB300 library (xtfem_gb300/libxtfem_gb300.so) in-tree.

Every translation unit is compiled in parallel with nvcc for sm_103a
(CUDA sources) or the host compiler (C++ sources), then linked into one
shared object that exports the C ABI of include/xtfem_gb300*.h.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT = HERE / "_build"
LIB = HERE / "libxtfem_gb300.so"
# debug build: host C++ under AddressSanitizer and UBSan, in its own folder
# and file (load it with XTFEM_LIB and the sanitizer runtimes preloaded)
OUT_SAN = HERE / "_build_san"
LIB_SAN = HERE / "libxtfem_gb300_san.so"
SAN = ["-fsanitize=address", "-fsanitize=undefined", "-fno-omit-frame-pointer"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# per-file extra flags: the damage kernel keeps the reference's operation
# order in its exact FP64 path, so multiply-adds are not contracted there
EXTRA = {"dev_damage.cu": ["-fmad=false"]}


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build xtfem_gb300")


def _sources():
    cu = sorted(CSRC.glob("*.cu"))
    cpp = sorted(CSRC.glob("*.cpp"))
    return cu, cpp


def _needs(obj: Path, deps) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, jobs: int | None = None, sanitize: bool = False) -> Path:
    nvcc = _nvcc()
    out_dir, lib = (OUT_SAN, LIB_SAN) if sanitize else (OUT, LIB)
    host_san = [f for s in SAN for f in ("-Xcompiler", s)] if sanitize else []
    out_dir.mkdir(exist_ok=True)
    cu, cpp = _sources()
    headers = (list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) +
               list((HERE.parent / "include").glob("*.h")))
    cmds = []
    objs = []
    for src in cu:
        obj = out_dir / (src.name + ".o")
        objs.append(obj)
        if _needs(obj, [src, *headers]):
            cmds.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-Xcompiler", "-ffp-contract=off",
                         "--expt-relaxed-constexpr", *EXTRA.get(src.name, []),
                         "-c", str(src), "-o", str(obj)])
    for src in cpp:
        obj = out_dir / (src.name + ".o")
        objs.append(obj)
        if _needs(obj, [src, *headers]):
            # host code: no FMA contraction, so x86 and Arm hosts assemble
            # bit-identical K and M
            cmds.append([nvcc, "-O1" if sanitize else "-O2", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-Xcompiler", "-ffp-contract=off", *host_san, "-c", str(src), "-o",
                         str(obj)])
    jobs = jobs or max(1, min(len(cmds), os.cpu_count() or 4))

    def run(cmd):
        p = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, p

    failed = []
    with cf.ThreadPoolExecutor(jobs) as ex:
        for cmd, p in ex.map(run, cmds):
            if verbose or p.returncode:
                sys.stderr.write(" ".join(cmd) + "\n" + p.stdout + p.stderr)
            if p.returncode:
                failed.append(cmd[-3])
    if failed:
        raise RuntimeError(f"compilation failed: {failed}")
    if cmds or not lib.exists():
        link = [nvcc, *ARCH, "-shared", "-o", str(lib), *map(str, objs), "-lcudart", *host_san]
        p = subprocess.run(link, capture_output=True, text=True)
        if p.returncode:
            raise RuntimeError("link failed:\n" + p.stdout + p.stderr)
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, sanitize="--sanitize" in sys.argv))
