"""In-tree build of the native library ``libgpudsm.so`` (sm_103a kernels + C ABI)
and of the ``gpu_DSM`` command-line driver.

nvcc compiles each translation unit in parallel with
``-gencode arch=compute_103a,code=sm_103a``.  ``-fmad=false`` keeps nvcc from
contracting a*b+c into FMA behind the code's back: the kMC decision arithmetic
is written with explicit ``__fmaf_rn`` where a fused multiply-add is meant, so
that a host restatement of the same operations gives identical bits.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libgpudsm.so"
# debug build with the step kernel's phase clocks (gpu_dsm_gb300/phases.py)
BUILD_PHASES = PKG / "_build_phases"
LIB_PHASES = PKG / "libgpudsm_phases.so"
CLI = PKG / "gpu_DSM"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-ffp-contract=off", "-I", str(ROOT / "include")]
SOURCES = ["dsm_kernels.cu", "dsm_host.cu", "dsm_compat.cu", "dsm_noalloc.cu", "dsm_serve.cu", "dsm_distr.cu", "dsm_gex.cpp",
           "dsm_checkpoint.cu", "dsm_refapi.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout)


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False, phases: bool = False) -> Path:
    """Compile libgpudsm.so and gpu_DSM if any source is newer than them.
    phases=True builds libgpudsm_phases.so instead: the same sources with the
    step kernel's phase clocks (-DDSM_PHASE_CLOCKS), in a build folder of its
    own."""
    bdir, lib = (BUILD_PHASES, LIB_PHASES) if phases else (BUILD, LIB)
    flags = NVFLAGS + (["-DDSM_PHASE_CLOCKS"] if phases else [])
    bdir.mkdir(exist_ok=True)
    nv = nvcc()
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h"))
    objs = []
    jobs = []
    for src in SOURCES:
        s = CSRC / src
        o = bdir / (s.stem + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nv, *ARCH, *flags, "-c", str(s), "-o", str(o)])
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        list(ex.map(_run, jobs))
    if force or jobs or _stale(lib, objs):
        _run([nv, *ARCH, "-shared", "-cudart", "static", "-o", str(lib), *map(str, objs)])
    if phases:
        return lib
    cli_src = CSRC / "cli_main.cpp"
    if cli_src.exists() and (force or _stale(CLI, [cli_src, LIB])):
        _run([nv, *ARCH, "-O2", "-std=c++17", "-I", str(ROOT / "include"), str(cli_src), "-o", str(CLI),
              "-L", str(PKG), "-lgpudsm", "-Xlinker", "-rpath", "-Xlinker", "$ORIGIN"])
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
