"""Build recipe of the GB300 GGEM library (libggem_gb300.so).

Compiles every translation unit of ``csrc/`` for sm_103a in parallel with
nvcc (device code) and links one shared library with the CUDA runtime linked
statically, so the library loads on its own and exports only the C ABI of
``include/ggem_gb300.h`` and ``include/ggem_workloads.h``.

    python -m ggem_gb300.build          (from copss-hydrodynamics-private_gb300/)
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = ROOT / "csrc"
INCLUDE = ROOT.parent / "include"
OUT_DIR = PKG / "_lib"
LIB = OUT_DIR / "libggem_gb300.so"
OBJ_DIR = ROOT / "_build"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr", "-Xptxas", "-O3"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the GGEM library needs the CUDA toolkit")


def sources():
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _compile(src: Path, verbose_ptxas: bool) -> Path:
    obj = OBJ_DIR / (src.name + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, f"-I{INCLUDE}", f"-I{CSRC}", "-c", str(src), "-o", str(obj)]
    if src.suffix == ".cpp":
        cmd = [nvcc(), "-x", "c++", *NVCC_FLAGS, f"-I{INCLUDE}", f"-I{CSRC}", "-c", str(src),
               "-o", str(obj)]
    elif verbose_ptxas:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
    if verbose_ptxas and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    deps = (list(sources()) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h")) +
            list((ROOT / "cpp").glob("*")) + [Path(__file__)])
    tools = [OUT_DIR / s.stem for s in (ROOT / "cpp").glob("*.cpp")]
    return all(x.exists() for x in tools) and all(d.stat().st_mtime <= t for d in deps)


def build(force: bool = False, verbose_ptxas: bool = False) -> Path:
    if not force and up_to_date():
        return LIB
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    OUT_DIR.mkdir(parents=True, exist_ok=True)
    srcs = sources()
    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose_ptxas), srcs))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-cudart", "static",
           "-lpthread", "-ldl", "-lrt"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    build_tools()
    return LIB


CPP = ROOT / "cpp"


def build_tools() -> list:
    """C++ host programs over the C ABI (cpp/*.cpp), linked to the library
    with an $ORIGIN rpath so they run from ggem_gb300/_lib/."""
    outs = []
    for src in sorted(CPP.glob("*.cpp")):
        exe = OUT_DIR / src.stem
        cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", f"-I{INCLUDE}", f"-I{CPP}",
               str(src), "-o", str(exe), f"-L{OUT_DIR}", "-lggem_gb300",
               "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"g++ failed on {src.name}:\n{r.stdout}\n{r.stderr}")
        outs.append(exe)
    return outs


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
