"""Build recipe of the engine library (libslaph_gb300.so).

Host C++ translation units are compiled with g++, CUDA translation units with
nvcc for sm_103a only, in parallel, and linked into one shared library that
lives next to this file (in-tree, so the loaded .so is the one from this
checkout).  Object files go to ``slaph-contractions_gb300/_build``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
ROOT = PKG_DIR.parent
CSRC = ROOT / "csrc"
BUILD = ROOT / "_build"
LIB = PKG_DIR / "libslaph_gb300.so"
REPO = ROOT.parent

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
CXXFLAGS = ["-std=c++17", "-O2", "-fPIC", "-Wall", "-Wextra", "-Wno-unused-parameter"]
NVCCFLAGS = ["-std=c++17", "-O3", ARCH, "-lineinfo", "-Xcompiler", "-fPIC",
             "--expt-relaxed-constexpr", "-Xptxas=-v"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the engine")


def _sources():
    cpp = sorted((CSRC / "host").glob("*.cpp"))
    cu = sorted((CSRC / "kernels").glob("*.cu")) + sorted((CSRC / "host").glob("*.cu"))
    return cpp, cu


def _headers():
    hs = list((CSRC).rglob("*.hpp")) + list((CSRC).rglob("*.cuh")) + list((REPO / "include").glob("*.h"))
    return hs


def _stale(obj: Path, src: Path, newest_header: float) -> bool:
    if not obj.exists():
        return True
    m = obj.stat().st_mtime
    return m < src.stat().st_mtime or m < newest_header


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    """Compile (incrementally) and link libslaph_gb300.so; returns its path."""
    nvcc = _nvcc()
    BUILD.mkdir(parents=True, exist_ok=True)
    cpp, cu = _sources()
    hdr_m = max((h.stat().st_mtime for h in _headers()), default=0.0)
    cuda_inc = str(Path(nvcc).resolve().parent.parent / "include")
    cmds = []
    objs = []
    for s in cpp:
        o = BUILD / (s.stem + ".cpp.o")
        objs.append(o)
        if _stale(o, s, hdr_m):
            cmds.append((["g++", *CXXFLAGS, f"-I{cuda_inc}", "-c", str(s), "-o", str(o)], s))
    for s in cu:
        o = BUILD / (s.stem + ".cu.o")
        objs.append(o)
        if _stale(o, s, hdr_m):
            cmds.append(([nvcc, *NVCCFLAGS, "-c", str(s), "-o", str(o)], s))

    def run(cmd_src):
        cmd, src = cmd_src
        r = subprocess.run(cmd, capture_output=True, text=True)
        return src, r

    logs = []
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        for src, r in ex.map(run, cmds):
            logs.append((src, r))
            if r.returncode != 0:
                raise RuntimeError(f"compilation of {src.name} failed:\n{r.stdout}\n{r.stderr}")
            if verbose and (r.stdout or r.stderr):
                print(f"--- {src.name}\n{r.stdout}{r.stderr}")
    lib_m = LIB.stat().st_mtime if LIB.exists() else -1.0
    if cmds or lib_m < max(o.stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(".so.tmp")
        # No -lcuda: driver entry points are fetched through the runtime, so the
        # library also loads on machines without a driver (for CPU-only tests).
        link = [nvcc, ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
        r = subprocess.run(link, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    (BUILD / "ptxas.log").write_text(
        "".join(f"--- {s.name}\n{r.stderr}" for s, r in logs if s.suffix == ".cu"))
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
