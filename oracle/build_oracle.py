"""Build recipe of the oracle (test infrastructure).

Compiles oracle/oracle.cpp into oracle/_build/liboracle.so with g++ -O2 and
OpenMP (the reference's Release flags, CMakeLists.txt:159).  When the
reference source tree is present, also compiles the reference's own
dependency-free dilution-iterator sources (src/dilution-iterator.cpp and
main/test-iterator.cpp) into oracle/_ref/test-dilution-iterator, used only to
cross-check the oracle's dilution enumeration.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"
LIB = OUT / "liboracle.so"
REF_OUT = HERE / "_ref"
# The reference source tree: $SLAPH_REFERENCE_DIR, else a directory named
# "reference" beside this repository's root.
REFERENCE = Path(os.environ.get("SLAPH_REFERENCE_DIR", str(HERE.parent.parent / "reference")))


def build() -> Path:
    OUT.mkdir(exist_ok=True)
    srcs = [HERE / "oracle.cpp"]
    deps = srcs + [HERE / "oracle.h", HERE.parent / "include" / "slaph_gb300.h"]
    if not LIB.exists() or LIB.stat().st_mtime < max(p.stat().st_mtime for p in deps):
        tmp = LIB.with_suffix(".so.tmp")
        cmd = ["g++", "-std=c++17", "-O2", "-fopenmp", "-fPIC", "-shared", "-o", str(tmp),
               *map(str, srcs)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


def build_ref() -> Path | None:
    """Reference dilution-iterator test program, if the reference is present."""
    src_dir = REFERENCE / "src"
    if not (src_dir / "dilution-iterator.cpp").exists():
        return None
    REF_OUT.mkdir(exist_ok=True)
    exe = REF_OUT / "test-dilution-iterator"
    if not exe.exists():
        cmd = ["g++", "-std=c++11", "-O2", "-I", str(REFERENCE / "include"),
               str(src_dir / "dilution-iterator.cpp"), str(REFERENCE / "main" / "test-iterator.cpp"),
               "-o", str(exe)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            print(f"reference dilution iterator did not build:\n{r.stderr}", file=sys.stderr)
            return None
    return exe


if __name__ == "__main__":
    print(build())
    print(build_ref())
