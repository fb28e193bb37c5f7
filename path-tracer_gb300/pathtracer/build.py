"""Build the native libraries in-tree.

Outputs (git-ignored):
  path-tracer_gb300/_build/libpt.so     CUDA kernels + C ABI (include/pt.h, include/pt_world.h)
  path-tracer_gb300/_build/pt-render    headless `render` command line (headless.rs flags)
  oracle/_build/liboracle.so            CPU oracle (test infrastructure only)

Device code targets sm_103a only and is compiled with IEEE-exact float
semantics (-fmad=false -prec-div=true -prec-sqrt=true -ftz=false); host code
with -ffp-contract=off.  Both are required for the kernels to reproduce the
oracle's bits.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent.parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
ORACLE = ROOT / "oracle"
ORACLE_OUT = ORACLE / "_build"
INCLUDE = ROOT / "include"

NVCC = os.environ.get("NVCC", "nvcc")
CXX = os.environ.get("CXX", "g++")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-lineinfo", "-O3", "-std=c++17", "--expt-relaxed-constexpr",
    "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
    "-Xcudafe", "--diag_suppress=177",
]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function"]
# extra device-compiler flags (e.g. launch-shape -D overrides for tuning sweeps)
NVCC_FLAGS += os.environ.get("PT_EXTRA_NVCC_FLAGS", "").split()

LIB = OUT / "libpt.so"
CLI = OUT / "pt-render"
ORACLE_LIB = ORACLE_OUT / "liboracle.so"


def _headers(directory: Path) -> list[Path]:
    return sorted(list(directory.glob("*.h")) + list(directory.glob("*.cuh")))


def _stale(target: Path, sources: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources)


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + proc.stdout + proc.stderr)
        raise RuntimeError(f"build step failed: {cmd[0]} {cmd[-1]}")


def _compile(src: Path, headers: list[Path]) -> Path:
    obj = OUT / (src.name + ".o")
    if not _stale(obj, [src, *headers]):
        return obj
    if src.suffix == ".cu":
        _run([NVCC, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)])
    else:
        _run([CXX, *CXX_FLAGS, "-c", str(src), "-o", str(obj)])
    return obj


def build(verbose: bool = False) -> dict[str, Path]:
    OUT.mkdir(parents=True, exist_ok=True)
    ORACLE_OUT.mkdir(parents=True, exist_ok=True)
    headers = _headers(CSRC) + _headers(INCLUDE)
    lib_sources = sorted(p for p in list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")) if p.name != "pt_render_main.cpp")
    with ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as pool:
        objs_f = [pool.submit(_compile, s, headers) for s in lib_sources]
        oracle_src = [ORACLE / "trace_oracle.cpp"]
        oracle_headers = [ORACLE / "oracle.h", CSRC / "pt_fmath.h", INCLUDE / "pt.h"]
        oracle_f = None
        if _stale(ORACLE_LIB, oracle_src + oracle_headers):
            oracle_f = pool.submit(_run, [CXX, *CXX_FLAGS, "-fopenmp", "-shared", *map(str, oracle_src),
                                          "-o", str(ORACLE_LIB)])
        objs = [f.result() for f in objs_f]
        if oracle_f is not None:
            oracle_f.result()
    if _stale(LIB, objs):
        _run([NVCC, *ARCH, "-shared", "-Xcompiler", "-fPIC", *map(str, objs), "-o", str(LIB)])
    cli_main = CSRC / "pt_render_main.cpp"
    if cli_main.exists() and _stale(CLI, [cli_main, LIB, *headers]):
        _run([CXX, *CXX_FLAGS, str(cli_main), "-o", str(CLI), f"-L{OUT}", "-lpt", f"-Wl,-rpath,{OUT}"])
    if verbose:
        print(f"built {LIB}, {ORACLE_LIB}")
    return {"lib": LIB, "oracle": ORACLE_LIB, "cli": CLI}


if __name__ == "__main__":
    build(verbose=True)
