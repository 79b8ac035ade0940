"""Build the native library ``_build/libacg.so`` for sm_103a, and the tools
``_build/acg_main`` (drop-in for the reference program) and
``_build/acg_prob2bin`` (its CSV-to-binary converter).

Every ``csrc/*.cu`` is compiled by nvcc for ``sm_103a`` only, every
``csrc/*.cpp`` by the host compiler; translation units compile in parallel and
are rebuilt only when a source or header is newer than its object.  The link
uses nvcc with the static CUDA runtime, so the library loads on a machine
without a GPU (its entry points then return ACG_ERR_CUDA).
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
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB = BUILD / "libacg.so"

ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found; the CUDA 13 toolkit is required")
    return cand


def _cxx() -> str:
    return os.environ.get("CXX", "g++")


def _headers() -> list[Path]:
    return sorted(list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h")))


def _stale(obj: Path, src: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(p.stat().st_mtime > t for p in [src, *deps])


def _compile(src: Path, verbose: bool, out: Path = BUILD, defines: tuple = ()) -> Path:
    obj = out / (src.name + ".o")
    if src.suffix == ".cu":
        cmd = [
            _nvcc(), ARCH, "-lineinfo", "-O3", "-std=c++20", "-c", str(src), "-o", str(obj),
            "-Xcompiler", "-fPIC", "-Xcompiler", "-fopenmp", "--expt-relaxed-constexpr",
            "-I", str(INCLUDE), "-I", str(CSRC), *[f"-D{d}" for d in defines],
        ]
        if os.environ.get("ACG_PTXAS_VERBOSE"):
            cmd += ["-Xptxas", "-v"]
    else:
        cmd = [
            _cxx(), "-std=c++17", "-O3", "-fPIC", "-fopenmp", "-Wall", "-Wno-unused-function",
            "-c", str(src), "-o", str(obj), "-I", str(INCLUDE), "-I", str(CSRC),
            "-I", "/usr/local/cuda/include",
        ]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {src.name}\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr:
        print(r.stderr, file=sys.stderr)
    return obj


def build(verbose: bool = False, force: bool = False, out_dir: Path | None = None,
          defines: tuple = ()) -> Path:
    """Compile and link ``libacg.so``; return its path.

    ``out_dir`` and ``defines`` (``NAME=VALUE`` preprocessor definitions for the
    CUDA sources) build a variant elsewhere, e.g. to compare tuning constants;
    load one with the environment variable ``ACG_LIBRARY``."""
    out = Path(out_dir) if out_dir else BUILD
    lib = out / "libacg.so"
    out.mkdir(parents=True, exist_ok=True)
    srcs = sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))
    deps = _headers()
    todo = [s for s in srcs if force or _stale(out / (s.name + ".o"), s, deps)]
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(todo)))) as ex:
        list(ex.map(lambda s: _compile(s, verbose, out, tuple(defines)), todo))
    objs = [out / (s.name + ".o") for s in srcs]
    if force or todo or not lib.exists() or any(o.stat().st_mtime > lib.stat().st_mtime for o in objs):
        tmp = out / "libacg.so.tmp"
        cmd = [_nvcc(), ARCH, "-shared", "-o", str(tmp), *map(str, objs),
               "-Xcompiler", "-fopenmp", "-lgomp", "-ldl", "-cudart", "static"]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, lib)
    _build_tools(out, lib, verbose, force)
    return lib


CLI = PKG / "cli"
TOOLS = {"acg_main": "acg_main.cpp", "acg_prob2bin": "acg_prob2bin.cpp"}


def _build_tools(out: Path, lib: Path, verbose: bool, force: bool) -> None:
    """The command-line tools next to the library (rpath $ORIGIN): ``acg_main``
    (drop-in for the reference program) and ``acg_prob2bin``."""
    for name, src in TOOLS.items():
        exe, srcp = out / name, CLI / src
        if not force and exe.exists() and exe.stat().st_mtime > max(
                srcp.stat().st_mtime, lib.stat().st_mtime):
            continue
        cmd = [_nvcc(), ARCH, "-O2", "-std=c++17", "-x", "cu", str(srcp), "-o", str(exe),
               "-I", str(INCLUDE), "-L", str(out), "-lacg", "-Xlinker", "-rpath=$ORIGIN",
               "-Xcompiler", "-fopenmp", "-cudart", "static"]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"build of {name} failed\n{r.stdout}\n{r.stderr}")


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
