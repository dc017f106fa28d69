"""Build recipe for libbale_gb300.so (CUDA for sm_103a + host C), in-tree.

    python bale_old_gb300/build.py          # incremental
    python bale_old_gb300/build.py --force  # rebuild everything

(run as a script: importing the package itself requires the built library)

Every ``csrc/*.cu`` file is compiled by nvcc for sm_103a only, every
``csrc/host/*.c`` file by the host C compiler, in parallel, into
``bale_old_gb300/_build/``; the objects are linked into
``bale_old_gb300/libbale_gb300.so`` with the CUDA runtime linked statically,
so the library needs only the NVIDIA driver at run time.
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
OBJDIR = PKG / "_build"
LIB = PKG / "libbale_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
    "-I", str(INCLUDE), "-I", str(CSRC),
]
CC_FLAGS = ["-O3", "-std=gnu11", "-fPIC", "-fvisibility=hidden", "-Wall", "-Wextra", "-ffp-contract=off",
            "-I", str(INCLUDE)]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found (set NVCC or put it on PATH)")


def _cc() -> str:
    return os.environ.get("CC") or shutil.which("gcc") or "cc"


def _headers() -> list[Path]:
    return sorted(INCLUDE.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("**/*.h"))


def _stale(obj: Path, src: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(p.stat().st_mtime > t for p in [src, *deps])


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile and link libbale_gb300.so; returns its path."""
    OBJDIR.mkdir(exist_ok=True)
    nvcc, cc = _nvcc(), _cc()
    deps = _headers()
    jobs: list[tuple[Path, list[str]]] = []
    objs: list[Path] = []
    for src in sorted(CSRC.glob("*.cu")):
        obj = OBJDIR / (src.stem + ".o")
        objs.append(obj)
        if force or _stale(obj, src, deps):
            jobs.append((obj, [nvcc, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]))
    for src in sorted((CSRC / "host").glob("*.c")):
        obj = OBJDIR / (src.stem + "_host.o")
        objs.append(obj)
        if force or _stale(obj, src, deps):
            jobs.append((obj, [cc, *CC_FLAGS, "-c", str(src), "-o", str(obj)]))
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for (obj, cmd), _ in zip(jobs, ex.map(lambda j: _run(j[1]), jobs)):
                if verbose:
                    print("built", obj.name)
    if force or jobs or not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(".so.tmp")
        _run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs),
              "-lpthread", "-lm"])
        os.replace(tmp, LIB)
    return LIB


def main(argv: list[str] | None = None) -> int:
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args(argv)
    print(build(force=a.force, verbose=a.verbose))
    return 0


if __name__ == "__main__":
    sys.exit(main())
