"""In-tree build of libqsgpu.so (CUDA for sm_103a + host C++), no cmake.

Each translation unit under ``csrc/`` is compiled in parallel with nvcc for
``-gencode arch=compute_103a,code=sm_103a``; objects and the shared library go
to ``qspace_gb300/_lib/`` (git-ignored).  Rebuilds only what changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "_lib"
OBJDIR = LIBDIR / "obj"
LIBNAME = "libqsgpu.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
          f"-I{INCLUDE}"]
CUFLAGS = ARCH + ["-lineinfo", "--expt-relaxed-constexpr"]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(p).exists():
        raise RuntimeError("nvcc not found (CUDA 13 toolkit required)")
    return p


def lib_path() -> Path:
    return LIBDIR / LIBNAME


def _headers_mtime() -> float:
    hs = list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))
    return max((h.stat().st_mtime for h in hs), default=0.0)


def _compile(src: Path, obj: Path, extra: list[str]) -> tuple[Path, str]:
    cmd = [nvcc()] + COMMON + (CUFLAGS if src.suffix == ".cu" else []) + extra + \
        ["-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(verbose: bool = False, force: bool = False, jobs: int | None = None,
          extra: list[str] | None = None) -> Path:
    """Compile every CUDA/C++ source of the library and link libqsgpu.so."""
    extra = list(extra or [])
    OBJDIR.mkdir(parents=True, exist_ok=True)
    srcs = sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))
    hm = _headers_mtime()
    todo = []
    objs = []
    for s in srcs:
        o = OBJDIR / (s.name + ".o")
        objs.append(o)
        if force or not o.exists() or o.stat().st_mtime < max(s.stat().st_mtime, hm):
            todo.append((s, o))
    jobs = jobs or min(len(todo) or 1, os.cpu_count() or 4)
    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
            futs = [ex.submit(_compile, s, o, extra) for s, o in todo]
            for f in futs:
                obj, err = f.result()
                if verbose and err.strip():
                    print(err)
    lib = lib_path()
    if force or todo or not lib.exists():
        cmd = [nvcc()] + ARCH + ["-shared", "-o", str(lib)] + [str(o) for o in objs] + \
            ["-lcusolver", "-lcublas"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return lib


if __name__ == "__main__":
    import sys
    print(build(verbose=True, force="--force" in sys.argv))
