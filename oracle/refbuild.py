"""Build recipe of the reference oracle (test infrastructure only).

Compiles the reference's own MEX sources unmodified, from where they lie
under the reference checkout, against the project's fake MATLAB runtime
(oracle/refshim) and numpy's bundled ILP64 OpenBLAS:

    g++ -std=c++17 -O2 -fPIC -shared -fopenmp -DMATLAB_MEX_FILE -DQS_SKIP_MPFR
        -I oracle/refshim -I <reference>/Source <reference>/Source/<name>.cc
        -o oracle/_ref/<name>.so -loracle/_ref/libfakemx.so -l<openblas64>

QS_SKIP_MPFR is the reference's own switch for building without MPFR/GMP
headers (its CG coefficients are then computed in double precision).
Outputs go to oracle/_ref/ only (git-ignored).  Nothing here runs on the GPU
box: the reference checkout is not there.

    python -m oracle.refbuild [--source=<reference>/Source] [names...]
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SHIM = HERE / "refshim"
OUT = HERE / "_ref"
# Where the reference's Source/ directory is: QS_REFERENCE_SOURCE, a
# --source=PATH argument, or else a checkout named "reference" beside this
# repository's root.
REF_SRC = Path(os.environ.get("QS_REFERENCE_SOURCE") or (HERE.parent.parent / "reference" / "Source"))
DEFAULT = ("contractQS", "permuteQS", "eigQS", "svdQS", "orthoQS", "getIdentityQS", "plusQS")


def reference_present() -> bool:
    return (REF_SRC / "contractQS.cc").exists()


def openblas() -> Path:
    import numpy
    libs = Path(numpy.__file__).resolve().parent.parent / "numpy.libs"
    c = sorted(glob.glob(str(libs / "libscipy_openblas64_*.so")))
    if not c:
        raise RuntimeError(f"numpy's bundled OpenBLAS (ILP64) not found under {libs}")
    return Path(c[0])


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("failed: " + " ".join(cmd) + "\n" + r.stderr[-4000:])


def build_fakemx(force=False) -> Path:
    OUT.mkdir(parents=True, exist_ok=True)
    so = OUT / "libfakemx.so"
    src = SHIM / "fakemx.cpp"
    deps = [src] + list(SHIM.glob("*.h"))
    if force or not so.exists() or so.stat().st_mtime < max(d.stat().st_mtime for d in deps):
        ob = openblas()
        _run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", f"-I{SHIM}", str(src), "-o", str(so),
              f"-L{ob.parent}", f"-l:{ob.name}", f"-Wl,-rpath,{ob.parent}"])
    return so


def build_one(name: str, force=False) -> Path:
    so = OUT / f"{name}.so"
    src = REF_SRC / f"{name}.cc"
    if not force and so.exists() and so.stat().st_mtime >= max(src.stat().st_mtime,
                                                              (OUT / "libfakemx.so").stat().st_mtime):
        return so
    ob = openblas()
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-fopenmp", "-w",
           "-DMATLAB_MEX_FILE", "-DQS_SKIP_MPFR", f"-I{SHIM}", f"-I{REF_SRC}", str(src), "-o", str(so),
           f"-L{OUT}", "-lfakemx", f"-L{ob.parent}", f"-l:{ob.name}",
           "-Wl,-rpath,$ORIGIN", f"-Wl,-rpath,{ob.parent}"]
    _run(cmd)
    return so


def build(names=DEFAULT, force=False, jobs=None) -> list[Path]:
    if not reference_present():
        raise RuntimeError(f"reference sources not found at {REF_SRC}")
    build_fakemx(force)
    jobs = jobs or min(len(names), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        return list(ex.map(lambda n: build_one(n, force), names))


if __name__ == "__main__":
    for a in sys.argv[1:]:
        if a.startswith("--source="):
            REF_SRC = Path(a.split("=", 1)[1])
    names = tuple(a for a in sys.argv[1:] if not a.startswith("-")) or DEFAULT
    for p in build(names, force="--force" in sys.argv):
        print(p)
