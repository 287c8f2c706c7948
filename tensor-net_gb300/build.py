"""Build libtnmps (the CUDA kernels + C ABI) in-tree for sm_103a.

Produces ``tensor-net_gb300/lib/libtnmps.so`` (loaded through ctypes) and
``tensor-net_gb300/lib/libtnmps.a`` (for a Rust/C host that links statically).
Translation units compile in parallel; a rebuild happens only when a source,
header or this file is newer than the shared library.
"""
from __future__ import annotations

import os
import pathlib
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = pathlib.Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
LIBDIR = PKG / "lib"
OBJDIR = PKG / "_build"
SO = LIBDIR / "libtnmps.so"
STATIC = LIBDIR / "libtnmps.a"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -ffp-contract=off: host arithmetic (the input generator) gives the same bits
# on x86-64 and on aarch64, where gcc would otherwise fuse a*b + c into FMAs.
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          f"-I{INCLUDE}", f"-I{CSRC}"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and pathlib.Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libtnmps")


def sources():
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _stale() -> bool:
    if not SO.exists() or not STATIC.exists():
        return True
    t = SO.stat().st_mtime
    deps = sources() + sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + \
        sorted(INCLUDE.glob("*.h")) + [pathlib.Path(__file__)]
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> pathlib.Path:
    """Compile every translation unit for sm_103a and link libtnmps.{so,a}."""
    if not force and not _stale():
        return SO
    nvcc = _nvcc()
    LIBDIR.mkdir(exist_ok=True)
    OBJDIR.mkdir(exist_ok=True)
    jobs = []
    for src in sources():
        obj = OBJDIR / (src.name + ".o")
        cmd = [nvcc, *ARCH, *COMMON, "-c", str(src), "-o", str(obj)]
        if src.suffix == ".cu":
            cmd += ["-Xptxas", "-v"] if verbose else []
        jobs.append((src, obj, cmd))

    def run(job):
        src, obj, cmd = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        objs = list(ex.map(run, jobs))
    tmp_so = SO.with_suffix(".so.tmp")
    r = subprocess.run([nvcc, *ARCH, "-shared", "-o", str(tmp_so), *map(str, objs)],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp_so, SO)
    if STATIC.exists():
        STATIC.unlink()
    r = subprocess.run([nvcc, *ARCH, "-lib", "-o", str(STATIC), *map(str, objs)],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"static archive failed:\n{r.stdout}\n{r.stderr}")
    os.utime(SO)
    return SO


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
