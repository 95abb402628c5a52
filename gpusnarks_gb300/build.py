"""Build the native library libgpusnarks_gb300.so in-tree.

Every CUDA translation unit under csrc/ is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``) by nvcc, in parallel, into
gpusnarks_gb300/_build/, then linked into gpusnarks_gb300/_lib/.  Objects
are rebuilt when their source or any header in csrc/ or include/ is newer,
or when the build-time options below change.

Build-time options (environment variables, passed to nvcc as -D defines):
  GSN_MONT_SCHEDULE  Montgomery product schedule of the multi-limb fields:
                     1 even/odd accumulators (default), 0 row chains.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess

PKG = pathlib.Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIBDIR = PKG / "_lib"
LIBNAME = "libgpusnarks_gb300.so"
LIB = LIBDIR / LIBNAME

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              f"-I{CSRC}", f"-I{INCLUDE}"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and pathlib.Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build gpusnarks_gb300")


def sources() -> list[pathlib.Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _headers_mtime() -> float:
    hs = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    return max((h.stat().st_mtime for h in hs), default=0.0)


OPTIONS = ("GSN_MONT_SCHEDULE",)


def _defines() -> list[str]:
    out = []
    for name in OPTIONS:
        v = os.environ.get(name)
        if v:
            if not v.isdigit():
                raise ValueError(f"{name} must be a number, got {v!r}")
            out.append(f"-D{name}={v}")
    return out


def _compile(src: pathlib.Path, obj: pathlib.Path, verbose: bool) -> str:
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *_defines(), "-c", str(src), "-o", str(obj)]
    if src.suffix == ".cpp":
        cmd[1:1] = ["-x", "cu"]
    if verbose:
        cmd.append("-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stdout}\n{res.stderr}")
    return res.stderr


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> pathlib.Path:
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    stamp = BUILD / "options.txt"
    opts = " ".join(_defines())
    if not stamp.exists() or stamp.read_text() != opts:
        force = True
    hdr_t = _headers_mtime()
    todo = []
    objs = []
    for src in sources():
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if force or not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, hdr_t):
            todo.append((src, obj))
    if todo:
        workers = jobs or min(len(todo), os.cpu_count() or 4)
        with cf.ThreadPoolExecutor(max_workers=workers) as ex:
            futs = {ex.submit(_compile, s, o, verbose): s for s, o in todo}
            for f in cf.as_completed(futs):
                out = f.result()
                if verbose and out:
                    print(f"== {futs[f].name}\n{out}")
    if todo or not LIB.exists():
        tmp = LIBDIR / (LIBNAME + ".tmp")
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lpthread"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
        os.replace(tmp, LIB)
    stamp.write_text(opts)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
