"""Build recipe for the oracle (test infrastructure only).

* ``build_oracle()`` compiles oracle/oracle.cpp (the CPU restatement) into
  oracle/_build/liboracle.so with g++ and OpenMP.  Portable C++: no intrinsics,
  no -march flags, so the same recipe works on x86-64 and aarch64.
* ``build_ref()`` compiles oracle/ref_driver.cpp against the reference's own
  headers, unmodified, where the reference checkout lies (``REFERENCE_ROOT``,
  default /root/reference), into oracle/_ref/libref.so.  The reference is a
  few header files, so a direct g++ call replaces its CMake build.  When the
  checkout is absent (for example on a machine that only runs the GPU tests)
  this is skipped and the tests that need it skip too.
"""
from __future__ import annotations

import os
import pathlib
import subprocess

HERE = pathlib.Path(__file__).resolve().parent
BUILD_DIR = HERE / "_build"
REF_DIR = HERE / "_ref"
ORACLE_SO = BUILD_DIR / "liboracle.so"
REF_SO = REF_DIR / "libref.so"
REFERENCE_ROOT = pathlib.Path(os.environ.get("GSN_REFERENCE_ROOT", "/root/reference"))

CXXFLAGS = ["-O2", "-std=c++17", "-fopenmp", "-shared", "-fPIC", "-Wall", "-Wno-unused-function"]


def _stale(target: pathlib.Path, sources) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(pathlib.Path(s).stat().st_mtime > t for s in sources)


def build_oracle(force: bool = False) -> pathlib.Path:
    BUILD_DIR.mkdir(exist_ok=True)
    srcs = [HERE / "oracle.cpp", HERE / "oracle_field.h"]
    if force or _stale(ORACLE_SO, srcs):
        tmp = ORACLE_SO.with_suffix(".so.tmp")
        subprocess.run(["g++", *CXXFLAGS, str(HERE / "oracle.cpp"), "-o", str(tmp)], check=True)
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def reference_present() -> bool:
    return (REFERENCE_ROOT / "test" / "fft_host.h").exists() and \
        (REFERENCE_ROOT / "cuda" / "device_field_operators.h").exists()


def build_ref(force: bool = False) -> pathlib.Path | None:
    if not reference_present():
        return REF_SO if REF_SO.exists() else None
    REF_DIR.mkdir(exist_ok=True)
    srcs = [HERE / "ref_driver.cpp", HERE / "oracle_field.h",
            REFERENCE_ROOT / "test" / "fft_host.h",
            REFERENCE_ROOT / "test" / "multiexp.h",
            REFERENCE_ROOT / "cuda" / "device_field.h",
            REFERENCE_ROOT / "cuda" / "device_field_operators.h"]
    if force or _stale(REF_SO, srcs):
        tmp = REF_SO.with_suffix(".so.tmp")
        # -w: the reference headers are compiled as shipped and warn a lot.
        subprocess.run(["g++", *CXXFLAGS, "-w", "-DDEBUG", f"-I{REFERENCE_ROOT}", f"-I{HERE}",
                        str(HERE / "ref_driver.cpp"), "-o", str(tmp)], check=True)
        os.replace(tmp, REF_SO)
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_ref(force=True))
