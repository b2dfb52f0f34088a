"""Build the CPU oracle (test infrastructure) and, where the reference
sources are present, the reference itself.

* ``build_oracle()`` compiles this directory's C restatements
  (vcp_oracle.c, ozaki_model.c) into ``oracle/_build/liboracle.so`` with gcc.
  Flags: -frounding-math (the code switches rounding modes) and
  -ffp-contract=off (no FMA contraction beyond the explicit fma() calls);
  on x86_64 -mfma -mavx2 so fma() is one instruction, on aarch64 FMA is
  baseline.
* ``build_reference()`` compiles the reference's own vblas/rmatmul.hpp and
  vcp/pidblas.hpp (through oracle/kvshim, a project-written stand-in for the
  absent kv library) from the reference tree into ``oracle/_ref/libvcpref.so``
  by the recipe in ``ref_wrap.cpp``.  The reference tree only exists where
  the sources are mounted; elsewhere this is a no-op returning None.
"""
from __future__ import annotations

import os
import platform
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
LIB = BUILD / "liboracle.so"
REF_LIB = REF_OUT / "libvcpref.so"
# Where this recipe looks for the reference sources: the directory named by
# VCP_REFERENCE_ROOT, else the mount point of the build container.  Callers
# use reference_root(), which gives None (and the callers skip) when neither
# holds the reference tree.
_REFERENCE_MOUNT = Path("/root/reference")


def reference_root() -> Path | None:
    env = os.environ.get("VCP_REFERENCE_ROOT")
    root = Path(env) if env else _REFERENCE_MOUNT
    return root if (root / "vblas" / "rmatmul.hpp").exists() else None


def _arch_flags() -> list[str]:
    m = platform.machine().lower()
    if m in ("x86_64", "amd64"):
        return ["-mfma", "-mavx2"]
    return []


def _stale(out: Path, srcs: list[Path]) -> bool:
    return not out.exists() or out.stat().st_mtime < max(s.stat().st_mtime for s in srcs)


def build_oracle(force: bool = False) -> Path:
    srcs = [HERE / "vcp_oracle.c", HERE / "ozaki_model.c"]
    srcs = [s for s in srcs if s.exists()]
    BUILD.mkdir(exist_ok=True)
    if force or _stale(LIB, srcs):
        cmd = ["gcc", "-O3", "-std=gnu11", "-fopenmp", "-frounding-math", "-ffp-contract=off",
               "-fPIC", "-shared", *_arch_flags(), "-o", str(LIB), *map(str, srcs), "-lm"]
        subprocess.run(cmd, check=True)
    return LIB


def build_reference(force: bool = False) -> Path | None:
    ref = reference_root()
    if ref is None:
        return None
    wrap = HERE / "ref_wrap.cpp"
    shim = sorted((HERE / "kvshim" / "kv").glob("*.hpp"))
    REF_OUT.mkdir(exist_ok=True)
    deps = [wrap, *shim]
    if force or _stale(REF_LIB, deps):
        cmd = ["g++", "-O3", "-std=c++11", "-fopenmp", "-fPIC", "-shared", "-DNDEBUG",
               "-DKV_FASTROUND", *_arch_flags(),
               f"-I{HERE / 'kvshim'}", f"-I{ref}", f"-I{ref / 'vblas'}",
               "-o", str(REF_LIB), str(wrap), "-lm"]
        subprocess.run(cmd, check=True)
    return REF_LIB


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_reference(force=True))
