"""Build of the in-tree native libraries.

* ``libsphdem.so``  -- the CUDA step library, sm_103a only, one nvcc process per
  translation unit (run in parallel), linked with the static CUDA runtime.
* ``oracle/_build/liboracle_{f32,f64}.so`` -- the CPU oracle (test
  infrastructure; built here so that one call prepares a fresh machine).

Outputs stay inside the repository (git-ignored), so a machine that receives
the sources and rebuilds them loads exactly these files.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB = BUILD / "libsphdem.so"
ORACLE_SRC = ROOT / "oracle" / "sphdem_oracle.c"
ORACLE_BUILD = ROOT / "oracle" / "_build"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -ftz=true: denormals flush to zero.  Membership thresholds are normal
# numbers (>= 1e-12), so no neighbour or contact decision can change.
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-ftz=true", "-Xcompiler", "-fPIC", "-Xptxas", "-v",
              f"-I{INCLUDE}", f"-I{CSRC}"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libsphdem.so")


def _sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> str:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed ({proc.returncode}): {' '.join(cmd)}\n"
                           f"{proc.stdout}\n{proc.stderr}")
    return proc.stdout + proc.stderr


def build_cuda(force: bool = False, verbose: bool = False) -> Path:
    """Compile every csrc/*.cu for sm_103a and link libsphdem.so."""
    BUILD.mkdir(parents=True, exist_ok=True)
    srcs = _sources()
    headers = _headers()
    objs = [BUILD / (s.stem + ".o") for s in srcs]
    todo = [(s, o) for s, o in zip(srcs, objs) if force or _stale(o, [s] + headers)]
    logs = {}
    if todo:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(todo))) as ex:
            futs = {ex.submit(_run, [nvcc(), *ARCH, *NVCC_FLAGS, "-c", str(s), "-o", str(o)]): s
                    for s, o in todo}
            for f in cf.as_completed(futs):
                logs[futs[f].name] = f.result()
    if force or todo or _stale(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp")
        _run([nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs)])
        os.replace(tmp, LIB)
    if verbose:
        for name, log in sorted(logs.items()):
            print(f"--- {name}\n{log}")
    (BUILD / "ptxas.log").write_text("".join(f"--- {k}\n{v}" for k, v in sorted(logs.items())))
    return LIB


def build_oracle(force: bool = False) -> dict[str, Path]:
    """Compile the CPU oracle twice (FP32 reference semantics and FP64)."""
    ORACLE_BUILD.mkdir(parents=True, exist_ok=True)
    cc = os.environ.get("CC") or shutil.which("gcc") or "cc"
    out = {}
    for tag, real in (("f32", "float"), ("f64", "double")):
        target = ORACLE_BUILD / f"liboracle_{tag}.so"
        if force or _stale(target, [ORACLE_SRC, INCLUDE / "sphdem.h"]):
            tmp = target.with_suffix(".so.tmp")
            _run([cc, "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
                  f"-I{INCLUDE}", f"-DORACLE_REAL={real}", str(ORACLE_SRC), "-o", str(tmp),
                  "-lpthread", "-lm"])
            os.replace(tmp, target)
        out[tag] = target
    return out


def build_all(force: bool = False, verbose: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        a = ex.submit(build_cuda, force, verbose)
        b = ex.submit(build_oracle, force)
        a.result()
        b.result()


if __name__ == "__main__":
    import sys
    build_all(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
