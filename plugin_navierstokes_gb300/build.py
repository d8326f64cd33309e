"""In-tree build of the native library libnsfv1_gb300.so (sm_103a).

Compiles the CUDA / C++ translation units of ``csrc/`` in parallel with nvcc
(one ``-gencode arch=compute_103a,code=sm_103a``) and links them into
``plugin_navierstokes_gb300/lib/libnsfv1_gb300.so``. No cmake, no torch.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT_DIR = HERE / "lib"
BUILD_DIR = HERE / "_build"
LIB = OUT_DIR / "libnsfv1_gb300.so"
SOURCES = ["nsfv1_assemble.cu", "nsfv1_jac_lanes.cu", "nsfv1_ipshape.cu", "nsfv1_tools.cu", "nsfv1_solver.cu", "nsfv1_capi.cpp", "nsfv1_noalloc.cu", "nsfv1_batch.cu",
           "nsfv1_mlp.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _flags(extra: list[str] | None = None) -> list[str]:
    f = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
                "-Xcompiler", "-ffp-contract=on", "-I", str(HERE.parent / "include")]
    return f + (extra or [])


BOUNDS_CHECKED_SOURCES = ["nsfv1_assemble.cu", "nsfv1_jac_lanes.cu"]


def compile_bounds_checked(out: Path) -> list[Path]:
    """Compiles the assembly kernels with NSFV1_BOUNDS_CHECK (every node id and
    block index checked, out-of-range accesses skipped and reported through the
    error word): one object file per assembly source, named after out."""
    def one(src: str) -> Path:
        obj = out.with_name(out.stem + "_" + Path(src).stem + out.suffix)
        cmd = [nvcc_path()] + _flags(["-DNSFV1_BOUNDS_CHECK"]) + ["-c", str(CSRC / src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for the bounds-checked {src}:\n" + r.stdout + r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(BOUNDS_CHECKED_SOURCES)) as ex:
        return list(ex.map(one, BOUNDS_CHECKED_SOURCES))


def _needs_rebuild() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = list(CSRC.glob("*")) + [HERE.parent / "include" / "nsfv1_gb300.h", Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps)


def build(force: bool = False, verbose: bool = False, ptxas_v: bool = False) -> Path:
    """Build libnsfv1_gb300.so if any source is newer than it; returns its path."""
    if not force and not _needs_rebuild():
        return LIB
    nvcc = nvcc_path()
    BUILD_DIR.mkdir(exist_ok=True)
    OUT_DIR.mkdir(exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_v else []

    def compile_one(src: str) -> Path:
        obj = BUILD_DIR / (src + ".o")
        cmd = [nvcc] + _flags(extra) + ["-c", str(CSRC / src), "-o", str(obj)]
        if src.endswith(".cpp"):
            cmd = [nvcc] + _flags() + ["-x", "cu", "-c", str(CSRC / src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or ptxas_v or r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}")
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc] + ARCH + ["-shared", "-o", str(tmp)] + [str(o) for o in objs] + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("link failed")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_v="--ptxas" in sys.argv)
    print(LIB)
