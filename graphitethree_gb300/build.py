"""Build recipe for libnl_gb300.so (sm_103a only, in-tree).

Compiles every translation unit under ``csrc/`` in parallel with nvcc for
``-gencode arch=compute_103a,code=sm_103a`` and links one shared library,
``graphitethree_gb300/lib/libnl_gb300.so``, whose C ABI is declared in
``include/nl.h`` and ``include/nl_gb300.h``.  No CMake, no torch extension:
the library depends only on the CUDA runtime (linked statically).
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
LIB_DIR = PKG / "lib"
LIB_NAME = "libnl_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["nlgb_solver.cu", "nlgb_assembly.cu", "nlgb_blas.cu", "nlgb_batch.cu",
              "nlgb_noalloc.cu", "nlgb_build.cu", "nlgb_krylov.cu", "nlgb_ssor.cu"]
CPP_SOURCES = ["nl_api.cpp", "nl_matrix_api.cpp", "nlgb_api.cpp", "nlgb_server.cpp"]


def lib_path() -> Path:
    return LIB_DIR / LIB_NAME


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build libnl_gb300")


def _deps() -> list[Path]:
    return sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(p.stat().st_mtime > t for p in [src, *_deps()])


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compile (if stale) and link the library; returns its path."""
    nvcc = _nvcc()
    obj_dir = PKG / "_build" / os.uname().machine
    obj_dir.mkdir(parents=True, exist_ok=True)
    LIB_DIR.mkdir(parents=True, exist_ok=True)
    common = ["-std=c++17", "-O3", "-Xcompiler", "-fPIC", "-I", str(INCLUDE), "-I", str(CSRC)]
    jobs = []
    for name in CU_SOURCES + CPP_SOURCES:
        src = CSRC / name
        if not src.exists():
            continue
        obj = obj_dir / (name + ".o")
        if name.endswith(".cu"):
            cmd = [nvcc, *ARCH, "-lineinfo", *common, "-c", str(src), "-o", str(obj)]
        else:
            # host code that includes the device-side structs: compiled as CUDA
            cmd = [nvcc, *ARCH, *common, "-Xcompiler", "-Wall", "-x", "cu", "-c", str(src),
                   "-o", str(obj)]
        jobs.append((obj, src, cmd))

    def run(job):
        obj, src, cmd = job
        if not force and not _stale(obj, src):
            return None
        if verbose:
            print(" ".join(cmd), flush=True)
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            return f"{src.name}:\n{p.stdout}\n{p.stderr}"
        return None

    with ThreadPoolExecutor(max_workers=min(8, len(jobs) or 1)) as ex:
        errors = [e for e in ex.map(run, jobs) if e]
    if errors:
        raise RuntimeError("libnl_gb300 build failed:\n" + "\n".join(errors))
    out = lib_path()
    objs = [str(j[0]) for j in jobs]
    if force or not out.exists() or any(Path(o).stat().st_mtime > out.stat().st_mtime for o in objs):
        tmp = out.with_suffix(".so.tmp")
        cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *objs, "-cudart", "static", "-lpthread", "-ldl", "-lrt"]
        if verbose:
            print(" ".join(cmd), flush=True)
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"libnl_gb300 link failed:\n{p.stdout}\n{p.stderr}")
        os.replace(tmp, out)
    return out


if __name__ == "__main__":
    print(build(verbose=True))
