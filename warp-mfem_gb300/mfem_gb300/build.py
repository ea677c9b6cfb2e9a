"""Builds libmfem_gb300.so in-tree with nvcc for sm_103a.

Every translation unit under ``csrc/`` is compiled in parallel to an object
file in ``_build/`` and linked into ``mfem_gb300/libmfem_gb300.so`` (static
CUDA runtime, so the library loads with or without PyTorch in the process).
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
PROJECT_DIR = PKG_DIR.parent
REPO_DIR = PROJECT_DIR.parent
CSRC = PROJECT_DIR / "csrc"
INCLUDE = REPO_DIR / "include"
BUILD_DIR = PROJECT_DIR / "_build"
LIB_PATH = PKG_DIR / "libmfem_gb300.so"

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall", "-Xcompiler", "-Wno-unknown-pragmas",
                f"-I{INCLUDE}", f"-I{CSRC}"]


def nvcc_path() -> str:
    cand = shutil.which("nvcc")
    if cand:
        return cand
    for root in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if root and (Path(root) / "bin" / "nvcc").exists():
            return str(Path(root) / "bin" / "nvcc")
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmfem_gb300")


def sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _compile(nvcc: str, src: Path, verbose: bool, ptxas_verbose: bool) -> Path:
    obj = BUILD_DIR / (src.name + ".o")
    cmd = [nvcc, "-c", str(src), "-o", str(obj), *ARCH_FLAGS, *COMMON_FLAGS]
    if src.suffix == ".cpp":
        cmd = [nvcc, "-x", "cu", "-c", str(src), "-o", str(obj), *ARCH_FLAGS, *COMMON_FLAGS]
    if ptxas_verbose and src.suffix == ".cu":
        cmd += ["-Xptxas", "-v"]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")
    if verbose or ptxas_verbose:
        out = (proc.stdout + proc.stderr).strip()
        if out:
            print(f"[{src.name}]\n{out}", file=sys.stderr)
    return obj


def _stale() -> bool:
    if not LIB_PATH.exists():
        return True
    lib_mtime = LIB_PATH.stat().st_mtime
    deps = sources() + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    return any(p.stat().st_mtime > lib_mtime for p in deps)


def build(force: bool = False, verbose: bool = False, ptxas_verbose: bool = False) -> Path:
    """Compiles the library if any source is newer than it; returns its path."""
    if not force and not _stale():
        return LIB_PATH
    nvcc = nvcc_path()
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    srcs = sources()
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(nvcc, s, verbose, ptxas_verbose), srcs))
    tmp = LIB_PATH.with_suffix(".so.tmp")
    cmd = [nvcc, "-shared", *ARCH_FLAGS, "-o", str(tmp), *map(str, objs), "-cudart", "static"]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    p = build(force="--force" in sys.argv, verbose=True, ptxas_verbose="-v" in sys.argv)
    print(p)
