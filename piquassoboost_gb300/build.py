"""Build the native library in-tree with nvcc (no CMake, no setuptools).

``build_native()`` compiles every ``csrc/*.cu`` for sm_103a in parallel and
links ``_lib/libgbperm.so``.  Objects are rebuilt only when a source or header
is newer than them.  Run ``python -m piquassoboost_gb300.build`` to build.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
INCLUDE = os.path.join(REPO_DIR, "include")
LIB_DIR = os.path.join(PKG_DIR, "_lib")
OBJ_DIR = os.path.join(PKG_DIR, "_build")
LIB_PATH = os.path.join(LIB_DIR, "libgbperm.so")

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-O3",
              "--expt-relaxed-constexpr"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgbperm")
    return cand


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_native(verbose: bool = False, jobs: int | None = None) -> str:
    """Compile and link libgbperm.so; return its path."""
    nvcc = _nvcc()
    os.makedirs(LIB_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    sources = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))
    headers = _headers()
    objs = []
    todo = []
    for src in sources:
        obj = os.path.join(OBJ_DIR, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            cmd = [nvcc, *ARCH_FLAGS, *NVCC_FLAGS, "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj]
            todo.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {cmd[-3]}:\n{r.stdout}\n{r.stderr}")
        return r.stderr

    if todo:
        with ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            for err in ex.map(run, todo):
                if verbose and err:
                    print(err, file=sys.stderr)
    if todo or _stale(LIB_PATH, objs):
        cmd = [nvcc, *ARCH_FLAGS, "-shared", "-o", LIB_PATH, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB_PATH


def build_oracle(verbose: bool = False) -> str:
    """Compile the C oracle (test infrastructure) into oracle/_build."""
    src = os.path.join(REPO_DIR, "oracle", "perm_oracle.c")
    body = os.path.join(REPO_DIR, "oracle", "perm_oracle_body.h")
    out_dir = os.path.join(REPO_DIR, "oracle", "_build")
    out = os.path.join(out_dir, "libperm_oracle.so")
    os.makedirs(out_dir, exist_ok=True)
    if _stale(out, [src, body]):
        cc = shutil.which("gcc") or "cc"
        cmd = [cc, "-std=gnu11", "-O3", "-fPIC", "-shared", "-o", out, src, "-lpthread", "-lm"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return out


def build_reference_oracle(verbose: bool = False) -> str | None:
    """Build oracle/_ref (the reference's own calculators, test
    infrastructure) with oracle/build_ref.sh.  The script locates the
    reference tree (PQB_REFERENCE_ROOT, or its default) and exits with status
    3 where there is none, as on the GPU machine; then this returns None."""
    script = os.path.join(REPO_DIR, "oracle", "build_ref.sh")
    shim = os.path.join(REPO_DIR, "oracle", "ref_capi.cpp")
    out = os.path.join(REPO_DIR, "oracle", "_ref", "libpqbref.so")
    if not _stale(out, [script, shim]):
        return out
    r = subprocess.run(["bash", script], capture_output=True, text=True)
    if verbose:
        print(r.stdout, r.stderr)
    return out if r.returncode == 0 else None


if __name__ == "__main__":
    print(build_native(verbose=True))
    print(build_oracle(verbose=True))
    print(build_reference_oracle(verbose=True))
