"""Build the in-tree CUDA library `libhmclab_gb300.so` for sm_103a.

Each translation unit under `csrc/` is compiled by nvcc in parallel
(`-gencode arch=compute_103a,code=sm_103a`) and linked into one shared
library next to this file.  The build is incremental: a unit is recompiled
when its source or any header under `csrc/`/`include/` is newer than its
object file.
"""
import concurrent.futures as _cf
import glob as _glob
import os as _os
import shutil as _shutil
import subprocess as _sp

PKG_DIR = _os.path.dirname(_os.path.abspath(__file__))
REPO_DIR = _os.path.dirname(PKG_DIR)
CSRC = _os.path.join(PKG_DIR, "csrc")
INCLUDE = _os.path.join(REPO_DIR, "include")
BUILD_DIR = _os.path.join(PKG_DIR, "_build")
LIB_NAME = "libhmclab_gb300.so"
LIB_PATH = _os.path.join(PKG_DIR, LIB_NAME)

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3",
    "-std=c++17",
    "-lineinfo",
    "-Xcompiler",
    "-fPIC",
    "-Xcompiler",
    "-fvisibility=hidden",
    "--expt-relaxed-constexpr",
    "-DHMC_BUILDING_LIBRARY",
]


def _nvcc():
    path = _shutil.which("nvcc")
    if path is None:
        cand = "/usr/local/cuda/bin/nvcc"
        if _os.path.exists(cand):
            return cand
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build hmclab_gb300")
    return path


def _headers():
    return _glob.glob(_os.path.join(CSRC, "*.cuh")) + _glob.glob(_os.path.join(INCLUDE, "*.h"))


def _stale(src, obj, headers):
    if not _os.path.exists(obj):
        return True
    t = _os.path.getmtime(obj)
    return any(_os.path.getmtime(f) > t for f in [src] + headers)


def _compile(src, obj, verbose):
    cmd = [_nvcc()] + ARCH_FLAGS + NVCC_FLAGS + ["-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    res = _sp.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {_os.path.basename(src)}:\n{res.stdout}\n{res.stderr}")
    return res.stderr if verbose else ""


def build(force: bool = False, verbose: bool = False, jobs: int = None) -> str:
    """Compile every `csrc/*.cu` and link the shared library; returns its path."""
    _os.makedirs(BUILD_DIR, exist_ok=True)
    sources = sorted(_glob.glob(_os.path.join(CSRC, "*.cu")))
    headers = _headers()
    objs = [_os.path.join(BUILD_DIR, _os.path.basename(s)[:-3] + ".o") for s in sources]
    todo = [(s, o) for s, o in zip(sources, objs) if force or _stale(s, o, headers)]
    logs = []
    if todo:
        jobs = jobs or min(len(todo), max(1, _os.cpu_count() or 1))
        with _cf.ThreadPoolExecutor(max_workers=jobs) as ex:
            for log in ex.map(lambda so: _compile(so[0], so[1], verbose), todo):
                logs.append(log)
    if todo or not _os.path.exists(LIB_PATH) or force:
        tmp = LIB_PATH + ".tmp"
        cmd = [_nvcc()] + ARCH_FLAGS + ["-shared", "-o", tmp] + objs + ["-lcuda"]
        res = _sp.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
        _os.replace(tmp, LIB_PATH)
    if verbose:
        print("\n".join(l for l in logs if l))
    return LIB_PATH


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
