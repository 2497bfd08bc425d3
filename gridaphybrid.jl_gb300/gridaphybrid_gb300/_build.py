"""Build of libgridaphybrid_gb300.so (sm_103a) from csrc/, in tree.

Each translation unit is compiled by nvcc in parallel with
``-gencode arch=compute_103a,code=sm_103a`` and linked into one shared
library next to this package.  No CMake, no torch extension machinery.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(PKG_ROOT, "csrc")
BUILD_DIR = os.path.join(PKG_ROOT, "_build")
LIB_NAME = "libgridaphybrid_gb300.so"
LIB_PATH = os.path.join(PKG_ROOT, LIB_NAME)

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgridaphybrid_gb300")


def sources():
    return sorted(
        os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp"))
    )


def _needs_rebuild(objs_and_srcs, lib):
    if not os.path.exists(lib):
        return True
    lib_t = os.path.getmtime(lib)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.abspath(os.path.join(PKG_ROOT, "..", "include", "hdg_gb300.h")))
    return any(os.path.getmtime(d) > lib_t for d in deps if os.path.exists(d))


def build(force=False, verbose=False, extra_flags=()):
    """Compile csrc/*.cu|*.cpp and link LIB_PATH; returns the library path."""
    srcs = sources()
    if not force and not _needs_rebuild(srcs, LIB_PATH):
        return LIB_PATH
    nvcc = _nvcc()
    os.makedirs(BUILD_DIR, exist_ok=True)

    def compile_one(src):
        obj = os.path.join(BUILD_DIR, os.path.basename(src) + ".o")
        cmd = [nvcc, *ARCH_FLAGS, *COMMON_FLAGS, *extra_flags, "-c", src, "-o", obj]
        if src.endswith(".cpp"):
            cmd[1:1] = ["-x", "cu"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("nvcc failed on %s:\n%s\n%s" % (src, " ".join(cmd), res.stderr))
        if verbose and res.stderr:
            print(res.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc, *ARCH_FLAGS, "-shared", "-o", tmp, *objs]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), res.stderr))
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force=True, verbose=True))
