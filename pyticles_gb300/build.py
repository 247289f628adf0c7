"""Builds libsph.so in-tree for sm_103a (GB300).

Each translation unit under csrc/ is compiled by its own nvcc process in
parallel, then linked into pyticles_gb300/_build/libsph.so with the static
CUDA runtime.  No cmake, no torch extension machinery: the library exports a
plain C ABI (include/sph.h) and is loaded with ctypes.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libsph.so")
SOURCES = ["sph_engine.cu", "sph_sort.cu", "sph_pairs.cu", "sph_force_f32.cu",
           "sph_force_f64.cu", "sph_noalloc.cu", "sph_splat.cu", "sph_collide.cu",
           "sph_cluster.cu", "sph_kfunc.cu", "sph_vlist.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "--expt-relaxed-constexpr"]


def nvcc():
    path = shutil.which("nvcc")
    if path:
        return path
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(os.path.dirname(HERE), "include", "sph.h"))
    return files


def lib_path(checks=False):
    return os.path.join(OUT, "libsph_checks.so" if checks else "libsph.so")


def up_to_date(checks=False):
    path = lib_path(checks)
    if not os.path.exists(path):
        return False
    t = os.path.getmtime(path)
    return all(os.path.getmtime(f) <= t for f in _deps())


def _compile(src, checks=False):
    suffix = "_checks.o" if checks else ".o"
    obj = os.path.join(OUT, os.path.basename(src).replace(".cu", suffix))
    extra = ["-DSPH_DEBUG_CHECKS"] if checks else []
    cmd = [nvcc()] + ARCH + FLAGS + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stderr}")
    return obj


def build(force=False, verbose=False, checks=False):
    """Compiles every CUDA translation unit and links libsph.so; with checks,
    libsph_checks.so, whose kernels test their cell and particle indices and
    report SPH_EBOUNDS instead of accessing out of range."""
    path = lib_path(checks)
    if not force and up_to_date(checks):
        return path
    os.makedirs(OUT, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda src: _compile(src, checks), SOURCES))
    tmp = path + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stderr}")
    os.replace(tmp, path)
    if verbose:
        print("built", path)
    return path


if __name__ == "__main__":
    build(force=True, verbose=True)
