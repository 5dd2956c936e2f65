"""Builds libglasma_gb300.so from csrc/ with nvcc for sm_103a (in-tree, no CMake).

Translation units are compiled in parallel, then linked into one shared library
next to this file.  Re-running only rebuilds when a source or header is newer
than the library.
"""
import concurrent.futures
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libglasma_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
    return _sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(CSRC, "*.inc")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


STAMP = LIB + ".flags"


def _extra_flags():
    """Extra nvcc flags for tuning sweeps, e.g. GLASMA_NVCC_EXTRA="-DGLASMA_FP32_MIN_BLOCKS=4"."""
    return os.environ.get("GLASMA_NVCC_EXTRA", "").split()


def needs_build():
    if not os.path.exists(LIB):
        return True
    try:
        if open(STAMP).read() != " ".join(_extra_flags()):
            return True
    except OSError:
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(d) > t for d in _deps())


def build(force=False, verbose=False, ptxas_verbose=False):
    if not force and not needs_build():
        return LIB
    nvcc = _nvcc()
    objdir = os.path.join(os.path.dirname(HERE), "_build", "obj")
    os.makedirs(objdir, exist_ok=True)
    extra = (["-Xptxas", "-v"] if ptxas_verbose else []) + _extra_flags()

    def compile_one(src):
        obj = os.path.join(objdir, os.path.basename(src) + ".o")
        cmd = [nvcc] + ARCH + NVCC_FLAGS + extra + ["-I", INCLUDE, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s" % (src, r.stderr[-4000:]))
        if verbose:
            print(r.stderr)
        return obj

    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, _sources()))
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-cudart", "shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stderr[-4000:])
    os.replace(tmp, LIB)
    with open(STAMP, "w") as f:
        f.write(" ".join(_extra_flags()))
    return LIB


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, ptxas_verbose="-v" in sys.argv))
