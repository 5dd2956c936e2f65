"""Build recipe for the oracle (TEST INFRASTRUCTURE ONLY).

* ``oracle/liboracle.so``  -- the CPU restatement (glasma_oracle.cpp), built on
  every machine (x86 here, aarch64 on the GPU host).
* ``oracle/_ref/libglasma_ref.so`` -- the reference's own SU(3) code path
  compiled from its unmodified sources plus the shims in ``oracle/ref``.  Built
  only where the reference checkout exists; its location comes from the
  ``GLASMA_REFERENCE_SRC`` environment variable, else the checkout's source
  directory next to this repository (``../reference/...`` from the repository
  root).  Where neither exists (the GPU host) nothing is built.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_REF_SRC = os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference", "Pragya_workingdirectory_worksonm1",
                               "Workingdirectory", "SourceCode")
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libglasma_ref.so")


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(force=False):
    src = os.path.join(HERE, "glasma_oracle.cpp")
    if force or _stale(ORACLE_SO, [src]):
        cmd = ["g++", "-O3", "-fopenmp", "-std=c++17", "-fPIC", "-shared", "-o", ORACLE_SO, src]
        subprocess.check_call(cmd)
    return ORACLE_SO


def reference_source_dir():
    d = os.environ.get("GLASMA_REFERENCE_SRC", DEFAULT_REF_SRC)
    return d if os.path.isdir(d) else None


def build_reference(force=False):
    ref = reference_source_dir()
    if ref is None:
        return None
    srcs = [os.path.join(HERE, "ref", "ref_harness.cpp"), os.path.join(HERE, "ref", "fftw3.h")]
    os.makedirs(os.path.dirname(REF_SO), exist_ok=True)
    if force or _stale(REF_SO, srcs):
        cmd = ["g++", "-O3", "-fopenmp", "-std=c++14", "-w", "-fPIC", "-shared",
               "-I", os.path.join(HERE, "ref"), "-I", ref, srcs[0], "-o", REF_SO]
        subprocess.check_call(cmd)
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_reference(force="--force" in sys.argv))
