"""Build recipe of the in-tree C-ABI library (no cmake, no torch).

``build()`` compiles ``csrc/*.cu`` with nvcc for sm_103a only and
``csrc/*.cpp`` with g++ (-ffp-contract=off: the host geometry must round like
the reference's x86-64 build), in parallel, and links
``build/libsonar_gb300.so``.  ``build/libcuda_project.so`` is a link to it
under the name the reference's ctypes wrapper loads
(run_scripts/modules/api.py:4).
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "build")
LIB = os.path.join(BUILD, "libsonar_gb300.so")
COMPAT = os.path.join(BUILD, "libcuda_project.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu"))), sorted(glob.glob(os.path.join(CSRC, "*.cpp")))


def _deps():
    return (glob.glob(os.path.join(CSRC, "*")) + glob.glob(os.path.join(INCLUDE, "*.h"))
            + [os.path.abspath(__file__)])


def _stale(target):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in _deps())


def _compile(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile and link the library if any source changed; return its path."""
    if not force and not _stale(LIB):
        _link_compat()
        return LIB
    if not os.path.exists(NVCC):
        raise RuntimeError("nvcc not found at %s" % NVCC)
    obj_dir = os.path.join(BUILD, "obj")
    os.makedirs(obj_dir, exist_ok=True)
    cus, cpps = _sources()
    jobs = []
    for src in cus:
        obj = os.path.join(obj_dir, os.path.basename(src) + ".o")
        cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE,
               "-c", src, "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        jobs.append((obj, cmd))
    for src in cpps:
        obj = os.path.join(obj_dir, os.path.basename(src) + ".o")
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-I", INCLUDE,
               "-I", os.path.join(CUDA_HOME, "include"), "-c", src, "-o", obj]
        jobs.append((obj, cmd))
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        outs = list(ex.map(lambda j: _compile(j[1]), jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    tmp = LIB + ".tmp%d" % os.getpid()
    _compile([NVCC, *ARCH, "-shared", "-o", tmp, *[o for o, _ in jobs], "-cudart", "static"])
    os.replace(tmp, LIB)
    _link_compat()
    return LIB


def _link_compat():
    try:
        if os.path.islink(COMPAT) or os.path.exists(COMPAT):
            if os.path.islink(COMPAT) and os.readlink(COMPAT) == os.path.basename(LIB):
                return
            os.remove(COMPAT)
        os.symlink(os.path.basename(LIB), COMPAT)
    except OSError:
        shutil.copyfile(LIB, COMPAT)


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
