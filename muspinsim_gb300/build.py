"""Compile ``libmspgpu.so`` (the CUDA kernels and their C ABI) for sm_103a.

The translation units under ``csrc/`` are compiled in parallel with nvcc
(``-gencode arch=compute_103a,code=sm_103a -O3 -lineinfo``) and linked into
``muspinsim_gb300/_build/libmspgpu.so`` (git-ignored, rebuilt on every
machine that runs it).  ``python -m muspinsim_gb300.build`` or
:func:`build`.
"""

import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD_DIR = os.path.join(HERE, "_build")
LIB_NAME = "libmspgpu.so"
SOURCES = ["msp_snap.cu", "msp_jacobi_warp.cu", "msp_ql_warp.cu", "msp_phase.cu", "msp_api.cu", "msp_static.cu", "msp_adjoint.cu", "msp_large.cu",
           "msp_large_mixed.cu",
           "msp_multi.cu", "msp_orient.cu", "msp_assemble.cu",
           "msp_lindblad.cu", "msp_celio.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3"]


def nvcc_path():
    cand = shutil.which("nvcc")
    if cand:
        return cand
    for root in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if root and os.path.exists(os.path.join(root, "bin", "nvcc")):
            return os.path.join(root, "bin", "nvcc")
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmspgpu")


def lib_path():
    return os.path.join(BUILD_DIR, LIB_NAME)


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(os.path.dirname(HERE), "include", "mspgpu.h"))
    return files


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{proc.stdout}")
    return proc.stdout


def build(force=False, verbose=False, extra_flags=()):
    """Compile the library if any source is newer than it; return its path."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    out = lib_path()
    deps = _deps()
    if not force and not _stale(out, deps):
        return out
    nvcc = nvcc_path()
    objs = []
    cmds = []
    for src in SOURCES:
        obj = os.path.join(BUILD_DIR, src.replace(".cu", ".o"))
        objs.append(obj)
        cmds.append([nvcc, *ARCH, *FLAGS, *extra_flags, "-c", os.path.join(CSRC, src), "-o", obj])
    with concurrent.futures.ThreadPoolExecutor(len(cmds)) as pool:
        logs = list(pool.map(_run, cmds))
    if verbose:
        for log in logs:
            sys.stdout.write(log)
    tmp = out + ".tmp"
    _run([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"])
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv,
                extra_flags=("-Xptxas", "-v") if "--ptxas" in sys.argv else ()))
