"""Build recipe for the CPU oracle (test infrastructure only).

Two outputs, both git-ignored:

* ``oracle/_build/liboracle.so`` -- the plain-C restatement of the phase-sum
  kernel (``oracle/fast_cos_sum.c``), compiled with gcc and OpenMP.
* ``oracle/_ref/cpp<EXT_SUFFIX>`` -- the reference's pybind11 module of
  Celio's method (``muspinsim/cpp/*.cpp``), compiled from its sources with
  g++ and OpenMP where both the reference tree and pybind11 are present
  (the golden-vector generator only; nothing on a machine without them
  needs it).
* ``oracle/_ref/_ref_parallel<EXT_SUFFIX>`` -- the reference's own Cython
  kernel (``muspinsim/cython/parallel.pyx``), compiled from the reference
  sources.  Where the reference tree is present, Cython first translates the
  ``.pyx`` into ``oracle/_ref/_ref_parallel.c``; where only that generated C
  file is present (a machine without the reference tree or Cython), it is
  compiled as is.  Flags follow the reference's own build
  (``setup.py:49-53``: ``-O3 -funroll-loops`` plus ``-fopenmp``).

Run ``python oracle/build.py`` or call :func:`build_all`.
"""

import os
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
REFERENCE_ROOT = "/root/reference"
REF_PYX = os.path.join(REFERENCE_ROOT, "muspinsim", "cython", "parallel.pyx")
REF_MODULE = "_ref_parallel"


def _run(cmd):
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed ({proc.returncode}): {' '.join(cmd)}\n{proc.stdout}")
    return proc.stdout


def oracle_lib_path():
    return os.path.join(BUILD_DIR, "liboracle.so")


def ref_module_path():
    return os.path.join(REF_DIR, REF_MODULE + sysconfig.get_config_var("EXT_SUFFIX"))


def build_port(force=False):
    """Compile the C restatement into oracle/_build/liboracle.so."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    srcs = [os.path.join(HERE, f) for f in ("fast_cos_sum.c", "celio.c")]
    out = oracle_lib_path()
    if not force and os.path.exists(out) and all(
            os.path.getmtime(out) >= os.path.getmtime(s) for s in srcs):
        return out
    _run(["gcc", "-O3", "-fopenmp", "-fPIC", "-shared"] + srcs + ["-o", out, "-lm"])
    return out


def build_ref(force=False):
    """Compile the reference's Cython kernel into oracle/_ref.

    Returns the path of the extension module, or None when neither the
    reference tree nor a previously generated C file is available."""
    os.makedirs(REF_DIR, exist_ok=True)
    csrc = os.path.join(REF_DIR, REF_MODULE + ".c")
    if os.path.exists(REF_PYX) and (force or not os.path.exists(csrc)):
        _run([sys.executable, "-m", "cython", "-3", "--module-name", REF_MODULE,
              REF_PYX, "-o", csrc])
    if not os.path.exists(csrc):
        return None
    out = ref_module_path()
    if not force and os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(csrc):
        return out
    import numpy

    inc = [sysconfig.get_paths()["include"], numpy.get_include()]
    cmd = ["gcc", "-w", "-O3", "-funroll-loops", "-fopenmp", "-fPIC", "-shared"]
    cmd += [f"-I{p}" for p in inc]
    cmd += [csrc, "-o", out, "-fopenmp", "-lm"]
    _run(cmd)
    return out


REF_CPP = os.path.join(REFERENCE_ROOT, "muspinsim", "cpp")


def ref_cpp_path():
    return os.path.join(REF_DIR, "cpp" + sysconfig.get_config_var("EXT_SUFFIX"))


def build_ref_cpp(force=False):
    """Compile the reference's pybind11 module (Celio's method) from its own
    sources into oracle/_ref; returns its path, or None where the reference
    tree or pybind11 is missing."""
    try:
        import pybind11
    except ImportError:
        return None
    if not os.path.isdir(REF_CPP):
        return None
    os.makedirs(REF_DIR, exist_ok=True)
    srcs = sorted(os.path.join(REF_CPP, f) for f in os.listdir(REF_CPP) if f.endswith(".cpp"))
    out = ref_cpp_path()
    if not force and os.path.exists(out) and all(
            os.path.getmtime(out) >= os.path.getmtime(s) for s in srcs):
        return out
    inc = [sysconfig.get_paths()["include"], pybind11.get_include()]
    cmd = ["g++", "-w", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared"]
    cmd += [f"-I{p}" for p in inc] + srcs + ["-o", out]
    _run(cmd)
    return out


def build_all(force=False):
    port = build_port(force)
    ref = build_ref(force)
    return port, ref


if __name__ == "__main__":
    print(build_all(force="--force" in sys.argv))
