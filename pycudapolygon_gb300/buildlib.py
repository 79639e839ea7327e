"""Build recipe for the GB300 (sm_103a) library and its Python module.

Outputs, all under pycudapolygon_gb300/_build/ (git-ignored):
  libpcp_gb300.so                 CUDA kernels + the C ABI of include/pcp_gb300.h
  libpyCudaPolygon<ext-suffix>    pybind11 module with the reference's Model table

Only nvcc and g++ are used (no cmake); the four CUDA/C++ translation units
compile in parallel with one -gencode (arch=compute_103a, code=sm_103a).
pybind11's headers come from the installed torch package (torch ships them),
so the module builds on machines without a separate pybind11 install.
"""
import importlib.util
import os
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libpcp_gb300.so")
EXT = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
MODULE = os.path.join(OUT, "libpyCudaPolygon" + EXT)

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["geometry.cu", "contacts.cu", "constraints.cu", "gradient.cu", "warmstart.cu"]
CPP_SOURCES = ["model.cpp"]
HEADERS = ["pcp_common.cuh", "pcp_internal.h", "pcp_fire.cuh"]


def _pybind_include():
    spec = importlib.util.find_spec("torch")
    if spec is not None and spec.origin:
        inc = os.path.join(os.path.dirname(spec.origin), "include")
        if os.path.exists(os.path.join(inc, "pybind11", "pybind11.h")):
            return inc
    try:
        import pybind11
        return pybind11.get_include()
    except ImportError as e:
        raise RuntimeError("pybind11 headers not found (neither torch/include nor pybind11)") from e


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + p.stdout)
    return p.stdout


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "pcp_gb300.h")]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if force or _newer(o, [s] + hdrs):
            jobs.append([NVCC, "-std=c++17", *ARCH, "-O3", "-lineinfo", "-Xcompiler", "-fPIC",
                         "-I" + INCLUDE, "-I" + CSRC, "-c", s, "-o", o])
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if force or _newer(o, [s] + hdrs):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-I" + INCLUDE, "-I" + CSRC,
                         "-I" + os.path.join(CUDA_HOME, "include"), "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            print(o)
    if force or jobs or _newer(LIB, objs):
        _run([NVCC, *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-lcudart"])
        os.replace(LIB + ".tmp", LIB)
    pyb = os.path.join(CSRC, "pybind_module.cpp")
    if force or _newer(MODULE, [pyb, LIB, os.path.join(INCLUDE, "pcp_gb300.h")]):
        py_inc = sysconfig.get_paths()["include"]
        _run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-fvisibility=hidden",
              "-I" + INCLUDE, "-I" + _pybind_include(), "-I" + py_inc, pyb,
              "-L" + OUT, "-lpcp_gb300", "-Wl,-rpath,$ORIGIN", "-o", MODULE + ".tmp"])
        os.replace(MODULE + ".tmp", MODULE)
    return LIB, MODULE


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
