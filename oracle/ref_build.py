"""Recipe for building the reference's own evaluation path (TEST INFRASTRUCTURE).

The reference (camdennis/pyCudaPolygon) is CUDA-only: it has no CPU
implementation of the path, so the golden vectors that pin the CPU oracle
come from the reference's own kernels, rebuilt for sm_103a and run on a GPU.

  stage   copy the reference's sources (src/kernels.cuh, model.cu, model.cpp,
          model.hpp, cuda_check.h, enumTypes.h) from the reference checkout
          named by PCP_REFERENCE into oracle/_ref/src/, and its unchanged
          Python layer (pyCudaPolygon/*.py with polygonMixins/) into
          oracle/_ref/py/pyCudaPolygon/, which the drop-in test imports on
          top of this repository's module.  oracle/_ref/ is git-ignored: the
          copies are inputs for the GPU machine, which has no reference
          checkout, and are never committed.
  build   compile oracle/_ref/src with the shims in oracle/ref_shim/ (CUDA 13
          removed cub::TransformInputIterator, src/model.cu:12,92; the
          reference does not ship src/FIRE.h and src/shake.h, model.cu:15-16)
          and the driver oracle/ref_golden.cpp into oracle/_ref/ref_golden.
          The sources compile unmodified; nothing of the reference is edited.

Only nvcc and g++ are used (no cmake; the reference's CMakeLists.txt fetches
CUB over the network, CUDA 13's bundled CCCL is used instead).  Outputs go to
oracle/_ref/ only.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
STAGED = os.path.join(REF_DIR, "src")
SHIM = os.path.join(HERE, "ref_shim")
DRIVER = os.path.join(HERE, "ref_golden.cpp")
BIN = os.path.join(REF_DIR, "ref_golden")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
SOURCES = ["kernels.cuh", "model.cu", "model.cpp", "model.hpp", "cuda_check.h", "enumTypes.h"]
PY_STAGED = os.path.join(REF_DIR, "py", "pyCudaPolygon")
PY_SOURCES = ["__init__.py", "enums.py", "pyCudaPolygon.py", "pyCudaPolygonLink.py",
              os.path.join("polygonMixins", "polygonDraw.py"),
              os.path.join("polygonMixins", "polygonUtils.py")]


def reference_root():
    root = os.environ.get("PCP_REFERENCE")
    if not root:
        raise SystemExit("set PCP_REFERENCE to the root of the reference checkout")
    return root


def stage(ref=None):
    """Copy the reference sources the path needs into oracle/_ref/src."""
    src = os.path.join(ref or reference_root(), "src")
    if not os.path.isdir(src):
        raise FileNotFoundError("reference sources not found at " + src)
    os.makedirs(STAGED, exist_ok=True)
    for f in SOURCES:
        shutil.copyfile(os.path.join(src, f), os.path.join(STAGED, f))
    pysrc = os.path.join(ref or reference_root(), "pyCudaPolygon")
    os.makedirs(os.path.join(PY_STAGED, "polygonMixins"), exist_ok=True)
    for f in PY_SOURCES:
        shutil.copyfile(os.path.join(pysrc, f), os.path.join(PY_STAGED, f))
    return STAGED


def python_staged():
    """The staged Python layer's package directory, or None."""
    ok = all(os.path.exists(os.path.join(PY_STAGED, f)) for f in PY_SOURCES)
    return PY_STAGED if ok else None


def staged():
    return all(os.path.exists(os.path.join(STAGED, f)) for f in SOURCES)


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("reference build failed:\n" + " ".join(cmd) + "\n" + p.stdout)


def build(force=False):
    """Build oracle/_ref/ref_golden from the staged sources."""
    if not staged():
        raise FileNotFoundError("reference sources are not staged in " + STAGED)
    deps = [os.path.join(STAGED, f) for f in SOURCES] + [DRIVER] + [
        os.path.join(dp, f) for dp, _, fs in os.walk(SHIM) for f in fs]
    if not force and os.path.exists(BIN) and all(
            os.path.getmtime(BIN) >= os.path.getmtime(d) for d in deps):
        return BIN
    obj = os.path.join(REF_DIR, "obj")
    os.makedirs(obj, exist_ok=True)
    inc = ["-I" + SHIM, "-I" + STAGED]
    arch = ["-gencode", "arch=compute_103a,code=sm_103a"]
    cu_o = os.path.join(obj, "model.cu.o")
    cpp_o = os.path.join(obj, "model.cpp.o")
    drv_o = os.path.join(obj, "ref_golden.o")
    jobs = [
        [NVCC, "-std=c++17", "-O2", *arch, *inc, "-c", os.path.join(STAGED, "model.cu"), "-o", cu_o],
        [NVCC, "-std=c++17", "-O2", *arch, *inc, "-x", "cu", "-c",
         os.path.join(STAGED, "model.cpp"), "-o", cpp_o],
        [NVCC, "-std=c++17", "-O2", *arch, *inc, "-x", "cu", "-c", DRIVER, "-o", drv_o],
    ]
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(max_workers=3) as ex:
        list(ex.map(_run, jobs))
    _run([NVCC, *arch, "-o", BIN + ".tmp", cu_o, cpp_o, drv_o, "-lcusolver", "-lcudart"])
    os.replace(BIN + ".tmp", BIN)
    return BIN


if __name__ == "__main__":
    what = sys.argv[1] if len(sys.argv) > 1 else "build"
    if what == "stage":
        print(stage())
    elif what == "build":
        print(build(force="--force" in sys.argv))
    else:
        raise SystemExit("usage: ref_build.py stage|build [--force]")
