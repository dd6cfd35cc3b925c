"""ORACLE — test infrastructure only.

Builds the reference's CPU backend from its own sources, where they lie in the
reference checkout, into ``oracle/_ref/libneon_ref.so`` (git-ignored), together
with ``oracle/ref_driver.cu``, the harness that runs the reference's D3Q19
cavity iteration and hands back its populations. The library pins the oracle
to outputs of the reference itself (``tests/test_ref_pin_cpu.py``).

What the recipe adds, and why (the reference's CMake build cannot run here: it
fetches spdlog, rapidjson, glm, libigl and GoogleTest from the network):

* ``oracle/ref_shim/``: stand-ins for the spdlog/rapidjson names that
  ``Neon/core/tools/Logger.h`` and ``Report.h`` use, for the two
  CMake-generated export headers and for the git-state source CMake
  configures from ``cmake/git_sha1.cpp.in``;
* ``-include cstring -include cassert`` on every file: a few reference headers
  use ``std::memcpy`` / ``assert`` without including them (older standard
  libraries pulled them in transitively);
* ``cub::Sum`` for the three files that name it (CUDA 13's CUB dropped it in
  favour of ``cuda::std::plus``): a forced include defines it;
* the GPU-information printouts of ``gpuDeviceTools.cpp`` and
  ``libNeonSys/src/sys/Report.cpp`` read ``cudaDeviceProp`` fields that CUDA 13
  removed (``clockRate``, ``memoryClockRate``, ``computeMode``); for those two
  files the names are mapped to fields that still exist. A CPU run never
  reaches them.

Every source is compiled with nvcc as CUDA (the headers carry device lambdas;
the device code is compiled but never run) and linked with OpenMP.

    python oracle/ref_build.py [--force]
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("NEON_REFERENCE", "/root/reference")
OUT = os.path.join(HERE, "_ref")
OBJ = os.path.join(OUT, "obj")
LIB = os.path.join(OUT, "libneon_ref.so")
LIBS = ["libNeonCore", "libNeonSys", "libNeonSet", "libNeonDomain", "libNeonSkeleton"]
CAVITY = os.path.join("benchmarks", "lbm-lid-driven-cavity-flow", "src")

CUB_SUM = {"libNeonSys/src/sys/patterns/Blas.cu", "libNeonDomain/src/domain/details/dGrid/dFieldReduceKernels.cu",
           "libNeonDomain/src/domain/details/bGrid/bFieldReduceKernels.cu"}
PROP_NAMES = {"libNeonSys/src/sys/devices/gpu/gpuDeviceTools.cpp", "libNeonSys/src/sys/Report.cpp"}


def available():
    return os.path.isdir(os.path.join(REF, "libNeonCore")) and shutil.which("nvcc") is not None


def sources():
    out = []
    for lib in LIBS:
        for root, _, files in os.walk(os.path.join(REF, lib, "src")):
            for f in sorted(files):
                if f.endswith((".cpp", ".cu")):
                    out.append(os.path.relpath(os.path.join(root, f), REF))
    out.append(os.path.join(CAVITY, "Config.cpp"))
    return sorted(out)


def _flags():
    inc = ["-I", os.path.join(HERE, "ref_shim")] + sum([["-I", os.path.join(REF, l, "include")] for l in LIBS], [])
    inc += ["-I", os.path.join(REF, CAVITY)]
    return ["-std=c++17", "-O2", "-x", "cu", "--expt-extended-lambda", "--expt-relaxed-constexpr",
            "-gencode", "arch=compute_90,code=compute_90", "-w",
            "-Xcompiler", "-fopenmp", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
            "-include", "cstring", "-include", "cassert"] + inc


def _compile(rel, src_path):
    obj = os.path.join(OBJ, rel.replace("/", "_") + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= os.path.getmtime(src_path):
        return obj
    cmd = ["nvcc"] + _flags()
    if rel in CUB_SUM:
        cmd += ["-include", os.path.join(HERE, "ref_shim", "cub_sum.h")]
    if rel in PROP_NAMES:
        cmd += ["-DclockRate=clockRateRemovedInCuda13", "-DmemoryClockRate=memoryBusWidth",
                "-DcomputeMode=asyncEngineCount", "-DclockRateRemovedInCuda13=multiProcessorCount"]
    cmd += ["-c", src_path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed on %s:\n%s" % (rel, r.stderr[-4000:]))
    return obj


def build(force=False, jobs=None):
    """Compile the reference's libraries and the harness into oracle/_ref/. Returns the library path."""
    if not available():
        raise RuntimeError("reference sources or nvcc not available")
    if force and os.path.isdir(OUT):
        shutil.rmtree(OUT)
    os.makedirs(OBJ, exist_ok=True)
    units = [(s, os.path.join(REF, s)) for s in sources()] + [("ref_driver.cu", os.path.join(HERE, "ref_driver.cu")),
                                                                ("git_sha1.cpp", os.path.join(HERE, "ref_shim", "git_sha1.cpp"))]
    with cf.ThreadPoolExecutor(max_workers=jobs or os.cpu_count() or 4) as ex:
        objs = list(ex.map(lambda u: _compile(*u), units))
    newest = max(os.path.getmtime(o) for o in objs)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = ["nvcc", "-shared", "-Xcompiler", "-fopenmp", "-o", tmp] + objs + ["-lcudart", "-lcublas"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s" % r.stderr[-4000:])
        os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    """The loaded reference library (built on first use)."""
    global _lib
    if _lib is None:
        import ctypes
        build()
        L = ctypes.CDLL(LIB)
        L.ref_cavity_run.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                     ctypes.c_void_p, ctypes.c_void_p]
        L.ref_cavity_run.restype = ctypes.c_int
        _lib = L
    return _lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
