"""Builds the neon_gb300 CUDA library in-tree (sm_103a only).

Every ``csrc/*.cu`` and ``csrc/*.cpp`` file is compiled in parallel with nvcc
(``-gencode arch=compute_103a,code=sm_103a -lineinfo -O3``) into
``neon_gb300/_build/libneon_gb300.so``. Translation units that must keep the
IEEE operation order of FP64 reference arithmetic are compiled with
``--fmad=false``.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD_DIR = os.path.join(HERE, "_build")
LIB_NAME = "libneon_gb300.so"
LIB_PATH = os.path.join(BUILD_DIR, LIB_NAME)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "--expt-relaxed-constexpr",
          "-I", INCLUDE, "-I", CSRC]
# FP64 reference-arithmetic units: no contraction into FMA.
NO_FMAD = {"lbm_dense_f64.cu", "lbm_shifted.cu", "bgrid_lbm.cu", "poisson.cu"}


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h", ".hpp"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _compile(src, extra, verbose):
    obj = os.path.join(BUILD_DIR, src + ".o")
    flags = list(COMMON) + list(extra)
    if src in NO_FMAD:
        flags.append("--fmad=false")
    cmd = [nvcc()] + ARCH + flags + ["-c", os.path.join(CSRC, src), "-o", obj]
    if src.endswith(".cpp"):
        cmd = [nvcc()] + ARCH + flags + ["-x", "cu", "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    if verbose and r.stderr.strip():
        print(r.stderr)
    return obj


def stale():
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    files = [os.path.join(CSRC, s) for s in _sources()] + _headers() + [os.path.abspath(__file__)]
    return any(os.path.getmtime(f) > t for f in files)


def build(force=False, verbose=False, extra=()):
    """Compile the library if any source is newer than it. Returns its path."""
    if not force and not stale():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(16, max(1, os.cpu_count() or 1))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra, verbose), srcs))
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    cudalib = os.path.join(os.path.dirname(os.path.dirname(nvcc())), "lib64")
    cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "shared", "-o", tmp] + objs + \
        ["-Xlinker", "-rpath," + cudalib]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True))
