"""Build the CUDA library libfjgpu.so in-tree for sm_103a.

    python -m fjmodels_gb300.build [--verbose]

Each translation unit compiles in parallel with nvcc, then one link step.
The library is rebuilt only when a source is newer than it.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfjgpu.so")
# Per translation unit: the FP64 plain form and the multipole kernels are built
# without FMA contraction.  The reference's algorithm has rounding-sensitive
# branches (bracket sign tests, the |f| < 5e-4 root shortcut, the switch of the
# quadratic interpolation point at mid-interval); with contracted arithmetic
# they take the other branch at a few nodes and densities move by ~1e-7,
# exactly as the reference's own sources do when compiled with contraction.
# The mixed-precision form is not a rounding-faithful restatement: it keeps
# contraction and uses the 2-ulp FP32 division and square root.
SOURCES = {"fj_moments.cu": ["--fmad=false"], "fj_multipole.cu": ["--fmad=false"], "fj_api.cu": [],
           "fj_peak.cu": [], "fj_noalloc.cu": [], "fj_moments_mixed.cu": ["-prec-div=false", "-prec-sqrt=false"], "fj_mlp.cu": [],
           "fj_los.cu": ["--fmad=false"], "fj_delta.cu": ["--fmad=false"]}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-Xcompiler", "-Wall,-Wno-unused-function,-Wno-unknown-pragmas,-ffp-contract=off"]


def nvcc():
    for c in (os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc"), "nvcc"):
        if os.path.sep not in c or os.path.exists(c):
            return c
    return "nvcc"


def _deps():
    root = os.path.dirname(HERE)
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".h"))]
    files.append(os.path.join(root, "include", "fjgpu.h"))
    return files


def needs_build():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(f) > t for f in _deps())


def build(verbose=False, force=False):
    if not force and not needs_build():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()

    def one(src):
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        cmd = [cc, *ARCH, *FLAGS, *SOURCES[src], "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        return obj, r.stderr

    with cf.ThreadPoolExecutor(len(SOURCES)) as ex:
        results = list(ex.map(one, SOURCES))
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    tmp = LIB + ".tmp"
    r = subprocess.run([cc, *ARCH, "-shared", "-o", tmp, *[o for o, _ in results], "-lcudart", "-lpthread"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="--verbose" in sys.argv, force="--force" in sys.argv))
