"""Build the SWE step library ``libsamoa_swe.so`` in-tree for sm_103a.

The C ABI (include/samoa_swe.h) is the product boundary; the library needs no
torch at build or run time. Compiled with ``--fmad=false`` so the FP64
arithmetic rounds exactly as the strict-IEEE CPU restatement does.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libsamoa_swe.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC,-O2,-fno-fast-math",
              "-Xcompiler", "-ffp-contract=off"]
SOURCES = ["swe_step.cu", "swe_mesh.cpp", "swe_geometry.cpp", "swe_noalloc.cu", "swe_step_fma.cu", "swe_adapt.cpp"]
# the FMA-contraction variant of the step kernels (an opt-in arithmetic mode)
FLAGS_OVERRIDE = {"swe_step_fma.cu": ["--fmad=true"]}


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(HERE, "..", "include", "samoa_swe.h"))
    return files


def _compile(src, extra):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    flags = [f for f in NVCC_FLAGS if not (f.startswith("--fmad") and src in FLAGS_OVERRIDE)]
    cmd = [_nvcc(), *ARCH, *flags, *FLAGS_OVERRIDE.get(src, []), *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    if src.endswith(".cpp"):
        cmd = [_nvcc(), "-x", "cu", *ARCH, *NVCC_FLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    subprocess.check_call(cmd)
    return obj


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    """Compile every CUDA/C++ source for sm_103a and link the shared library."""
    os.makedirs(BUILD, exist_ok=True)
    newest = max(os.path.getmtime(f) for f in _deps())
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.check_call([_nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force=True, verbose_ptxas="-v" in sys.argv))
