"""In-tree build of libasv.so (CUDA kernels for sm_103a + host C++).

The kernels with floating-point arithmetic are compiled with -fmad=false:
every float operation is one IEEE operation in the written order, which is
what makes the labels, metrics and flow bit-exact against the CPU
restatement.  The integer-only kernels (connectivity, evaluation, the
no-allocation post-processing) have no float multiply-add to contract, so
they build without the flag.
"""
import concurrent.futures
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libasv.so")
INCLUDE = os.path.join(ROOT, "include")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["asv_volume.cu", "asv_metric.cu", "asv_noalloc.cu", "asv_stream.cu", "asv_connect.cu",
              "asv_flow.cu", "asv_eval.cu"]
CPP_SOURCES = ["asv_api.cpp", "asv_synth.cpp", "asv_server.cpp", "asv_png.cpp", "asv_frames.cpp", "asv_render.cpp"]
HEADERS = ["asv_common.cuh", "asv_internal.h", "asv_stream.cuh", "asv_connect.cuh", "asv_flow.cuh",
           "asv_eval.cuh"]
PUBLIC_HEADERS = ["asv.h", "asv_host.h"]


def _sources():
    return ([os.path.join(CSRC, f) for f in CU_SOURCES + CPP_SOURCES + HEADERS]
            + [os.path.join(INCLUDE, f) for f in PUBLIC_HEADERS])


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(s) > t for s in _sources() if os.path.exists(s))


# translation units without floating-point arithmetic
INTEGER_ONLY = {"asv_connect.cu", "asv_eval.cu", "asv_noalloc.cu"}


def _nvcc_cmd(src, obj):
    fmad = [] if os.path.basename(src) in INTEGER_ONLY else ["-fmad=false"]
    return [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", *fmad, "-Xptxas", "-v",
            "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj]


def _cxx_cmd(src, obj):
    cxx = shutil.which("g++") or "g++"
    return [cxx, "-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-Wall",
            "-I", INCLUDE, "-I", CSRC, "-I", os.path.join(CUDA_HOME, "include"), "-c", src, "-o", obj]


def _run(cmd):
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("build failed:\n$ " + " ".join(cmd) + "\n" + p.stdout + p.stderr)
    return p.stdout + p.stderr


def build(force=False, verbose=False):
    """Compiles libasv.so in place (skipped when it is newer than its sources)."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    jobs = []
    for f in CU_SOURCES:
        jobs.append(_nvcc_cmd(os.path.join(CSRC, f), os.path.join(BUILD, f + ".o")))
    for f in CPP_SOURCES:
        jobs.append(_cxx_cmd(os.path.join(CSRC, f), os.path.join(BUILD, f + ".o")))
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        logs = list(ex.map(_run, jobs))
    with open(os.path.join(BUILD, "ptxas.log"), "w") as f:
        f.write("\n".join(logs))
    objs = [os.path.join(BUILD, f + ".o") for f in CU_SOURCES + CPP_SOURCES]
    tmp = LIB + ".tmp"
    _run([NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-Xcompiler", "-fopenmp", "-lgomp"])
    os.replace(tmp, LIB)
    if verbose:
        print("\n".join(logs))
    return LIB


if __name__ == "__main__":
    build(force=True, verbose=True)
