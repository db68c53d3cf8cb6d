"""Builds the CUDA library librast.so (sm_103a) in-tree under rusterizer_gb300/_build/.

nvcc flags that the pipeline's bit-exactness depends on: --fmad=false (no a*b+c contraction
on the device), IEEE division and square root (no --use_fast_math), and -ffp-contract=off for
the host compiler (the host folds P*V*W with the reference's dot order).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "librast.so")
SOURCES = ["rast_kernels.cu", "rast_api.cu", "rast_noalloc.cu", "rast_batch.cu", "rast_server.cu"]
HEADERS = ["rast_device.cuh", "rast_raster_warp.cuh", "rast_types.h", "rast_kernels.h", "rast_internal.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-prec-div=true",
                  "-prec-sqrt=true", "-ftz=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
                  "-I" + os.path.join(os.path.dirname(HERE), "include")]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    deps = [os.path.join(CSRC, f) for f in SOURCES + HEADERS]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "rast.h"))
    deps.append(__file__)
    newest = max(os.path.getmtime(p) for p in deps)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    nvcc = _nvcc()
    procs, objs = [], []
    for src in SOURCES:
        obj = os.path.join(OUT, src.replace(".cu", ".o"))
        objs.append(obj)
        cmd = [nvcc] + NVFLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0 or verbose:
            sys.stderr.write(out.decode(errors="replace"))
        if p.returncode != 0:
            raise RuntimeError("nvcc failed: " + " ".join(cmd))
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
