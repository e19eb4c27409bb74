"""Builds libcovgpu.so in place: every .cu with nvcc for sm_103a, every .c
with gcc, linked into one shared library next to this file.  Also
libcovsynth.so, the synthetic-alignment generator alone (host code of
cov_synth.cu), which the benchmark's CPU reference arm uses to make its
input without loading the GPU library."""
import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INC = os.path.join(ROOT, "include")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libcovgpu.so")
SYNTHLIB = os.path.join(HERE, "libcovsynth.so")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fopenmp", "-I", INC,
                  "-I", CSRC]
CFLAGS = ["-O2", "-fPIC", "-std=c11", "-fopenmp", "-D_DEFAULT_SOURCE", "-Wall", "-I", INC]


def _needs(src, obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in [src] + deps)


def _compile(job):
    src, obj, cmd = job
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj


def build(verbose=False, force=False):
    os.makedirs(OBJ, exist_ok=True)
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INC, "*.h"))
    jobs, objs = [], []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or _needs(src, obj, headers):
            jobs.append((src, obj, [NVCC] + NVFLAGS + ["-c", src, "-o", obj]))
    for src in sorted(glob.glob(os.path.join(CSRC, "*.c"))):
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or _needs(src, obj, headers):
            jobs.append((src, obj, ["gcc"] + CFLAGS + ["-c", src, "-o", obj]))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            for o in ex.map(_compile, jobs):
                if verbose:
                    print("built", os.path.basename(o))
    if force or jobs or not os.path.exists(LIB):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lm", "-Xcompiler", "-fopenmp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    if force or jobs or not os.path.exists(SYNTHLIB):
        cmd = [NVCC] + ARCH + ["-shared", "-o", SYNTHLIB, os.path.join(OBJ, "cov_synth.cu.o"), "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
