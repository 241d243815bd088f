"""Build the sm_103a library liborgpu.so in place (nvcc, no cmake).

Every CUDA source is compiled with -fmad=false: the kernels round each float
operation once, like the CPU oracle and a reference build at -fmad=false.

build(fmad=True) makes a second image, liborgpu_fmad1.so, with nvcc's default
multiply-add contraction -- the arithmetic of the reference as its Makefile
builds it.  It is a measurement variant for the parity report against that
build (tests/golden/make_golden.py), not the product.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "liborgpu.so")
OUT_FMAD1 = os.path.join(HERE, "liborgpu_fmad1.so")
BUILD = os.path.join(HERE, "_build")
CU = ["er_kernel.cu", "xz_kernel.cu", "yz_kernel.cu", "clean_kernel.cu", "global_kernel.cu", "pack_kernel.cu",
      "collect_kernel.cu", "learned_kernel.cu", "mlp_kernel.cu", "select_kernel.cu", "physics_kernel.cu", "output_kernel.cu",
      "yz_noalloc.cu",
      "capi.cu"]
CPP = ["geometry.cpp", "rt_calib.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
                     "-ftz=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build liborgpu.so")


def _deps():
    inc = os.path.join(os.path.dirname(HERE), "include")
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(inc, f) for f in os.listdir(inc)]
    return files + [os.path.abspath(__file__)]


def up_to_date(out=OUT):
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(force=False, verbose=False, fmad=False):
    out = OUT_FMAD1 if fmad else OUT
    if not force and up_to_date(out):
        return out
    nvcc = _nvcc()
    bdir = BUILD + ("_fmad1" if fmad else "")
    flags = [f.replace("-fmad=false", "-fmad=true") for f in NVCC_FLAGS] if fmad else NVCC_FLAGS
    os.makedirs(bdir, exist_ok=True)
    jobs = []
    for f in CU:
        jobs.append([nvcc] + flags + ["-c", os.path.join(CSRC, f), "-o", os.path.join(bdir, f + ".o")])
    for f in CPP:
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-c", os.path.join(CSRC, f),
                     "-o", os.path.join(bdir, f + ".o")])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)

    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        list(ex.map(run, jobs))
    objs = [os.path.join(bdir, f + ".o") for f in CU + CPP]
    run([nvcc] + ARCH + ["-shared", "-o", out + ".tmp"] + objs)
    os.replace(out + ".tmp", out)
    return out


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
