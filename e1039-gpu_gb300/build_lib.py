"""Build the sm_103a library liborgpu.so in place (nvcc, no cmake).

Every CUDA source is compiled with -fmad=false: the kernels round each float
operation once, like the CPU oracle and a reference build at -fmad=false.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "liborgpu.so")
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


def up_to_date():
    if not os.path.exists(OUT):
        return False
    t = os.path.getmtime(OUT)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(force=False, verbose=False):
    if not force and up_to_date():
        return OUT
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    jobs = []
    for f in CU:
        jobs.append([nvcc] + NVCC_FLAGS + ["-c", os.path.join(CSRC, f), "-o", os.path.join(BUILD, f + ".o")])
    for f in CPP:
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-c", os.path.join(CSRC, f),
                     "-o", os.path.join(BUILD, f + ".o")])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)

    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        list(ex.map(run, jobs))
    objs = [os.path.join(BUILD, f + ".o") for f in CU + CPP]
    run([nvcc] + ARCH + ["-shared", "-o", OUT + ".tmp"] + objs)
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
