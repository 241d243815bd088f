"""Compile the reference's own path kernels into device images under
oracle/_ref/.  TEST INFRASTRUCTURE ONLY: the images pin the CPU oracle
against the reference; the library never loads them.

The reference is CUDA whose helpers are all __device__ functions, so it has
no CPU build; its kernels (OnlineReconstruction/reconstruction_kernels.cuh and
the headers it includes) compile as they are, with nvcc, from the reference
tree.  ref_kernels.cu includes them; this script passes the include path.

Two images are built:
  ref_kernels_fmad0.cubin   -fmad=false: one rounding per operation, the
                            arithmetic the oracle and the library use, so
                            the comparison is bit for bit;
  ref_kernels_fmad1.cubin   nvcc's default (-fmad=true), as the reference's
                            own Makefile builds it; fit parameters differ in
                            the last bits and are compared within 1e-5.
Both use -DNDEBUG so that the reference's device asserts compile out.

Only run where the reference sources exist; the images are device code and
are used unchanged on any host.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
# the reference tree: OR_REFERENCE_SRC, else a checkout named `reference`
# beside this repository
REF_SRC = os.environ.get("OR_REFERENCE_SRC",
                         os.path.join(os.path.dirname(ORACLE), "..", "reference", "OnlineReconstruction"))
WRAP = os.path.join(HERE, "ref_kernels.cu")
HARNESS = [os.path.join(HERE, "xz_pin.cuh")]
VARIANTS = {"fmad0": ["-fmad=false"], "fmad1": []}


def image_path(variant):
    return os.path.join(OUT, f"ref_kernels_{variant}.cubin")


def _headers():
    return [os.path.join(REF_SRC, f) for f in os.listdir(REF_SRC) if f.endswith((".cuh", ".h"))]


def _stale(path):
    if not os.path.exists(path):
        return True
    t = os.path.getmtime(path)
    return any(os.path.getmtime(s) > t for s in [WRAP, __file__] + HARNESS + _headers())


def _compile(variant):
    dst = image_path(variant)
    cmd = ["nvcc", "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O3", "-DNDEBUG",
           "-w", "-I", REF_SRC] + VARIANTS[variant] + ["-o", dst + ".tmp", WRAP]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference kernels ({variant}) failed to compile:\n{r.stderr[-4000:]}")
    os.replace(dst + ".tmp", dst)
    return dst


def build_if_sources(force=False):
    """Build both images when the reference tree is present; else do nothing.
    Returns the list of images (possibly empty)."""
    if not os.path.isfile(os.path.join(REF_SRC, "reconstruction_kernels.cuh")):
        return [image_path(v) for v in VARIANTS if os.path.exists(image_path(v))]
    os.makedirs(OUT, exist_ok=True)
    todo = [v for v in VARIANTS if force or _stale(image_path(v))]
    with ThreadPoolExecutor(len(VARIANTS)) as ex:
        list(ex.map(_compile, todo))
    return [image_path(v) for v in VARIANTS]


if __name__ == "__main__":
    print(build_if_sources(force="--force" in sys.argv))
