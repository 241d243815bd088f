// ref_kernels.cu -- translation unit that compiles the reference's own path
// kernels, unchanged, from their sources (OnlineReconstruction/
// reconstruction_kernels.cuh and the headers it includes) into a device
// image.  TEST INFRASTRUCTURE ONLY: the image is the reference the oracle is
// pinned against; nothing in the library loads it.
//
// The reference's headers are found through -I at build time
// (oracle/ref/build_ref.py); this file holds no reference code.  xz_pin.cuh
// adds a test-only kernel that runs the XZ stage's per-thread candidate loop
// on the reference's helpers (its XZ kernel itself cannot be run).
#include <cassert>
#include <thrust/pair.h>

#include "reconstruction_kernels.cuh"
#include "xz_pin.cuh"
