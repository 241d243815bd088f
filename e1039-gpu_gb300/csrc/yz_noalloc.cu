// yz_noalloc.cu -- the YZ tracklet stage on a statically reserved scratch area.
//
// or_yz() runs on the scratch that or_create() allocates (about 10.8 GB: the
// work queue, per-warp arenas, the survivor pool and the window images).  Some callers cannot
// allocate device memory when they call: a trigger or serving process that
// hands all free HBM to its own pool at start-up, or a latency-critical loop
// that must not call cudaMalloc/cudaFree (both synchronise the device).
// or_yz_noalloc() serves them: it needs no library context, allocates
// nothing, and runs the same plan/work/apply kernels as or_yz() on a fixed
// area reserved in this file:
//
//   - the area is a file-scope __device__ array of OR_YZ_NOALLOC_SCRATCH_BYTES
//     (56 MiB), reserved by the CUDA runtime when this module is loaded on a
//     device;
//   - the first call on a device, with that device current, looks the
//     array's address up once (cudaGetSymbolAddress) and caches it per
//     device; later calls reuse it.  Make that first call before any stream
//     capture.  The cached address is that of the device's context at the
//     first call: cudaDeviceReset() reloads the module, the array may move,
//     and later calls on that device would use a stale address, so a
//     process that resets a device must not call or_yz_noalloc() on it
//     again;
//   - a call takes at most OR_YZ_NOALLOC_MAX_EVENTS events; larger batches are
//     rejected with OR_ERR_CAPACITY before anything is launched;
//   - the queue counters, the only part that must start at zero, are cleared
//     on the caller's stream by each call (cudaMemsetAsync);
//   - there is one area per device: calls that overlap on a device (two
//     streams, or two host threads) race on it and corrupt each other's
//     results.  Serialise them.
//
// The queue is smaller than or_yz()'s (65,536 units and 16,384 heavy
// tracklets against a context's 4 Mi and 2 Mi; 1,216 work warps).  A
// tracklet that finds the queue full is evaluated by its planning warp
// instead, so the results are the same as or_yz()'s for every batch; only the
// time changes.
#include <mutex>

#include "../../include/or_gb300.h"
#include "or_device.cuh"

namespace orgpu {
cudaError_t launch_yz(const or_plane_t *, or_hits_view_t, or_tracks_view_t, const uint8_t *, int, uint32_t *, void *,
                      int, int, int, cudaStream_t, int);
size_t yz_scratch_bytes(int, int, int);

namespace {
constexpr int NOALLOC_UNITS = 65536;
constexpr int NOALLOC_HEAVY = 16384;
constexpr int NOALLOC_WARPS_MAX = 1216;  // 8 warps per SM on 152 SMs
constexpr int NOALLOC_MAX_DEVICES = 64;

static __device__ __align__(256) unsigned char g_yz_static_scratch[OR_YZ_NOALLOC_SCRATCH_BYTES];

struct DeviceScratch {
    bool ready = false;
    void *ptr = nullptr;
    int sm_count = 0;
    int warps = 0;
};
std::mutex g_setup_mutex;
DeviceScratch g_dev[NOALLOC_MAX_DEVICES];
}  // namespace

// Look the static area up on the current device (first call only).
// Returns the cudaError_t of the failing call; cudaErrorInvalidDevice with
// *why set when the device index is above the per-device table, and
// cudaErrorInvalidValue with *why set when the area is smaller than the queue.
cudaError_t yz_noalloc_scratch(int *device, DeviceScratch **out, const char **why) {
    *why = nullptr;
    cudaError_t e = cudaGetDevice(device);
    if (e != cudaSuccess) return e;
    if (*device < 0 || *device >= NOALLOC_MAX_DEVICES) {
        *why = "device index above the static scratch table (64 devices)";
        return cudaErrorInvalidDevice;
    }
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    DeviceScratch &d = g_dev[*device];
    if (!d.ready) {
        void *ptr = nullptr;
        if ((e = cudaGetSymbolAddress(&ptr, g_yz_static_scratch)) != cudaSuccess) return e;
        int sm = 0;
        if ((e = cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, *device)) != cudaSuccess) return e;
        int warps = sm * 8;
        if (warps > NOALLOC_WARPS_MAX) warps = NOALLOC_WARPS_MAX;
        warps &= ~3;  // whole 4-warp blocks
        if (warps < 4) warps = 4;
        if (yz_scratch_bytes(NOALLOC_UNITS, NOALLOC_HEAVY, warps) > sizeof(g_yz_static_scratch)) {
            *why = "static scratch smaller than the queue it must hold";
            return cudaErrorInvalidValue;
        }
        d.ptr = ptr;
        d.sm_count = sm;
        d.warps = warps;
        d.ready = true;
    }
    *out = &d;
    return cudaSuccess;
}

cudaError_t launch_yz_noalloc(const or_plane_t *d_plane, or_hits_view_t hv, or_tracks_view_t tv,
                              const uint8_t *toomany, int n_events, uint32_t *errw, cudaStream_t stream,
                              const char **why) {
    int dev = 0;
    DeviceScratch *d = nullptr;
    cudaError_t e = yz_noalloc_scratch(&dev, &d, why);
    if (e != cudaSuccess) return e;
    return launch_yz(d_plane, hv, tv, toomany, n_events, errw, d->ptr, NOALLOC_UNITS, NOALLOC_HEAVY, d->warps,
                     stream, d->sm_count);
}

}  // namespace orgpu
