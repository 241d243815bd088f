// collect_kernel.cu -- gather the final tracks of a batch into one dense
// buffer for the device-to-host copy.
//
// The reference copies whole collections back and walks them on the host to
// fill its output tree (OnlineReconstruction/online_reconstruction.cu
// :1023-1224, OROutput.h:25-102); a 10000-event track collection is 3 GB.
// Here the tracks with stationID == `stid` (6 = global tracks) are written as
// OR_COLLECT_STRIDE-float rows [event, slot*16+position, 148-float record],
// so only the tracks cross PCIe/C2C.  One thread per event counts its tracks,
// a block scan orders them, one atomicAdd per block reserves output rows.
// Row order across blocks is not fixed; every row carries its event and slot.
#include "or_device.cuh"

namespace orgpu {

constexpr int CO_THREADS = 256;

__global__ void __launch_bounds__(CO_THREADS)
    collect_kernel(or_tracks_view_t tv, const uint8_t *__restrict__ toomany, int n_events, float stid,
                   float *__restrict__ out, long long capacity, unsigned long long *__restrict__ cursor) {
    __shared__ int warp_tot[CO_THREADS / 32];
    __shared__ unsigned long long base;
    const long e = (long)blockIdx.x * CO_THREADS + threadIdx.x;
    int cnt = 0;
    if (e < n_events && !toomany[e]) {
        for (int s = 0; s < OR_NSLOTS; ++s) {
            const int n = min((int)tv.ntracks[e * OR_NSLOTS + s], OR_SLOTCAP);
            for (int k = 0; k < n; ++k) cnt += trk_rec(tv, e, s, k)[OR_TRK_STID] == stid;
        }
    }
    // block exclusive scan of the counts
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    if (lane == 31) warp_tot[w] = incl;
    __syncthreads();
    if (threadIdx.x == 0) {
        int s = 0;
        for (int i = 0; i < CO_THREADS / 32; ++i) {
            const int t = warp_tot[i];
            warp_tot[i] = s;
            s += t;
        }
        base = s ? atomicAdd(cursor, (unsigned long long)s) : 0ull;
    }
    __syncthreads();
    long long row = (long long)base + warp_tot[w] + incl - cnt;
    if (cnt == 0) return;
    for (int s = 0; s < OR_NSLOTS; ++s) {
        const int n = min((int)tv.ntracks[e * OR_NSLOTS + s], OR_SLOTCAP);
        for (int k = 0; k < n; ++k) {
            const float *r = trk_rec(tv, e, s, k);
            if (r[OR_TRK_STID] != stid) continue;
            if (row < capacity) {
                float *o = out + row * OR_COLLECT_STRIDE;
                o[0] = (float)e;
                o[1] = (float)(s * OR_SLOTCAP + k);
                for (int f = 0; f < OR_NTRKPARAM; ++f) o[2 + f] = r[f];
            }
            ++row;
        }
    }
}

cudaError_t launch_collect(or_tracks_view_t tv, const uint8_t *toomany, int n_events, float stid, float *out,
                           long long capacity, unsigned long long *cursor, cudaStream_t stream) {
    if (n_events <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(cursor, 0, sizeof(unsigned long long), stream);
    if (e != cudaSuccess) return e;
    const unsigned blocks = (unsigned)((n_events + CO_THREADS - 1) / CO_THREADS);
    collect_kernel<<<blocks, CO_THREADS, 0, stream>>>(tv, toomany, n_events, stid, out, capacity, cursor);
    return cudaGetLastError();
}

}  // namespace orgpu
