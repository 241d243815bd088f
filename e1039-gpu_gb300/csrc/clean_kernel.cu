// clean_kernel.cu -- duplicate removal among YZ tracks (back-track cleaning).
//
// Replaces gKernel_BackTrackCleaning (OnlineReconstruction/
// reconstruction_helper.cuh:1789-1843) and
// gKernel_BackTrackCleaning_crossthreads (:1846-1909).
//
// For two tracks with stationID >= 5 the one with the worse chi2/(nhits-4)
// is demoted to stationID 3 when the shared (detector, element) hits exceed a
// third of its hits; the shared-hit counter keeps accumulating over the
// partners of one track, as the reference's does.  The reference's
// cross-slot pass runs its 32 threads concurrently on shared records, so its
// outcome depends on timing; here the slots are visited in order 0..31, a
// deterministic order the CPU oracle shares.  One warp per event: the loops
// over tracks are warp-uniform and each hit-overlap count is done by the
// lanes (one hit of the first track per lane) with a ballot.
#include "or_device.cuh"

namespace orgpu {

constexpr int CL_WARPS = 4;

__device__ __forceinline__ int common_hits(const float *A, int na, const float *B, int nb) {
    const int lane = lane_id();
    bool f = false;
    if (lane < na) {
        const float d = A[OR_TRK_HIT_DETID + lane], c = A[OR_TRK_HIT_CHAN + lane];
        for (int j = 0; j < nb; ++j) {
            if (B[OR_TRK_HIT_DETID + j] == d && B[OR_TRK_HIT_CHAN + j] == c) {
                f = true;
                break;
            }
        }
    }
    return __popc(__ballot_sync(0xffffffffu, f));
}

// one comparison step of either pass (H:1819-1838 / H:1886-1904)
__device__ __forceinline__ void clean_pair(float *Ti, float *Tj, int &nc) {
    const short ni = (short)min((int)Ti[OR_TRK_NHITS], OR_MAXHITS_PER_TRACK);
    const short nj = (short)min((int)Tj[OR_TRK_NHITS], OR_MAXHITS_PER_TRACK);
    nc += common_hits(Ti, ni, Tj, nj);
    if (lane_id() == 0) {
        if (Ti[OR_TRK_CHI2] / (float)(ni - 4) < Tj[OR_TRK_CHI2] / (float)(nj - 4)) {
            if ((float)nc > (float)ni * 0.3333f) Tj[OR_TRK_STID] = 3.f;
        } else {
            if ((float)nc > (float)nj * 0.3333f) Ti[OR_TRK_STID] = 3.f;
        }
    }
    __syncwarp();
}

__global__ void __launch_bounds__(CL_WARPS * 32)
    clean_kernel(or_tracks_view_t tv, const uint8_t *__restrict__ toomany, int n_events) {
    const int w = threadIdx.x >> 5;
    for (long e = (long)blockIdx.x * CL_WARPS + w; e < n_events; e += (long)gridDim.x * CL_WARPS) {
        if (toomany[e]) continue;
        const uint16_t *nt = tv.ntracks + e * OR_NSLOTS;
        // within each slot
        for (int s = 0; s < OR_NSLOTS; ++s) {
            const int n = min((int)nt[s], OR_SLOTCAP);
            for (int i = 0; i < n; ++i) {
                float *Ti = trk_rec(tv, e, s, i);
                if (Ti[OR_TRK_STID] < 5) continue;
                int nc = 0;
                for (int j = i + 1; j < n; ++j) {
                    float *Tj = trk_rec(tv, e, s, j);
                    if (Tj[OR_TRK_STID] < 5) continue;
                    clean_pair(Ti, Tj, nc);
                }
            }
        }
        // across slots, slot t against every other slot u
        for (int t = 0; t < OR_NSLOTS; ++t) {
            const int n = min((int)nt[t], OR_SLOTCAP);
            if (n == 0) continue;
            for (int u = 0; u < OR_NSLOTS; ++u) {
                if (u == t) continue;
                const int m = min((int)nt[u], OR_SLOTCAP);
                if (m == 0) continue;
                for (int i = 0; i < n; ++i) {
                    float *Ti = trk_rec(tv, e, t, i);
                    if (Ti[OR_TRK_STID] < 5) continue;
                    int nc = 0;
                    for (int j = 0; j < m; ++j) {
                        float *Tj = trk_rec(tv, e, u, j);
                        if (Tj[OR_TRK_STID] < 5) continue;
                        clean_pair(Ti, Tj, nc);
                    }
                }
            }
        }
    }
}

cudaError_t launch_back_clean(or_tracks_view_t tv, const uint8_t *toomany, int n_events, cudaStream_t stream,
                              int sm_count) {
    if (n_events <= 0) return cudaSuccess;
    long blocks = (n_events + CL_WARPS - 1) / CL_WARPS;
    const long cap = (long)sm_count * 16;
    if (blocks > cap) blocks = cap;
    clean_kernel<<<(unsigned)blocks, CL_WARPS * 32, 0, stream>>>(tv, toomany, n_events);
    return cudaGetLastError();
}

}  // namespace orgpu
