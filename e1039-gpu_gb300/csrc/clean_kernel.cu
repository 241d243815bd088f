// clean_kernel.cu -- duplicate removal among YZ tracks (back-track cleaning).
//
// Replaces gKernel_BackTrackCleaning (OnlineReconstruction/
// reconstruction_helper.cuh:1789-1843) and
// gKernel_BackTrackCleaning_crossthreads (:1846-1909).
//
// For two tracks with stationID >= 5 the one with the worse chi2/(nhits-4)
// is demoted to stationID 3 when the shared (detector, element) hits exceed a
// third of its hits; the shared-hit counter keeps accumulating over the
// partners of one track, as the reference's does.
//
// One warp per event, lane t = the reference's thread t = track slot t.
//  - The first pass touches only the lane's own slot, as in the reference.
//  - In the cross-slot pass the reference's 32 threads run the same loop
//    nest together: at step (i_trd, i, j) every thread t != i_trd compares
//    its track i with track j of slot i_trd, reading the stationIDs the
//    earlier steps left, and the demotions of the step land after it.  The
//    lanes follow that lockstep order exactly: read and decide, __syncwarp,
//    write, __syncwarp.  All writes store the same value (3), so lanes
//    demoting the same track do not conflict.
#include "or_device.cuh"

namespace orgpu {

// shared (detector, element) hits of A's hits found among B's, H:1810-1817
__device__ __forceinline__ int common_hits(const float *A, int na, const float *B, int nb) {
    int acc = 0;
    for (int ih = 0; ih < na; ++ih) {
        const float d = A[OR_TRK_HIT_DETID + ih], c = A[OR_TRK_HIT_CHAN + ih];
        for (int jh = 0; jh < nb; ++jh) {
            if (B[OR_TRK_HIT_DETID + jh] == d && B[OR_TRK_HIT_CHAN + jh] == c) {
                ++acc;
                break;
            }
        }
    }
    return acc;
}

// the comparison of H:1819-1838 / H:1886-1904: 1 = demote j, 2 = demote i
__device__ __forceinline__ int clean_decide(const float *Ti, int ni, const float *Tj, int nj, int nc) {
    if (Ti[OR_TRK_CHI2] / (float)(ni - 4) < Tj[OR_TRK_CHI2] / (float)(nj - 4))
        return ((float)nc > (float)ni * 0.3333f) ? 1 : 0;
    return ((float)nc > (float)nj * 0.3333f) ? 2 : 0;
}

template <int W>
__global__ void __launch_bounds__(W * 32)
    clean_kernel(or_tracks_view_t tv, const uint8_t *__restrict__ toomany, int n_events) {
    const int w = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    for (long e = (long)blockIdx.x * W + w; e < n_events; e += (long)gridDim.x * W) {
        if (toomany[e]) continue;
        const int n_own = min((int)tv.ntracks[e * OR_NSLOTS + lane], OR_SLOTCAP);
        // --- pass 1: the lane's own slot (H:1789-1843) ------------------------
        for (int i = 0; i < n_own; ++i) {
            float *Ti = trk_rec(tv, e, lane, i);
            if (Ti[OR_TRK_STID] < 5) continue;
            const int ni = min((int)(short)Ti[OR_TRK_NHITS], OR_MAXHITS_PER_TRACK);
            int nc = 0;
            for (int j = i + 1; j < n_own; ++j) {
                float *Tj = trk_rec(tv, e, lane, j);
                if (Tj[OR_TRK_STID] < 5) continue;
                const int nj = min((int)(short)Tj[OR_TRK_NHITS], OR_MAXHITS_PER_TRACK);
                nc += common_hits(Ti, ni, Tj, nj);
                const int d = clean_decide(Ti, ni, Tj, nj, nc);
                if (d == 1) Tj[OR_TRK_STID] = 3.f;
                else if (d == 2) Ti[OR_TRK_STID] = 3.f;
            }
        }
        __syncwarp();
        // --- pass 2: across slots, in lockstep (H:1846-1909) ------------------
        const int maxn = __reduce_max_sync(0xffffffffu, (unsigned)n_own);
        for (int u = 0; u < OR_NSLOTS; ++u) {
            const int m = __shfl_sync(0xffffffffu, n_own, u);
            if (m == 0) continue;
            for (int i = 0; i < maxn; ++i) {
                float *Ti = (i < n_own) ? trk_rec(tv, e, lane, i) : nullptr;
                const bool act = lane != u && Ti && Ti[OR_TRK_STID] >= 5;
                const int ni = act ? min((int)(short)Ti[OR_TRK_NHITS], OR_MAXHITS_PER_TRACK) : 0;
                if (!__any_sync(0xffffffffu, act)) continue;
                int nc = 0;
                for (int j = 0; j < m; ++j) {
                    float *Tj = trk_rec(tv, e, u, j);
                    const bool alive_j = Tj[OR_TRK_STID] >= 5;  // same record for every lane
                    int d = 0;
                    if (act && alive_j) {
                        const int nj = min((int)(short)Tj[OR_TRK_NHITS], OR_MAXHITS_PER_TRACK);
                        nc += common_hits(Ti, ni, Tj, nj);
                        d = clean_decide(Ti, ni, Tj, nj, nc);
                    }
                    __syncwarp();
                    if (d == 1) Tj[OR_TRK_STID] = 3.f;
                    else if (d == 2) Ti[OR_TRK_STID] = 3.f;
                    __syncwarp();
                }
            }
        }
    }
}

template <int W>
static cudaError_t clean_launch(or_tracks_view_t tv, const uint8_t *toomany, int n_events, cudaStream_t stream,
                                int sm_count) {
    long blocks = (n_events + W - 1) / W;
    const long cap = (long)sm_count * (64 / W);
    if (blocks > cap) blocks = cap;
    clean_kernel<W><<<(unsigned)blocks, W * 32, 0, stream>>>(tv, toomany, n_events);
    return cudaGetLastError();
}

cudaError_t launch_back_clean(or_tracks_view_t tv, const uint8_t *toomany, int n_events, cudaStream_t stream,
                              int sm_count, int warps) {
    if (n_events <= 0) return cudaSuccess;
    switch (warps) {
    case 1: return clean_launch<1>(tv, toomany, n_events, stream, sm_count);
    case 2: return clean_launch<2>(tv, toomany, n_events, stream, sm_count);
    case 8: return clean_launch<8>(tv, toomany, n_events, stream, sm_count);
    case 16: return clean_launch<16>(tv, toomany, n_events, stream, sm_count);
    default: return clean_launch<4>(tv, toomany, n_events, stream, sm_count);
    }
}

}  // namespace orgpu
