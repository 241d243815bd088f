// select_kernel.cu -- post-global selection: prop-tube segment matching and
// global-track cleaning.
//
// Replaces gKernel_PropSegmentMatching (OnlineReconstruction/
// reconstruction_helper.cuh:1916-2277), gKernel_GlobalTrackCleaning
// (:2289-2331) and gKernel_GlobalTrackCleaning_crossthreads (:2333-2380),
// launched after global tracking (online_reconstruction.cu:914-933).
//
//  - Every track of a slot, whatever its stationID, that has no x and y
//    segment in the two prop-tube stations agreeing with it is given
//    stationID 5.  The reference's loops only raise a flag, so each test is
//    an existence test over the hits of the two stations.
//  - Global tracks (stationID 6) with chi2/(nhits-5) above 250 are demoted
//    to 5; of two same-charge global tracks whose 1/p agree within the merge
//    threshold (0.015, relative and signed), the worse chi2/(nhits-5) one is
//    demoted.  The within-slot pass compares invP(i) with itself in its
//    second branch (H:2323), so there the charge test alone decides.
//  - The cross-slot pass runs the reference block's 32 threads in lockstep,
//    as clean_kernel does: lane = slot, decisions of a step on the state
//    before it, demotions after a __syncwarp.
// One warp per event.
#include "or_device.cuh"

namespace orgpu {

constexpr float SEL_CHI2DOF_MAX = 250.f;  // reconstruction_constants.h:194
constexpr float SEL_MERGE_THRES = 0.015f; // :196

__device__ __forceinline__ bool prop_segment(float x0, float tx, const HitPlane &p1a, float z1a, const HitPlane &p1b,
                                             float z1b, const HitPlane &p2a, float z2a, const HitPlane &p2b, float z2b,
                                             float win1, float win2, float slope_max, float inter_max) {
    const float cut = 0.03f;  // H:1992, H:2000
    for (int s1 = 0; s1 < 2; ++s1) {
        const HitPlane &h1 = s1 ? p1b : p1a;
        const float z1 = s1 ? z1b : z1a;
        for (int n = 0; n < h1.n; ++n) {
            const float ipos1 = h1.pos(n);
            if (!(fabsf(ipos1 - (tx * z1 + x0)) < win1)) continue;
            for (int s2 = 0; s2 < 2; ++s2) {
                const HitPlane &h2 = s2 ? p2b : p2a;
                const float z2 = s2 ? z2b : z2a;
                for (int m = 0; m < h2.n; ++m) {
                    const float ipos2 = h2.pos(m);
                    if (fabsf(ipos2 - (tx * z2 + x0)) > win2) continue;
                    const float a = (ipos2 - ipos1) / (z2 - z1);
                    if (fabsf(a) > slope_max) continue;
                    if (fabsf(a - tx) > cut) continue;
                    const float b = ipos1 - a * z1;
                    if (fabsf(b) > inter_max) continue;
                    if (fabsf((tx * 2028.19f + x0) - (a * 2028.19f + b)) > 3.0f) continue;
                    return true;
                }
            }
        }
    }
    return false;
}

__device__ __forceinline__ float chi2dof(const float *T) { return T[OR_TRK_CHI2] / (T[OR_TRK_NHITS] - 5); }

template <int W>
__global__ void __launch_bounds__(W * 32)
    select_kernel(const or_plane_t *__restrict__ gplane, or_hits_view_t hv, or_tracks_view_t tv,
                  const uint8_t *__restrict__ toomany, int n_events, int do_prop, int do_clean) {
    __shared__ float zs[OR_NDET];
    for (int i = threadIdx.x; i < OR_NDET; i += blockDim.x) zs[i] = gplane->z[i];
    __syncthreads();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // prop-tube planes: x 50/49 and 52/51, y 48/47 and 54/53
    const int px1 = c_detsuperid[5][0] * 2, px2 = c_detsuperid[6][0] * 2;
    const int py1 = c_detsuperid[5][1] * 2, py2 = c_detsuperid[6][1] * 2;
    for (long e = (long)blockIdx.x * W + w; e < n_events; e += (long)gridDim.x * W) {
        if (toomany[e]) continue;
        const int n_own = min((int)tv.ntracks[e * OR_NSLOTS + lane], OR_SLOTCAP);
        if (do_prop) {
            const HitPlane p1x1 = hits_of(hv, e, px1), p1x2 = hits_of(hv, e, px1 - 1);
            const HitPlane p2x1 = hits_of(hv, e, px2), p2x2 = hits_of(hv, e, px2 - 1);
            const HitPlane p1y1 = hits_of(hv, e, py1), p1y2 = hits_of(hv, e, py1 - 1);
            const HitPlane p2y1 = hits_of(hv, e, py2), p2y2 = hits_of(hv, e, py2 - 1);
            for (int i = 0; i < n_own; ++i) {
                float *T = trk_rec(tv, e, lane, i);
                const float x0 = T[OR_TRK_X0], y0 = T[OR_TRK_Y0], tx = T[OR_TRK_TX], ty = T[OR_TRK_TY];
                if (!prop_segment(x0, tx, p1x1, zs[px1], p1x2, zs[px1 - 1], p2x1, zs[px2], p2x2, zs[px2 - 1], 5.08f,
                                  7.62f, 0.15f, 150.f) ||
                    !prop_segment(y0, ty, p1y1, zs[py1], p1y2, zs[py1 - 1], p2y1, zs[py2], p2y2, zs[py2 - 1], 5.08f,
                                  10.16f, 0.1f, 50.f))
                    T[OR_TRK_STID] = 5.f;
            }
            __syncwarp();
        }
        if (!do_clean) continue;
        // --- within the lane's slot (H:2289-2331) -----------------------------
        for (int i = 0; i < n_own; ++i) {
            float *Ti = trk_rec(tv, e, lane, i);
            if (Ti[OR_TRK_STID] < 6) continue;
            if (chi2dof(Ti) > SEL_CHI2DOF_MAX) {
                Ti[OR_TRK_STID] = 5.f;
                continue;
            }
            for (int j = i + 1; j < n_own; ++j) {
                float *Tj = trk_rec(tv, e, lane, j);
                if (Tj[OR_TRK_STID] < 6) continue;
                const bool same_q = Ti[OR_TRK_CHARGE] * Tj[OR_TRK_CHARGE] > 0;
                if (chi2dof(Ti) < chi2dof(Tj)) {
                    if ((Ti[OR_TRK_INVP] - Tj[OR_TRK_INVP]) / Ti[OR_TRK_INVP] < SEL_MERGE_THRES && same_q)
                        Tj[OR_TRK_STID] = 5.f;
                } else {
                    if ((Ti[OR_TRK_INVP] - Ti[OR_TRK_INVP]) / Tj[OR_TRK_INVP] < SEL_MERGE_THRES && same_q)
                        Ti[OR_TRK_STID] = 5.f;
                }
            }
        }
        __syncwarp();
        // --- across slots, in lockstep (H:2333-2380) --------------------------
        const int maxn = __reduce_max_sync(0xffffffffu, (unsigned)n_own);
        for (int u = 0; u < OR_NSLOTS; ++u) {
            const int m = __shfl_sync(0xffffffffu, n_own, u);
            if (m == 0) continue;
            for (int i = 0; i < maxn; ++i) {
                float *Ti = (i < n_own) ? trk_rec(tv, e, lane, i) : nullptr;
                const bool act = lane != u && Ti && Ti[OR_TRK_STID] >= 6;
                if (!__any_sync(0xffffffffu, act)) continue;
                for (int j = 0; j < m; ++j) {
                    float *Tj = trk_rec(tv, e, u, j);
                    const bool alive_j = Tj[OR_TRK_STID] >= 6;
                    int d = 0;
                    if (act && alive_j) {
                        const bool same_q = Ti[OR_TRK_CHARGE] * Tj[OR_TRK_CHARGE] > 0;
                        if (chi2dof(Ti) < chi2dof(Tj)) {
                            if ((Ti[OR_TRK_INVP] - Tj[OR_TRK_INVP]) / Ti[OR_TRK_INVP] < SEL_MERGE_THRES && same_q) d = 1;
                        } else {
                            if ((Ti[OR_TRK_INVP] - Tj[OR_TRK_INVP]) / Tj[OR_TRK_INVP] < SEL_MERGE_THRES && same_q) d = 2;
                        }
                    }
                    __syncwarp();
                    if (d == 1) Tj[OR_TRK_STID] = 5.f;
                    else if (d == 2) Ti[OR_TRK_STID] = 5.f;
                    __syncwarp();
                }
            }
        }
    }
}

template <int W>
static cudaError_t select_launch(const or_plane_t *d_plane, or_hits_view_t hv, or_tracks_view_t tv,
                                 const uint8_t *toomany, int n_events, int do_prop, int do_clean, cudaStream_t stream,
                                 int sm_count) {
    long blocks = (n_events + W - 1) / W;
    const long cap = (long)sm_count * (64 / W);
    if (blocks > cap) blocks = cap;
    select_kernel<W><<<(unsigned)blocks, W * 32, 0, stream>>>(d_plane, hv, tv, toomany, n_events, do_prop, do_clean);
    return cudaGetLastError();
}

cudaError_t launch_select(const or_plane_t *d_plane, or_hits_view_t hv, or_tracks_view_t tv, const uint8_t *toomany,
                          int n_events, int do_prop, int do_clean, cudaStream_t stream, int sm_count, int warps) {
    if (n_events <= 0) return cudaSuccess;
    switch (warps) {
    case 1: return select_launch<1>(d_plane, hv, tv, toomany, n_events, do_prop, do_clean, stream, sm_count);
    case 2: return select_launch<2>(d_plane, hv, tv, toomany, n_events, do_prop, do_clean, stream, sm_count);
    case 8: return select_launch<8>(d_plane, hv, tv, toomany, n_events, do_prop, do_clean, stream, sm_count);
    case 16: return select_launch<16>(d_plane, hv, tv, toomany, n_events, do_prop, do_clean, stream, sm_count);
    default: return select_launch<4>(d_plane, hv, tv, toomany, n_events, do_prop, do_clean, stream, sm_count);
    }
}

}  // namespace orgpu
