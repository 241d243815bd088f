// window_pairs.cuh -- make_hitpairs_in_station with an x window
// (OnlineReconstruction/reconstruction_helper.cuh:464-549), warp-cooperative.
//
// Hits of the two planes of one projection whose wire spans overlap
// [xmin, xmax] are kept in order; pairs closer than the projection's
// spacing are listed in (hit1, hit2) order, then the unpaired hits of plane
// 1, then those of plane 2 -- the reference's order, kept with ballot ranks.
#pragma once
#include "or_device.cuh"

namespace orgpu {

constexpr int WP_MAXHITS = 200;

struct WindowScratch {
    short idx1[WP_MAXHITS], idx2[WP_MAXHITS];
    uint8_t fl1[WP_MAXHITS], fl2[WP_MAXHITS];
};

// Ordered append of the taking lanes' entries to out[*count...]; returns
// nothing, advances *count (warp-uniform) even beyond cap.
__device__ __forceinline__ void wp_append(bool take, short2 v, short2 *out, int cap, int &count) {
    const unsigned m = __ballot_sync(0xffffffffu, take);
    if (take) {
        const int k = count + __popc(m & lanemask_lt());
        if (k < cap) out[k] = v;
    }
    count += __popc(m);
}

__device__ __forceinline__ bool wp_in_window(int det, float chan, float xmin, float xmax, const or_plane_t &P) {
    const int el = (int)chan;
    float p1x, p2x;
    if (P.deltapx[det] > 0) {
        p1x = x_bep(det, el, P);
        p2x = x_tep(det, el, P);
    } else {
        p1x = x_tep(det, el, P);
        p2x = x_bep(det, el, P);
    }
    return (p1x <= xmax) && (p2x >= xmin);
}

// Returns the pair count (may exceed cap: entries past cap are not stored).
__device__ inline int window_pairs(const HitPlane &h1, int det1, const HitPlane &h2, int det2, float spacing, float xmin,
                            float xmax, const or_plane_t &P, short2 *out, int cap, WindowScratch &W) {
    const int lane = lane_id();
    const int n1 = min(h1.n, WP_MAXHITS), n2 = min(h2.n, WP_MAXHITS);
    int c1 = 0, c2 = 0;
#pragma unroll 1
    for (int b = 0; b < n1; b += 32) {
        const int i = b + lane;
        const bool in = i < n1 && wp_in_window(det1, h1.chan(i), xmin, xmax, P);
        const unsigned m = __ballot_sync(0xffffffffu, in);
        if (in) {
            const int k = c1 + __popc(m & lanemask_lt());
            W.idx1[k] = (short)i;
            W.fl1[k] = 0;
        }
        c1 += __popc(m);
    }
#pragma unroll 1
    for (int b = 0; b < n2; b += 32) {
        const int i = b + lane;
        const bool in = i < n2 && wp_in_window(det2, h2.chan(i), xmin, xmax, P);
        const unsigned m = __ballot_sync(0xffffffffu, in);
        if (in) {
            const int k = c2 + __popc(m & lanemask_lt());
            W.idx2[k] = (short)i;
            W.fl2[k] = 0;
        }
        c2 += __popc(m);
    }
    __syncwarp();
    int np = 0;
    const int nn = c1 * c2;
#pragma unroll 1
    for (int b = 0; b < nn; b += 32) {
        const int c = b + lane;
        bool take = false;
        short2 v = make_short2(0, 0);
        if (c < nn) {
            const int a = c / c2, bb = c - a * c2;
            const int i = W.idx1[a], j = W.idx2[bb];
            if (!(fabsf(h1.pos(i) - h2.pos(j)) > spacing)) {
                take = true;
                v = make_short2((short)i, (short)j);
                W.fl1[a] = 1;
                W.fl2[bb] = 1;
            }
        }
        wp_append(take, v, out, cap, np);
    }
    __syncwarp();
#pragma unroll 1
    for (int b = 0; b < c1; b += 32) {
        const int a = b + lane;
        const bool take = a < c1 && !W.fl1[a];
        wp_append(take, make_short2(take ? W.idx1[a] : 0, -1), out, cap, np);
    }
#pragma unroll 1
    for (int b = 0; b < c2; b += 32) {
        const int a = b + lane;
        const bool take = a < c2 && !W.fl2[a];
        wp_append(take, make_short2(-1, take ? W.idx2[a] : 0), out, cap, np);
    }
    __syncwarp();
    return np;
}

}  // namespace orgpu
