// learned_kernel.cu -- inputs and outputs of the learned tracklet scorer.
//
// The scorer decides, per XZ tracklet, whether its YZ combinatorics
// (K:1320-1825, the dominant cost of the path) are worth evaluating.  This
// file holds the three kernels around it:
//
//   rows_kernel      row index of every tracklet: row_off[e] = tracklets of
//                    the events before e (slots in order, tracklets in slot
//                    order); flagged events own no rows;
//   features_kernel  16 float features per tracklet (OR_NFEAT), one row each:
//                    the XZ fit (x0, tx, errors, hit count, station-3 half),
//                    the hits in the eight u/v planes, and, per u2/v2/u3/v3
//                    projection, how many hits
//                    lie in the YZ window and how many of those give a y in
//                    the acceptance -- the window test of make_hitpairs_in
//                    _station (H:480-511) and calculate_y_uvhit (H:75-100) on
//                    the tracklet's windows (K:1252-1283);
//   keep_kernel      keep mask from the scores: a tracklet is kept when its
//                    score reaches t_keep; an event with any score in
//                    [t_unc, t_keep) is uncertain and keeps all its
//                    tracklets (re-run plain).
//
// Rows past the caller's capacity (max_rows) get no features and no score and
// are always kept.  A pruned tracklet is left exactly as the plain YZ stage
// leaves a tracklet that no combination extends (stationID 3, K:1285); kept
// tracklets get the plain result bit for bit.
#include "../../include/or_gb300.h"
#include "or_device.cuh"
#include "window_pairs.cuh"

namespace orgpu {

constexpr int RW_THREADS = 1024;

// one block: per-thread segment sums, a block scan, segment rewrites
__global__ void __launch_bounds__(RW_THREADS)
    rows_kernel(const uint16_t *__restrict__ ntracks, const uint8_t *__restrict__ toomany, int n_events,
                int32_t *__restrict__ row_off) {
    __shared__ int warp_sum[RW_THREADS / 32];
    const int t = threadIdx.x;
    const int per = (n_events + RW_THREADS - 1) / RW_THREADS;
    const int e0 = min(t * per, n_events), e1 = min(e0 + per, n_events);
    auto count = [&](int e) -> int {
        if (toomany[e]) return 0;
        int c = 0;
        for (int s = 0; s < OR_NSLOTS; ++s) c += min((int)ntracks[(long)e * OR_NSLOTS + s], OR_SLOTCAP);
        return c;
    };
    int mine = 0;
    for (int e = e0; e < e1; ++e) mine += count(e);
    // block-wide exclusive scan of `mine`
    const int lane = t & 31, w = t >> 5;
    int incl = mine;
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    if (lane == 31) warp_sum[w] = incl;
    __syncthreads();
    if (w == 0) {
        int ws = warp_sum[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, ws, o);
            if (lane >= o) ws += v;
        }
        warp_sum[lane] = ws;  // inclusive
    }
    __syncthreads();
    int run = incl - mine + (w > 0 ? warp_sum[w - 1] : 0);
    for (int e = e0; e < e1; ++e) {
        row_off[e] = run;
        run += count(e);
    }
    if (t == RW_THREADS - 1) row_off[n_events] = warp_sum[RW_THREADS / 32 - 1];
}


template <int W>
__global__ void __launch_bounds__(W * 32)
    features_kernel(const or_plane_t *__restrict__ gplane, or_hits_view_t hv, or_tracks_view_t tv,
                    const uint8_t *__restrict__ toomany, int n_events, const int32_t *__restrict__ row_off,
                    float *__restrict__ feat, long max_rows) {
    __shared__ or_plane_t P;
    load_plane_smem(&P, gplane);
    __syncthreads();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (long e = (long)blockIdx.x * W + w; e < n_events; e += (long)gridDim.x * W) {
        if (toomany[e]) continue;
        // first row of every slot
        const int nslot = min((int)tv.ntracks[e * OR_NSLOTS + lane], OR_SLOTCAP);
        int incl = nslot;
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        const int slot_row = row_off[e] + incl - nslot;
        for (int slot = 0; slot < OR_NSLOTS; ++slot) {
            const int ntr = __shfl_sync(0xffffffffu, nslot, slot);
            const int r0 = __shfl_sync(0xffffffffu, slot_row, slot);
            if (ntr == 0) continue;
            const int st3 = 3 + (slot & 1);
            const short dl[8] = {DET_U2, DET_UP2, DET_V2, DET_VP2, (short)det_u3(st3), (short)(det_u3(st3) - 1),
                                 (short)det_v3(st3), (short)(det_v3(st3) - 1)};
            for (int it = 0; it < ntr; ++it) {
                const float *T = trk_rec(tv, e, slot, it);
                const float x0 = T[OR_TRK_X0], tx = T[OR_TRK_TX], ex0 = T[OR_TRK_ERR_X0], etx = T[OR_TRK_ERR_TX];
                int nwin[4], nacc[4], nall = 0;
                for (int q = 0; q < 4; ++q) {
                    const int a = 2 * q;
                    const float za = P.z[dl[a]], zb = P.z[dl[a + 1]];
                    const float sp = P.spacing[dl[a]];
                    const float xmin = fminf((tx - etx) * za, (tx - etx) * zb) + x0 - ex0 - sp;
                    const float xmax = fmaxf((tx + etx) * za, (tx + etx) * zb) + x0 + ex0 + sp;
                    int cw = 0, ca = 0;
                    for (int side = 0; side < 2; ++side) {
                        const int det = dl[a + side];
                        const HitPlane h = hits_of(hv, e, det);
                        nall += h.n;
                        for (int b0 = 0; b0 < h.n; b0 += 32) {
                            const int i = b0 + lane;
                            bool in = false, acc = false;
                            if (i < h.n) {
                                in = wp_in_window(det, h.chan(i), xmin, xmax, P);
                                if (in) {
                                    float yy, ey;
                                    acc = calculate_y_uvhit(det, (int)h.chan(i), h.drift(i), 0, x0, tx, P, yy, ey);
                                }
                            }
                            cw += __popc(__ballot_sync(0xffffffffu, in));
                            ca += __popc(__ballot_sync(0xffffffffu, acc));
                        }
                    }
                    nwin[q] = cw;
                    nacc[q] = ca;
                }
                if (lane < OR_NFEAT && (long)(r0 + it) < max_rows) {
                    float f = 0.f;
                    switch (lane) {
                    case 0: f = x0 * 0.01f; break;
                    case 1: f = tx * 10.f; break;
                    case 2: f = ex0; break;
                    case 3: f = etx * 100.f; break;
                    case 4: f = log1pf((float)nall); break;
                    case 5: f = T[OR_TRK_NHITS]; break;
                    case 6: f = (float)(slot & 1); break;
                    case 7: case 8: case 9: case 10: f = log1pf((float)nwin[lane - 7]); break;
                    case 11: case 12: case 13: case 14: f = log1pf((float)nacc[lane - 11]); break;
                    default:
                        f = log1pf((float)nacc[0]) + log1pf((float)nacc[1]) + log1pf((float)nacc[2]) +
                            log1pf((float)nacc[3]);
                        break;
                    }
                    feat[(long)(r0 + it) * OR_NFEAT + lane] = f;
                }
            }
        }
    }
}

__global__ void keep_kernel(const float *__restrict__ score, const int32_t *__restrict__ row_off, int n_events,
                            float t_keep, float t_unc, uint8_t *__restrict__ keep, long max_rows) {
    const int lane = threadIdx.x & 31;
    const long warp = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long nwarps = ((long)gridDim.x * blockDim.x) >> 5;
    for (long e = warp; e < n_events; e += nwarps) {
        const int r0 = row_off[e], r1 = (int)min((long)row_off[e + 1], max_rows);
        bool unc = false;
        for (int r = r0 + lane; r < r1; r += 32) unc |= (score[r] >= t_unc && score[r] < t_keep);
        unc = __any_sync(0xffffffffu, unc);
        for (int r = r0 + lane; r < r1; r += 32) keep[r] = (unc || score[r] >= t_keep) ? 1 : 0;
    }
}

// label of every row: 1 when the tracklet ended as a global track
// (stationID 6) in the run that produced `tv`
__global__ void labels_kernel(or_tracks_view_t tv, const uint8_t *__restrict__ toomany, int n_events,
                              const int32_t *__restrict__ row_off, uint8_t *__restrict__ label, long max_rows) {
    const int lane = threadIdx.x & 31;
    const long warp = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long nwarps = ((long)gridDim.x * blockDim.x) >> 5;
    for (long e = warp; e < n_events; e += nwarps) {
        if (toomany[e]) continue;
        const int nslot = min((int)tv.ntracks[e * OR_NSLOTS + lane], OR_SLOTCAP);
        int incl = nslot;
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        const long r0 = row_off[e] + incl - nslot;
        for (int k = 0; k < nslot; ++k)
            if (r0 + k < max_rows) label[r0 + k] = trk_rec(tv, e, lane, k)[OR_TRK_STID] == 6.f ? 1 : 0;
    }
}

// agreement of two runs on the same events: [0] global tracks (stationID 6)
// of run a, [1] of those the identical record in run b, [2] global tracks of b
__global__ void agreement_kernel(or_tracks_view_t ta, or_tracks_view_t tb, const uint8_t *__restrict__ toomany,
                                 int n_events, unsigned long long *__restrict__ counts) {
    const int lane = threadIdx.x & 31;
    const long warp = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long nwarps = ((long)gridDim.x * blockDim.x) >> 5;
    unsigned long long na = 0, nm = 0, nb = 0;
    for (long e = warp; e < n_events; e += nwarps) {
        if (toomany[e]) continue;
        const int n = min((int)ta.ntracks[e * OR_NSLOTS + lane], OR_SLOTCAP);
        const int m = min((int)tb.ntracks[e * OR_NSLOTS + lane], OR_SLOTCAP);
        for (int k = 0; k < max(n, m); ++k) {
            const uint32_t *ra = k < n ? reinterpret_cast<const uint32_t *>(trk_rec(ta, e, lane, k)) : nullptr;
            const uint32_t *rb = k < m ? reinterpret_cast<const uint32_t *>(trk_rec(tb, e, lane, k)) : nullptr;
            const bool ga = ra && __uint_as_float(ra[OR_TRK_STID]) == 6.f;
            const bool gb = rb && __uint_as_float(rb[OR_TRK_STID]) == 6.f;
            na += ga;
            nb += gb;
            if (ga && gb) {
                bool same = true;
                for (int f = 0; f < OR_NTRKPARAM && same; ++f) same = ra[f] == rb[f];
                nm += same;
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        na += __shfl_xor_sync(0xffffffffu, na, o);
        nm += __shfl_xor_sync(0xffffffffu, nm, o);
        nb += __shfl_xor_sync(0xffffffffu, nb, o);
    }
    if (lane == 0) {
        atomicAdd(&counts[0], na);
        atomicAdd(&counts[1], nm);
        atomicAdd(&counts[2], nb);
    }
}

cudaError_t launch_labels(or_tracks_view_t tv, const uint8_t *toomany, int n_events, const int32_t *row_off,
                          uint8_t *label, long max_rows, cudaStream_t stream, int sm_count) {
    if (n_events <= 0) return cudaSuccess;
    long blocks = (n_events + 7) / 8;
    const long cap = (long)sm_count * 16;
    if (blocks > cap) blocks = cap;
    labels_kernel<<<(unsigned)blocks, 256, 0, stream>>>(tv, toomany, n_events, row_off, label, max_rows);
    return cudaGetLastError();
}

cudaError_t launch_agreement(or_tracks_view_t ta, or_tracks_view_t tb, const uint8_t *toomany, int n_events,
                             unsigned long long *counts, cudaStream_t stream, int sm_count) {
    cudaError_t err = cudaMemsetAsync(counts, 0, 3 * sizeof(unsigned long long), stream);
    if (err != cudaSuccess || n_events <= 0) return err;
    long blocks = (n_events + 7) / 8;
    const long cap = (long)sm_count * 16;
    if (blocks > cap) blocks = cap;
    agreement_kernel<<<(unsigned)blocks, 256, 0, stream>>>(ta, tb, toomany, n_events, counts);
    return cudaGetLastError();
}

cudaError_t launch_rows(const uint16_t *ntracks, const uint8_t *toomany, int n_events, int32_t *row_off,
                        cudaStream_t stream) {
    if (n_events <= 0) return cudaMemsetAsync(row_off, 0, sizeof(int32_t), stream);
    rows_kernel<<<1, RW_THREADS, 0, stream>>>(ntracks, toomany, n_events, row_off);
    return cudaGetLastError();
}

template <int W>
static cudaError_t features_launch(const or_plane_t *d_plane, or_hits_view_t hv, or_tracks_view_t tv,
                                   const uint8_t *toomany, int n_events, const int32_t *row_off, float *feat,
                                   long max_rows, cudaStream_t stream, int sm_count) {
    long blocks = (n_events + W - 1) / W;
    const long cap = (long)sm_count * (64 / W);
    if (blocks > cap) blocks = cap;
    features_kernel<W><<<(unsigned)blocks, W * 32, 0, stream>>>(d_plane, hv, tv, toomany, n_events, row_off, feat,
                                                               max_rows);
    return cudaGetLastError();
}

cudaError_t launch_features(const or_plane_t *d_plane, or_hits_view_t hv, or_tracks_view_t tv, const uint8_t *toomany,
                            int n_events, const int32_t *row_off, float *feat, long max_rows, cudaStream_t stream,
                            int sm_count, int warps) {
    if (n_events <= 0) return cudaSuccess;
    switch (warps) {
    case 1: return features_launch<1>(d_plane, hv, tv, toomany, n_events, row_off, feat, max_rows, stream, sm_count);
    case 2: return features_launch<2>(d_plane, hv, tv, toomany, n_events, row_off, feat, max_rows, stream, sm_count);
    case 8: return features_launch<8>(d_plane, hv, tv, toomany, n_events, row_off, feat, max_rows, stream, sm_count);
    case 16: return features_launch<16>(d_plane, hv, tv, toomany, n_events, row_off, feat, max_rows, stream, sm_count);
    default: return features_launch<4>(d_plane, hv, tv, toomany, n_events, row_off, feat, max_rows, stream, sm_count);
    }
}

cudaError_t launch_keep(const float *score, const int32_t *row_off, int n_events, float t_keep, float t_unc,
                        uint8_t *keep, long max_rows, cudaStream_t stream, int sm_count) {
    if (n_events <= 0) return cudaSuccess;
    long blocks = (n_events + 7) / 8;
    const long cap = (long)sm_count * 16;
    if (blocks > cap) blocks = cap;
    keep_kernel<<<(unsigned)blocks, 256, 0, stream>>>(score, row_off, n_events, t_keep, t_unc, keep, max_rows);
    return cudaGetLastError();
}

}  // namespace orgpu
