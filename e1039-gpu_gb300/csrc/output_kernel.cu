// output_kernel.cu -- the reference's per-event output as flat rows.
//
// Replaces the host loop online_reconstruction.cu:1063-1222, which walks the
// copied-back collections and pushes every field into the ROOT tree
// ORoutput_tree (OnlineReconstruction/OROutput.h:25-102): for each event with
// raw hits and no reject flag, its reduced hits (chambers, hodoscopes, prop
// tubes in plane order), its tracks with stationID >= 7 (the build without
// SAVE_ALL_TRACKS) with their hits, and its dimuons.  Here the same fields, in
// the tree's order, go into five row tables in device memory, events in batch
// order, so a host reads back only the rows (one copy per table).
//
// Three launches: counts per event (one warp per event), one block that scans
// them into row offsets, then the writes (one warp per event).
#include "or_device.cuh"

namespace orgpu {

struct OutCount {
    int acc, hits, tracks, thits, dims;
};
struct OutOffset {
    long long ev, hits, tracks, thits, dims;
};

__device__ __forceinline__ int plane_count(const or_hits_view_t &hv, long e, int det) {
    if (det <= OR_NCHAM) return (int)hv.nhits_cham[e * OR_NCHAM + det - 1];
    if (det <= OR_NCHAM + OR_NHODO) return (int)hv.nhits_hodo[e * OR_NHODO + det - OR_NCHAM - 1];
    return (int)hv.nhits_prop[e * OR_NPROP + det - OR_NCHAM - OR_NHODO - 1];
}

// the track's hit count as the host reads it (M:1138), within the record's 18
__device__ __forceinline__ int track_nhits(const float *T) {
    return max(0, min((int)T[OR_TRK_NHITS], OR_MAXHITS_PER_TRACK));
}

__global__ void __launch_bounds__(256)
    out_count_kernel(or_hits_view_t hv, or_tracks_view_t tv, or_dimuons_view_t dv, const uint8_t *__restrict__ toomany,
                     const int32_t *__restrict__ raw_hits, float min_stid, int n_events, OutCount *cnt) {
    const int lane = threadIdx.x & 31;
    for (long e = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; e < n_events;
         e += ((long)gridDim.x * blockDim.x) >> 5) {
        const bool acc = !toomany[e] && (!raw_hits || raw_hits[e] > 0);  // M:1066-1072
        int hits = 0;
        for (int d = 1 + lane; d < OR_NDET; d += 32) hits += plane_count(hv, e, d);
        const int n = min((int)tv.ntracks[e * OR_NSLOTS + lane], OR_SLOTCAP);
        int ntr = 0, nth = 0;
        for (int k = 0; k < n; ++k) {
            const float *T = trk_rec(tv, e, lane, k);
            if (T[OR_TRK_STID] < min_stid) continue;  // M:1130
            ++ntr;
            nth += track_nhits(T);
        }
        hits = __reduce_add_sync(0xffffffffu, hits);
        ntr = __reduce_add_sync(0xffffffffu, ntr);
        nth = __reduce_add_sync(0xffffffffu, nth);
        if (lane == 0) {
            OutCount c;
            c.acc = acc ? 1 : 0;
            c.hits = acc ? hits : 0;
            c.tracks = acc ? ntr : 0;
            c.thits = acc ? nth : 0;
            c.dims = acc ? min((int)dv.ndimuons[e], OR_DIMUON_MAX) : 0;
            cnt[e] = c;
        }
    }
}

// one block: exclusive offsets of every event's rows, totals into counts[5]
__global__ void __launch_bounds__(1024)
    out_scan_kernel(const OutCount *__restrict__ cnt, int n_events, OutOffset *off, long long *counts) {
    __shared__ long long part[5][1024];
    const int t = threadIdx.x;
    const long per = ((long)n_events + blockDim.x - 1) / blockDim.x;
    const long e0 = min((long)n_events, t * per), e1 = min((long)n_events, e0 + per);
    long long s[5] = {0, 0, 0, 0, 0};
    for (long e = e0; e < e1; ++e) {
        const OutCount c = cnt[e];
        s[0] += c.acc; s[1] += c.hits; s[2] += c.tracks; s[3] += c.thits; s[4] += c.dims;
    }
    for (int q = 0; q < 5; ++q) part[q][t] = s[q];
    __syncthreads();
    // inclusive scan of the per-thread sums (Hillis-Steele in shared memory)
    for (int o = 1; o < (int)blockDim.x; o <<= 1) {
        long long v[5];
        for (int q = 0; q < 5; ++q) v[q] = t >= o ? part[q][t - o] : 0;
        __syncthreads();
        for (int q = 0; q < 5; ++q) part[q][t] += v[q];
        __syncthreads();
    }
    long long run[5];
    for (int q = 0; q < 5; ++q) run[q] = part[q][t] - s[q];
    for (long e = e0; e < e1; ++e) {
        const OutCount c = cnt[e];
        off[e] = OutOffset{run[0], run[1], run[2], run[3], run[4]};
        run[0] += c.acc; run[1] += c.hits; run[2] += c.tracks; run[3] += c.thits; run[4] += c.dims;
    }
    if (t == blockDim.x - 1)
        for (int q = 0; q < 5; ++q) counts[q] = part[q][t];
}

__constant__ int c_dim_out_src[OR_OUT_DIMUON_FIELDS] = {
    // OROutput.h:61-100 order from the dimuon record (M:1186-1219); -1..-3 = sums
    OR_DIM_MASS, OR_DIM_PT, OR_DIM_XF, OR_DIM_X1, OR_DIM_X2, OR_DIM_COSTHETA, OR_DIM_PHI, OR_DIM_MASS_SINGLE,
    OR_DIM_CHI2_SINGLE, OR_DIM_VTX, OR_DIM_VTX + 1, OR_DIM_VTX + 2, -1, -2, -3, OR_DIM_POS_VTX, OR_DIM_POS_VTX + 1,
    OR_DIM_POS_VTX + 2, OR_DIM_NEG_VTX, OR_DIM_NEG_VTX + 1, OR_DIM_NEG_VTX + 2, OR_DIM_POS_P + 3, OR_DIM_POS_P,
    OR_DIM_POS_P + 1, OR_DIM_POS_P + 2, OR_DIM_NEG_P + 3, OR_DIM_NEG_P, OR_DIM_NEG_P + 1, OR_DIM_NEG_P + 2,
    OR_DIM_POS_P_SINGLE + 3, OR_DIM_POS_P_SINGLE, OR_DIM_POS_P_SINGLE + 1, OR_DIM_POS_P_SINGLE + 2,
    OR_DIM_NEG_P_SINGLE + 3, OR_DIM_NEG_P_SINGLE, OR_DIM_NEG_P_SINGLE + 1, OR_DIM_NEG_P_SINGLE + 2, OR_DIM_CHI2_VTX,
    OR_DIM_CHI2_KF};
__constant__ int c_trk_out_src[OR_OUT_TRACK_FIELDS] = {
    // OROutput.h:32-51 order from the track record (M:1137-1155)
    OR_TRK_STID, OR_TRK_NHITS, OR_TRK_CHI2, OR_TRK_X0, OR_TRK_Y0, OR_TRK_TX, OR_TRK_TY, OR_TRK_INVP, OR_TRK_ERR_X0,
    OR_TRK_ERR_Y0, OR_TRK_ERR_TX, OR_TRK_ERR_TY, OR_TRK_ERR_INVP, OR_TRK_CHARGE, OR_TRK_VX, OR_TRK_VX + 1,
    OR_TRK_VX + 2, OR_TRK_PX, OR_TRK_PX + 1, OR_TRK_PX + 2};

__global__ void __launch_bounds__(256)
    out_write_kernel(or_hits_view_t hv, or_tracks_view_t tv, or_dimuons_view_t dv, const int32_t *__restrict__ event_ids,
                     float min_stid, int n_events, const OutCount *__restrict__ cnt,
                     const OutOffset *__restrict__ off, or_output_view_t out) {
    const int lane = threadIdx.x & 31;
    for (long e = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; e < n_events;
         e += ((long)gridDim.x * blockDim.x) >> 5) {
        const OutCount c = cnt[e];
        if (!c.acc) continue;
        const OutOffset o = off[e];
        if (lane == 0 && o.ev < out.cap_events) {
            int64_t *R = out.events + o.ev * OR_OUT_EV_FIELDS;
            R[OR_OUT_EV_INDEX] = e;
            R[OR_OUT_EV_ID] = event_ids ? event_ids[e] : e;
            R[OR_OUT_EV_NHITS] = c.hits;
            R[OR_OUT_EV_NTRACKS] = c.tracks;
            R[OR_OUT_EV_NDIMUONS] = c.dims;
            R[OR_OUT_EV_HIT0] = o.hits;
            R[OR_OUT_EV_TRACK0] = o.tracks;
            R[OR_OUT_EV_TRACKHIT0] = o.thits;
            R[OR_OUT_EV_DIMUON0] = o.dims;
        }
        // hits, planes 1..54 in order (M:1082-1116): plane offsets by a warp scan
        long long row = o.hits;
        for (int d0 = 1; d0 < OR_NDET; d0 += 32) {
            const int d = d0 + lane;
            const int n = d < OR_NDET ? plane_count(hv, e, d) : 0;
            int incl = n;
#pragma unroll
            for (int s = 1; s < 32; s <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, incl, s);
                if (lane >= s) incl += v;
            }
            const int total = __shfl_sync(0xffffffffu, incl, 31);
            for (int src = 0; src < 32 && d0 + src < OR_NDET; ++src) {
                const int np = __shfl_sync(0xffffffffu, n, src);
                if (np == 0) continue;
                const long long r0 = row + __shfl_sync(0xffffffffu, incl - n, src);
                const HitPlane h = hits_of(hv, e, d0 + src);
                for (int l = lane; l < np; l += 32) {
                    const long long r = r0 + l;
                    if (r >= out.cap_hits) continue;
                    float *R = out.hits + r * OR_OUT_HIT_FIELDS;
                    R[0] = (float)(d0 + src);
                    R[1] = h.chan(l);
                    R[2] = h.pos(l);
                    R[3] = h.tdc(l);
                    R[4] = h.drift(l);
                }
            }
            row += total;
        }
        // tracks in (slot, position) order with their hits (M:1122-1162)
        {
            const int n = min((int)tv.ntracks[e * OR_NSLOTS + lane], OR_SLOTCAP);
            int ntr = 0, nth = 0;
            for (int k = 0; k < n; ++k) {
                const float *T = trk_rec(tv, e, lane, k);
                if (T[OR_TRK_STID] < min_stid) continue;
                ++ntr;
                nth += track_nhits(T);
            }
            int itr = ntr, ith = nth;
#pragma unroll
            for (int s = 1; s < 32; s <<= 1) {
                const int a = __shfl_up_sync(0xffffffffu, itr, s), b = __shfl_up_sync(0xffffffffu, ith, s);
                if (lane >= s) {
                    itr += a;
                    ith += b;
                }
            }
            long long tr = o.tracks + itr - ntr, th = o.thits + ith - nth;
            for (int k = 0; k < n; ++k) {
                const float *T = trk_rec(tv, e, lane, k);
                if (T[OR_TRK_STID] < min_stid) continue;
                if (tr < out.cap_tracks) {
                    float *R = out.tracks + tr * OR_OUT_TRACK_FIELDS;
                    for (int f = 0; f < OR_OUT_TRACK_FIELDS; ++f) R[f] = T[c_trk_out_src[f]];
                }
                const int nh = track_nhits(T);
                for (int l = 0; l < nh; ++l, ++th) {
                    if (th >= out.cap_track_hits) continue;
                    float *R = out.track_hits + th * OR_OUT_TRACKHIT_FIELDS;
                    R[0] = T[OR_TRK_HIT_DETID + l];
                    R[1] = T[OR_TRK_HIT_CHAN + l];
                    R[2] = T[OR_TRK_HIT_POS + l];
                    R[3] = T[OR_TRK_HIT_DRIFT + l];
                    R[4] = T[OR_TRK_HIT_SIGN + l];
                    R[5] = T[OR_TRK_HIT_TDC + l];
                    R[6] = T[OR_TRK_HIT_RESID + l];
                }
                ++tr;
            }
        }
        // dimuons (M:1166-1220)
        for (int i = lane; i < c.dims; i += 32) {
            const long long r = o.dims + i;
            if (r >= out.cap_dimuons) continue;
            const float *D = dv.dimuons + (size_t)e * OR_EVT_DIM_FLOATS + (size_t)i * OR_NDIMUONPARAM;
            float *R = out.dimuons + r * OR_OUT_DIMUON_FIELDS;
            for (int f = 0; f < OR_OUT_DIMUON_FIELDS; ++f) {
                const int sidx = c_dim_out_src[f];
                R[f] = sidx >= 0 ? D[sidx] : D[OR_DIM_POS_P - 1 - sidx] + D[OR_DIM_NEG_P - 1 - sidx];
            }
        }
    }
}

size_t output_scratch_bytes(int n_events) {
    return ((sizeof(OutCount) * (size_t)n_events + 255) & ~size_t(255)) + sizeof(OutOffset) * (size_t)n_events;
}

cudaError_t launch_output_rows(or_hits_view_t hv, or_tracks_view_t tv, or_dimuons_view_t dv, const uint8_t *toomany,
                               const int32_t *raw_hits, const int32_t *event_ids, float min_stid, or_output_view_t out,
                               int n_events, void *scratch, cudaStream_t stream, int sm_count) {
    OutCount *cnt = static_cast<OutCount *>(scratch);
    OutOffset *off = reinterpret_cast<OutOffset *>(static_cast<char *>(scratch) +
                                                   ((sizeof(OutCount) * (size_t)n_events + 255) & ~size_t(255)));
    if (n_events <= 0) return cudaMemsetAsync(out.counts, 0, 5 * sizeof(long long), stream);
    long blocks = ((long)n_events * 32 + 255) / 256;
    blocks = blocks > (long)sm_count * 16 ? (long)sm_count * 16 : blocks;
    out_count_kernel<<<(unsigned)blocks, 256, 0, stream>>>(hv, tv, dv, toomany, raw_hits, min_stid, n_events, cnt);
    cudaError_t err = cudaGetLastError();
    if (err) return err;
    out_scan_kernel<<<1, 1024, 0, stream>>>(cnt, n_events, off, reinterpret_cast<long long *>(out.counts));
    if ((err = cudaGetLastError())) return err;
    out_write_kernel<<<(unsigned)blocks, 256, 0, stream>>>(hv, tv, dv, event_ids, min_stid, n_events, cnt, off, out);
    return cudaGetLastError();
}

}  // namespace orgpu
