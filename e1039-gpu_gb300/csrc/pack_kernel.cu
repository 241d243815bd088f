// pack_kernel.cu -- device-side hit packer: compact hit records to the
// reference hit layout.
//
// Does on the GPU what the reference host loop does per event
// (OnlineReconstruction/online_reconstruction.cu:589-636): for every plane
// write the hit count and the five SoA fields [chan | pos | tdc | flag |
// drift] with stride = count, pos = (float)wire_position[det][elem].
// Records of an event must be sorted by (det, elem, tdc); hits beyond a
// plane's slot capacity are dropped (the reference host would write past the
// slot).  One warp per event: a shared-memory histogram per plane, an
// exclusive scan, then coalesced field writes.
#include "or_device.cuh"

namespace orgpu {

constexpr int PK_WARPS = 8;

__global__ void __launch_bounds__(PK_WARPS * 32)
    pack_kernel(const or_hit_record_t *__restrict__ rec, const int64_t *__restrict__ off, int n_events,
                const float *__restrict__ wire_pos_f, or_hits_view_t hv) {
    __shared__ int cnt[PK_WARPS][64];
    __shared__ int start[PK_WARPS][64];
    const int w = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    for (long e = (long)blockIdx.x * PK_WARPS + w; e < n_events; e += (long)gridDim.x * PK_WARPS) {
        const int64_t r0 = off[e], r1 = off[e + 1];
        const int nrec = (int)(r1 - r0);
        cnt[w][lane] = 0;
        cnt[w][lane + 32] = 0;
        __syncwarp();
        for (int r = lane; r < nrec; r += 32) {
            const int d = rec[r0 + r].det;
            if (d >= 1 && d < OR_NDET) atomicAdd(&cnt[w][d], 1);
        }
        __syncwarp();
        // records are sorted by det: plane d's run starts at the sum of the
        // counts of the planes before it (records with det out of range sort
        // first or last and are skipped)
        if (lane == 0) {
            int lead = 0;
            for (int r = 0; r < nrec && rec[r0 + r].det < 1; ++r) ++lead;
            int s = lead;
            for (int d = 1; d < OR_NDET; ++d) {
                start[w][d] = s;
                s += cnt[w][d];
            }
        }
        __syncwarp();
        // counts (capped) for all 54 planes
        for (int d = 1 + lane; d < OR_NDET; d += 32) {
            const int n = cnt[w][d];
            if (d <= OR_NCHAM)
                hv.nhits_cham[e * OR_NCHAM + d - 1] = (uint32_t)min(n, OR_MAXHITS_CHAM);
            else if (d <= OR_NCHAM + OR_NHODO)
                hv.nhits_hodo[e * OR_NHODO + d - OR_NCHAM - 1] = (uint32_t)min(n, OR_MAXHITS_HODO);
            else
                hv.nhits_prop[e * OR_NPROP + d - OR_NCHAM - OR_NHODO - 1] = (uint32_t)min(n, OR_MAXHITS_PROP);
        }
        for (int r = lane; r < nrec; r += 32) {
            const or_hit_record_t h = rec[r0 + r];
            const int d = h.det;
            if (d < 1 || d >= OR_NDET) continue;
            const int k = r - start[w][d];
            float *slot;
            int cap;
            if (d <= OR_NCHAM) {
                slot = hv.hits_cham + e * OR_EVT_CHAM_FLOATS + (long)OR_NHITSPARAM * OR_MAXHITS_CHAM * (d - 1);
                cap = OR_MAXHITS_CHAM;
            } else if (d <= OR_NCHAM + OR_NHODO) {
                slot = hv.hits_hodo + e * OR_EVT_HODO_FLOATS + (long)OR_NHITSPARAM * OR_MAXHITS_HODO * (d - OR_NCHAM - 1);
                cap = OR_MAXHITS_HODO;
            } else {
                slot = hv.hits_prop + e * OR_EVT_PROP_FLOATS +
                       (long)OR_NHITSPARAM * OR_MAXHITS_PROP * (d - OR_NCHAM - OR_NHODO - 1);
                cap = OR_MAXHITS_PROP;
            }
            const int n = min(cnt[w][d], cap);
            if (k >= n) continue;
            const int el = h.elem;
            const float pos = (el >= 0 && el < OR_WIREPOS_STRIDE) ? wire_pos_f[d * OR_WIREPOS_STRIDE + el] : 0.f;
            slot[k] = (float)el;
            slot[n + k] = pos;
            slot[2 * n + k] = h.tdc;
            slot[3 * n + k] = (float)h.flag;
            slot[4 * n + k] = h.drift;
        }
        __syncwarp();
    }
}

cudaError_t launch_pack(const or_hit_record_t *rec, const int64_t *off, int n_events, const float *wire_pos_f,
                        or_hits_view_t hv, cudaStream_t stream, int sm_count) {
    if (n_events <= 0) return cudaSuccess;
    long blocks = (n_events + PK_WARPS - 1) / PK_WARPS;
    const long cap = (long)sm_count * 8;
    if (blocks > cap) blocks = cap;
    pack_kernel<<<(unsigned)blocks, PK_WARPS * 32, 0, stream>>>(rec, off, n_events, wire_pos_f, hv);
    return cudaGetLastError();
}

}  // namespace orgpu
