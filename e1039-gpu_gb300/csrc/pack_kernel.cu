// pack_kernel.cu -- device-side hit packer: compact hit records to the
// reference hit layout.
//
// Does on the GPU what the reference host loop does per event
// (OnlineReconstruction/online_reconstruction.cu:589-636): for every plane
// write the hit count and the five SoA fields [chan | pos | tdc | flag |
// drift] with stride = count, pos = (float)wire_position[det][elem].
// Records of an event must be sorted by (det, elem, tdc); hits beyond a
// plane's slot capacity are dropped (the reference host would write past the
// slot).  An event whose records are out of that order raises ERRW_INPUT
// (or_stream_sync reports it as an argument error); its slots are then
// undefined but every write stays inside them.  Records whose det is outside
// 1..54 (they sort first or last) are skipped.  One warp per event: a shared-memory histogram per plane, an
// exclusive scan, then coalesced field writes.
//
// With an R-T table the drift field is computed from the tdc as the
// reference host does while packing (online_reconstruction.cu:387-396); the
// same conversion also runs in place on hits packed elsewhere (rt_apply).
#include "or_device.cuh"

namespace orgpu {

constexpr int PK_WARPS = 8;

// Drift distance of a hit on plane det from the R-T calibration, or `drift`
// unchanged when the plane has no profile (hodoscopes never have one).
// Evaluation follows the spline's piece convention: piece k covers
// (t[k], t[k+1]]; x <= t[0] uses piece 0 and x >= t[n-1] piece n-2.  The
// cubic is evaluated in double in nested form and rounded to float once, as
// the reference's float drift_distance receives the double result (:332, :395).
static __device__ __forceinline__ float rt_drift(const or_rt_table_t *__restrict__ rt, int det, float tdc,
                                                 float drift) {
    const int n = rt->nknots[det];
    if (n <= 0) return drift;
    if (tdc < rt->tmin[det]) return (float)((double)rt->cellwidth[det] * 0.5);
    if (tdc > rt->tmax[det]) return 0.f;
    const double *t = rt->t[det];
    const double x = (double)tdc;
    int k = 0;
    if (n > 1) {
        if (x >= t[n - 1]) {
            k = n - 2;
        } else if (x > t[0]) {
            int lo = 0, hi = n - 1;
            while (hi - lo > 1) {
                const int mid = (lo + hi) >> 1;
                if (x > t[mid]) lo = mid;
                else hi = mid;
            }
            k = lo;
        }
    }
    const double dx = x - t[k];
    const double v = rt->r[det][k] + dx * (rt->b[det][k] + dx * (rt->c[det][k] + dx * rt->d[det][k]));
    return (float)v;
}

static __device__ __forceinline__ bool rt_plane(int det) {
    return (det >= 1 && det <= OR_NCHAM) || (det > OR_NCHAM + OR_NHODO && det < OR_NDET);
}

template <bool RT>
__global__ void __launch_bounds__(PK_WARPS * 32)
    pack_kernel(const or_hit_record_t *__restrict__ rec, const int64_t *__restrict__ off, int n_events,
                const float *__restrict__ wire_pos_f, const or_rt_table_t *__restrict__ rt, or_hits_view_t hv,
                uint32_t *__restrict__ errw) {
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
        bool unsorted = false;
        for (int r = lane; r < nrec; r += 32) {
            const or_hit_record_t h = rec[r0 + r];
            if (r > 0) {
                const or_hit_record_t q = rec[r0 + r - 1];
                unsorted |= h.det < q.det || (h.det == q.det && (h.elem < q.elem || (h.elem == q.elem && h.tdc < q.tdc)));
            }
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
            if (k < 0 || k >= n) continue;  // k < 0 only for records out of order
            const int el = h.elem;
            const float pos = (el >= 0 && el < OR_WIREPOS_STRIDE) ? wire_pos_f[d * OR_WIREPOS_STRIDE + el] : 0.f;
            slot[k] = (float)el;
            slot[n + k] = pos;
            slot[2 * n + k] = h.tdc;
            slot[3 * n + k] = (float)h.flag;
            slot[4 * n + k] = (RT && rt_plane(d)) ? rt_drift(rt, d, h.tdc, h.drift) : h.drift;
        }
        if (__any_sync(0xffffffffu, unsorted) && lane == 0) atomicOr(errw, ERRW_INPUT);
        __syncwarp();
    }
}

// In-place R-T conversion on the reference layout: one warp per event, the
// chamber and prop-tube planes in turn, lanes over a plane's hits.
__global__ void __launch_bounds__(PK_WARPS * 32)
    rt_apply_kernel(const or_rt_table_t *__restrict__ rt, or_hits_view_t hv, int n_events) {
    const int w = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    for (long e = (long)blockIdx.x * PK_WARPS + w; e < n_events; e += (long)gridDim.x * PK_WARPS) {
        for (int p = 0; p < OR_NCHAM + OR_NPROP; ++p) {
            const bool cham = p < OR_NCHAM;
            const int d = cham ? 1 + p : OR_NCHAM + OR_NHODO + 1 + (p - OR_NCHAM);
            if (rt->nknots[d] <= 0) continue;
            float *slot;
            int n;
            if (cham) {
                n = min((int)hv.nhits_cham[e * OR_NCHAM + p], OR_MAXHITS_CHAM);
                slot = hv.hits_cham + e * OR_EVT_CHAM_FLOATS + (long)OR_NHITSPARAM * OR_MAXHITS_CHAM * p;
            } else {
                n = min((int)hv.nhits_prop[e * OR_NPROP + p - OR_NCHAM], OR_MAXHITS_PROP);
                slot = hv.hits_prop + e * OR_EVT_PROP_FLOATS + (long)OR_NHITSPARAM * OR_MAXHITS_PROP * (p - OR_NCHAM);
            }
            for (int k = lane; k < n; k += 32) slot[4 * n + k] = rt_drift(rt, d, slot[2 * n + k], slot[4 * n + k]);
        }
    }
}

static long pack_blocks(int n_events, int sm_count) {
    long blocks = (n_events + PK_WARPS - 1) / PK_WARPS;
    const long cap = (long)sm_count * 8;
    return blocks > cap ? cap : blocks;
}

cudaError_t launch_pack(const or_hit_record_t *rec, const int64_t *off, int n_events, const float *wire_pos_f,
                        const or_rt_table_t *rt, or_hits_view_t hv, uint32_t *errw, cudaStream_t stream,
                        int sm_count) {
    if (n_events <= 0) return cudaSuccess;
    const unsigned blocks = (unsigned)pack_blocks(n_events, sm_count);
    if (rt)
        pack_kernel<true><<<blocks, PK_WARPS * 32, 0, stream>>>(rec, off, n_events, wire_pos_f, rt, hv, errw);
    else
        pack_kernel<false><<<blocks, PK_WARPS * 32, 0, stream>>>(rec, off, n_events, wire_pos_f, nullptr, hv, errw);
    return cudaGetLastError();
}

cudaError_t launch_rt_apply(const or_rt_table_t *rt, or_hits_view_t hv, int n_events, cudaStream_t stream,
                            int sm_count) {
    if (n_events <= 0) return cudaSuccess;
    rt_apply_kernel<<<(unsigned)pack_blocks(n_events, sm_count), PK_WARPS * 32, 0, stream>>>(rt, hv, n_events);
    return cudaGetLastError();
}

}  // namespace orgpu
