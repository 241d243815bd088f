// er_kernel.cu -- event reducer (hit filtering, declustering, per-channel
// de-duplication, in-place compaction, station-multiplicity reject).
//
// Replaces gkernel_eR<<<N,8>>> (OnlineReconstruction/reconstruction_kernels
// .cuh:8-172) and event_reduction() (reconstruction_helper.cuh:168-361).
//
// Layout on the GPU: one warp per event.  The warp stages the
// occupied part of each plane slot (5*n floats, rounded up to 16 bytes --
// slot capacities are multiples of 16 bytes, so the round-up stays inside the
// slot) into shared memory with 1-D TMA bulk copies completing on an
// mbarrier; planes are taken in batches that fit the warp's buffer (a warp
// prefix sum over the planes' sizes), each lane issuing the copies of its
// planes.  Each lane then runs the reference's per-plane state machine on one
// plane out of shared memory and writes that plane's survivors back, with the
// new SoA stride, into the same slot.  Bytes beyond the survivors are left as
// they were, as the reference leaves them.
#include "or_device.cuh"

namespace orgpu {

constexpr int ER_BUF_FLOATS = 2048;                 // 8 KB staging buffer per warp
constexpr int ER_MAX_STAGED_HITS = ER_BUF_FLOATS / 5 + 8;
constexpr int ER_NPLANES = 48;
constexpr uint32_t ER_WAIT_LIMIT = 1u << 26;        // bounded mbarrier wait
constexpr uint32_t ER_DRAIN_LIMIT = 1u << 28;       // ... and the wait for copies in flight after it gave up

// the 48 planes the reducer touches: the 24 chambers of the E1039 set
// (reconstruction_constants.h:60), 16 hodoscopes, 8 prop tubes (K:25-57)
__device__ __constant__ unsigned char c_er_det[ER_NPLANES] = {
    1,  2,  3,  4,  5,  6,  13, 14, 15, 16, 17, 18, 19, 20, 21, 22, 23, 24, 25, 26, 27, 28, 29, 30,
    31, 32, 33, 34, 35, 36, 37, 38, 39, 40, 41, 42, 43, 44, 45, 46, 47, 48, 49, 50, 51, 52, 53, 54};

struct __align__(16) ErWarp {
    float buf[ER_BUF_FLOATS];
    uint64_t bar;
    int n[ER_NPLANES];
    int kept[ER_NPLANES];
    int soff[ER_NPLANES];
    int hoff[ER_NPLANES];
    uint8_t keep[ER_MAX_STAGED_HITS];
    uint16_t surv[ER_MAX_STAGED_HITS];
    uint32_t seen[32][8];  // per-lane channel bitmap, 202 channels
};

struct PlaneRef {
    float *slot;
    uint32_t *count;
    int cap;
};

__device__ __forceinline__ PlaneRef er_plane(const or_hits_view_t &hv, long e, int det) {
    PlaneRef r;
    if (det <= OR_NCHAM) {
        r.slot = hv.hits_cham + e * OR_EVT_CHAM_FLOATS + (long)OR_NHITSPARAM * OR_MAXHITS_CHAM * (det - 1);
        r.count = hv.nhits_cham + e * OR_NCHAM + det - 1;
        r.cap = OR_MAXHITS_CHAM;
    } else if (det <= OR_NCHAM + OR_NHODO) {
        const int k = det - OR_NCHAM - 1;
        r.slot = hv.hits_hodo + e * OR_EVT_HODO_FLOATS + (long)OR_NHITSPARAM * OR_MAXHITS_HODO * k;
        r.count = hv.nhits_hodo + e * OR_NHODO + k;
        r.cap = OR_MAXHITS_HODO;
    } else {
        const int k = det - OR_NCHAM - OR_NHODO - 1;
        r.slot = hv.hits_prop + e * OR_EVT_PROP_FLOATS + (long)OR_NHITSPARAM * OR_MAXHITS_PROP * k;
        r.count = hv.nhits_prop + e * OR_NPROP + k;
        r.cap = OR_MAXHITS_PROP;
    }
    return r;
}

// event_reduction() on one staged plane (reconstruction_helper.cuh:168-361).
// Returns the survivor count; keep[] gets 1/0 per hit, surv[] the survivor
// indices in order.
static __device__ int er_reduce_plane(const float *h, int n, int det, uint8_t *keep, uint16_t *surv, uint32_t *seen) {
    auto chan = [&](int i) { return h[i]; };
    auto pos = [&](int i) { return h[n + i]; };
    auto tdc = [&](int i) { return h[2 * n + i]; };
    auto intime = [&](int i) { return (((int)h[3 * n + i]) & 2) != 0; };
    auto drift = [&](int i) { return h[4 * n + i]; };

    int cl_first = 0, cl_last = 0, cls = 0;
    for (int i = 0; i < n; ++i) {
        keep[i] = 1;
        if (!intime(i)) {  // H:198
            keep[i] = 0;
            continue;
        }
        // H:204-230 never changes a flag: uniqueID_curr is reset every hit.
        if (det > OR_NCHAM) continue;
        if (cls == 0) {  // H:241-243
            cl_first = cl_last = i;
            cls = 1;
            continue;
        }
        const float dc = fabsf(chan(i) - chan(cl_last));
        if (dc > 1 || i == n - 1) {  // H:258
            if (i == n - 1 && dc <= 1) {
                cl_last = i;
                ++cls;
            }
            if (cls == 2) {  // H:267-295
                const int a = cl_first, b = cl_last;
                const float w_max = (float)(0.9 * 0.5 * (double)(pos(b) - pos(a)));
                const float w_min = (float)(4.0 / 9.0 * (double)w_max);
                if ((drift(a) > w_max && drift(b) > w_min) || (drift(a) > w_min && drift(b) > w_max)) {
                    if (drift(a) > drift(b))
                        keep[a] = 0;
                    else
                        keep[b] = 0;
                } else {
                    const float dt = tdc(a) - tdc(b);
                    if ((((double)dt >= 0.0 && (double)dt < 8.0) || ((double)dt <= 0.0 && (double)dt > -8.0)) &&
                        (det >= 19 && det <= 24)) {
                        keep[a] = 0;
                        keep[b] = 0;
                    }
                }
            }
            if (cls >= 3) {  // H:297-318: members are the in-time hits in [first, last]
                float dt_mean = 0.0f;
                int prev = cl_first;
                for (int m = cl_first + 1; m <= cl_last; ++m) {
                    if (!intime(m)) continue;
                    const float d = tdc(m) - tdc(prev);
                    dt_mean += ((double)d > 0.0 ? d : (tdc(prev) - tdc(m)));
                    prev = m;
                }
                dt_mean = dt_mean / (float)(cls - 1);
                const bool all = (double)dt_mean < 10.0;
                for (int m = cl_first; m <= cl_last; ++m) {
                    if (!intime(m)) continue;
                    if (all || m != cl_first) keep[m] = 0;
                }
            }
            cls = 0;
        } else {
            cl_last = i;
            ++cls;
        }
    }
    // H:334-349, first survivor per channel wins
#pragma unroll
    for (int w = 0; w < 8; ++w) seen[w] = 0u;
    int nred = 0;
    for (int i = 0; i < n; ++i) {
        if (!keep[i]) continue;
        const int c = (short)chan(i);
        if (c >= 0 && c < 202) {
            const uint32_t bit = 1u << (c & 31);
            if (seen[c >> 5] & bit) {
                keep[i] = 0;
                continue;
            }
            seen[c >> 5] |= bit;
        }
        surv[nred++] = (uint16_t)i;
    }
    return nred;
}

template <int W>
__global__ void __launch_bounds__(W * 32) er_kernel(or_hits_view_t hv, uint8_t *__restrict__ toomany, int n_events,
                                                    uint32_t *__restrict__ errw) {
    extern __shared__ __align__(16) unsigned char er_smem[];
    ErWarp *sm = reinterpret_cast<ErWarp *>(er_smem);
    const int w = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    ErWarp &S = sm[w];
    if (lane == 0) mbar_init(&S.bar, 1);
    __syncwarp();
    uint32_t phase = 0;

    for (long e = (long)blockIdx.x * W + w; e < n_events; e += (long)gridDim.x * W) {
        for (int p = lane; p < ER_NPLANES; p += 32) {
            const PlaneRef r = er_plane(hv, e, c_er_det[p]);
            const int n = (int)*r.count;
            S.n[p] = n < r.cap ? n : r.cap;
        }
        __syncwarp();
        int p0 = 0;
        while (p0 < ER_NPLANES) {
            // batch [p0, p1): planes whose staged images fit the buffer
            int p1 = p0, off = 0, hits = 0;
            // 32 planes at a time: prefix sums of the staged sizes and hit
            // counts over the lanes; the planes that fit form a prefix
            for (;;) {
                const int p = p1 + lane;
                const int n_l = p < ER_NPLANES ? S.n[p] : 0;
                const int sz_l = p < ER_NPLANES ? ((5 * n_l + 3) & ~3) : ER_BUF_FLOATS + 1;
                int csz = sz_l, cn = n_l;
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const int a = __shfl_up_sync(0xffffffffu, csz, d);
                    const int b = __shfl_up_sync(0xffffffffu, cn, d);
                    if (lane >= d) {
                        csz += a;
                        cn += b;
                    }
                }
                const bool fit = off + csz <= ER_BUF_FLOATS;
                const int nfit = __popc(__ballot_sync(0xffffffffu, fit));
                if (fit) {
                    S.soff[p] = off + csz - sz_l;
                    S.hoff[p] = hits + cn - n_l;
                }
                if (nfit == 0) break;
                off += __shfl_sync(0xffffffffu, csz, nfit - 1);
                hits += __shfl_sync(0xffffffffu, cn, nfit - 1);
                p1 += nfit;
                if (nfit < 32 || p1 >= ER_NPLANES) break;
            }
            __syncwarp();
            if (off > 0) {
                // lane 0 announces the batch's bytes before any copy is
                // issued; then every lane issues the copies of its planes
                if (lane == 0) mbar_arrive_expect_tx(&S.bar, (uint32_t)off * 4u);
                __syncwarp();
                fence_proxy_async_smem();  // buffer was read by the generic proxy
                for (int p = p0 + lane; p < p1; p += 32) {
                    const int sz = (5 * S.n[p] + 3) & ~3;
                    if (sz == 0) continue;
                    const PlaneRef r = er_plane(hv, e, c_er_det[p]);
                    tma_load_1d(S.buf + S.soff[p], r.slot, (uint32_t)sz * 4u, &S.bar);
                }
                if (!__all_sync(0xffffffffu, mbar_wait_bounded(&S.bar, phase, ER_WAIT_LIMIT))) {
                    // the wait gave up: raise the error word, then wait (again
                    // bounded) for this batch's copies still in flight, so that
                    // the warp leaves no bulk copy writing into shared memory
                    if (lane == 0) atomicOr(errw, ERRW_TMA_TIMEOUT);
                    mbar_wait_bounded(&S.bar, phase, ER_DRAIN_LIMIT);
                    __syncwarp();
                    return;
                }
                phase ^= 1u;
            }
            for (int p = p0 + lane; p < p1; p += 32) {
                S.kept[p] = er_reduce_plane(S.buf + S.soff[p], S.n[p], c_er_det[p], S.keep + S.hoff[p],
                                            S.surv + S.hoff[p], S.seen[lane]);
            }
            __syncwarp();
            // each lane writes back the planes it reduced
            for (int p = p0 + lane; p < p1; p += 32) {
                const int n = S.n[p], nk = S.kept[p];
                const PlaneRef r = er_plane(hv, e, c_er_det[p]);
                const float *src = S.buf + S.soff[p];
                const uint16_t *sv = S.surv + S.hoff[p];
                for (int f = 0; f < 5; ++f)
                    for (int k = 0; k < nk; ++k) r.slot[f * nk + k] = src[f * n + sv[k]];
                *r.count = (uint32_t)nk;
            }
            __syncwarp();
            p0 = p1;
        }
        // K:128-139: station sums of the reduced chamber counts
        if (lane == 0) {
            int m[4] = {0, 0, 0, 0};
            for (int p = 0; p < 24; ++p) {
                const int d = c_er_det[p];
                const int st = d <= 12 ? 0 : (d - 7) / 6;
                m[st] += S.kept[p];
            }
            toomany[e] = (uint8_t)((m[0] > MAXD0) || (m[1] > MAXD2) || (m[2] > MAXD3) || (m[3] > MAXD3));
        }
        __syncwarp();
    }
}

// Host launcher.
template <int W>
static cudaError_t er_launch(or_hits_view_t hv, uint8_t *toomany, int n_events, uint32_t *errw, cudaStream_t stream,
                             int sm_count) {
    const size_t smem = sizeof(ErWarp) * W;
    cudaError_t e = smem_attr_once((const void *)er_kernel<W>, (int)smem);
    if (e != cudaSuccess) return e;
    long blocks = (n_events + W - 1) / W;
    const long cap = (long)sm_count * (48 / W > 0 ? 48 / W : 1);  // up to 48 resident warps per SM
    if (blocks > cap) blocks = cap;
    er_kernel<W><<<(unsigned)blocks, W * 32, smem, stream>>>(hv, toomany, n_events, errw);
    return cudaGetLastError();
}

// Self-test of the bounded wait: one warp waits on an mbarrier that nothing
// arrives at and no bulk copy targets, `polls` polls at most.  The wait runs
// out, the kernel raises ERRW_TMA_TIMEOUT as the reducer does, invalidates the
// barrier and returns; the context stays usable.
__global__ void __launch_bounds__(32) wait_selftest_kernel(uint32_t *__restrict__ errw, uint32_t polls) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    __syncwarp();
    const bool done = __all_sync(0xffffffffu, mbar_wait_bounded(&bar, 0u, polls));
    if (!done && threadIdx.x == 0) atomicOr(errw, ERRW_TMA_TIMEOUT);
    __syncwarp();
    if (threadIdx.x == 0) asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(&bar)) : "memory");
}

cudaError_t launch_wait_selftest(uint32_t *errw, uint32_t polls, cudaStream_t stream) {
    wait_selftest_kernel<<<1, 32, 0, stream>>>(errw, polls);
    return cudaGetLastError();
}

// Host launcher; `warps` = events per CTA (1, 2, 4, 8 or 16).
cudaError_t launch_event_reduce(or_hits_view_t hv, uint8_t *toomany, int n_events, uint32_t *errw,
                                cudaStream_t stream, int sm_count, int warps) {
    if (n_events <= 0) return cudaSuccess;
    switch (warps) {
    case 1: return er_launch<1>(hv, toomany, n_events, errw, stream, sm_count);
    case 2: return er_launch<2>(hv, toomany, n_events, errw, stream, sm_count);
    case 8: return er_launch<8>(hv, toomany, n_events, errw, stream, sm_count);
    case 16: return er_launch<16>(hv, toomany, n_events, errw, stream, sm_count);
    default: return er_launch<4>(hv, toomany, n_events, errw, stream, sm_count);
    }
}

}  // namespace orgpu
