// yz_kernel.cu -- YZ extension of the XZ tracklets with U/V hits.
//
// Replaces gKernel_YZ_tracking<<<N,32>>> (OnlineReconstruction/
// reconstruction_kernels.cuh:864-1832).
//
// The reference gives each of its 32 threads one tracklet slot and, for every
// tracklet in it, loops u3 x v3 (outer) and u2 x v2 (inner) hit pairs
// sequentially, keeping the best chi2 (K:1320-1825).  Two pieces of state
// make that loop sequential:
//   - the station-3 hit signs chosen by the left/right resolution survive
//     from one inner iteration to the next: they are fixed by the first
//     combination of a (u3,v3) iteration that passes the first y cut, and on
//     station 3+ the last v3' hit can pair with the first u2 hit
//     (planes 19/18), whose resolution re-sets that sign whenever it
//     succeeds (H:714-780);
//   - the left/right walk reads the scratch entry just past the hit count
//     (H:725-735), which holds the last hit load attempted at that index --
//     possibly by an earlier combination, (u3,v3) iteration or tracklet of
//     the same slot.
// Work per event is heavily skewed (a few events hold most combinations),
// so the GPU version splits it:
//   yz_plan_kernel   one warp per event walks its slots and tracklets in
//                    order; builds each tracklet's hit windows once (y, error
//                    and acceptance of every windowed hit for this tracklet);
//                    evaluates light tracklets itself, and cuts heavy ones
//                    into units of whole (u3,v3) iterations on a device queue,
//                    storing each one's windows as an image;
//   yz_first_kernel  persistent warps (28 per SM, 72 registers) drain the
//                    queue with the first cut only: fit of the station-3 and
//                    station-2 y hits, 2-sigma cut, scratch-entry scan; each
//                    unit's survivors (about 6 %) go in order to a device pool;
//                    with the combination scorer it walks only the listed
//                    kept (u3,v3) iterations;
//   yz_second_kernel per unit, the survivors replayed in order with the sign
//                    carry: left/right walk, prop and hodoscope gates, chi2
//                    (28 warps per SM, 72 registers; a survivor's hits are
//                    register offsets into the arena); a unit whose survivors
//                    did not fit runs whole, first cut and survivors together
//                    (yz_work_kernel's path, which also serves contexts
//                    without a pool, such as the no-allocation entry);
//   yz_apply_kernel  writes each heavy tracklet's best combination.
// Inside a range, lanes evaluate 32 combinations at a time in the reference
// order; ballot/shuffle scans recover the sign state and the scratch entry.
// A unit starts with the scratch entries left by everything before it, which
// depend only on which hit loads were attempted (not on any fit), so the plan
// pass and each unit derive them without evaluating the earlier work.  The
// best combination of a tracklet is the minimum of (chi2, combination index),
// the reference's first-strictly-smaller rule.
#include "window_pairs.cuh"

namespace orgpu {

constexpr int YZ_MAXWIN = 100;          // windowed hits per plane (the reference's hitidx arrays)
constexpr int YZ_MAXPAIR = 100;         // pairs per projection (the reference's hitpairs arrays)
// Build-time tunables (-D...), with the values measured best on the
// 100,000-event uneven batch; results do not depend on any of them:
//   OR_YZ_ARENA          windowed hit records per warp in shared memory
//   OR_YZ_WARPS_SM       warps per SM of the combined work kernel
//   OR_YZ_SPLIT          first-cut / survivor kernels (1) or the combined one (0)
//   OR_YZ_PLAN_WARPS_SM, OR_YZ_FIRST_WARPS_SM, OR_YZ_SECOND_WARPS_SM
//                        warps per SM (register caps) of the other kernels
//   OR_YZ_POOL_PER_UNIT  survivor-pool entries per unit of queue capacity
//   OR_YZ_IMG_PER_UNIT   window-image 16-byte words per unit of queue capacity
//   OR_YZ_LIGHT          combinations a planning warp evaluates itself
//   OR_YZ_PLAN_CHUNK     slots per planning unit
//   OR_YZ_UNIT           live combinations per queued unit
//   OR_YZ_QCAP_CTX       per-warp survivor queue entries of a context
#ifndef OR_YZ_ARENA
#define OR_YZ_ARENA 64
#endif
#ifndef OR_YZ_WARPS_SM
#define OR_YZ_WARPS_SM 16
#endif
#ifndef OR_YZ_SPLIT
#define OR_YZ_SPLIT 1
#endif
#ifndef OR_YZ_PLAN_WARPS_SM
#define OR_YZ_PLAN_WARPS_SM 28
#endif
#ifndef OR_YZ_FIRST_WARPS_SM
#define OR_YZ_FIRST_WARPS_SM 28
#endif
#ifndef OR_YZ_POOL_PER_UNIT
#define OR_YZ_POOL_PER_UNIT 48
#endif
// survivor entries in the pool (32 B each), per unit of queue capacity: a
// context sized for the 100,000-event uneven batch (4 Mi units) holds
// 192 Mi, and that batch queues between 64 Mi and 128 Mi survivors; units
// that do not fit run on the combined path
constexpr long long YZ_POOL_PER_UNIT = OR_YZ_POOL_PER_UNIT;
#ifndef OR_YZ_IMG_PER_UNIT
#define OR_YZ_IMG_PER_UNIT 36
#endif
// window images (16-byte words) per unit of queue capacity: 144 Mi words
// (2.25 GiB) for 4 Mi units, and the 100,000-event uneven batch's queued
// tracklets take 128 Mi words (1.9 GiB); tracklets whose image does not fit
// are windowed again by each of their units
constexpr long long YZ_IMG_PER_UNIT = OR_YZ_IMG_PER_UNIT;
constexpr int YZ_ARENA_HITS = OR_YZ_ARENA;      // windowed hits kept in shared memory per warp
#ifndef OR_YZ_LIGHT
#define OR_YZ_LIGHT 32
#endif
constexpr long YZ_LIGHT = OR_YZ_LIGHT;         // combinations a planning warp evaluates itself per tracklet
constexpr long YZ_CHUNK_INLINE = OR_YZ_LIGHT;  // ... and per planning unit
#ifndef OR_YZ_PLAN_CHUNK
#define OR_YZ_PLAN_CHUNK 8
#endif
constexpr int YZ_PLAN_CHUNK = OR_YZ_PLAN_CHUNK;  // slots per planning unit
#ifndef OR_YZ_UNIT
#define OR_YZ_UNIT 8192
#endif
constexpr long YZ_UNIT = OR_YZ_UNIT;    // live combinations per queued unit (whole (u3,v3) iterations)
constexpr int YZ_GARENA_HITS = 8 * YZ_MAXWIN;  // per-warp global overflow arena
// survivors of the first cut wait in a per-warp queue in global memory and
// are evaluated in a batch when it fills or the range ends, so that the two
// phases do not alternate every 32 survivors (each switch refetches the
// other phase's instructions)
constexpr int YZ_QCAP_MIN = 64;     // queue entries per warp: the static (no-allocation) scratch
#ifndef OR_YZ_QCAP_CTX
#define OR_YZ_QCAP_CTX 2048
#endif
constexpr int YZ_QCAP_CTX = OR_YZ_QCAP_CTX;   // ... and a context's scratch

struct __align__(16) YzHit {
    float Y, eY, pos, drift;
    float tdc, z;  // z = the plane's z, read by every fit
    short det, el;
    int acc;  // calculate_y_uvhit accepted this hit for the tracklet
};
static_assert(sizeof(YzHit) == 32, "YzHit is two 16-byte words");

struct Stale {
    short det;
    float pos, drift;
};

// one queued unit: combinations [g0*C2, g1*C2) of heavy tracklet `heavy`,
// with the scratch entries 4..7 as they stand when the unit starts
struct YzUnit {
    int heavy;
    int g0, g1;
    int pad;
    Stale entry[4];
    // the unit's live outer iterations as the combination scorer's rows of
    // its tracklet: ranks [r0, r1)
    int r0, r1;
};
// a heavy tracklet
struct YzHeavy {
    int e, slot, k;
    int unit0, nunits;
    // outer-iteration scoring: the tracklet's first score row (-1: no rows,
    // nothing pruned), its row count (the live outer iterations), the inner
    // combinations per outer iteration, and the outer index of its best
    // combination (written by yz_apply_kernel; -1: none)
    int orow0, nrows, c2, best_g;
    // its window image in the image pool (16-byte words), -1: none
    int img;
};
// best combination of one unit
struct YzBest {
    unsigned long long key;
    int nuv;
    float chi2, ty, y0, ety, ey0;
    float det[8], el[8], pos[8], drift[8], sign[8], tdc[8], res[12];
    int pad;
};

// The first y fit of a combination (fit_2D_track over its accepted u/v hits,
// K:1602, AM:32-74) weighs every hit by its plane's error (calculate_y_uvhit,
// H:98: resolution * |dp_y / dp_x|) at its plane's z, so the normal matrix,
// its inverse and the parameter errors depend only on which of the eight
// planes (u3 u3' v3 v3' u2 u2' v2 v2', added in that order) gave a hit.  The
// fit needs at least one hit in each of the four projections: 3^4 = 81 plane
// sets per station-3 half.  yz_tab_kernel computes each entry with the same
// operations in the same order as the per-combination fit did (Fit2 then
// matinv_2x2 and sqrtf), so a combination's fit keeps only the right-hand
// side (B0, B1) and two dot products, bit for bit the same result.
constexpr int YZ_TAB_SETS = 81;
struct __align__(16) YzTab {
    float ai0, ai1, ai2, ai3;  // inverse of the normal matrix
    float thr_y0, thr_ty;      // Y0_MAX + 2 err_y0, TY_MAX + 2 err_ty (the first cut, K:1611)
    float ey0, ety;            // err_y0, err_ty
};
static_assert(sizeof(YzTab) == 32, "YzTab is two 16-byte words");
constexpr size_t YZ_TAB_BYTES = (2 * YZ_TAB_SETS * sizeof(YzTab) + 255) & ~size_t(255);

// index of a plane set: group values g = (second plane << 1 | first plane)
// in 1..3 for u3, v3, u2, v2
__device__ __forceinline__ int yz_tab_index(int gu3, int gv3, int gu2, int gv2) {
    return ((gu3 - 1) * 3 + (gv3 - 1)) * 9 + (gu2 - 1) * 3 + (gv2 - 1);
}

// Work counters of one YZ call (64-bit, in the counters area): combinations
// that reach the first y fit, the sum of their hit counts, and combinations
// that pass its 2-sigma cut (the survivors of the first cut).
constexpr int YZ_CTR_FITTED = 16, YZ_CTR_HITSUM = 18, YZ_CTR_SURVIVORS = 20;

struct YzScratch {
    const YzTab *tab;        // 2 x YZ_TAB_SETS entries: station-3 half 0 (D3p) then 1 (D3m)
    YzUnit *units;
    YzHeavy *heavy;
    YzBest *best;
    unsigned int *counters;  // [0] units reserved, [1] heavy reserved, [2] queue head, [3] survivor-kernel
                             // head, [4..5] planning units, [8..9] pool entries, [10..11] image words,
                             // [16..21] work counters
    YzHit *garena;           // per-warp overflow arenas
    struct PassEntryStore *qbuf;  // per-warp survivor queues (qcap entries each)
    int cap_units, cap_heavy, garena_warps, qcap;
    // split first-cut / survivor kernels: each unit's survivors in order in
    // pool[useg[u].x .. + useg[u].y); useg[u].x < 0: the unit runs combined
    struct PassEntryStore *pool;
    int2 *useg;
    long long pool_cap;  // 0: no pool, the combined kernel runs
    // window images of the queued tracklets (YzImgHead, arena, pairs),
    // written by the planning pass; counter [10..11] allocates them
    uint4 *img;
    long long img_cap;   // 16-byte words; 0: no images, every unit windows its tracklet
    int count_work;      // nonzero: the kernels add up the work counters
};

// optional pruning: tracklet rows (row_off, as the scorer's) and keep flags
struct YzPrune {
    // tracklet keep flags of the tracklet scorer
    const int32_t *row_off;
    const uint8_t *keep;  // nullptr: plain
    long max_rows;
    // the combination scorer: one feature row per live (u3, v3) outer
    // iteration of every queued (heavy) tracklet, written by the planning
    // pass; scores filled before the first cut; an outer iteration scoring
    // below t_keep is skipped, unless its event is uncertain (unc[e])
    float *ofeat;          // [cap_orows * OR_NFEAT]; nullptr: no outer rows
    int32_t *og;           // [cap_orows] outer index g of each row
    float *oscore;         // [cap_orows]
    uint32_t *orows;       // row counter
    uint8_t *unc;          // [n_events] uncertain events
    const or_mlp_t *model; // nullptr: rows written, nothing scored or pruned
    long cap_orows;
    float t_keep, t_unc;
};


struct PassEntryStore {
    int c;
    float y0, ty, ey0, ety, stpos, stdrift;
    int stdet;
};

struct YzEvent {
    HitPlane hc[8];
    HitPlane p1y1, p1y2, p2y1, p2y2;
    HitPlane hod[3][2];
    short dl[8];
};

// the first cut's listed iterations at a time (yz_first_kept)
constexpr int YZ_KEPT_BATCH = 32;
// inner-pair records (yz_s2_record) the first cut keeps in shared memory
constexpr int YZ_REC_SMEM = (8 * YZ_MAXWIN * 2 + 2 * YZ_MAXWIN) / 8;

struct YzWarp {
    union {
        YzEvent ev;  // the event's plane views, the same for every lane
        // first cut (the event's views are not read there): the scratch
        // writes of the pruned iterations before each listed one
        unsigned long long kgap[YZ_KEPT_BATCH];
    };
    Stale st[4];  // scratch entries 4..7 as the next combination finds them, the same for every lane
    YzHit arena[YZ_ARENA_HITS];
    short2 pair[4][YZ_MAXPAIR];  // windowed indices (or -1) in sides 0, 1 of list q
    union {
        struct {
            short widx[8][YZ_MAXWIN];  // plane hit index of each windowed hit
            uint8_t wfl[2][YZ_MAXWIN];
        } w;                           // while the windows are built
        unsigned long long rec[YZ_REC_SMEM];  // first cut: the inner pairs' records
    };
    unsigned short kuv[YZ_KEPT_BATCH];  // first cut: the listed iterations, iu3 | iv3 << 8
    int np[4], nw[8], woff[8];
    float x0, tx, ex0, etx;
    int nhx;
    float xdd[4], xres[4], xp1x[4], xp1y[4], xp1z[4], xdpx[4], xdpy[4], xdpz[4];
    short xhs[4];
    // survivors this warp evaluated (work counter)
    unsigned long long nsurv;
    YzBest b;
};

// The event's plane views for a tracklet of station half st3, one plane per
// lane (every lane calls): u2 u2' v2 v2' u3 u3' v3 v3' (K:910-984), the
// prop-tube y planes and the x hodoscopes of stations 2-4.
__device__ __forceinline__ void yz_event_planes(YzEvent &E, const or_hits_view_t &hv, long e, int st3) {
    const int lane = lane_id();
    int det = 0;
    HitPlane *dst = nullptr;
    if (lane < 8) {
        const int u3 = det_u3(st3), v3 = det_v3(st3);
        det = lane == 0 ? DET_U2 : lane == 1 ? DET_UP2 : lane == 2 ? DET_V2 : lane == 3 ? DET_VP2
            : lane == 4 ? u3 : lane == 5 ? u3 - 1 : lane == 6 ? v3 : v3 - 1;
        E.dl[lane] = (short)det;
        dst = &E.hc[lane];
    } else if (lane < 12) {
        det = lane == 8 ? DET_P1Y1 : lane == 9 ? DET_P1Y2 : lane == 10 ? DET_P2Y1 : DET_P2Y2;
        dst = lane == 8 ? &E.p1y1 : lane == 9 ? &E.p1y2 : lane == 10 ? &E.p2y1 : &E.p2y2;
    } else if (lane < 18) {
        const int q = (lane - 12) >> 1, c = (lane - 12) & 1;
        det = c_hodoplanesx[q + 1][c];
        dst = &E.hod[q][c];
    }
    if (dst) *dst = hits_of(hv, e, det);
}

// Build the tracklet's windows (make_hitpairs_in_station, H:464-549) with the
// per-hit y of this tracklet (calculate_y_uvhit, H:75-100).  Returns false
// when a window or a pair list exceeds the reference's 100-entry arrays.
__device__ bool yz_build(YzWarp &S, const YzEvent &E, const float *T, const or_plane_t &P, int st3,
                         const YzHit *&base, YzHit *garena) {
    const int lane = lane_id();
    const float x0 = T[OR_TRK_X0], tx = T[OR_TRK_TX], ex0 = T[OR_TRK_ERR_X0], etx = T[OR_TRK_ERR_TX];
    const int stid_of[4] = {2, 2, st3, st3}, proj_of[4] = {1, 2, 1, 2};
    bool ok = true;
    int total = 0;
    // windowed hit lists, in plane order (H:480-511)
#pragma unroll 1
    for (int q = 0; q < 4; ++q) {
        const int a = 2 * q;
        const float za = P.z[E.dl[a]], zb = P.z[E.dl[a + 1]];
        const float sp = P.spacing[E.dl[a]];
        const float xmin = fminf((tx - etx) * za, (tx - etx) * zb) + x0 - ex0 - sp;
        const float xmax = fmaxf((tx + etx) * za, (tx + etx) * zb) + x0 + ex0 + sp;
#pragma unroll 1
        for (int side = 0; side < 2; ++side) {
            const HitPlane &h = E.hc[a + side];
            const int det = E.dl[a + side];
            int c = 0;
#pragma unroll 1
            for (int b0 = 0; b0 < h.n; b0 += 32) {
                const int i = b0 + lane;
                const bool in = i < h.n && wp_in_window(det, h.chan(i), xmin, xmax, P);
                const unsigned m = __ballot_sync(0xffffffffu, in);
                if (in) {
                    const int k = c + __popc(m & lanemask_lt());
                    if (k < YZ_MAXWIN) S.w.widx[a + side][k] = (short)i;
                }
                c += __popc(m);
            }
            if (c > YZ_MAXWIN) ok = false;
            c = min(c, YZ_MAXWIN);
            if (lane == 0) {
                S.nw[a + side] = c;
                S.woff[a + side] = total;
            }
            total += c;
        }
    }
    __syncwarp();
    // windowed hit records (K:1326-1355 computes these per combination)
    YzHit *dst = (total <= YZ_ARENA_HITS) ? S.arena : garena;
#pragma unroll 1
    for (int l = 0; l < 8; ++l) {
        const HitPlane &h = E.hc[l];
        const int det = E.dl[l];
#pragma unroll 1
        for (int i = lane; i < S.nw[l]; i += 32) {
            const int hi = S.w.widx[l][i];
            YzHit r;
            r.det = (short)det;
            r.el = (short)h.chan(hi);
            r.tdc = h.tdc(hi);
            r.drift = h.drift(hi);
            r.pos = h.pos(hi);
            float yy = 0.f, ey = 0.f;
            r.acc = calculate_y_uvhit(det, r.el, r.drift, 0, x0, tx, P, yy, ey) ? 1 : 0;
            r.Y = yy;
            r.eY = ey;
            r.z = P.z[det];
            dst[S.woff[l] + i] = r;
        }
    }
    __syncwarp();
    // pairs over each projection's two windowed lists (H:513-546)
#pragma unroll 1
    for (int q = 0; q < 4; ++q) {
        const int a = 2 * q;
        const int c1 = S.nw[a], c2 = S.nw[a + 1];
#pragma unroll 1
        for (int i = lane; i < c1; i += 32) S.w.wfl[0][i] = 0;
#pragma unroll 1
        for (int i = lane; i < c2; i += 32) S.w.wfl[1][i] = 0;
        __syncwarp();
        const float spacing = c_spacingplane[c_detsuperid[stid_of[q]][proj_of[q]]];
        int np = 0;
#pragma unroll 1
        for (int b0 = 0; b0 < c1 * c2; b0 += 32) {
            const int c = b0 + lane;
            bool take = false;
            short2 v = make_short2(0, 0);
            if (c < c1 * c2) {
                const int ia = c / c2, ib = c - ia * c2;
                if (!(fabsf(dst[S.woff[a] + ia].pos - dst[S.woff[a + 1] + ib].pos) > spacing)) {
                    take = true;
                    v = make_short2((short)ia, (short)ib);
                    S.w.wfl[0][ia] = 1;
                    S.w.wfl[1][ib] = 1;
                }
            }
            wp_append(take, v, S.pair[q], YZ_MAXPAIR, np);
        }
        __syncwarp();
#pragma unroll 1
        for (int b0 = 0; b0 < c1; b0 += 32) {
            const int ia = b0 + lane;
            const bool take = ia < c1 && !S.w.wfl[0][ia];
            wp_append(take, make_short2((short)ia, -1), S.pair[q], YZ_MAXPAIR, np);
        }
#pragma unroll 1
        for (int b0 = 0; b0 < c2; b0 += 32) {
            const int ib = b0 + lane;
            const bool take = ib < c2 && !S.w.wfl[1][ib];
            wp_append(take, make_short2(-1, (short)ib), S.pair[q], YZ_MAXPAIR, np);
        }
        if (np > YZ_MAXPAIR) ok = false;
        if (lane == 0) S.np[q] = min(np, YZ_MAXPAIR);
        __syncwarp();
    }
    base = dst;
    if (lane == 0) {
        S.x0 = x0;
        S.tx = tx;
        S.ex0 = ex0;
        S.etx = etx;
    }
    __syncwarp();
    return ok;
}

// A queued tracklet's windows as yz_build left them: the planning pass
// stores this image once, and the first-cut and survivor kernels load it
// for each of the tracklet's units instead of windowing the event's hits
// again.  Layout in 16-byte words: the head (7 words), the arena (2 words a
// hit), then the four pair lists back to back (4 pairs a word).
struct __align__(16) YzImgHead {
    int np[4];
    int nw[8], woff[8];
    float x0, tx, ex0, etx;
    int total, npair, pad[2];
};
static_assert(sizeof(YzImgHead) == 112, "YzImgHead is seven 16-byte words");
constexpr int YZ_IMG_HEAD_WORDS = sizeof(YzImgHead) / 16;

// Store the windows just built (base: their arena); returns the image's
// word offset, or -1 when the pool is full.
__device__ int yz_store_image(const YzWarp &S, const YzHit *base, const YzScratch &sc) {
    const int lane = lane_id();
    const int total = S.woff[7] + S.nw[7];
    const int npair = S.np[0] + S.np[1] + S.np[2] + S.np[3];
    const long long words = YZ_IMG_HEAD_WORDS + 2LL * total + (npair + 3) / 4;
    unsigned long long o = 0ull;
    if (lane == 0) o = atomicAdd(reinterpret_cast<unsigned long long *>(sc.counters + 10), (unsigned long long)words);
    o = __shfl_sync(0xffffffffu, o, 0);
    if ((long long)o + words > sc.img_cap) return -1;
    uint4 *dst = sc.img + o;
    if (lane == 0) {
        YzImgHead h;
#pragma unroll
        for (int q = 0; q < 4; ++q) h.np[q] = S.np[q];
#pragma unroll
        for (int l = 0; l < 8; ++l) {
            h.nw[l] = S.nw[l];
            h.woff[l] = S.woff[l];
        }
        h.x0 = S.x0;
        h.tx = S.tx;
        h.ex0 = S.ex0;
        h.etx = S.etx;
        h.total = total;
        h.npair = npair;
        h.pad[0] = h.pad[1] = 0;
        *reinterpret_cast<YzImgHead *>(dst) = h;
    }
    const uint4 *src = reinterpret_cast<const uint4 *>(base);
    uint4 *da = dst + YZ_IMG_HEAD_WORDS;
#pragma unroll 1
    for (int i = lane; i < 2 * total; i += 32) da[i] = src[i];
    short2 *dp = reinterpret_cast<short2 *>(da + 2 * total);
    int off = 0;
#pragma unroll 1
    for (int q = 0; q < 4; ++q) {
#pragma unroll 1
        for (int i = lane; i < S.np[q]; i += 32) dp[off + i] = S.pair[q][i];
        off += S.np[q];
    }
    return (int)o;
}

// Load a tracklet's windows from its image into the warp's state; returns
// the arena (in shared memory when it fits there, else the image itself).
__device__ const YzHit *yz_load_image(YzWarp &S, const uint4 *__restrict__ img) {
    const int lane = lane_id();
    const YzImgHead &h = *reinterpret_cast<const YzImgHead *>(img);
    const int total = h.total;
    if (lane < 4) S.np[lane] = h.np[lane];
    if (lane < 8) {
        S.nw[lane] = h.nw[lane];
        S.woff[lane] = h.woff[lane];
    }
    if (lane == 0) {
        S.x0 = h.x0;
        S.tx = h.tx;
        S.ex0 = h.ex0;
        S.etx = h.etx;
    }
    const uint4 *ia = img + YZ_IMG_HEAD_WORDS;
    const YzHit *base = reinterpret_cast<const YzHit *>(ia);
    if (total <= YZ_ARENA_HITS) {
        uint4 *da = reinterpret_cast<uint4 *>(S.arena);
#pragma unroll 1
        for (int i = lane; i < 2 * total; i += 32) da[i] = ia[i];
        base = S.arena;
    }
    const short2 *ip = reinterpret_cast<const short2 *>(ia + 2 * total);
    int off = 0;
#pragma unroll 1
    for (int q = 0; q < 4; ++q) {
        const int n = h.np[q];
#pragma unroll 1
        for (int i = lane; i < n; i += 32) S.pair[q][i] = ip[off + i];
        off += n;
    }
    __syncwarp();
    return base;
}

// x hits of the tracklet (K:1300-1316)
__device__ __forceinline__ void yz_xhits(YzWarp &S, const float *T, const or_plane_t &P) {
    const int lane = lane_id();
    const int nhx = min((int)T[OR_TRK_NHITS], 4);  // XZ tracklets carry 2-4 hits
    if (lane < nhx) {
        const short d = (short)T[OR_TRK_HIT_DETID + lane];
        const short ch = (short)T[OR_TRK_HIT_CHAN + lane];
        S.xdd[lane] = T[OR_TRK_HIT_DRIFT + lane];
        S.xhs[lane] = (short)T[OR_TRK_HIT_SIGN + lane];
        S.xres[lane] = P.resolution[d];
        S.xp1x[lane] = x_bep(d, ch, P);
        S.xp1y[lane] = y_bep(d, ch, P);
        S.xp1z[lane] = z_bep(d, ch, P);
        S.xdpx[lane] = P.deltapx[d];
        S.xdpy[lane] = P.deltapy[d];
        S.xdpz[lane] = P.deltapz[d];
    }
    if (lane == 0) S.nhx = nhx;
    __syncwarp();
}

// A survivor's accepted u/v hits in the reference order (K:1326-1597), kept
// in registers: arena offsets, 16 bits each (hits 0-3 in lo, 4-7 in hi), and
// the left/right signs, 2 bits each in two's complement (0, 1 or -1).  The
// hits' fields are read from the arena where they are needed.
struct UvSet {
    unsigned long long lo, hi;
    unsigned sign;
};

__device__ __forceinline__ int uv_off(const UvSet &U, int k) {
    return (int)(((k < 4 ? U.lo : U.hi) >> (16 * (k & 3))) & 0xFFFFull);
}
__device__ __forceinline__ short uv_sign(const UvSet &U, int k) {
    return (short)((int)(U.sign << (30 - 2 * k)) >> 30);
}
__device__ __forceinline__ void uv_set_sign(UvSet &U, int k, int s) {
    U.sign = (U.sign & ~(3u << (2 * k))) | (((unsigned)s & 3u) << (2 * k));
}

// resolve_leftright_newhits walk over the n hits of U with the scratch entry
// past the end given by `st` (H:714-780), then the singles (H:785-804).
__device__ __forceinline__ void walk_newhits(int n, UvSet &U, const YzHit *base, const Stale &st, float x0, float tx,
                                             float y0, float ty, float ex0, float etx, float ey0, float ety,
                                             const or_plane_t &P) {
#pragma unroll 1
    for (int i = 0; i < n;) {
        const int j = i + 1;
        const YzHit &hi = base[uv_off(U, i)];
        const short di = hi.det;
        short dj = st.det, sj = 0;
        float pj = st.pos, drj = st.drift;
        if (j < n) {
            const YzHit &hj = base[uv_off(U, j)];
            dj = hj.det;
            sj = uv_sign(U, j);
            pj = hj.pos;
            drj = hj.drift;
        }
        if (abs(di - dj) != 1) {
            i += 1;
            continue;
        }
        if (uv_sign(U, i) * sj == 0) {
            const int k = lr_pair_newhits(x0, tx, y0, ty, ex0, etx, ey0, ety, di, dj, hi.pos, hi.drift, pj, drj, P,
                                          150.f);
            if (k >= 0) {
                uv_set_sign(U, i, c_lrpossibility[k][0]);
                if (j < n) uv_set_sign(U, j, c_lrpossibility[k][1]);
            }
        }
        i += 2;
    }
#pragma unroll 1
    for (int k = 0; k < n; ++k) {
        if (uv_sign(U, k)) continue;
        const YzHit &h = base[uv_off(U, k)];
        uv_set_sign(U, k, single_sign_newhits(x0, tx, y0, ty, h.det, h.pos, P));
    }
}

// The per-survivor work below runs once per 32 queued survivors, between long
// stretches of the first-cut loop; it is kept out of line (one copy each) so
// that the loop's instructions stay resident in the instruction cache.  The
// walk takes and returns the hit set by value (registers, not a stack frame).
__device__ __noinline__ unsigned walk_uv(int n, UvSet U, const YzHit *base, Stale st, float x0, float tx, float y0,
                                         float ty, float ex0, float etx, float ey0, float ety, const or_plane_t &P) {
    walk_newhits(n, U, base, st, x0, tx, y0, ty, ex0, etx, ey0, ety, P);
    return U.sign;
}

// Index of the last station-3 hit when the walk pairs it with the first
// station-2 hit, else -1.  The walk's pairs depend only on plane ids.
__device__ __forceinline__ int cross_pair_index(int n3, const UvSet &U, const YzHit *base, int nuv) {
#pragma unroll 1
    for (int i = 0; i < n3;) {
        const int j = i + 1;
        if (j >= nuv) return -1;
        if (abs(base[uv_off(U, i)].det - base[uv_off(U, j)].det) != 1) {
            i += 1;
            continue;
        }
        if (j == n3) return i;
        i += 2;
    }
    return -1;
}

__device__ __forceinline__ const YzHit *yz_list(const YzWarp &S, const YzHit *base, int l) { return base + S.woff[l]; }

// accepted station-3 hits of the outer iteration (iu3, iv3)
__device__ __forceinline__ int s3_count(const YzWarp &S, const YzHit *base, int iu3, int iv3, bool &valid) {
    const short2 pu = S.pair[2][iu3], pv = S.pair[3][iv3];
    int nu = 0, nv = 0;
    if (pu.x >= 0) nu += yz_list(S, base, 4)[pu.x].acc;
    if (pu.y >= 0) nu += yz_list(S, base, 5)[pu.y].acc;
    if (nu > 0) {
        if (pv.x >= 0) nv += yz_list(S, base, 6)[pv.x].acc;
        if (pv.y >= 0) nv += yz_list(S, base, 7)[pv.y].acc;
    }
    valid = nu > 0 && nv > 0;
    return nu + nv;
}

// Walk the outer iterations of the current tracklet in order and track the
// scratch entries 4..7 from the load pattern alone (no fits): entry k is set
// by the last inner combination writing offset k-4+... of the last valid
// outer iteration that reaches it.  When `units` is given, the state at the
// start of every unit (each `gper` outer iterations) is stored there.  `st`
// goes in as the state before the tracklet and comes out as the state after.
// live outer iterations (both pairs alive) before outer index g, g <= G:
// the scorer-row rank of g when g is live
__device__ __forceinline__ int live_before(const unsigned mu[4], const unsigned mv[4], int nu3, int g) {
    const int iu = g % nu3, iv = g / nu3;
    int below_v = 0, below_u = 0, au = 0;
#pragma unroll
    for (int w = 0; w < 4; ++w) {
        au += __popc(mu[w]);
        if (w < (iv >> 5)) below_v += __popc(mv[w]);
        else if (w == (iv >> 5)) below_v += __popc(mv[w] & ((1u << (iv & 31)) - 1u));
        if (w < (iu >> 5)) below_u += __popc(mu[w]);
        else if (w == (iu >> 5)) below_u += __popc(mu[w] & ((1u << (iu & 31)) - 1u));
    }
    const bool v_live = iv < 128 && ((mv[iv >> 5] >> (iv & 31)) & 1u);
    return below_v * au + (v_live ? below_u : 0);
}

static_assert(8 * YZ_MAXWIN <= 1024, "arena offsets fit 10 bits");

// The station-2 record of the inner pair (iu2, iv2): its load attempts in
// the reference order (K:1467-1597) reduced to what the first cut needs, the
// same in every outer iteration.  16-bit field e (0..3) holds in bits 0-9 the
// arena offset of the last hit attempted when e of the pair's hits had been
// accepted -- for e below the accepted count, accepted hit e, in order -- so
// that after n3 station-3 hits the attempts write scratch entries e + n3 - 4;
// bits 10-13 which fields were written, bits 26-28 the accepted count, bits
// 42-45 the planes of the accepted hits (u2 u2' v2 v2'), bit 58 whether both
// the u2 and the v2 group gave a hit (the first fit is reached).
__device__ __forceinline__ unsigned long long yz_s2_record(const YzWarp &S, const YzHit *base, int iu2, int iv2) {
    const short2 pu = S.pair[0][iu2], pv = S.pair[1][iv2];
    const int offs[4] = {pu.x >= 0 ? S.woff[0] + pu.x : -1, pu.y >= 0 ? S.woff[1] + pu.y : -1,
                         pv.x >= 0 ? S.woff[2] + pv.x : -1, pv.y >= 0 ? S.woff[3] + pv.y : -1};
    unsigned long long rec = 0ull;
    unsigned pm = 0u, g2 = 0u;
    int nacc = 0, nu = 0;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        if (a == 2) {
            nu = nacc;
            if (nu == 0) break;  // no u2 hit: v2 is not loaded
        }
        const int off = offs[a];
        if (off < 0) continue;
        const int sh = 16 * nacc;
        rec = (rec & ~(0x3FFull << sh)) | ((unsigned long long)off << sh);
        pm |= 1u << nacc;
        if (base[off].acc) {
            g2 |= 1u << a;
            ++nacc;
        }
    }
    const unsigned fit = (nu > 0 && nacc > nu) ? 1u : 0u;
    return rec | ((unsigned long long)pm << 10) | ((unsigned long long)nacc << 26) | ((unsigned long long)g2 << 42) |
           ((unsigned long long)fit << 58);
}

// The station-2 load attempts of an outer iteration do not depend on the
// iteration (only on the inner pair, K:1467-1597): the last inner combination
// writing scratch offset m (past the station-3 hit count) is the same in
// every live outer iteration.  Returns those hits as arena offsets, 16 bits
// per offset m = 0..3, 0xFFFF where no combination writes m.
__device__ unsigned long long yz_last_writes(const YzWarp &S, const YzHit *base) {
    const int nu2 = S.np[0];
    const int C2 = S.np[0] * S.np[1];
    unsigned long long lasto = ~0ull;
#pragma unroll 1
    for (int b0 = 0; b0 < C2; b0 += 32) {
        const int c = b0 + lane_id();
        const unsigned long long rec = c < C2 ? yz_s2_record(S, base, c % nu2, c / nu2) : 0ull;
        const unsigned pm = (unsigned)(rec >> 10) & 0xFu;
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            const int l = last_lane(__ballot_sync(0xffffffffu, (pm >> m) & 1u));
            if (l >= 0) {
                const unsigned long long o =
                    (unsigned)__shfl_sync(0xffffffffu, (unsigned)((rec >> (16 * m)) & 0x3FFull), l);
                lasto = (lasto & ~(0xFFFFull << (16 * m))) | (o << (16 * m));
            }
        }
    }
    return lasto;
}

__device__ void yz_unit_states(const YzWarp &S, const YzHit *base, int G, int gper, Stale st[4], YzUnit *units,
                               int heavy, const unsigned *alive_u = nullptr, const unsigned *alive_v = nullptr) {
    const int lane = lane_id();
    const unsigned lt = lanemask_lt();
    const int nu3 = S.np[2];
    // the last inner combination's write of each offset m, as arena offsets
    const unsigned long long lasto = yz_last_writes(S, base);
    const Stale st_in[4] = {st[0], st[1], st[2], st[3]};
    // per entry k the arena offset of its last write so far (0xFFFF: st_in[k])
    unsigned long long carry = ~0ull;
    auto resolve = [&](int k, unsigned o) -> Stale {
        if (o == 0xFFFFu) return st_in[k];
        const YzHit &r = base[o];
        return Stale{r.det, r.pos, r.drift};
    };
#pragma unroll 1
    for (int b0 = 0; b0 < G; b0 += 32) {
        const int g = b0 + lane;
        unsigned long long mk = ~0ull;  // this outer iteration's writes of entries 4..7
        if (g < G) {
            bool valid;
            const int n3 = s3_count(S, base, g % nu3, g / nu3, valid);
            if (valid) {
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int mm = k + 4 - n3;
                    if (mm >= 0 && mm < 4)
                        mk = (mk & ~(0xFFFFull << (16 * k))) | (((lasto >> (16 * mm)) & 0xFFFFull) << (16 * k));
                }
            }
        }
        unsigned long long ent = 0ull;  // the entries as this outer iteration finds them
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const unsigned wk = (unsigned)((mk >> (16 * k)) & 0xFFFFull);
            const unsigned wm = __ballot_sync(0xffffffffu, wk != 0xFFFFu);
            const int src = last_lane(wm & lt);
            const unsigned v = __shfl_sync(0xffffffffu, wk, src < 0 ? 0 : src);
            const unsigned e = src >= 0 ? v : (unsigned)((carry >> (16 * k)) & 0xFFFFull);
            ent |= (unsigned long long)e << (16 * k);
            const int l = last_lane(wm);
            if (l >= 0) {
                const unsigned long long c = __shfl_sync(0xffffffffu, wk, l);
                carry = (carry & ~(0xFFFFull << (16 * k))) | (c << (16 * k));
            }
        }
        if (units && g < G && (g % gper) == 0) {
            YzUnit &u = units[g / gper];
            u.heavy = heavy;
            u.g0 = g;
            u.g1 = min(G, g + gper);
            u.pad = 0;
            u.r0 = alive_u ? live_before(alive_u, alive_v, nu3, u.g0) : 0;
            u.r1 = alive_u ? live_before(alive_u, alive_v, nu3, u.g1) : 0;
#pragma unroll
            for (int k = 0; k < 4; ++k) u.entry[k] = resolve(k, (unsigned)((ent >> (16 * k)) & 0xFFFFull));
        }
    }
    __syncwarp();  // every lane has read the entry states
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const Stale v = resolve(k, (unsigned)((carry >> (16 * k)) & 0xFFFFull));
        if (lane == 0) st[k] = v;
    }
    __syncwarp();
}

// A combination that passed the first y cut, queued for the full evaluation:
// index inside the tracklet, first fit, scratch entry past its hit count.
using PassEntry = PassEntryStore;

// Gather the accepted hits of combination c in the reference order
// (K:1326-1597), station 3 first; returns nuv, sets n3.
__device__ __forceinline__ int yz_gather(const YzWarp &S, const YzHit *base, int c, int C2, UvSet &U, int &n3) {
    const int iuv3 = c / C2, iuv2 = c - iuv3 * C2;
    const int nu2 = S.np[0], nu3 = S.np[2];
    const short2 p3u = S.pair[2][iuv3 % nu3], p3v = S.pair[3][iuv3 / nu3];
    const short2 p2u = S.pair[0][iuv2 % nu2], p2v = S.pair[1][iuv2 / nu2];
    U.lo = U.hi = 0ull;
    U.sign = 0u;
    int nuv = 0;
#pragma unroll
    for (int a = 0; a < 8; ++a) {
        if (a == 4) n3 = nuv;
        const short2 p = a < 2 ? p3u : a < 4 ? p3v : a < 6 ? p2u : p2v;
        const int wi = (a & 1) ? p.y : p.x;
        if (wi < 0) continue;
        const int l = (a + 4) & 7;  // lists u3 u3' v3 v3' u2 u2' v2 v2'
        const int off = S.woff[l] + wi;
        if (!base[off].acc) continue;
        const unsigned long long f = (unsigned long long)off << (16 * (nuv & 3));
        if (nuv < 4) U.lo |= f;
        else U.hi |= f;
        ++nuv;
    }
    return nuv;
}

// gates of a candidate after the refit: the hard cut (K:1638), the prop-tube
// y segments (K:1640-1702) and the hodoscopes with y (H:1002-1087)
__device__ __noinline__ bool yz_gates(const YzEvent &E, const or_plane_t &P, float x0, float y0, float tx, float ty,
                                      float ex0, float ey0, float etx, float ety) {
    if (fabsf(y0) > Y0_MAX || fabsf(ty) > TY_MAX) return false;
    const int nprop = prop_hits(E.p1y1, P.z[DET_P1Y1], E.p1y2, P.z[DET_P1Y2], 5.08f, y0, ty) +
                      prop_hits(E.p2y1, P.z[DET_P2Y1], E.p2y2, P.z[DET_P2Y2], 10.16f, y0, ty);
    if (nprop < NPROP_MIN) return false;
#pragma unroll 1
    for (int qq = 0; qq < 3; ++qq) {
        bool ok = false;
#pragma unroll 1
        for (int c = 0; c < 2 && !ok; ++c)
            ok = match_tracklet_to_hodo(qq + 1, c_hodoplanesx[qq + 1][c], E.hod[qq][c], x0, y0, tx, ty, ex0, ey0, etx,
                                        ety, P);
        if (!ok) return false;
    }
    return true;
}

// One residual of chi2_track (H:1149-1165): x hit m < nhx, else u/v hit
// m - nhx of U.
__device__ __forceinline__ float yz_residual(const YzWarp &S, const UvSet &U, const YzHit *base, int m, int nhx,
                                             const or_plane_t &P, float x0, float y0, float tx, float ty, float &res) {
    if (m < nhx) {
        res = S.xres[m];
        return residual_line(S.xp1x[m], S.xp1y[m], S.xp1z[m], S.xdpx[m], S.xdpy[m], S.xdpz[m], S.xdd[m], S.xhs[m], x0,
                             y0, tx, ty);
    }
    const int k = m - nhx;
    const YzHit &h = base[uv_off(U, k)];
    const short d = h.det;
    res = P.resolution[d];
    return residual_line(x_bep(d, h.el, P), y_bep(d, h.el, P), z_bep(d, h.el, P), P.deltapx[d], P.deltapy[d],
                         P.deltapz[d], h.drift, uv_sign(U, k), x0, y0, tx, ty);
}

// chi2_track over the x hits and the uv hits (H:1182-1204)
__device__ __noinline__ float yz_chi2(const YzWarp &S, UvSet U, const YzHit *base, int nuv, int nhx,
                                      const or_plane_t &P, float x0, float y0, float tx, float ty) {
    float chi2 = 0.f;
#pragma unroll 1
    for (int m = 0; m < nhx + nuv; ++m) {
        float res;
        const float r = yz_residual(S, U, base, m, nhx, P, x0, y0, tx, ty, res);
        chi2 += r * r / res / res;
    }
    return chi2;
}

// Sign state carried from one survivor chunk to the next (the first
// combination of an outer iteration fixes the station-3 signs), and the best
// key so far.
struct Phase2Carry {
    int g = -1;
    bool hasf = false, hascross = false;
    short sig[4] = {0, 0, 0, 0};
    short cross = 0;
    unsigned long long best = ~0ull;
};

// The full evaluation of n (<= 32) queued survivors Qc[0..n), in order: sign
// state, left/right walk, prop and hodoscope gates, chi2, best key
// (K:1613-1799).  Out of line: it runs once per 32 survivors, and inlined it
// would sit in the middle of the first-cut loop's instructions.
__device__ __noinline__ void yz_phase2(YzWarp &S, const YzEvent &E, const YzHit *base, int C2, const or_plane_t &P,
                                       const PassEntryStore *Qc, int n, Phase2Carry &cs) {
    const int lane = lane_id();
    const float x0 = S.x0, tx = S.tx, ex0 = S.ex0, etx = S.etx;
    const int nhx = S.nhx;
    if (lane == 0) S.nsurv += (unsigned long long)n;
    // --- one chunk of survivors ------------------------------------------
    const bool valid = lane < n;
    PassEntry q;
    if (valid) q = Qc[lane];
    const int c = valid ? q.c : 0;
    const int g = valid ? c / C2 : -1 - lane;
    UvSet U{0ull, 0ull, 0u};
    int n3 = 0, nuv = 0;
    if (valid) nuv = yz_gather(S, base, c, C2, U, n3);
    const Stale stj{(short)(valid ? q.stdet : DET_SENTINEL), valid ? q.stpos : 0.f, valid ? q.stdrift : 0.f};
    const float y0 = valid ? q.y0 : 0.f, ty = valid ? q.ty : 0.f;
    const float ey0 = valid ? q.ey0 : 0.f, ety = valid ? q.ety : 0.f;
    const unsigned seg = __match_any_sync(0xffffffffu, g);
    const unsigned vm = __ballot_sync(0xffffffffu, valid);
    const bool carried_f = (g == cs.g) && cs.hasf;
    const int fl = __ffs(vm & seg) - 1;
    const bool is_first = valid && !carried_f && fl == lane;
    // Every survivor walks at once.  A first survivor of its outer iteration
    // starts from unset signs; the others start with placeholder station-3
    // signs: the walk only asks whether a sign is set, so it passes over the
    // station-3 pairs and singles and resolves the station-2 hits and the
    // cross pair exactly as it does after their real signs, which are put in
    // below (the first survivor's, or the cross pair's where it resolved).
    if (valid) {
        if (!is_first) {
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (k < n3) uv_set_sign(U, k, 1);
        }
        U.sign = walk_uv(nuv, U, base, stj, x0, tx, y0, ty, ex0, etx, ey0, ety, P);
    }
    short sig[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const short mine = (k < n3) ? uv_sign(U, k) : (short)0;
        const short v = (short)__shfl_sync(0xffffffffu, (int)mine, fl < 0 ? 0 : fl);
        sig[k] = carried_f ? cs.sig[k] : v;
    }
    bool xok = false;
    short xval = 0;
    if (valid && !is_first) {
        const int xi = cross_pair_index(n3, U, base, nuv);
        if (xi >= 0) {
            const YzHit &ha = base[uv_off(U, xi)], &hb = base[uv_off(U, xi + 1)];
            const int k = lr_pair_newhits_ool(x0, tx, y0, ty, ex0, etx, ey0, ety, ha.det, hb.det, ha.pos, ha.drift,
                                              hb.pos, hb.drift, P, 150.f);
            if (k >= 0) {
                xok = true;
                xval = c_lrpossibility[k][0];
            }
        }
    }
    const unsigned xm = __ballot_sync(0xffffffffu, xok);
    const int xs = last_lane(xm & seg & lanemask_lt());
    const short xprev = (short)__shfl_sync(0xffffffffu, (int)xval, xs < 0 ? 0 : xs);
    bool pass = false;
    float chi2 = 0.f;
    if (valid && !is_first) {
        // the station-3 signs this survivor's walk would have started from:
        // the first survivor's, the last hit's re-set by an earlier survivor's
        // cross pair; its own cross pair, where resolved, already set the last
        // station-3 hit in the walk above
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < n3 && !(xok && k == n3 - 1)) uv_set_sign(U, k, sig[k]);
        if (n3 > 0 && !xok) {
            if (xs >= 0) uv_set_sign(U, n3 - 1, xprev);
            else if (g == cs.g && cs.hascross) uv_set_sign(U, n3 - 1, cs.cross);
        }
    }
    if (valid) {
        pass = yz_gates(E, P, x0, y0, tx, ty, ex0, ey0, etx, ety);
        if (pass) chi2 = yz_chi2(S, U, base, nuv, nhx, P, x0, y0, tx, ty);
    }
    // carry of the sign state to the next survivor chunk
    {
        const int last = last_lane(vm);
        const int gl = __shfl_sync(0xffffffffu, g, last < 0 ? 0 : last);
        const unsigned segl = __ballot_sync(0xffffffffu, valid && g == gl);
        const int fnew = __ffs(__ballot_sync(0xffffffffu, is_first) & segl) - 1;
        short ns[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) ns[k] = (short)__shfl_sync(0xffffffffu, (int)sig[k], fnew < 0 ? 0 : fnew);
        const int xl = last_lane(xm & segl);
        const short nx = (short)__shfl_sync(0xffffffffu, (int)xval, xl < 0 ? 0 : xl);
        const bool cont = (gl == cs.g);
        if (fnew >= 0) {
            cs.hasf = true;
#pragma unroll 1
            for (int k = 0; k < 4; ++k) cs.sig[k] = ns[k];
        } else if (!cont) {
            cs.hasf = false;
        }
        if (xl >= 0) {
            cs.hascross = true;
            cs.cross = nx;
        } else if (!cont) {
            cs.hascross = false;
        }
        cs.g = gl;
    }
    // best: min (chi2, index) over chi2 < 10000.1 (K:1778)
    const bool elig = pass && chi2 < 10000.1f;
    const unsigned key = elig ? __float_as_uint(chi2) : 0xffffffffu;
    const unsigned kmin = __reduce_min_sync(0xffffffffu, key);
    if (kmin != 0xffffffffu) {
        const int win = __ffs(__ballot_sync(0xffffffffu, key == kmin)) - 1;
        const int cw = __shfl_sync(0xffffffffu, c, win);
        const unsigned long long full = ((unsigned long long)kmin << 32) | (unsigned long long)(unsigned)cw;
        if (full < cs.best) {
            cs.best = full;
            if (lane == win) {
                S.b.key = full;
                S.b.nuv = nuv;
                S.b.chi2 = chi2;
                S.b.ty = ty;
                S.b.y0 = y0;
                S.b.ety = ety;
                S.b.ey0 = ey0;
#pragma unroll 1
                for (int n = 0; n < nuv; ++n) {
                    const YzHit &h = base[uv_off(U, n)];
                    S.b.det[n] = h.det;
                    S.b.el[n] = h.el;
                    S.b.pos[n] = h.pos;
                    S.b.drift[n] = h.drift;
                    S.b.sign[n] = uv_sign(U, n);
                    S.b.tdc[n] = h.tdc;
                }
                // the winner's residuals, recomputed as chi2 formed them
#pragma unroll 1
                for (int n = 0; n < nhx + nuv; ++n) {
                    float res;
                    S.b.res[n] = yz_residual(S, U, base, n, nhx, P, x0, y0, tx, ty, res);
                }
            }
        }
    }
    __syncwarp();
}

// Evaluate combinations [c0, c1) (whole outer iterations) of the current
// tracklet.  `st` is advanced to the scratch state after the range.  Returns
// the best key (chi2 bits << 32 | combination index) or ~0, with that
// combination's record in S.b.
//
// Phase 1 (every combination, registers only): station-3/2 load attempts in
// the reference order, the first y fit, its 2-sigma cut (K:1602-1611) and the
// scratch-entry scan.  Survivors (about 6% on the uneven batch) go to the
// warp's queue in global memory, in order.  Phase 2 (yz_phase2, 32 at a time,
// when the queue fills or the range ends): sign state, left/right walk, prop
// and hodoscope gates, chi2 (K:1613-1799).  This combined walk serves the
// planning kernel's light tracklets and the units whose survivors do not fit
// the pool; the first-cut kernel walks listed outer iterations with the
// inner pairs' records instead (yz_first_kept).
//
// Outer iterations (iu3, iv3) whose u3 pair or v3 pair gives no accepted hit
// are skipped whole: the reference leaves such an iteration before any
// station-2 load (K:1326-1390), so it neither writes a scratch entry past a
// count of 4 nor yields a candidate, and jumping over it changes nothing.

// Pairs of lists 2 (u3) and 3 (v3) with an accepted hit, as 128-bit masks
// (at most YZ_MAXPAIR = 100 pairs per list).
struct YzAlive {
    unsigned u[4], v[4];
};

__device__ __forceinline__ YzAlive yz_alive(const YzWarp &S, const YzHit *base) {
    const int lane = lane_id();
    const YzHit *l4 = yz_list(S, base, 4), *l5 = yz_list(S, base, 5);
    const YzHit *l6 = yz_list(S, base, 6), *l7 = yz_list(S, base, 7);
    YzAlive m;
#pragma unroll
    for (int w = 0; w < 4; ++w) {
        const int i = w * 32 + lane;
        bool a = false, b = false;
        if (i < S.np[2]) {
            const short2 p = S.pair[2][i];
            a = (p.x >= 0 && l4[p.x].acc) || (p.y >= 0 && l5[p.y].acc);
        }
        if (i < S.np[3]) {
            const short2 p = S.pair[3][i];
            b = (p.x >= 0 && l6[p.x].acc) || (p.y >= 0 && l7[p.y].acc);
        }
        m.u[w] = __ballot_sync(0xffffffffu, a);
        m.v[w] = __ballot_sync(0xffffffffu, b);
    }
    return m;
}

__device__ __forceinline__ int bits128(const unsigned m[4]) {
    return __popc(m[0]) + __popc(m[1]) + __popc(m[2]) + __popc(m[3]);
}

__device__ __forceinline__ bool bit128(const unsigned m[4], int i) {
    const unsigned w = i < 32 ? m[0] : (i < 64 ? m[1] : (i < 96 ? m[2] : m[3]));
    return (w >> (i & 31)) & 1u;
}

// first set bit at index >= p (0 <= p), or -1
__device__ __forceinline__ int next_bit128(const unsigned m[4], int p) {
#pragma unroll
    for (int w = 0; w < 4; ++w) {
        if (w < (p >> 5)) continue;
        unsigned v = m[w];
        if (w == (p >> 5)) v &= ~0u << (p & 31);
        if (v) return w * 32 + __ffs(v) - 1;
    }
    return -1;
}

// first outer iteration after (iu, iv), u fastest, with both pairs alive; -1 if none
__device__ __forceinline__ int next_alive_outer(const YzAlive &m, int nu3, int iu, int iv) {
    if (bit128(m.v, iv)) {
        const int u = next_bit128(m.u, iu + 1);
        if (u >= 0) return u + iv * nu3;
    }
    const int v = next_bit128(m.v, iv + 1);
    const int u = next_bit128(m.u, 0);
    return (v < 0 || u < 0) ? -1 : u + v * nu3;
}

// index of the k-th set bit (k from 0) of a 128-bit mask, or -1
__device__ __forceinline__ int nth_bit128(const unsigned m[4], int k) {
#pragma unroll 1
    for (int w = 0; w < 4; ++w) {
        const int c = __popc(m[w]);
        if (k < c) {
            unsigned v = m[w];
#pragma unroll 1
            for (int i = 0; i < k; ++i) v &= v - 1u;
            return w * 32 + __ffs(v) - 1;
        }
        k -= c;
    }
    return -1;
}

// set bits of a 128-bit mask below index i
__device__ __forceinline__ int bits_below128(const unsigned m[4], int i) {
    int c = 0;
#pragma unroll
    for (int w = 0; w < 4; ++w) {
        if (w < (i >> 5)) c += __popc(m[w]);
        else if (w == (i >> 5)) c += __popc(m[w] & ((1u << (i & 31)) - 1u));
    }
    return c;
}

// Distance from the hits of a prop-tube y plane at z = zp to the window of
// y the track can have there: through y3 at z3 with |ty| <= TY_MAX and
// |y0| <= Y0_MAX (the bounds the YZ hard cut enforces, K:1638), widened by
// the prop-tube match tolerance (K:1640-1702); 30 cm when there is no hit or
// no such line.
__device__ __forceinline__ float prop_gap(const HitPlane &h, float zp, float y3, float z3, float lo_t, float hi_t,
                                          float tol) {
    float d = 30.f;
    if (lo_t > hi_t) return d;
    const float ya = y3 + lo_t * (zp - z3), yb = y3 + hi_t * (zp - z3);
    const float lo = fminf(ya, yb) - tol, hi = fmaxf(ya, yb) + tol;
#pragma unroll 1
    for (int i = 0; i < h.n; ++i) {
        const float p = h.pos(i);
        d = fminf(d, fmaxf(fmaxf(lo - p, p - hi), 0.f));
    }
    return d;
}

// The combination scorer's 16 features of live outer iteration (iu, iv) of
// the current tracklet: the tracklet's x fit, the y of its u3 and v3 hits
// (mean of the accepted hits of each pair) and their difference against the
// x fit's error at station 3 -- the x error moves the two stereo estimates
// of y apart -- the distance of the P1 and P2 y-tube hits from the window
// the track's y can reach there, hit counts, the inner and outer loop sizes,
// the station-3 half and the tracklet's x-hit count.
__device__ void yz_outer_features(const YzWarp &S, const YzEvent &E, const YzHit *base, const or_plane_t &P, int iu,
                                  int iv, int st3, long C2, long Ga, float *f) {
    const short2 pu = S.pair[2][iu], pv = S.pair[3][iv];
    const YzHit *l4 = yz_list(S, base, 4), *l5 = yz_list(S, base, 5);
    const YzHit *l6 = yz_list(S, base, 6), *l7 = yz_list(S, base, 7);
    float su = 0.f, sv = 0.f;
    int nu = 0, nv = 0;
    if (pu.x >= 0 && l4[pu.x].acc) { su += l4[pu.x].Y; ++nu; }
    if (pu.y >= 0 && l5[pu.y].acc) { su += l5[pu.y].Y; ++nu; }
    if (pv.x >= 0 && l6[pv.x].acc) { sv += l6[pv.x].Y; ++nv; }
    if (pv.y >= 0 && l7[pv.y].acc) { sv += l7[pv.y].Y; ++nv; }
    const float yu = su / (float)max(nu, 1), yv = sv / (float)max(nv, 1);
    const float z3 = P.z[E.dl[4]];
    const float sig = fmaxf(S.ex0 + S.etx * z3, 1e-3f);
    const float y3 = 0.5f * (yu + yv);
    const float lo_t = fmaxf(-TY_MAX, (y3 - Y0_MAX) / z3), hi_t = fminf(TY_MAX, (y3 + Y0_MAX) / z3);
    const float d1 = fminf(prop_gap(E.p1y1, P.z[DET_P1Y1], y3, z3, lo_t, hi_t, 5.08f),
                           prop_gap(E.p1y2, P.z[DET_P1Y2], y3, z3, lo_t, hi_t, 5.08f));
    const float d2 = fminf(prop_gap(E.p2y1, P.z[DET_P2Y1], y3, z3, lo_t, hi_t, 10.16f),
                           prop_gap(E.p2y2, P.z[DET_P2Y2], y3, z3, lo_t, hi_t, 10.16f));
    f[0] = S.x0 * 0.01f;
    f[1] = S.tx * 10.f;
    f[2] = S.ex0;
    f[3] = S.etx * 100.f;
    f[4] = yu * 0.02f;
    f[5] = yv * 0.02f;
    f[6] = fminf(fmaxf((yu - yv) / sig, -20.f), 20.f) * 0.1f;
    f[7] = log1pf(fabsf(yu - yv));
    f[8] = d1 * 0.1f;
    f[9] = d2 * 0.1f;
    f[10] = (float)nu;
    f[11] = (float)nv;
    f[12] = log1pf((float)C2);
    f[13] = log1pf((float)Ga);
    f[14] = (float)(st3 - 3);
    f[15] = (float)S.nhx;
}


// Skip the pruned live outer iterations from rank r (the scorer's rows of
// the tracklet are its live outer iterations in loop order): returns the
// rank of the next kept one (nrows when none) and, when one follows, sets
// the scratch entries 4..7 as the skipped iterations' load attempts leave
// them in the reference -- for each entry, the last skipped iteration whose
// station-3 hit count puts one of its writes there -- so that the kept
// combinations read the same stale entries as in the plain run.
__device__ __noinline__ int yz_skip_pruned(const YzWarp &S, const YzHit *base, const YzAlive &al, int Au, int nrows,
                                           const float *__restrict__ osc, float t_keep, unsigned long long lasto,
                                           int r, int r_end, Stale st[4]) {
    const int lane = lane_id();
    int rk = nrows;  // no kept iteration before the range's end rank r_end
#pragma unroll 1
    for (int b = r; b < r_end; b += 32) {
        const int j = b + lane;
        const unsigned m = __ballot_sync(0xffffffffu, j < r_end && osc[j] >= t_keep);
        if (m) {
            rk = b + __ffs(m) - 1;
            break;
        }
    }
    if (rk >= nrows) return rk;
    unsigned done = 0u;
#pragma unroll 1
    for (int b = rk - 1; b >= r && done != 0xFu; b -= 32) {
        const int j = b - lane;  // lane 0 holds the latest rank of the chunk
        int n3 = 0;
        if (j >= r) {
            bool v;
            n3 = s3_count(S, base, nth_bit128(al.u, j % Au), nth_bit128(al.v, j / Au), v);
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (done & (1u << k)) continue;
            const int mm = k + 4 - n3;
            const bool ok = j >= r && mm >= 0 && mm < 4 && ((lasto >> (16 * mm)) & 0xFFFFull) != 0xFFFFull;
            const unsigned m = __ballot_sync(0xffffffffu, ok);
            if (m) {
                const int src = __shfl_sync(0xffffffffu, mm, __ffs(m) - 1);
                const YzHit &h = base[(int)((lasto >> (16 * src)) & 0xFFFFull)];
                const Stale v{h.det, h.pos, h.drift};
                __syncwarp();
                st[k] = v;
                done |= 1u << k;
            }
        }
    }
    __syncwarp();
    return rk;
}

// Station-3 part of the outer iteration (iu3, iv3) (K:1326-1390): the first
// y fit's right-hand side over its accepted hits in the reference order,
// their count and the table offset of the plane set.  False when the u3 or
// the v3 pair gives no accepted hit (the iteration ends before station 2).
struct Yz3 {
    float b0, b1;
    int n3, tab3;
};

__device__ __forceinline__ bool yz_station3(const YzWarp &S, const YzHit *base, int iu3, int iv3, Yz3 &o) {
    const short2 pu = S.pair[2][iu3], pv = S.pair[3][iv3];
    const unsigned long long offs = (unsigned long long)(pu.x >= 0 ? S.woff[4] + pu.x : 0xFFFF) |
                                    ((unsigned long long)(pu.y >= 0 ? S.woff[5] + pu.y : 0xFFFF) << 16) |
                                    ((unsigned long long)(pv.x >= 0 ? S.woff[6] + pv.x : 0xFFFF) << 32) |
                                    ((unsigned long long)(pv.y >= 0 ? S.woff[7] + pv.y : 0xFFFF) << 48);
    // B0 += w*y, B1 += w*y*z per accepted hit, as Fit2::add
    float b0 = 0.f, b1 = 0.f;
    int nu = 0, nv = 0, gu = 0, gv = 0;
#pragma unroll 1
    for (int a = 0; a < 4; ++a) {
        if (a == 2 && nu == 0) break;  // no u3 hit: v3 is not loaded
        const int off = (int)((offs >> (16 * a)) & 0xFFFFull);
        if (off == 0xFFFF) continue;
        const YzHit &r = base[off];
        if (!r.acc) continue;
        const float t = r.eY * r.Y;
        b0 += t;
        b1 += t * r.z;
        if (a < 2) {
            ++nu;
            gu |= 1 << a;
        } else {
            ++nv;
            gv |= 1 << (a - 2);
        }
    }
    const bool alive3 = nu > 0 && nv > 0;
    o.b0 = b0;
    o.b1 = b1;
    o.n3 = nu + nv;
    o.tab3 = alive3 ? yz_tab_index(gu, gv, 1, 1) : 0;
    return alive3;
}

// Station-2 load attempts of the inner pair (iu2, iv2) in the reference order
// (K:1467-1597) after the station-3 part s3: every attempted hit writes the
// scratch entry at the running count (4..7 at most: n3 <= 4, four attempts;
// `own` holds those writes as arena offsets, 16 bits per entry, `wmask` which
// entries), accepted ones enter the fit.  When the v2 group gives a hit and
// `fit` is set, the first y fit with the plane set's tabulated inverse and
// its 2-sigma cut (K:1602-1611).  Returns the accepted hit count.
__device__ __forceinline__ int yz_station2_fit(const YzWarp &S, const YzHit *base, int iu2, int iv2, const Yz3 &s3,
                                               bool fit, const YzTab *__restrict__ tab, unsigned long long &own,
                                               unsigned &wmask, bool &pass1, float &y0, float &ty, float &ey0,
                                               float &ety) {
    float b0 = s3.b0, b1 = s3.b1;
    int g2 = 0;  // plane bits u2 u2' v2 v2' of the accepted hits
    int nuv = s3.n3;
    const short2 pu = S.pair[0][iu2];
    auto attempt = [&](int off, int a) {
        const YzHit &r = base[off];
        const int k = nuv - 4;
        if (k >= 0) {
            const int sh = k << 4;
            own = (own & ~(0xFFFFull << sh)) | ((unsigned long long)off << sh);
            wmask |= 1u << k;
        }
        if (r.acc) {
            const float t = r.eY * r.Y;
            b0 += t;
            b1 += t * r.z;
            g2 |= 1 << a;
            ++nuv;
        }
    };
    // the four attempts as one loop body: arena offsets (0xFFFF = no hit) of
    // u2, u2', v2, v2' packed in 64 bits
    const short2 pv = S.pair[1][iv2];
    const unsigned long long offs = (unsigned long long)(pu.x >= 0 ? S.woff[0] + pu.x : 0xFFFF) |
                                    ((unsigned long long)(pu.y >= 0 ? S.woff[1] + pu.y : 0xFFFF) << 16) |
                                    ((unsigned long long)(pv.x >= 0 ? S.woff[2] + pv.x : 0xFFFF) << 32) |
                                    ((unsigned long long)(pv.y >= 0 ? S.woff[3] + pv.y : 0xFFFF) << 48);
    int nu2hits = s3.n3;
#pragma unroll 1
    for (int a = 0; a < 4; ++a) {
        if (a == 2) {
            nu2hits = nuv;
            if (nu2hits == s3.n3) break;  // the u2 group gave no hit
        }
        const int off = (int)((offs >> (16 * a)) & 0xFFFFull);
        if (off != 0xFFFF) attempt(off, a);
    }
    if (nu2hits > s3.n3 && nuv > nu2hits && fit) {  // the v2 group gave a hit: the fit is reached
        // Fit2::solve with the plane set's tabulated inverse
        const YzTab *te = tab + s3.tab3 + (g2 & 3) * 3 - 4 + (g2 >> 2);
        const float4 ai = __ldg(reinterpret_cast<const float4 *>(te));
        const float2 thr = __ldg(reinterpret_cast<const float2 *>(&te->thr_y0));
        y0 = 0.0f;
        y0 += ai.x * b0;
        y0 += ai.y * b1;
        ty = 0.0f;
        ty += ai.z * b0;
        ty += ai.w * b1;
        pass1 = !(fabsf(y0) > thr.x || fabsf(ty) > thr.y);
        if (pass1) {
            const float2 er = __ldg(reinterpret_cast<const float2 *>(&te->ey0));
            ey0 = er.x;
            ety = er.y;
        }
    }
    return nuv;
}

// One chunk's scratch entries and survivors.  Entry k+4 as the lane's
// combination c reads it: its own write, else the last earlier lane's write
// in this chunk, else the state st[] before the chunk; the chunk's last
// write becomes the new state.  `own` holds the lane's writes as arena
// offsets in the low 10 bits of 16-bit fields (entry k in field k; bits above
// them are ignored), `wmask` which entries it writes.  The survivors (pass1) go to Q[qn..] in lane
// order with the entry past their hit count; returns the new queue length.
__device__ __forceinline__ int yz_scan_queue(const YzHit *base, Stale st[4], unsigned long long own, unsigned wmask,
                                             int nuv, bool pass1, int c, float y0, float ty, float ey0, float ety,
                                             PassEntryStore *Q, int qn) {
    Stale stj{DET_SENTINEL, 0.f, 0.f};
    int stj_off = -1;
    {
        const int j = nuv;
        const unsigned lt = lanemask_lt();
#pragma unroll 1
        for (int k = 0; k < 4; ++k) {
            const bool mine = (wmask >> k) & 1u;
            const int ok = (int)((own >> (16 * k)) & 0x3FFull);  // arena offsets are below 1,024
            const unsigned m = __ballot_sync(0xffffffffu, mine);
            const int src = last_lane(m & lt);
            const int so = __shfl_sync(0xffffffffu, ok, src < 0 ? 0 : src);
            if (j == k + 4) {
                if (mine) stj_off = ok;
                else if (src >= 0) stj_off = so;
                else stj = st[k];
            }
            const int lw = last_lane(m);
            if (lw >= 0) {
                const YzHit &r = base[__shfl_sync(0xffffffffu, ok, lw)];
                __syncwarp();  // every lane has read entry k
                st[k] = Stale{r.det, r.pos, r.drift};
            }
        }
    }
    if (pass1 && stj_off >= 0) {
        const YzHit &r = base[stj_off];
        stj = Stale{r.det, r.pos, r.drift};
    }
    // --- queue the survivors in order ----------------------------------
    const unsigned pm = __ballot_sync(0xffffffffu, pass1);
    if (pass1) {
        PassEntryStore e;
        e.c = c;
        e.y0 = y0;
        e.ty = ty;
        e.ey0 = ey0;
        e.ety = ety;
        e.stdet = stj.det;
        e.stpos = stj.pos;
        e.stdrift = stj.drift;
        Q[qn + __popc(pm & lanemask_lt())] = e;
    }
    qn += __popc(pm);
    __syncwarp();
    return qn;
}

// yz_scan_queue for the first-cut kernel, with the scratch state in a
// register: field k (16 bits) of `stp` is the arena offset of the last write
// of entry k before this chunk, 0xFFFF while entry k still holds st[k] (the
// unit's starting state, which stays in shared memory unchanged).  Hits are
// read only for the survivors' entries, and a chunk without survivors only
// advances the state.
__device__ __forceinline__ int yz_scan_queue_off(const YzHit *base, const Stale *st, unsigned long long &stp,
                                                 unsigned long long own, unsigned wmask, int nuv, bool pass1, int c,
                                                 float y0, float ty, float ey0, float ety, PassEntryStore *Q, int qn) {
    const unsigned pm = __ballot_sync(0xffffffffu, pass1);
    if (pm == 0u) {
#pragma unroll 1
        for (int k = 0; k < 4; ++k) {
            const unsigned m = __ballot_sync(0xffffffffu, (wmask >> k) & 1u);
            if (m) {
                const int ok = (int)((own >> (16 * k)) & 0x3FFull);
                const unsigned long long v = (unsigned)__shfl_sync(0xffffffffu, ok, last_lane(m));
                stp = (stp & ~(0xFFFFull << (16 * k))) | (v << (16 * k));
            }
        }
        return qn;
    }
    const unsigned lt = lanemask_lt();
    int stj = -2;  // the entry past the hit count: -2 none, -1 st[kk], else an arena offset
    int kk = 0;
#pragma unroll 1
    for (int k = 0; k < 4; ++k) {
        const bool mine = (wmask >> k) & 1u;
        const int ok = (int)((own >> (16 * k)) & 0x3FFull);
        const unsigned m = __ballot_sync(0xffffffffu, mine);
        const int src = last_lane(m & lt);
        const int so = __shfl_sync(0xffffffffu, ok, src < 0 ? 0 : src);
        if (nuv == k + 4) {
            const int cur = (int)((stp >> (16 * k)) & 0xFFFFull);
            stj = mine ? ok : (src >= 0 ? so : (cur == 0xFFFF ? -1 : cur));
            kk = k;
        }
        if (m) {
            const unsigned long long v = (unsigned)__shfl_sync(0xffffffffu, ok, last_lane(m));
            stp = (stp & ~(0xFFFFull << (16 * k))) | (v << (16 * k));
        }
    }
    if (pass1) {
        Stale e3{DET_SENTINEL, 0.f, 0.f};
        if (stj >= 0) {
            const YzHit &r = base[stj];
            e3 = Stale{r.det, r.pos, r.drift};
        } else if (stj == -1) {
            e3 = st[kk];
        }
        PassEntryStore e;
        e.c = c;
        e.y0 = y0;
        e.ty = ty;
        e.ey0 = ey0;
        e.ety = ety;
        e.stdet = e3.det;
        e.stpos = e3.pos;
        e.stdrift = e3.drift;
        Q[qn + __popc(pm & lt)] = e;
    }
    qn += __popc(pm);
    __syncwarp();
    return qn;
}

template <bool PRUNE = false>
__device__ unsigned long long yz_range_t(YzWarp &S, const YzEvent &E, const YzHit *base, long c0l, long c1l,
                                         Stale st[4], const or_plane_t &P, const YzTab *__restrict__ tab,
                                         PassEntryStore *Q, int qcap, const float *__restrict__ osc = nullptr,
                                         float t_keep = 0.f) {
    const int lane = lane_id();
    const int nu2 = S.np[0], nu3 = S.np[2];
    const int C2 = S.np[0] * S.np[1];
    const int c0 = (int)c0l, c1 = (int)c1l;  // at most 100^4 combinations
    Phase2Carry cs;
    int qh = 0, qn = 0;  // survivors Q[qh..qn) wait for the full evaluation
    const int nv2 = S.np[1];
    // Lane's combination as digits (iu2, iv2, iu3, iv3) in radices (nu2, nv2,
    // nu3, nv3) -- the reference's index order (u2 fastest) -- advanced by 32
    // per chunk with carries instead of divisions.
    int d0, d1, d2, d3, s0, s1, s2, s3;
    auto set_digits = [&](int cb) {
        const int c = cb + lane;
        const int g = c / C2, r = c - g * C2;
        d0 = r % nu2;
        d1 = r / nu2;
        d2 = g % nu3;
        d3 = g / nu3;
    };
    set_digits(c0);
    {
        const int sg = 32 / C2, sr = 32 - sg * C2;
        s0 = sr % nu2;
        s1 = sr / nu2;
        s2 = sg % nu3;
        s3 = sg / nu3;
    }
    const YzAlive alive = yz_alive(S, base);
    // the combination scorer (PRUNE): live outer iterations scoring below
    // t_keep are skipped; `osc` holds the tracklet's scores in loop order
    int Au = 0, nrows = 0, r_end = 0;
    unsigned long long lasto = ~0ull;
    if constexpr (PRUNE) {
        if (osc) {
            Au = bits128(alive.u);
            nrows = Au * bits128(alive.v);
            r_end = live_before(alive.u, alive.v, nu3, (c1 + C2 - 1) / C2);  // rows of the range's outer iterations
            lasto = yz_last_writes(S, base);
        }
    }
    bool pruned3 = false;
    // station-3 part of the lane's current outer iteration (iu3, iv3): the
    // fit's right-hand side over its accepted hits in the reference order,
    // their count, the table offset of its plane set, and whether both u3
    // and v3 gave one (K:1326-1390); recomputed only when the outer digits
    // move.
    float b0_3 = 0.f, b1_3 = 0.f;
    int tab3 = 0;
    int n3 = 0;
    bool alive3 = false, need3 = true;
    int basec = c0;
    for (;;) {
        if (basec < c1) {
            // the chunk's first combination in a dead outer iteration: jump
            // to the next live one (every combination in between is dead);
            // lane 0 holds that combination's digits
            const int iu = __shfl_sync(0xffffffffu, d2, 0), iv = __shfl_sync(0xffffffffu, d3, 0);
            if (!(bit128(alive.u, iu) && bit128(alive.v, iv))) {
                const int gn = next_alive_outer(alive, nu3, iu, iv);
                basec = gn < 0 ? c1 : min(gn * C2, c1);
                if (basec < c1) set_digits(basec);
                need3 = true;
            }
        }
        if constexpr (PRUNE) {
            // the chunk's first combination in a pruned live outer
            // iteration: jump to the next kept one, with the scratch entries
            // the skipped ones write
            if (osc && basec < c1) {
                const int iu = __shfl_sync(0xffffffffu, d2, 0), iv = __shfl_sync(0xffffffffu, d3, 0);
                const int r = bits_below128(alive.v, iv) * Au + bits_below128(alive.u, iu);
                if (osc[r] < t_keep) {
                    const int rk = yz_skip_pruned(S, base, alive, Au, nrows, osc, t_keep, lasto, r, r_end, st);
                    if (rk >= nrows) {
                        basec = c1;
                    } else {
                        const int gk = nth_bit128(alive.u, rk % Au) + nth_bit128(alive.v, rk / Au) * nu3;
                        basec = min(gk * C2, c1);
                        if (basec < c1) set_digits(basec);
                    }
                    need3 = true;
                }
            }
        }
        const bool more = basec < c1;
        if (!more && qn == qh) break;
        if (more) {
            const int c = basec + lane;
            const bool valid = c < c1;
            int nuv = 0;
            // scratch entries this combination writes (offsets 4..7 past the
            // hit count): arena offsets of the hits, 16 bits each
            unsigned long long own = 0ull;
            unsigned wmask = 0u;
            float y0 = 0.f, ty = 0.f, ey0 = 0.f, ety = 0.f;
            bool pass1 = false;
            if (valid) {
                if (need3) {
                    Yz3 t3;
                    alive3 = yz_station3(S, base, d2, d3, t3);
                    b0_3 = t3.b0;
                    b1_3 = t3.b1;
                    n3 = t3.n3;
                    tab3 = t3.tab3;
                    if constexpr (PRUNE) {
                        pruned3 = osc && alive3 &&
                                  osc[bits_below128(alive.v, d3) * Au + bits_below128(alive.u, d2)] < t_keep;
                    }
                    need3 = false;
                }
                if (alive3)
                    nuv = yz_station2_fit(S, base, d0, d1, Yz3{b0_3, b1_3, n3, tab3}, !pruned3, tab, own, wmask, pass1,
                                          y0, ty, ey0, ety);
            }
            qn = yz_scan_queue(base, st, own, wmask, nuv, pass1, c, y0, ty, ey0, ety, Q, qn);
            // --- next chunk: digits + 32 -----------------------------------------
            basec += 32;
            d0 += s0;
            int cy = d0 >= nu2;
            d0 -= cy ? nu2 : 0;
            d1 += s1 + cy;
            cy = d1 >= nv2;
            d1 -= cy ? nv2 : 0;
            if (cy || s2 || s3) need3 = true;
            d2 += s2 + cy;
            cy = d2 >= nu3;
            d2 -= cy ? nu3 : 0;
            d3 += s3 + cy;
        }
        if (qn > qcap - 32 || (!more && qn > qh)) {
            // a full queue (the next chunk could add 32) or the end of the
            // range: evaluate every waiting survivor, 32 at a time, in order
            while (qh < qn) {
                const int n = min(qn - qh, 32);
                yz_phase2(S, E, base, C2, P, Q + qh, n, cs);
                qh += n;
                __syncwarp();
            }
            qh = qn = 0;
        }
    }
    return cs.best;
}


// The first cut of one unit over its live outer iterations, or with the
// combination scorer (`osc`) over the kept ones only (first kernel).  The unit's live outer iterations
// -- the scorer's rows [r0, r1) of its tracklet, in loop order -- are
// classified 32 at a time; the kept ones go, 32 at a time, into a list in
// the warp's shared memory, each with the scratch writes of
// the pruned iterations right before it (its gap: for every entry 4..7 the
// arena offset of the last pruned iteration's write there, from the load
// pattern alone, as yz_skip_pruned finds it).  The list's combinations are
// then walked densely, 32 a chunk, as yz_range_t walks a range; the first
// combination of a kept iteration counts its gap's writes as its own, made
// before its own loads, so every survivor reads the scratch entry of the
// plain run.  A combination's station-2 part comes from the record of its
// inner pair (R, yz_s2_record); its station-3 part is computed once per
// listed iteration.  Survivors go to Q in order; *nsurv = their count, or -1
// when the queue could overflow (the unit then runs on the combined path).

// inner-pair records (8 B) that fit the per-warp overflow arena, where the
// first cut keeps them when the shared ones do not suffice
constexpr int YZ_RECORDS_MAX = (int)(YZ_GARENA_HITS * sizeof(YzHit) / 8);
static_assert(sizeof(YzEvent) >= sizeof(unsigned long long) * YZ_KEPT_BATCH, "the listed gaps fit the event's views");

__device__ void yz_first_kept(YzWarp &S, const YzHit *base, int r0, int r1, Stale st[4],
                              const YzTab *__restrict__ tab, PassEntryStore *Q, int qcap, int *nsurv,
                              const float *__restrict__ osc, float t_keep, const unsigned long long *R) {
    const int lane = lane_id();
    const unsigned lt = lanemask_lt();
    const int nu2 = S.np[0], nv2 = S.np[1], nu3 = S.np[2];
    const int C2 = nu2 * nv2;
    const YzAlive alive = yz_alive(S, base);
    const int Au = bits128(alive.u);
    const unsigned long long lasto = osc ? yz_last_writes(S, base) : ~0ull;
    const int sg = 32 / C2, sr = 32 - sg * C2;
    const int s0 = sr % nu2, s1 = sr / nu2;  // a chunk's step in the inner digits ...
    int qn = 0;
    unsigned long long stp = ~0ull;  // scratch entries' last writes (yz_scan_queue_off)
    unsigned long long gapc = ~0ull;  // writes of the pruned iterations since the last kept one
    int r = r0;
    while (r < r1) {
        // --- the next kept iterations and their gaps ---------------------
        int nk = 0;
        __syncwarp();  // every lane is done with the previous list
        while (r < r1 && nk <= YZ_KEPT_BATCH - 32) {
            const int j = r + lane;
            const bool in = j < r1;
            bool kept = false;
            int iu = 0, iv = 0;
            unsigned long long w = ~0ull;  // this pruned iteration's writes
            if (in) {
                kept = !osc || osc[j] >= t_keep;
                iu = nth_bit128(alive.u, j % Au);
                iv = nth_bit128(alive.v, j / Au);
                if (!kept) {
                    bool v;
                    const int n3 = s3_count(S, base, iu, iv, v);
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const int mm = k + 4 - n3;
                        if (mm >= 0 && mm < 4)
                            w = (w & ~(0xFFFFull << (16 * k))) | (((lasto >> (16 * mm)) & 0xFFFFull) << (16 * k));
                    }
                }
            }
            const unsigned km = __ballot_sync(0xffffffffu, kept);
            const int lk = last_lane(km & lt);  // the last kept lane before this one
            const unsigned after = lk >= 0 ? ~((2u << lk) - 1u) : 0xffffffffu;
            const int lka = last_lane(km);  // ... and of the chunk
            const unsigned aftera = lka >= 0 ? ~((2u << lka) - 1u) : 0xffffffffu;
            unsigned long long gap = 0ull, carry = 0ull;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const unsigned wk = (unsigned)((w >> (16 * k)) & 0xFFFFull);
                const unsigned ck = (unsigned)((gapc >> (16 * k)) & 0xFFFFull);
                const unsigned pm = __ballot_sync(0xffffffffu, wk != 0xFFFFu);
                const int src = last_lane(pm & lt & after);
                const unsigned v = __shfl_sync(0xffffffffu, wk, src < 0 ? 0 : src);
                const unsigned g = src >= 0 ? v : (lk >= 0 ? 0xFFFFu : ck);
                gap |= (unsigned long long)g << (16 * k);
                const int srca = last_lane(pm & aftera);
                const unsigned va = __shfl_sync(0xffffffffu, wk, srca < 0 ? 0 : srca);
                const unsigned ga = srca >= 0 ? va : (lka >= 0 ? 0xFFFFu : ck);
                carry |= (unsigned long long)ga << (16 * k);
            }
            gapc = carry;
            if (kept) {
                const int pos = nk + __popc(km & lt);
                S.kuv[pos] = (unsigned short)(iu | (iv << 8));
                S.kgap[pos] = gap;
            }
            nk += __popc(km);
            r += 32;
        }
        __syncwarp();  // the list is written
        // --- their combinations, 32 a chunk ------------------------------
        const int ctot = nk * C2;
        int k = lane / C2, d0, d1;
        {
            const int rr = lane - k * C2;
            d0 = rr % nu2;
            d1 = rr / nu2;
        }
        int kl = -1;  // list index whose station-3 part the lane holds
        Yz3 t3{0.f, 0.f, 0, 0};
        bool alive3 = false;
#pragma unroll 1
        for (int cb = 0; cb < ctot; cb += 32) {
            const bool valid = cb + lane < ctot;
            int nuv = 0, c = 0;
            unsigned long long own = 0ull;
            unsigned wmask = 0u;
            float y0 = 0.f, ty = 0.f, ey0 = 0.f, ety = 0.f;
            bool pass1 = false;
            if (valid) {
                const unsigned uv = S.kuv[k];
                const int iu3 = (int)(uv & 0xFFu), iv3 = (int)(uv >> 8);
                if (k != kl) {
                    alive3 = yz_station3(S, base, iu3, iv3, t3);
                    kl = k;
                }
                const int r2 = d1 * nu2 + d0;
                c = (iu3 + iv3 * nu3) * C2 + r2;
                if (r2 == 0) {
                    // the gap's writes come before the iteration's own
                    own = S.kgap[k];
#pragma unroll
                    for (int e = 0; e < 4; ++e)
                        if (((own >> (16 * e)) & 0xFFFFull) != 0xFFFFull) wmask |= 1u << e;
                }
                if (alive3) {
                    // the inner pair's attempts: scratch writes shifted by the
                    // station-3 count (n3 = 2..4), accepted hits in order
                    const unsigned long long rec = R[r2];
                    const int sh = 4 - t3.n3;
                    const int nacc = (int)((rec >> 26) & 7u);
                    const unsigned wr = ((unsigned)(rec >> 10) & 0xFu) >> sh;
                    const unsigned long long mine = rec >> (16 * sh);
#pragma unroll
                    for (int e = 0; e < 4; ++e)
                        if ((wr >> e) & 1u) own = (own & ~(0xFFFFull << (16 * e))) | (mine & (0xFFFFull << (16 * e)));
                    wmask |= wr;
                    nuv = t3.n3 + nacc;
                    if ((rec >> 58) & 1u) {
                        // Fit2::solve with the plane set's tabulated inverse
                        float b0 = t3.b0, b1 = t3.b1;
#pragma unroll 1
                        for (int e = 0; e < nacc; ++e) {
                            const YzHit &h = base[(int)((rec >> (16 * e)) & 0x3FFull)];
                            const float t = h.eY * h.Y;
                            b0 += t;
                            b1 += t * h.z;
                        }
                        const unsigned g2 = (unsigned)(rec >> 42) & 0xFu;
                        const YzTab *te = tab + t3.tab3 + (g2 & 3u) * 3 - 4 + (g2 >> 2);
                        const float4 ai = __ldg(reinterpret_cast<const float4 *>(te));
                        const float2 thr = __ldg(reinterpret_cast<const float2 *>(&te->thr_y0));
                        y0 = 0.0f;
                        y0 += ai.x * b0;
                        y0 += ai.y * b1;
                        ty = 0.0f;
                        ty += ai.z * b0;
                        ty += ai.w * b1;
                        pass1 = !(fabsf(y0) > thr.x || fabsf(ty) > thr.y);
                        if (pass1) {
                            const float2 er = __ldg(reinterpret_cast<const float2 *>(&te->ey0));
                            ey0 = er.x;
                            ety = er.y;
                        }
                    }
                }
            }
            qn = yz_scan_queue_off(base, st, stp, own, wmask, nuv, pass1, c, y0, ty, ey0, ety, Q, qn);
            if (qn > qcap - 32) {
                *nsurv = -1;
                return;
            }
            d0 += s0;
            int cy = d0 >= nu2;
            d0 -= cy ? nu2 : 0;
            d1 += s1 + cy;
            cy = d1 >= nv2;
            d1 -= cy ? nv2 : 0;
            k += sg + cy;
        }
    }
    *nsurv = qn;
}


// The combined evaluation of a range, out of line: the survivor kernel runs
// it only for units whose survivors did not fit the pool, the planning
// kernel for light tracklets, and inlined its registers would weigh on the
// rest of those kernels.
template <bool PRUNE>
__device__ __noinline__ unsigned long long yz_range_ool(YzWarp &S, const YzEvent &E, const YzHit *base, long c0l,
                                                        long c1l, Stale *st, const or_plane_t &P, const YzTab *tab,
                                                        PassEntryStore *Q, int qcap, const float *osc, float t_keep) {
    return yz_range_t<PRUNE>(S, E, base, c0l, c1l, st, P, tab, Q, qcap, osc, t_keep);
}

// write the best combination into the track record (K:1804-1825)
__device__ __forceinline__ void yz_store(float *T, const YzBest &b, int nhx) {
    const int lane = lane_id();
    const int nuv = b.nuv;
    if (lane == 0) {
        T[OR_TRK_STID] = 5.f;
        T[OR_TRK_NHITS] = (float)nhx + (float)nuv;
        T[OR_TRK_CHI2] = b.chi2;
        T[OR_TRK_TY] = b.ty;
        T[OR_TRK_Y0] = b.y0;
        T[OR_TRK_ERR_TY] = b.ety;
        T[OR_TRK_ERR_Y0] = b.ey0;
    }
    if (lane < nuv) {
        const int n = lane;
        T[OR_TRK_HIT_DETID + nhx + n] = b.det[n];
        T[OR_TRK_HIT_CHAN + nhx + n] = b.el[n];
        T[OR_TRK_HIT_POS + nhx + n] = b.pos[n];
        T[OR_TRK_HIT_DRIFT + nhx + n] = b.drift[n];
        T[OR_TRK_HIT_SIGN + nhx + n] = b.sign[n];
        T[OR_TRK_HIT_TDC + nhx + n] = b.tdc[n];
        if (n < nhx) T[OR_TRK_HIT_RESID + n] = b.res[n];
        T[OR_TRK_HIT_RESID + nhx + n] = b.res[nhx + n];
    }
}

__device__ __forceinline__ YzHit *yz_garena(const YzScratch &sc, int gwarp) {
    return sc.garena + (long)(gwarp % sc.garena_warps) * YZ_GARENA_HITS;
}

// Work of a tracklet's first cut, from its pair lists: a combination reaches
// the first y fit when each of the u3, v3, u2 and v2 pairs gives an accepted
// hit, so the fitted combinations are the product of the four counts of such
// pairs, and the sum of their hit counts follows from each projection's
// accepted hits.  Returned on every lane.
__device__ void yz_fit_counts(const YzWarp &S, const YzHit *base, unsigned long long &fitted,
                              unsigned long long &hitsum) {
    const int lane = lane_id();
    unsigned long long A[4], H[4];
#pragma unroll 1
    for (int q = 0; q < 4; ++q) {
        const YzHit *la = yz_list(S, base, 2 * q), *lb = yz_list(S, base, 2 * q + 1);
        unsigned a = 0, h = 0;
#pragma unroll 1
        for (int i = lane; i < S.np[q]; i += 32) {
            const short2 p = S.pair[q][i];
            const unsigned k = (p.x >= 0 && la[p.x].acc ? 1u : 0u) + (p.y >= 0 && lb[p.y].acc ? 1u : 0u);
            a += k > 0;
            h += k;
        }
        A[q] = __reduce_add_sync(0xffffffffu, a);
        H[q] = __reduce_add_sync(0xffffffffu, h);
    }
    fitted = A[0] * A[1] * A[2] * A[3];
    hitsum = H[0] * A[1] * A[2] * A[3] + A[0] * H[1] * A[2] * A[3] + A[0] * A[1] * H[2] * A[3] +
             A[0] * A[1] * A[2] * H[3];
}

__device__ __forceinline__ void yz_flush_counts(const YzScratch &sc, unsigned long long fitted,
                                                unsigned long long hitsum, unsigned long long nsurv) {
    unsigned long long *c = reinterpret_cast<unsigned long long *>(sc.counters);
    if (fitted) atomicAdd(c + YZ_CTR_FITTED / 2, fitted);
    if (hitsum) atomicAdd(c + YZ_CTR_HITSUM / 2, hitsum);
    if (nsurv) atomicAdd(c + YZ_CTR_SURVIVORS / 2, nsurv);
}

template <int W>
__global__ void __launch_bounds__(W * 32, (OR_YZ_PLAN_WARPS_SM / W > 0 ? OR_YZ_PLAN_WARPS_SM / W : 1))
    yz_plan_kernel(const or_plane_t *__restrict__ gplane, or_hits_view_t hv, or_tracks_view_t tv,
                   const uint8_t *__restrict__ toomany, int n_events, YzScratch sc, uint32_t *__restrict__ errw,
                   YzPrune prune) {
    extern __shared__ __align__(16) unsigned char yz_smem[];
    or_plane_t &P = *reinterpret_cast<or_plane_t *>(yz_smem);
    YzWarp *warps = reinterpret_cast<YzWarp *>(yz_smem + ((sizeof(or_plane_t) + 15) & ~size_t(15)));
    load_plane_smem(&P, gplane);
    __syncthreads();
    const int w = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    YzWarp &S = warps[w];
    YzHit *garena = yz_garena(sc, blockIdx.x * W + w);
    PassEntryStore *Q = sc.qbuf + (long)((blockIdx.x * W + w) % sc.garena_warps) * sc.qcap;
    if (lane == 0) S.nsurv = 0ull;
    unsigned long long n_fitted = 0ull, n_hitsum = 0ull;  // lane 0's work counters

    // planning units (event, YZ_PLAN_CHUNK slots) from a device counter: slots
    // are independent (one reference thread each), events very uneven
    const unsigned long long nplan = (unsigned long long)n_events * (OR_NSLOTS / YZ_PLAN_CHUNK);
    unsigned long long *plan_ctr = reinterpret_cast<unsigned long long *>(sc.counters + 4);
    for (;;) {
        unsigned long long pu = 0;
        if (lane == 0) pu = atomicAdd(plan_ctr, 1ull);
        pu = __shfl_sync(0xffffffffu, pu, 0);
        if (pu >= nplan) break;
        const long e = (long)(pu / (OR_NSLOTS / YZ_PLAN_CHUNK));
        const int slot0 = (int)(pu % (OR_NSLOTS / YZ_PLAN_CHUNK)) * YZ_PLAN_CHUNK;
        if (toomany[e]) continue;  // K:873-878
        long budget = YZ_CHUNK_INLINE;
        long row = 0;  // scorer row of the next tracklet (slots in order, tracklets in slot order)
        if (prune.keep) {
            row = prune.row_off[e];
#pragma unroll 1
            for (int s = 0; s < slot0; ++s) row += min((int)tv.ntracks[e * OR_NSLOTS + s], OR_SLOTCAP);
        }
#pragma unroll 1
        for (int slot = slot0; slot < slot0 + YZ_PLAN_CHUNK; ++slot) {
            const int ntr = min((int)tv.ntracks[e * OR_NSLOTS + slot], OR_SLOTCAP);
            const long slot_row = row;
            row += ntr;
            if (ntr == 0) continue;
            const int st3 = 3 + (slot & 1);  // K:884
            YzEvent &E = S.ev;
            __syncwarp();  // every lane is done with the previous slot's views
            yz_event_planes(E, hv, e, st3);
            __syncwarp();
            Stale *st = S.st;
            __syncwarp();  // every lane is done with the previous slot's states
#pragma unroll 1
            for (int k = 0; k < 4; ++k) st[k] = Stale{DET_SENTINEL, 0.f, 0.f};
            __syncwarp();
#pragma unroll 1
            for (int it = 0; it < ntr; ++it) {
                float *T = trk_rec(tv, e, slot, it);
                const YzHit *base;
                const bool fits = yz_build(S, E, T, P, st3, base, garena);
                if (lane == 0) T[OR_TRK_STID] = 3.f;  // K:1285
                if (!fits) {
                    if (lane == 0) atomicOr(errw, ERRW_CAPACITY);
                    continue;
                }
                const int nu2 = S.np[0], nv2 = S.np[1], nu3 = S.np[2], nv3 = S.np[3];
                if (nu2 == 0 || nu3 == 0 || nv2 == 0 || nv3 == 0) continue;
                const long C2 = (long)nu2 * nv2;
                const long G = (long)nu3 * nv3;
                if (prune.keep) {
                    const long r = slot_row + it;
                    if (r < prune.max_rows && !prune.keep[r]) {
                        // pruned: no combination is evaluated, as when none
                        // passes; the scratch entries still advance over its
                        // load pattern so later tracklets of the slot see the
                        // plain state
                        yz_unit_states(S, base, (int)G, 1, st, nullptr, 0);
                        __syncwarp();
                        continue;
                    }
                }
                const YzAlive al = yz_alive(S, base);
                const long Ga = (long)bits128(al.u) * bits128(al.v);  // live outer iterations
                if (Ga == 0) continue;  // no candidate and no scratch entry past 3 written
                if (sc.count_work) {
                    unsigned long long f, h;
                    yz_fit_counts(S, base, f, h);
                    n_fitted += f;
                    n_hitsum += h;
                }
                yz_xhits(S, T, P);
                const long C = G * C2;
                const long Cl = Ga * C2 + G;  // live combinations, plus one step per outer iteration
                bool inline_it = Cl <= YZ_LIGHT && Cl <= budget;
                if (!inline_it) {
                    // whole outer iterations per unit, about YZ_UNIT live combinations each
                    const long gper = max(1L, min(G, (YZ_UNIT * G) / (Ga * C2)));
                    const int nunits = (int)((G + gper - 1) / gper);
                    int hid = 0, u0 = 0;
                    if (lane == 0) {
                        hid = (int)atomicAdd(&sc.counters[1], 1u);
                        u0 = (int)atomicAdd(&sc.counters[0], (unsigned)nunits);
                    }
                    hid = __shfl_sync(0xffffffffu, hid, 0);
                    u0 = __shfl_sync(0xffffffffu, u0, 0);
                    if (hid >= sc.cap_heavy || (long)u0 + nunits > sc.cap_units) {
                        // no room on the queue: evaluate here; void the reserved units
#pragma unroll 1
                        for (int u = lane; u < nunits; u += 32)
                            if (u0 + u < sc.cap_units) sc.units[u0 + u].heavy = -1;
                        if (lane == 0 && hid < sc.cap_heavy) sc.heavy[hid].nunits = 0;
                        inline_it = true;
                    } else {
                        // the combination scorer's rows: one per live outer iteration
                        int orow0 = -1;
                        if (prune.ofeat) {
                            unsigned r0 = 0u;
                            if (lane == 0) r0 = atomicAdd(prune.orows, (unsigned)Ga);
                            r0 = __shfl_sync(0xffffffffu, r0, 0);
                            if ((long)r0 + Ga <= prune.cap_orows) {
                                orow0 = (int)r0;
                                const int Au = bits128(al.u);
#pragma unroll 1
                                for (long r = lane; r < Ga; r += 32) {
                                    const int iu = nth_bit128(al.u, (int)(r % Au)), iv = nth_bit128(al.v, (int)(r / Au));
                                    float f[OR_NFEAT];
                                    yz_outer_features(S, E, base, P, iu, iv, st3, C2, Ga, f);
                                    float4 *dst = reinterpret_cast<float4 *>(prune.ofeat + (r0 + r) * OR_NFEAT);
#pragma unroll
                                    for (int q = 0; q < OR_NFEAT / 4; ++q)
                                        dst[q] = make_float4(f[4 * q], f[4 * q + 1], f[4 * q + 2], f[4 * q + 3]);
                                    prune.og[r0 + r] = iu + iv * nu3;
                                }
                            }
                        }
                        const int img = sc.img_cap > 0 ? yz_store_image(S, base, sc) : -1;
                        if (lane == 0) {
                            YzHeavy hv2;
                            hv2.img = img;
                            hv2.e = (int)e;
                            hv2.slot = slot;
                            hv2.k = it;
                            hv2.unit0 = u0;
                            hv2.nunits = nunits;
                            hv2.orow0 = orow0;
                            hv2.nrows = (int)Ga;
                            hv2.c2 = (int)C2;
                            hv2.best_g = -1;
                            sc.heavy[hid] = hv2;
                        }
                        yz_unit_states(S, base, (int)G, (int)gper, st, sc.units + u0, hid, al.u, al.v);
                    }
                }
                if (inline_it) {
                    budget -= Cl;
                    const unsigned long long bk =
                        yz_range_ool<false>(S, E, base, 0, C, st, P, sc.tab + YZ_TAB_SETS * (st3 - 3), Q, sc.qcap,
                                            nullptr, 0.f);
                    __syncwarp();
                    if (bk != ~0ull) yz_store(T, S.b, S.nhx);
                }
                __syncwarp();
            }
        }
    }
    __syncwarp();
    if (lane == 0 && sc.count_work) yz_flush_counts(sc, n_fitted, n_hitsum, S.nsurv);
}

// the scores of a queued tracklet's live outer iterations, when the
// combination scorer prunes it (rows written, event not uncertain)
__device__ __forceinline__ const float *yz_tracklet_scores(const YzPrune &prune, const YzHeavy &h) {
    if (!prune.model || h.orow0 < 0 || (prune.unc && prune.unc[h.e])) return nullptr;
    return prune.oscore + h.orow0;
}

// persistent warps drain the unit queue
template <int W, bool PRUNE>
__global__ void __launch_bounds__(W * 32, (OR_YZ_WARPS_SM / W > 0 ? OR_YZ_WARPS_SM / W : 1))
    yz_work_kernel(const or_plane_t *__restrict__ gplane, or_hits_view_t hv, or_tracks_view_t tv, YzScratch sc,
                   YzPrune prune) {
    extern __shared__ __align__(16) unsigned char yz_smem[];
    or_plane_t &P = *reinterpret_cast<or_plane_t *>(yz_smem);
    YzWarp *warps = reinterpret_cast<YzWarp *>(yz_smem + ((sizeof(or_plane_t) + 15) & ~size_t(15)));
    load_plane_smem(&P, gplane);
    __syncthreads();
    const int w = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    YzWarp &S = warps[w];
    YzHit *garena = yz_garena(sc, blockIdx.x * W + w);
    PassEntryStore *Q = sc.qbuf + (long)((blockIdx.x * W + w) % sc.garena_warps) * sc.qcap;
    if (lane == 0) S.nsurv = 0ull;
    __syncwarp();
    const int nunits = min((int)sc.counters[0], sc.cap_units);
    for (;;) {
        int u = 0;
        if (lane == 0) u = (int)atomicAdd(&sc.counters[2], 1u);
        u = __shfl_sync(0xffffffffu, u, 0);
        if (u >= nunits) break;
        const YzUnit un = sc.units[u];
        if (un.heavy < 0) continue;
        const YzHeavy hv2 = sc.heavy[un.heavy];
        const float *T = trk_rec(tv, hv2.e, hv2.slot, hv2.k);
        const int st3 = 3 + (hv2.slot & 1);
        YzEvent &E = S.ev;
        __syncwarp();  // every lane is done with the previous unit's views
        yz_event_planes(E, hv, hv2.e, st3);
        __syncwarp();
        const YzHit *base;
        if (hv2.img >= 0) base = yz_load_image(S, sc.img + hv2.img);
        else yz_build(S, E, T, P, st3, base, garena);
        yz_xhits(S, T, P);
        Stale *st = S.st;
        __syncwarp();  // every lane is done with the previous unit's states
#pragma unroll 1
        for (int k = 0; k < 4; ++k) st[k] = un.entry[k];
        __syncwarp();
        const long C2 = (long)S.np[0] * S.np[1];
        const float *osc = PRUNE ? yz_tracklet_scores(prune, hv2) : nullptr;
        const unsigned long long bk =
            yz_range_t<PRUNE>(S, E, base, (long)un.g0 * C2, (long)un.g1 * C2, st, P,
                              sc.tab + YZ_TAB_SETS * (st3 - 3), Q, sc.qcap, osc, prune.t_keep);
        __syncwarp();
        YzBest *dst = sc.best + u;
        if (bk == ~0ull) {
            if (lane == 0) dst->key = ~0ull;
        } else {
            const unsigned *src = reinterpret_cast<const unsigned *>(&S.b);
            unsigned *d = reinterpret_cast<unsigned *>(dst);
#pragma unroll 1
            for (int i = lane; i < (int)(sizeof(YzBest) / 4); i += 32) d[i] = src[i];
        }
        __syncwarp();
    }
    if (lane == 0 && sc.count_work) yz_flush_counts(sc, 0ull, 0ull, S.nsurv);
}


// Split path, first kernel: the first cut of every queued unit (no survivor
// evaluation, so it needs far fewer registers and no per-lane hit arrays);
// a unit's survivors go, in order, to one contiguous piece of the pool.

template <int W, bool PRUNE>
__global__ void __launch_bounds__(W * 32, (OR_YZ_FIRST_WARPS_SM / W > 0 ? OR_YZ_FIRST_WARPS_SM / W : 1))
    yz_first_kernel(const or_plane_t *__restrict__ gplane, or_hits_view_t hv, or_tracks_view_t tv, YzScratch sc,
                    YzPrune prune) {
    extern __shared__ __align__(16) unsigned char yz_smem[];
    or_plane_t &P = *reinterpret_cast<or_plane_t *>(yz_smem);
    YzWarp *warps = reinterpret_cast<YzWarp *>(yz_smem + ((sizeof(or_plane_t) + 15) & ~size_t(15)));
    load_plane_smem(&P, gplane);
    __syncthreads();
    const int w = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    YzWarp &S = warps[w];
    const int gw = blockIdx.x * W + w;
    if (gw >= sc.garena_warps) return;  // queues and arenas exist for garena_warps warps
    YzHit *garena = yz_garena(sc, gw);
    PassEntryStore *Q = sc.qbuf + (long)gw * sc.qcap;
    unsigned long long *pool_ctr = reinterpret_cast<unsigned long long *>(sc.counters + 8);
    const int nunits = min((int)sc.counters[0], sc.cap_units);
    for (;;) {
        int u = 0;
        if (lane == 0) u = (int)atomicAdd(&sc.counters[2], 1u);
        u = __shfl_sync(0xffffffffu, u, 0);
        if (u >= nunits) break;
        const YzUnit un = sc.units[u];
        if (un.heavy < 0) continue;
        const YzHeavy hv2 = sc.heavy[un.heavy];
        const float *T = trk_rec(tv, hv2.e, hv2.slot, hv2.k);
        const int st3 = 3 + (hv2.slot & 1);
        YzEvent &E = S.ev;
        const YzHit *base;
        __syncwarp();  // every lane is done with the previous unit's state
        if (hv2.img >= 0) {
            base = yz_load_image(S, sc.img + hv2.img);
        } else {
            yz_event_planes(E, hv, hv2.e, st3);
            __syncwarp();
            yz_build(S, E, T, P, st3, base, garena);
        }
        Stale *st = S.st;
        __syncwarp();
#pragma unroll 1
        for (int k = 0; k < 4; ++k) st[k] = un.entry[k];
        __syncwarp();
        const int C2 = S.np[0] * S.np[1];
        int ns = -1;  // -1: the unit runs on the combined path (survivor kernel)
        if (C2 <= YZ_REC_SMEM || (hv2.img >= 0 && C2 <= YZ_RECORDS_MAX)) {
            // the inner pairs' records: in shared memory (the window indices
            // are not needed once the windows exist), else in the per-warp
            // overflow arena, free when the windows came from an image
            unsigned long long *R = C2 <= YZ_REC_SMEM ? S.rec : reinterpret_cast<unsigned long long *>(garena);
            const int nu2 = S.np[0];
#pragma unroll 1
            for (int r = lane; r < C2; r += 32) R[r] = yz_s2_record(S, base, r % nu2, r / nu2);
            __syncwarp();
            const float *osc = PRUNE ? yz_tracklet_scores(prune, hv2) : nullptr;
            yz_first_kept(S, base, un.r0, un.r1, st, sc.tab + YZ_TAB_SETS * (st3 - 3), Q, sc.qcap, &ns, osc,
                          prune.t_keep, R);
        }
        __syncwarp();
        long long off = -1;
        if (lane == 0 && ns >= 0) {
            const unsigned long long o = atomicAdd(pool_ctr, (unsigned long long)ns);
            if (o + (unsigned long long)ns <= (unsigned long long)sc.pool_cap) off = (long long)o;
        }
        off = __shfl_sync(0xffffffffu, off, 0);
        if (off >= 0) {
            const uint4 *src = reinterpret_cast<const uint4 *>(Q);
            uint4 *dst = reinterpret_cast<uint4 *>(sc.pool + off);
#pragma unroll 1
            for (int i = lane; i < ns * 2; i += 32) dst[i] = src[i];
        }
        if (lane == 0) sc.useg[u] = make_int2(off >= 0 ? (int)off : -1, off >= 0 ? ns : 0);
        __syncwarp();
    }
}

// Split path, second kernel: per unit, the windows again and then its
// survivors replayed in order with the sign carry (or the whole unit on the
// combined path when its survivors did not fit); writes the unit's best.
#ifndef OR_YZ_SECOND_WARPS_SM
#define OR_YZ_SECOND_WARPS_SM 28
#endif
template <int W, bool PRUNE>
__global__ void __launch_bounds__(W * 32, (OR_YZ_SECOND_WARPS_SM / W > 0 ? OR_YZ_SECOND_WARPS_SM / W : 1))
    yz_second_kernel(const or_plane_t *__restrict__ gplane, or_hits_view_t hv, or_tracks_view_t tv, YzScratch sc,
                     YzPrune prune) {
    extern __shared__ __align__(16) unsigned char yz_smem[];
    or_plane_t &P = *reinterpret_cast<or_plane_t *>(yz_smem);
    YzWarp *warps = reinterpret_cast<YzWarp *>(yz_smem + ((sizeof(or_plane_t) + 15) & ~size_t(15)));
    load_plane_smem(&P, gplane);
    __syncthreads();
    const int w = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    YzWarp &S = warps[w];
    const int gw = blockIdx.x * W + w;
    if (gw >= sc.garena_warps) return;
    YzHit *garena = yz_garena(sc, gw);
    PassEntryStore *Q = sc.qbuf + (long)gw * sc.qcap;
    if (lane == 0) S.nsurv = 0ull;
    __syncwarp();
    const int nunits = min((int)sc.counters[0], sc.cap_units);
    for (;;) {
        int u = 0;
        if (lane == 0) u = (int)atomicAdd(&sc.counters[3], 1u);
        u = __shfl_sync(0xffffffffu, u, 0);
        if (u >= nunits) break;
        const YzUnit un = sc.units[u];
        if (un.heavy < 0) continue;
        const int2 seg = sc.useg[u];
        if (seg.x >= 0 && seg.y == 0) {  // no survivor: nothing to evaluate
            if (lane == 0) sc.best[u].key = ~0ull;
            continue;
        }
        const YzHeavy hv2 = sc.heavy[un.heavy];
        const float *T = trk_rec(tv, hv2.e, hv2.slot, hv2.k);
        const int st3 = 3 + (hv2.slot & 1);
        YzEvent &E = S.ev;
        __syncwarp();
        yz_event_planes(E, hv, hv2.e, st3);
        __syncwarp();
        const YzHit *base;
        if (hv2.img >= 0) base = yz_load_image(S, sc.img + hv2.img);
        else yz_build(S, E, T, P, st3, base, garena);
        yz_xhits(S, T, P);
        const long C2 = (long)S.np[0] * S.np[1];
        unsigned long long bk;
        if (seg.x < 0) {
            Stale *st = S.st;
            __syncwarp();
#pragma unroll 1
            for (int k = 0; k < 4; ++k) st[k] = un.entry[k];
            __syncwarp();
            const float *osc = PRUNE ? yz_tracklet_scores(prune, hv2) : nullptr;
            bk = yz_range_ool<PRUNE>(S, E, base, (long)un.g0 * C2, (long)un.g1 * C2, st, P,
                                     sc.tab + YZ_TAB_SETS * (st3 - 3), Q, sc.qcap, osc, prune.t_keep);
        } else {
            Phase2Carry cs;
#pragma unroll 1
            for (int i = 0; i < seg.y; i += 32) {
                yz_phase2(S, E, base, (int)C2, P, sc.pool + seg.x + i, min(seg.y - i, 32), cs);
                __syncwarp();
            }
            bk = cs.best;
        }
        __syncwarp();
        YzBest *dst = sc.best + u;
        if (bk == ~0ull) {
            if (lane == 0) dst->key = ~0ull;
        } else {
            const unsigned *src = reinterpret_cast<const unsigned *>(&S.b);
            unsigned *d = reinterpret_cast<unsigned *>(dst);
#pragma unroll 1
            for (int i = lane; i < (int)(sizeof(YzBest) / 4); i += 32) d[i] = src[i];
        }
        __syncwarp();
    }
    if (lane == 0 && sc.count_work) yz_flush_counts(sc, 0ull, 0ull, S.nsurv);
}


// one warp per heavy tracklet: its units' minimum key wins
__global__ void __launch_bounds__(128) yz_apply_kernel(or_tracks_view_t tv, YzScratch sc) {
    const int lane = threadIdx.x & 31;
    const int nheavy = min((int)sc.counters[1], sc.cap_heavy);
#pragma unroll 1
    for (int h = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; h < nheavy; h += (gridDim.x * blockDim.x) >> 5) {
        const YzHeavy hv2 = sc.heavy[h];
        if (hv2.nunits <= 0 || (long)hv2.unit0 + hv2.nunits > sc.cap_units) continue;
        unsigned long long best = ~0ull;
        int bu = -1;
#pragma unroll 1
        for (int u = lane; u < hv2.nunits; u += 32) {
            const unsigned long long k = sc.best[hv2.unit0 + u].key;
            if (k < best) {
                best = k;
                bu = hv2.unit0 + u;
            }
        }
#pragma unroll 1
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long ok = __shfl_xor_sync(0xffffffffu, best, o);
            const int ou = __shfl_xor_sync(0xffffffffu, bu, o);
            if (ok < best) {
                best = ok;
                bu = ou;
            }
        }
        if (lane == 0) sc.heavy[h].best_g = best == ~0ull ? -1 : (int)((unsigned)best / (unsigned)max(hv2.c2, 1));
        if (best == ~0ull) continue;
        float *T = trk_rec(tv, hv2.e, hv2.slot, hv2.k);
        const int nhx = min((int)T[OR_TRK_NHITS], 4);
        yz_store(T, sc.best[bu], nhx);
    }
}

// The 2 x 81 plane-set entries of the first y fit (see YzTab): for every
// set, Fit2's normal matrix accumulated over the set's planes in the order
// u3 u3' v3 v3' u2 u2' v2 v2' with the plane's weight and z, then
// matinv_2x2 and the errors as in Fit2::solve, and the first cut's bounds.
__global__ void __launch_bounds__(256) yz_tab_kernel(const or_plane_t *__restrict__ gplane, YzTab *__restrict__ tab) {
    const int t = threadIdx.x;
    if (t >= 2 * YZ_TAB_SETS) return;
    const or_plane_t &P = *gplane;
    const int st3 = 3 + t / YZ_TAB_SETS;
    const int i = t % YZ_TAB_SETS;
    const int g[4] = {i / 27 + 1, (i / 9) % 3 + 1, (i / 3) % 3 + 1, i % 3 + 1};  // u3 v3 u2 v2
    const int det[8] = {det_u3(st3), det_u3(st3) - 1, det_v3(st3), det_v3(st3) - 1, DET_U2, DET_UP2, DET_V2, DET_VP2};
    Fit2 f;
#pragma unroll 1
    for (int k = 0; k < 8; ++k) {
        if (!((g[k >> 1] >> (k & 1)) & 1)) continue;
        const int d = det[k];
        const float w = P.resolution[d] * fabsf(P.deltapy[d] / P.deltapx[d]);  // calculate_y_uvhit's err_y, H:98
        f.add(0.f, P.z[d], w);
    }
    const float A[4] = {f.A0, f.A1, f.A2, f.A3};
    float Ai[4];
    matinv_2x2(A, Ai);
    YzTab e;
    e.ai0 = Ai[0];
    e.ai1 = Ai[1];
    e.ai2 = Ai[2];
    e.ai3 = Ai[3];
    e.ey0 = sqrtf(fabsf(Ai[0]));
    e.ety = sqrtf(fabsf(Ai[3]));
    e.thr_y0 = Y0_MAX + 2 * e.ey0;
    e.thr_ty = TY_MAX + 2 * e.ety;
    tab[t] = e;
}

// Events the combination scorer leaves to the plain method: a queued
// tracklet all of whose live outer iterations score below t_keep, the best
// of them at or above t_unc -- the scorer would drop the whole tracklet
// without a clear margin.  Such an event is evaluated without pruning.
__global__ void __launch_bounds__(128) yz_unc_kernel(YzScratch sc, YzPrune prune) {
    const int lane = threadIdx.x & 31;
    const int nheavy = min((int)sc.counters[1], sc.cap_heavy);
    const long ncap = min((long)*prune.orows, prune.cap_orows);
#pragma unroll 1
    for (int h = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; h < nheavy; h += (gridDim.x * blockDim.x) >> 5) {
        const YzHeavy hv2 = sc.heavy[h];
        if (hv2.nunits <= 0 || hv2.orow0 < 0 || (long)hv2.orow0 + hv2.nrows > ncap) continue;
        float mx = -1.f;
#pragma unroll 1
        for (int r = lane; r < hv2.nrows; r += 32) mx = fmaxf(mx, prune.oscore[hv2.orow0 + r]);
#pragma unroll 1
        for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if (lane == 0 && mx < prune.t_keep && mx >= prune.t_unc) prune.unc[hv2.e] = 1;
    }
}

// Units of pruned tracklets with no kept row in their rank range are dropped
// before the first cut (their best key is "none"); everything they would
// have done is skipped anyway, including the window rebuild.
__global__ void __launch_bounds__(128) yz_kill_units_kernel(YzScratch sc, YzPrune prune) {
    const int lane = threadIdx.x & 31;
    const int nunits = min((int)sc.counters[0], sc.cap_units);
    const long ncap = min((long)*prune.orows, prune.cap_orows);
#pragma unroll 1
    for (int u = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < nunits; u += (gridDim.x * blockDim.x) >> 5) {
        const YzUnit un = sc.units[u];
        if (un.heavy < 0) continue;
        const YzHeavy hv2 = sc.heavy[un.heavy];
        if (hv2.orow0 < 0 || (long)hv2.orow0 + hv2.nrows > ncap || prune.unc[hv2.e]) continue;
        bool kept = false;
#pragma unroll 1
        for (int r = un.r0 + lane; r < un.r1 && !kept; r += 32) kept = prune.oscore[hv2.orow0 + r] >= prune.t_keep;
        if (!__any_sync(0xffffffffu, kept) && lane == 0) {
            sc.units[u].heavy = -1;
            sc.best[u].key = ~0ull;
        }
    }
}

// Labels of the scorer's rows after the plain chain: 1 for the row of the
// outer iteration that holds its tracklet's best combination when the
// tracklet ended as a global track (stationID 6 after global tracking), else
// 0.  The scratch still holds the last YZ call's heavy tracklets.
__global__ void __launch_bounds__(128) yz_outer_labels_kernel(YzScratch sc, or_tracks_view_t tv,
                                                              const uint8_t *__restrict__ toomany,
                                                              const int32_t *__restrict__ og, const uint32_t *orows,
                                                              long cap, uint8_t *__restrict__ labels) {
    const int lane = threadIdx.x & 31;
    const int nheavy = min((int)sc.counters[1], sc.cap_heavy);
    const long ncap = min((long)*orows, cap);
#pragma unroll 1
    for (int h = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; h < nheavy; h += (gridDim.x * blockDim.x) >> 5) {
        const YzHeavy hv2 = sc.heavy[h];
        if (hv2.nunits <= 0 || hv2.orow0 < 0 || (long)hv2.orow0 + hv2.nrows > ncap) continue;
        const float *T = trk_rec(tv, hv2.e, hv2.slot, hv2.k);
        const bool global = !toomany[hv2.e] && T[OR_TRK_STID] == 6.f;
#pragma unroll 1
        for (int r = lane; r < hv2.nrows; r += 32)
            labels[hv2.orow0 + r] = (global && og[hv2.orow0 + r] == hv2.best_g) ? 1 : 0;
    }
}

size_t yz_smem_bytes(int warps) {
    return ((sizeof(or_plane_t) + 15) & ~size_t(15)) + sizeof(YzWarp) * (size_t)warps;
}

// Scratch the YZ stage needs: queue of units, per-unit best records, heavy
// tracklets, per-warp overflow arenas.
static long long yz_pool_cap(int qcap, int cap_units) {
    return (OR_YZ_SPLIT && qcap == YZ_QCAP_CTX) ? YZ_POOL_PER_UNIT * cap_units : 0;
}
static long long yz_img_cap(int qcap, int cap_units) {
    return (OR_YZ_SPLIT && qcap == YZ_QCAP_CTX) ? YZ_IMG_PER_UNIT * cap_units : 0;
}

size_t yz_scratch_bytes_q(int cap_units, int cap_heavy, int garena_warps, int qcap) {
    size_t b = 256 + YZ_TAB_BYTES + (sizeof(YzUnit) + sizeof(YzBest)) * (size_t)cap_units +
               sizeof(YzHeavy) * (size_t)cap_heavy;
    b = (b + 255) & ~size_t(255);
    b += sizeof(YzHit) * YZ_GARENA_HITS * (size_t)garena_warps;
    b += sizeof(PassEntryStore) * (size_t)qcap * (size_t)garena_warps;
    if (yz_pool_cap(qcap, cap_units) > 0) {
        b = (b + 255) & ~size_t(255);
        b += sizeof(int2) * (size_t)cap_units;
        b = (b + 255) & ~size_t(255);
        b += sizeof(PassEntryStore) * (size_t)yz_pool_cap(qcap, cap_units);
    }
    if (yz_img_cap(qcap, cap_units) > 0) {
        b = (b + 255) & ~size_t(255);
        b += 16 * (size_t)yz_img_cap(qcap, cap_units);
    }
    return b;
}

// the static (no-allocation) scratch: survivor queues of YZ_QCAP_MIN entries
size_t yz_scratch_bytes(int cap_units, int cap_heavy, int garena_warps) {
    return yz_scratch_bytes_q(cap_units, cap_heavy, garena_warps, YZ_QCAP_MIN);
}

// a context's scratch
size_t yz_scratch_bytes_ctx(int cap_units, int cap_heavy, int garena_warps) {
    return yz_scratch_bytes_q(cap_units, cap_heavy, garena_warps, YZ_QCAP_CTX);
}

// the work counters of the last YZ call on `scratch` (synchronous copy)
cudaError_t yz_read_counts(const void *scratch, long long out[3]) {
    unsigned long long c[32];
    const cudaError_t e = cudaMemcpy(c, scratch, sizeof(c), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return e;
    out[0] = (long long)c[YZ_CTR_FITTED / 2];
    out[1] = (long long)c[YZ_CTR_HITSUM / 2];
    out[2] = (long long)c[YZ_CTR_SURVIVORS / 2];
    return cudaSuccess;
}

// The pointers into a YZ scratch area (the layout yz_scratch_bytes_q sizes).
static YzScratch yz_scratch_layout(void *scratch, int cap_units, int cap_heavy, int garena_warps, int qcap,
                                   long long pool_limit) {
    char *p = static_cast<char *>(scratch);
    YzScratch sc;
    sc.counters = reinterpret_cast<unsigned int *>(p);
    p += 256;
    sc.tab = reinterpret_cast<YzTab *>(p);
    p += YZ_TAB_BYTES;
    sc.units = reinterpret_cast<YzUnit *>(p);
    p += sizeof(YzUnit) * (size_t)cap_units;
    sc.best = reinterpret_cast<YzBest *>(p);
    p += sizeof(YzBest) * (size_t)cap_units;
    sc.heavy = reinterpret_cast<YzHeavy *>(p);
    p += sizeof(YzHeavy) * (size_t)cap_heavy;
    p = reinterpret_cast<char *>((reinterpret_cast<uintptr_t>(p) + 255) & ~uintptr_t(255));
    sc.garena = reinterpret_cast<YzHit *>(p);
    p += sizeof(YzHit) * YZ_GARENA_HITS * (size_t)garena_warps;
    sc.qbuf = reinterpret_cast<PassEntryStore *>(p);
    p += sizeof(PassEntryStore) * (size_t)qcap * (size_t)garena_warps;
    sc.pool_cap = yz_pool_cap(qcap, cap_units);
    if (pool_limit >= 0 && pool_limit < sc.pool_cap) sc.pool_cap = pool_limit;  // the rest of the pool goes unused
    sc.useg = nullptr;
    sc.pool = nullptr;
    if (sc.pool_cap > 0) {
        p = reinterpret_cast<char *>((reinterpret_cast<uintptr_t>(p) + 255) & ~uintptr_t(255));
        sc.useg = reinterpret_cast<int2 *>(p);
        p += sizeof(int2) * (size_t)cap_units;
        p = reinterpret_cast<char *>((reinterpret_cast<uintptr_t>(p) + 255) & ~uintptr_t(255));
        sc.pool = reinterpret_cast<PassEntryStore *>(p);
    }
    // the images follow the whole pool (pool_limit only narrows its use)
    p = reinterpret_cast<char *>(scratch) + yz_scratch_bytes_q(cap_units, cap_heavy, garena_warps, qcap) -
        16 * (size_t)yz_img_cap(qcap, cap_units);
    sc.img = yz_img_cap(qcap, cap_units) > 0 ? reinterpret_cast<uint4 *>(p) : nullptr;
    sc.img_cap = yz_img_cap(qcap, cap_units);
    sc.cap_units = cap_units;
    sc.cap_heavy = cap_heavy;
    sc.garena_warps = garena_warps;
    sc.qcap = qcap;
    sc.count_work = 0;
    return sc;
}

cudaError_t launch_mlp_score(const or_mlp_t *, const float *, long, const int32_t *, float *, uint32_t *, cudaStream_t,
                             int);

template <int W>
static cudaError_t launch_yz_impl(const or_plane_t *d_plane, or_hits_view_t hv, or_tracks_view_t tv,
                                  const uint8_t *toomany, int n_events, uint32_t *errw, void *scratch, int cap_units,
                                  int cap_heavy, int garena_warps, cudaStream_t stream, int sm_count, YzPrune prune,
                                  int qcap, long long pool_limit, int count_work) {
    if (n_events <= 0) return cudaSuccess;
    const size_t smem = yz_smem_bytes(W);
    cudaError_t err;
    if (prune.ofeat) {
        if ((err = cudaMemsetAsync(prune.orows, 0, sizeof(uint32_t), stream))) return err;
        if (prune.unc && (err = cudaMemsetAsync(prune.unc, 0, (size_t)n_events, stream))) return err;
    } else {
        prune.model = nullptr;  // no rows: nothing to score or prune
    }
    if ((err = smem_attr_once((const void *)yz_plan_kernel<W>, (int)smem)))
        return err;
    YzScratch sc = yz_scratch_layout(scratch, cap_units, cap_heavy, garena_warps, qcap, pool_limit);
    YzTab *tab = const_cast<YzTab *>(sc.tab);
    sc.count_work = count_work;
    if ((err = cudaMemsetAsync(sc.counters, 0, 256, stream))) return err;
    yz_tab_kernel<<<1, 256, 0, stream>>>(d_plane, tab);
    if ((err = cudaGetLastError())) return err;
    const long blocks = garena_warps / W;
    const long blocks_plan = min(((long)n_events * (OR_NSLOTS / YZ_PLAN_CHUNK) + W - 1) / W, blocks);
    yz_plan_kernel<W><<<(unsigned)blocks_plan, W * 32, smem, stream>>>(d_plane, hv, tv, toomany, n_events, sc, errw,
                                                                       prune);
    if ((err = cudaGetLastError())) return err;
    if (prune.model) {
        // score the rows on the tensor cores (the row count stays on the
        // device), then the uncertain events
        if ((err = launch_mlp_score(prune.model, prune.ofeat, prune.cap_orows,
                                    reinterpret_cast<const int32_t *>(prune.orows), prune.oscore, errw, stream,
                                    sm_count)))
            return err;
        yz_unc_kernel<<<(unsigned)(sm_count * 4), 128, 0, stream>>>(sc, prune);
        if ((err = cudaGetLastError())) return err;
        yz_kill_units_kernel<<<(unsigned)(sm_count * 8), 128, 0, stream>>>(sc, prune);
        if ((err = cudaGetLastError())) return err;
    }
    if (sc.pool_cap > 0) {
        const long res = (long)sm_count * (OR_YZ_SECOND_WARPS_SM / W > 0 ? OR_YZ_SECOND_WARPS_SM / W : 1);
        if (prune.model) {
            if ((err = smem_attr_once((const void *)yz_first_kernel<W, true>, (int)smem))) return err;
            if ((err = smem_attr_once((const void *)yz_second_kernel<W, true>, (int)smem))) return err;
            yz_first_kernel<W, true><<<(unsigned)blocks, W * 32, smem, stream>>>(d_plane, hv, tv, sc, prune);
            if ((err = cudaGetLastError())) return err;
            yz_second_kernel<W, true><<<(unsigned)min(blocks, res), W * 32, smem, stream>>>(d_plane, hv, tv, sc, prune);
        } else {
            if ((err = smem_attr_once((const void *)yz_first_kernel<W, false>, (int)smem))) return err;
            if ((err = smem_attr_once((const void *)yz_second_kernel<W, false>, (int)smem))) return err;
            yz_first_kernel<W, false><<<(unsigned)blocks, W * 32, smem, stream>>>(d_plane, hv, tv, sc, prune);
            if ((err = cudaGetLastError())) return err;
            yz_second_kernel<W, false><<<(unsigned)min(blocks, res), W * 32, smem, stream>>>(d_plane, hv, tv, sc,
                                                                                          prune);
        }
    } else if (prune.model) {
        if ((err = smem_attr_once((const void *)yz_work_kernel<W, true>, (int)smem))) return err;
        yz_work_kernel<W, true><<<(unsigned)blocks, W * 32, smem, stream>>>(d_plane, hv, tv, sc, prune);
    } else {
        if ((err = smem_attr_once((const void *)yz_work_kernel<W, false>, (int)smem))) return err;
        yz_work_kernel<W, false><<<(unsigned)blocks, W * 32, smem, stream>>>(d_plane, hv, tv, sc, prune);
    }
    if ((err = cudaGetLastError())) return err;
    yz_apply_kernel<<<(unsigned)(sm_count * 4), 128, 0, stream>>>(tv, sc);
    return cudaGetLastError();
}

static cudaError_t launch_yz_w(const or_plane_t *d_plane, or_hits_view_t hv, or_tracks_view_t tv,
                               const uint8_t *toomany, int n_events, uint32_t *errw, void *scratch, int cap_units,
                               int cap_heavy, int garena_warps, cudaStream_t stream, int sm_count, YzPrune prune,
                               int warps, int qcap, long long pool_limit, int count_work) {
#define OR_YZ_LAUNCH(W)                                                                                         \
    launch_yz_impl<W>(d_plane, hv, tv, toomany, n_events, errw, scratch, cap_units, cap_heavy, garena_warps, stream, \
                      sm_count, prune, qcap, pool_limit, count_work)
    switch (warps) {
    case 1: return OR_YZ_LAUNCH(1);
    case 2: return OR_YZ_LAUNCH(2);
    case 8: return OR_YZ_LAUNCH(8);
    case 16: return OR_YZ_LAUNCH(16);
    default: return OR_YZ_LAUNCH(4);
    }
#undef OR_YZ_LAUNCH
}

cudaError_t launch_yz(const or_plane_t *d_plane, or_hits_view_t hv, or_tracks_view_t tv, const uint8_t *toomany,
                      int n_events, uint32_t *errw, void *scratch, int cap_units, int cap_heavy, int garena_warps,
                      cudaStream_t stream, int sm_count) {
    return launch_yz_w(d_plane, hv, tv, toomany, n_events, errw, scratch, cap_units, cap_heavy, garena_warps, stream,
                       sm_count, YzPrune{}, 4, YZ_QCAP_MIN, -1, 0);
}

// with `warps` events (work units) per CTA: 1, 2, 4, 8 or 16
cudaError_t launch_yz_tuned(const or_plane_t *d_plane, or_hits_view_t hv, or_tracks_view_t tv,
                            const uint8_t *toomany, int n_events, uint32_t *errw, void *scratch, int cap_units,
                            int cap_heavy, int garena_warps, cudaStream_t stream, int sm_count, int warps,
                            long long pool_limit, int count_work) {
    return launch_yz_w(d_plane, hv, tv, toomany, n_events, errw, scratch, cap_units, cap_heavy, garena_warps, stream,
                       sm_count, YzPrune{}, warps, YZ_QCAP_CTX, pool_limit, count_work);
}

// YZ with the scorer's keep flags: pruned tracklets are left as tracklets no
// combination extends; kept ones get the plain result
cudaError_t launch_yz_pruned(const or_plane_t *d_plane, or_hits_view_t hv, or_tracks_view_t tv,
                             const uint8_t *toomany, int n_events, uint32_t *errw, void *scratch, int cap_units,
                             int cap_heavy, int garena_warps, cudaStream_t stream, int sm_count,
                             const int32_t *row_off, const uint8_t *keep, long max_rows, int warps,
                             long long pool_limit, int count_work) {
    YzPrune pr{};
    pr.row_off = row_off;
    pr.keep = keep;
    pr.max_rows = max_rows;
    return launch_yz_w(d_plane, hv, tv, toomany, n_events, errw, scratch, cap_units, cap_heavy, garena_warps, stream,
                       sm_count, pr, warps, YZ_QCAP_CTX, pool_limit, count_work);
}

// YZ with the combination scorer: rows of features for every live outer
// iteration of each queued tracklet, scored by `prune.model` (nullptr: rows
// only), outer iterations below t_keep skipped
cudaError_t launch_yz_scored(const or_plane_t *d_plane, or_hits_view_t hv, or_tracks_view_t tv,
                             const uint8_t *toomany, int n_events, uint32_t *errw, void *scratch, int cap_units,
                             int cap_heavy, int garena_warps, cudaStream_t stream, int sm_count, const or_mlp_t *model,
                             float t_keep, float t_unc, float *feat, int32_t *og, float *score, uint32_t *rows,
                             uint8_t *unc, long max_rows, int warps, long long pool_limit, int count_work) {
    YzPrune pr{};
    pr.ofeat = feat;
    pr.og = og;
    pr.oscore = score;
    pr.orows = rows;
    pr.unc = unc;
    pr.model = model;
    pr.cap_orows = max_rows;
    pr.t_keep = t_keep;
    pr.t_unc = t_unc;
    return launch_yz_w(d_plane, hv, tv, toomany, n_events, errw, scratch, cap_units, cap_heavy, garena_warps, stream,
                       sm_count, pr, warps, YZ_QCAP_CTX, pool_limit, count_work);
}

// labels of the last scored YZ call's rows (see yz_outer_labels_kernel)
cudaError_t launch_yz_outer_labels(void *scratch, int cap_units, int cap_heavy, int garena_warps, or_tracks_view_t tv,
                                   const uint8_t *toomany, const int32_t *og, const uint32_t *rows, long max_rows,
                                   uint8_t *labels, cudaStream_t stream, int sm_count) {
    const YzScratch sc = yz_scratch_layout(scratch, cap_units, cap_heavy, garena_warps, YZ_QCAP_CTX, -1);
    yz_outer_labels_kernel<<<(unsigned)(sm_count * 4), 128, 0, stream>>>(sc, tv, toomany, og, rows, max_rows, labels);
    return cudaGetLastError();
}

}  // namespace orgpu
