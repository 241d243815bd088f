// or_device.cuh -- device-side constants and helpers shared by the sm_103a
// kernels of the online-reconstruction path.
//
// Every translation unit that includes this header is compiled with
// -fmad=false (and IEEE division/sqrt, no flush-to-zero): each float
// operation rounds once, in the order the reference source writes it, so the
// kernels are bit-exact with a reference build at -fmad=false and with the
// CPU oracle.  Citations are file:line inside the reference project
// (OnlineReconstruction/...): K = reconstruction_kernels.cuh,
// H = reconstruction_helper.cuh, AM = trackanalyticalminimizer.cuh,
// FT = trackfittingtools.cuh, K0 = reconstruction_constants.h.
#pragma once

#include <cuda_runtime.h>
#include <mutex>
#include <stdint.h>

#include "../../include/or_layout.h"

// Small and per-hit loops on the combinatorial paths are kept rolled
// (`#pragma unroll 1`): those kernels are limited by instruction-cache
// misses, and one copy of a loop body costs less there than unrolled copies
// save in issue slots (measured per loop group on the 100,000-event uneven
// batch: YZ 191 -> 122 ms, global 33 -> 16 ms, outputs bit-identical).
// The XZ kernel is the exception: there the unrolled loops are faster.


namespace orgpu {

// ---------------------------------------------------------------------------
// constants, K0:29-207
// ---------------------------------------------------------------------------
constexpr float TX_MAX = 0.15f, TY_MAX = 0.1f, X0_MAX = 150.f, Y0_MAX = 50.f;
constexpr float INVP_MAX = 0.2f, INVP_MIN = 0.01f;
constexpr float Z_DUMP = 42.f;
constexpr float SAGITTA_TARGET_CENTER = 1.85f, SAGITTA_TARGET_WIDTH = 0.25f;
constexpr float SAGITTA_DUMP_CENTER = 1.5f, SAGITTA_DUMP_WIDTH = 0.3f;
constexpr float PT_KICK_KMAG = -0.3819216f;
constexpr float FMAGSTR = -1.054f;
constexpr float Z_KMAG_BEND = 1064.26f;
constexpr float Z_TARGET = -300.f;
constexpr int MAXHITS_PROJ_X = 20;
constexpr int MAXD0 = 210, MAXD2 = 120, MAXD3 = 90;
constexpr int NPROP_MIN = 2;
constexpr short DET_SENTINEL = -100;  // never adjacent to a plane id

// planes of the hot path
constexpr int DET_X2 = 16, DET_XP2 = 15;           // st2 x/x'  (detsuperid[2][0]*2)
constexpr int DET_U2 = 18, DET_UP2 = 17;           // st2 u/u'
constexpr int DET_V2 = 14, DET_VP2 = 13;           // st2 v/v'
__host__ __device__ constexpr int det_x3(int st3) { return st3 == 3 ? 22 : 28; }   // detsuperid[3|4][0]*2
__host__ __device__ constexpr int det_u3(int st3) { return st3 == 3 ? 24 : 30; }
__host__ __device__ constexpr int det_v3(int st3) { return st3 == 3 ? 20 : 26; }
constexpr int DET_P1X1 = 50, DET_P1X2 = 49, DET_P2X1 = 52, DET_P2X2 = 51;  // detsuperid[5|6][0]
constexpr int DET_P1Y1 = 48, DET_P1Y2 = 47, DET_P2Y1 = 54, DET_P2Y2 = 53;  // detsuperid[5|6][1]

__device__ __constant__ short c_eff_detid_chambers[24] = {1,  2,  3,  4,  5,  6,  13, 14, 15, 16, 17, 18,
                                                          19, 20, 21, 22, 23, 24, 25, 26, 27, 28, 29, 30};
__device__ __constant__ short c_hodoplanesx[4][2] = {{31, 32}, {37, 38}, {39, 40}, {45, 46}};
__device__ __constant__ float c_hodofudgefac[4] = {0.25f, 0.2f, 0.15f, 0.0f};
__device__ __constant__ float c_hodoXcellwidth[4] = {7.32f, 13.0f, 14.5875f, 19.6475f};
__device__ __constant__ short c_lrpossibility[4][2] = {{1, 1}, {1, -1}, {-1, 1}, {-1, -1}};
__device__ __constant__ float c_spacingplane[28] = {0.f,  0.40f, 0.40f, 0.40f, 0.40f, 0.40f, 0.40f, 1.3f,  1.3f, 1.3f,
                                                    1.2f, 1.2f,  1.2f,  1.2f,  1.2f,  1.2f,  4.0f,  4.0f,  7.0f, 7.0f,
                                                    8.0f, 12.0f, 12.0f, 10.0f, 3.0f,  3.0f,  3.0f,  3.0f};
__device__ __constant__ short c_detsuperid[7][3] = {{2, 1, 3},    {5, 6, 4},    {8, 9, 7},  {11, 12, 10},
                                                    {14, 15, 13}, {25, 24, -1}, {26, 27, -1}};
__device__ __constant__ short c_planetype[15] = {1, 0, 2, 1, 0, 2, 2, 0, 1, 2, 0, 1, 2, 0, 1};
// last element of the x element bins: st2 bins end at 112, st3 bins at 116 (K0:155-161)
__host__ __device__ inline int x_bin_of(int st, float chan) {
    // bins b = 0..27 cover elements [1+4b, 4+4b]; the last bin of station 3
    // reaches 116 (K0:159, :161).  Elements outside every bin get -1.
    if (!(chan >= 1.f)) return -1;
    const float hi_last = (st == 2) ? 112.f : 116.f;
    if (chan > hi_last) return -1;
    if (chan >= 109.f) return 27;
    const int b = (int)((chan - 1.f) * 0.25f);  // chan < 109 here
    return (chan >= (float)(4 * b + 1) && chan <= (float)(4 * b + 4)) ? b : -1;
}

// ---------------------------------------------------------------------------
// geometry in shared memory
// ---------------------------------------------------------------------------
__device__ __forceinline__ void load_plane_smem(or_plane_t *dst, const or_plane_t *__restrict__ src) {
    const uint32_t *s = reinterpret_cast<const uint32_t *>(src);
    uint32_t *d = reinterpret_cast<uint32_t *>(dst);
    for (int i = threadIdx.x; i < (int)(sizeof(or_plane_t) / 4); i += blockDim.x) d[i] = __ldg(s + i);
}

// H:8-36
__device__ __forceinline__ float x_bep(int d, int elid, const or_plane_t &P) { return P.p1x_w1[d] + P.dp1x[d] * (float)(elid - 1); }
__device__ __forceinline__ float y_bep(int d, int elid, const or_plane_t &P) { return P.p1y_w1[d] + P.dp1y[d] * (float)(elid - 1); }
__device__ __forceinline__ float z_bep(int d, int elid, const or_plane_t &P) { return P.p1z_w1[d] + P.dp1z[d] * (float)(elid - 1); }
__device__ __forceinline__ float x_tep(int d, int elid, const or_plane_t &P) { return x_bep(d, elid, P) + P.deltapx[d]; }
__device__ __forceinline__ float position(float pos, float drift, short sign) { return pos + (float)sign * drift; }

// H:75-100
__device__ __forceinline__ bool calculate_y_uvhit(int d, int elid, float drift, short hitsign, float x0, float tx,
                                                  const or_plane_t &P, float &y, float &err_y) {
    const float p1x = x_bep(d, elid, P);
    const float p2x = p1x + P.deltapx[d];
    const float x_trk = x0 + P.z[d] * tx;
    if (x_trk - drift > p1x && x_trk - drift > p2x) return false;
    if (x_trk + drift < p1x && x_trk + drift < p2x) return false;
    const float p1y = y_bep(d, elid, P);
    float yy = p1y + (x_trk - p1x) * P.deltapy[d] / P.deltapx[d];
    if (hitsign != 0) yy += copysignf(1.f, P.sintheta[d]) * 2.f * (drift - 0.5f * (float)hitsign);
    yy = fmaxf(yy, p1y);
    yy = fminf(yy, p1y + P.deltapy[d]);
    y = yy;
    err_y = P.resolution[d] * fabsf(P.deltapy[d] / P.deltapx[d]);
    return true;
}

// H:140-158
__device__ __forceinline__ void calculate_xz_fy(int d, int elid, float drift, short hitsign, float y0, float ty,
                                                const or_plane_t &P, float &x, float &z) {
    const float p1x = x_bep(d, elid, P);
    const float p1y = y_bep(d, elid, P);
    const float p1z = z_bep(d, elid, P);
    const float dpy = P.deltapy[d];
    const float dpz = P.deltapz[d];
    float zz = p1z - p1y * dpz / dpy;
    const float y_trk = y0 + zz * ty;
    float xx = p1x + (y_trk - p1y) * P.deltapx[d] / dpy;
    zz = p1z + (y_trk - p1y) * dpz / dpy;
    if (hitsign != 0) xx += (float)hitsign * drift;
    x = xx;
    z = zz;
}

// FT:3-82, Gauss-Jordan with partial pivoting (operations.h:39-62)
__device__ __forceinline__ void matinv_2x2(const float A[4], float Ainv[4]) {
    int perm0 = 0, perm1 = 1;
    float AA00 = A[0], AA10 = A[1], AA01 = A[2], AA11 = A[3], tmp;
    if (fabsf(AA10) > fabsf(AA00)) {
        tmp = AA00; AA00 = AA10; AA10 = tmp;
        tmp = AA01; AA01 = AA11; AA11 = tmp;
        perm0 = 1; perm1 = 0;
    }
    tmp = 1.0f / AA00;
    const int icol0 = perm0;
    AA00 = tmp;
    AA01 = tmp * AA01;
    tmp = AA10;
    AA10 = (-tmp) * AA00;
    AA11 = -(tmp * AA01) + AA11;
    tmp = 1.0f / AA11;
    const int icol1 = perm1;
    AA10 = tmp * AA10;
    AA11 = tmp;
    tmp = AA01;
    AA00 = -(tmp * AA10) + AA00;
    AA01 = (-tmp) * AA11;
    // icol0 and icol1 are 0/1 or 1/0
    if (icol0 == 0) {
        Ainv[0] = AA00; Ainv[2] = AA10; Ainv[1] = AA01; Ainv[3] = AA11;
    } else {
        Ainv[1] = AA00; Ainv[3] = AA10; Ainv[0] = AA01; Ainv[2] = AA11;
    }
    (void)icol1;
}

// Normal-equation accumulator of fit_2D_track / fit_2D_track_drift
// (AM:32-119): weights are the plane resolutions, as the callers pass them.
struct Fit2 {
    float A0 = 0.f, A1 = 0.f, A2 = 0.f, A3 = 0.f, B0 = 0.f, B1 = 0.f;
    __device__ __forceinline__ void add(float x, float z, float w) {
        B0 += w * x;
        B1 += w * x * z;
        A0 += w;
        A1 += w * z;
        A2 += w * z;
        A3 += w * z * z;
    }
    __device__ __forceinline__ void add_drift(float x, float drift, short sign, float z, float w) {
        B0 += w * (x + drift * (float)sign);
        B1 += w * (x + drift * (float)sign) * z;
        A0 += w;
        A1 += w * z;
        A2 += w * z;
        A3 += w * z * z;
    }
    __device__ __forceinline__ void solve(float &p0, float &p1, float &e0, float &e1) const {
        const float A[4] = {A0, A1, A2, A3};
        float Ai[4];
        matinv_2x2(A, Ai);
        p0 = 0.0f;
        p0 += Ai[0] * B0;
        p0 += Ai[1] * B1;
        p1 = 0.0f;
        p1 += Ai[2] * B0;
        p1 += Ai[3] * B1;
        e0 = sqrtf(fabsf(Ai[0]));
        e1 = sqrtf(fabsf(Ai[3]));
    }
};

// pull of one LR hypothesis, H:755-760 / H:847-852
__device__ __forceinline__ float lr_pull(float slope_exp, float err_slope, float inter_exp, float err_inter,
                                         float slope_local, float inter_local) {
    return sqrtf((slope_exp - slope_local) * (slope_exp - slope_local) / err_slope / err_slope +
                 (inter_exp - inter_local) * (inter_exp - inter_local) / err_inter / err_inter);
}

// Resolve one adjacent pair (i, j) of resolve_leftright_newhits, H:737-776.
// Returns the lrpossibility index to apply, or -1.
__device__ __forceinline__ int lr_pair_newhits(float x0, float tx, float y0, float ty, float err_x0, float err_tx,
                                               float err_y0, float err_ty, short di, short dj, float pos_i, float dr_i,
                                               float pos_j, float dr_j, const or_plane_t &P, float thr) {
    const float slope_exp = P.costheta[di] * tx + P.sintheta[di] * ty;
    const float err_slope = fabsf(P.costheta[di] * err_tx) + fabsf(P.sintheta[di] * err_ty);
    const float inter_exp = P.costheta[di] * x0 + P.sintheta[di] * y0;
    const float err_inter = fabsf(P.costheta[di] * err_x0) + fabsf(P.sintheta[di] * err_y0);
    int indexmin = -1;
    float pull_min = 1.e6f;
#pragma unroll 1
    for (int k = 0; k < 4; k++) {
        const float pi = position(pos_i, dr_i, c_lrpossibility[k][0]);
        const float pj = position(pos_j, dr_j, c_lrpossibility[k][1]);
        const float slope_local = (pi - pj) / (P.z[di] - P.z[dj]);
        const float inter_local = pi - slope_local * P.z[di];
        if (fabsf(slope_local) > P.slope_max[di] || fabsf(inter_local) > P.inter_max[di]) continue;
        const float pull = lr_pull(slope_exp, err_slope, inter_exp, err_inter, slope_local, inter_local);
        if (pull < pull_min) {
            indexmin = k;
            pull_min = pull;
        }
    }
    return (indexmin > 0 && pull_min < thr) ? indexmin : -1;
}

// The same, out of line: for call sites outside a kernel's hot loop, so that
// the loop's instructions stay resident in the instruction cache.
static __device__ __noinline__ int lr_pair_newhits_ool(float x0, float tx, float y0, float ty, float err_x0, float err_tx,
                                                float err_y0, float err_ty, short di, short dj, float pos_i,
                                                float dr_i, float pos_j, float dr_j, const or_plane_t &P, float thr) {
    return lr_pair_newhits(x0, tx, y0, ty, err_x0, err_tx, err_y0, err_ty, di, dj, pos_i, dr_i, pos_j, dr_j, P, thr);
}

// Resolve one adjacent pair of resolve_leftright_xhits, H:829-868.
__device__ __forceinline__ int lr_pair_xhits(float x0, float tx, float err_x0, float err_tx, short di, short dj,
                                             float pos_i, float dr_i, float pos_j, float dr_j, const float *zarr,
                                             float thr) {
    int indexmin = -1;
    float pull_min = 1.e6f;
#pragma unroll 1
    for (int k = 0; k < 4; k++) {
        const float pi = position(pos_i, dr_i, c_lrpossibility[k][0]);
        const float pj = position(pos_j, dr_j, c_lrpossibility[k][1]);
        const float slope_local = (pi - pj) / (zarr[di] - zarr[dj]);
        const float inter_local = pi - slope_local * zarr[di];
        const float pull = lr_pull(tx, err_tx, x0, err_x0, slope_local, inter_local);
        if (pull < pull_min) {
            indexmin = k;
            pull_min = pull;
        }
    }
    return (indexmin > 0 && pull_min < thr) ? indexmin : -1;
}

// H:796-797
__device__ __forceinline__ short single_sign_newhits(float x0, float tx, float y0, float ty, short d, float pos,
                                                     const or_plane_t &P) {
    const float pos_exp = (P.z[d] * tx + x0) * P.costheta[d] + (P.z[d] * ty + y0) * P.sintheta[d];
    return pos_exp > pos ? (short)1 : (short)-1;
}
// H:885-886
__device__ __forceinline__ short single_sign_xhits(float x0, float tx, short d, float pos, const float *zarr) {
    const float pos_exp = zarr[d] * tx + x0;
    return pos_exp > pos ? (short)1 : (short)-1;
}

// H:1158-1164, one term of chi2_track / residual
__device__ __forceinline__ float residual_line(float p1x, float p1y, float p1z, float dpx, float dpy, float dpz,
                                               float drift, short sign, float x0, float y0, float tx, float ty) {
    const float den2 = dpy * dpy * (1 + tx * tx) + dpx * dpx * (1 + ty * ty) -
                       2 * (ty * dpx * dpz + ty * dpy * dpz + tx * ty * dpx * dpy);
    const float dca =
        ((ty * dpz - dpy) * (p1x - x0) + (dpx - tx * dpz) * (p1y - y0) + p1z * (tx * dpy - ty * dpx)) / sqrtf(den2);
    return drift * (float)sign - dca;
}

// H:684-691 (E1039): the product is formed in double
__device__ __forceinline__ short calculate_charge(float tx, float x0) {
    return (-0.0033f * copysign(1.0, (double)FMAGSTR) * (double)x0 < (double)tx) ? (short)1 : (short)-1;
}

// ---------------------------------------------------------------------------
// hit-collection access
// ---------------------------------------------------------------------------
struct HitPlane {
    const float *d;  // slot base
    int n;           // count = SoA stride
    __device__ __forceinline__ float chan(int i) const { return d[i]; }
    __device__ __forceinline__ float pos(int i) const { return d[n + i]; }
    __device__ __forceinline__ float tdc(int i) const { return d[2 * n + i]; }
    __device__ __forceinline__ float flag(int i) const { return d[3 * n + i]; }
    __device__ __forceinline__ float drift(int i) const { return d[4 * n + i]; }
};

__device__ __forceinline__ HitPlane hits_of(const or_hits_view_t &hv, long e, int det) {
    HitPlane h;
    if (det <= OR_NCHAM) {
        h.n = (int)hv.nhits_cham[e * OR_NCHAM + det - 1];
        h.d = hv.hits_cham + e * OR_EVT_CHAM_FLOATS + (long)OR_NHITSPARAM * OR_MAXHITS_CHAM * (det - 1);
    } else if (det <= OR_NCHAM + OR_NHODO) {
        h.n = (int)hv.nhits_hodo[e * OR_NHODO + det - OR_NCHAM - 1];
        h.d = hv.hits_hodo + e * OR_EVT_HODO_FLOATS + (long)OR_NHITSPARAM * OR_MAXHITS_HODO * (det - OR_NCHAM - 1);
    } else {
        h.n = (int)hv.nhits_prop[e * OR_NPROP + det - OR_NCHAM - OR_NHODO - 1];
        h.d = hv.hits_prop + e * OR_EVT_PROP_FLOATS +
              (long)OR_NHITSPARAM * OR_MAXHITS_PROP * (det - OR_NCHAM - OR_NHODO - 1);
    }
    return h;
}

__device__ __forceinline__ float *trk_rec(const or_tracks_view_t &tv, long e, int slot, int k) {
    return tv.tracks + e * OR_EVT_TRK_FLOATS + (long)slot * OR_SLOTCAP * OR_NTRKPARAM + (long)k * OR_NTRKPARAM;
}

// H:1090-1144
__device__ __forceinline__ bool match_track_XZ_to_hodo(int stid, int detid, const HitPlane &h, float x0, float tx,
                                                       float err_x0, float err_tx, const float *zarr) {
    if (h.n == 0) return false;
    if (detid > 40) stid = 3;
    const float xhodo = zarr[detid] * tx + x0;
    const float fudgefac = c_hodofudgefac[stid];
    const float cellwidth = c_hodoXcellwidth[stid];
    float err_x = 3.f * (fabsf(zarr[detid] * err_tx) + err_x0);
#pragma unroll 1
    for (int i = 0; i < h.n; i++) {
        const float p = h.pos(i);
        float xmin = p - cellwidth * 0.5f;
        float xmax = p + cellwidth * 0.5f;
        xmin -= (xmax - xmin) * fudgefac;
        xmax += (xmax - xmin) * fudgefac;
        err_x += (xmax - xmin) * 0.15f;
        xmin -= err_x;
        xmax += err_x;
        if (xmin <= xhodo && xhodo <= xmax) return true;
    }
    return false;
}

// H:1002-1087 (MATCH_Y_HODO undefined in the reference)
__device__ __forceinline__ bool match_tracklet_to_hodo(int stid, int detid, const HitPlane &h, float x0, float y0,
                                                       float tx, float ty, float err_x0, float err_y0, float err_tx,
                                                       float err_ty, const or_plane_t &P) {
    if (h.n == 0) return false;
    if (detid > 40) stid = 3;
    const float fudgefac = c_hodofudgefac[stid];
    const float cellwidth = P.cellwidth[detid];
    const float xhodo = P.z[detid] * tx + x0;
    const float yhodo = P.z[detid] * ty + y0;
    float err_x = 3.f * (fabsf(P.z[detid] * err_tx) + err_x0);
    const float err_y = 3.f * (fabsf(P.z[detid] * err_ty) + err_y0);
#pragma unroll 1
    for (int i = 0; i < h.n; i++) {
        const float p = h.pos(i);
        float xmin = p - cellwidth * 0.5f;
        float xmax = p + cellwidth * 0.5f;
        float ymin = P.y1[detid];
        float ymax = P.y2[detid];
        xmin -= (xmax - xmin) * fudgefac;
        xmax += (xmax - xmin) * fudgefac;
        ymin -= (ymax - ymin) * fudgefac;
        ymax += (ymax - ymin) * fudgefac;
        err_x += (xmax - xmin) * 0.15f;
        xmin -= err_x;
        xmax += err_x;
        ymin -= err_y;
        ymax += err_y;
        if (xmin <= xhodo && xhodo <= xmax && ymin <= yhodo && yhodo <= ymax) return true;
    }
    return false;
}

// Prop-tube gate: a hit within `tol1` on plane a (else plane b), plus one
// within `tol2` on plane c (else d) -- K:577-640 for x, K:1640-1701 for y.
// `proj0`/`slope` are the track's intercept and slope in that projection.
__device__ __forceinline__ int prop_hits(const HitPlane &a, float za, const HitPlane &b, float zb, float tol,
                                         float proj0, float slope) {
#pragma unroll 1
    for (int n = 0; n < a.n; n++) {
        const float e = slope * za + proj0;
        if (fabsf(a.pos(n) - e) < tol) return 1;
    }
#pragma unroll 1
    for (int n = 0; n < b.n; n++) {
        const float e = slope * zb + proj0;
        if (fabsf(b.pos(n) - e) < tol) return 1;
    }
    return 0;
}

// ---------------------------------------------------------------------------
// warp helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ unsigned lanemask_lt() { return (1u << lane_id()) - 1u; }
// highest set lane index of m, or -1
__device__ __forceinline__ int last_lane(unsigned m) { return m ? 31 - __clz(m) : -1; }

// Raise a kernel's dynamic shared-memory limit once per device; the
// attribute persists, so later launches -- also those recorded into a CUDA
// graph by stream capture -- make no further runtime calls for it.  The
// table holds SMEM_ATTR_FUNCS kernels per device, above the library's count
// of kernel instantiations that use it (about 40: the launch-shape templates
// of every stage); a kernel beyond it would set the attribute on each launch.
constexpr int SMEM_ATTR_FUNCS = 128;
inline cudaError_t smem_attr_once(const void *func, int bytes) {
    static std::mutex mu;
    static const void *fn[64][SMEM_ATTR_FUNCS];
    static int nfn[64];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    std::lock_guard<std::mutex> lock(mu);
    for (int i = 0; i < nfn[dev]; ++i)
        if (fn[dev][i] == func) return cudaSuccess;
    e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess && nfn[dev] < SMEM_ATTR_FUNCS) fn[dev][nfn[dev]++] = func;
    return e;
}

// Error words the kernels raise (bounded waits, capacity overruns).
enum : uint32_t {
    ERRW_NONE = 0u,
    ERRW_TMA_TIMEOUT = 1u,
    ERRW_CAPACITY = 2u,
    ERRW_INPUT = 4u,  // hit records of an event not sorted by (det, elem, tdc)
};

// ---------------------------------------------------------------------------
// TMA bulk copies and mbarriers (sm_90+ PTX, used on sm_103a)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
// 1-D bulk copy global -> shared, completing on `bar` (16-byte aligned
// addresses, size a multiple of 16)
__device__ __forceinline__ void tma_load_1d(void *dst_smem, const void *src_gmem, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst_smem)),
        "l"(src_gmem), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
// Bounded wait for phase `parity` of `bar`; false when the limit ran out.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, uint32_t max_iter) {
    const uint32_t a = smem_u32(bar);
    for (uint32_t it = 0; it < max_iter; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

}  // namespace orgpu
