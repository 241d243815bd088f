// physics_kernel.cu -- the stages after global tracking: vertexing, dimuon
// building and the monitoring histograms.
//
// Replaces gKernel_Vertexing (OnlineReconstruction/reconstruction_kernels.cuh
// :2542-2810), gKernel_DimuonBuilding (:2820-3090, with
// FindDimuonClosestApproach, reconstruction_helper.cuh:1269-1477) and
// gKernel_fill_display_histograms (:3100-3195), launched in that order after
// the post-global selection (online_reconstruction.cu:939-983).
//
//  - Vertexing swims each global track (stationID >= 6) back through FMag in
//    double, 100 magnet steps with energy loss and 100 target steps, and keeps
//    the point of closest approach to the beam line: stationID 7, vertex
//    position and momentum.  The reference gives a thread to each slot, so a
//    warp works for the one or two lanes whose slot holds a global track;
//    here a warp gathers the global tracks of 32 events into a shared list
//    and swims them one per lane, which keeps the lanes of the double-
//    precision loop busy (FP64 is the scarce unit of this GPU).  The swim is
//    not stored: the closest-approach scan visits the points in step order
//    with a strict "smaller than" test, so it runs as the points are made.
//  - Dimuons: one thread per event, as in the reference (its pair loop
//    carries state from one pair to the next: the swum momenta of the
//    current track stay in p_pos / p_neg), visiting only slots that hold a
//    vertexed track.
//  - Histograms: one warp per event, lanes over the bins of one (trigger,
//    variable) table; counts go in with atomics, so the result is the exact
//    count whatever the order (the reference's plain "+=" from concurrent
//    blocks loses updates).
//
// Every expression keeps the operand types of the reference expression it
// restates (float track parameters, double step and energy-loss constants,
// sqrtf on double expressions), so promotions and roundings are the same.
#include "or_device.cuh"

namespace orgpu {

namespace phys {
constexpr float X_BEAM = 0.f, Y_BEAM = 0.f;          // K0:75-76
constexpr double PTKICK_UNIT = -0.006096568;         // K0:93
constexpr double FMAG_LENGTH = 502.92;               // K0:110
constexpr double FMAG_HOLE_LENGTH = 27.94;           // K0:111
constexpr double FMAG_HOLE_RADIUS = 1.27;            // K0:112
constexpr int NSTEPS_FMAG = 100;                     // K0:113
constexpr double STEP_FMAG = 2.514600;               // K0:114
constexpr double DEDX_UNIT_0 = 0.014282073;          // K0:115-119
constexpr double DEDX_UNIT_1 = 7.1869681e-05;
constexpr double DEDX_UNIT_2 = -1.4279150e-06;
constexpr double DEDX_UNIT_3 = 1.5853655e-08;
constexpr double DEDX_UNIT_4 = -6.0741470e-11;
constexpr int NSTEPS_TARGET = 100;                   // K0:120
constexpr double STEP_TARGET = 5.0;                  // K0:121
constexpr float EBEAM = 120.f, MP = 0.938272f, PBEAM = 119.996331801f, MMU = 0.105658f;  // K0:210-213
constexpr float CHI2DOF_MAX = 250.f;                 // K0:194
constexpr int VTX_LIST = 256;                        // vertexing list entries per warp
}  // namespace phys

// gTracks::get_firsthitdetid (reconstruction_classes.cuh:517-532)
__device__ __forceinline__ short first_hit_detid(const float *T, const float *z) {
    const int nhits = (int)T[OR_TRK_NHITS];
    short detid_min = 30;
    float z_min = 10000.f;
    for (int i = 0; i < nhits && i < OR_MAXHITS_PER_TRACK; ++i) {
        const short d = (short)T[OR_TRK_HIT_DETID + i];
        if (d > 0 && z[d] < z_min) {
            detid_min = d;
            z_min = z[d];
        }
    }
    return detid_min;
}

// calculate_x0_tx_st1 (H:622-626)
__device__ __forceinline__ void x0_tx_st1(float x0, float tx, float invP, short charge, float &x0_st1, float &tx_st1) {
    tx_st1 = tx + PT_KICK_KMAG * invP * charge;
    x0_st1 = tx * Z_KMAG_BEND + x0 - tx_st1 * Z_KMAG_BEND;
}

__device__ __forceinline__ double dedx_poly(double p) {
    using namespace phys;
    return DEDX_UNIT_0 + DEDX_UNIT_1 * p + DEDX_UNIT_2 * p * p + DEDX_UNIT_3 * p * p * p + DEDX_UNIT_4 * p * p * p * p;
}

// ---------------------------------------------------------------------------
// vertexing (K:2594-2803)

__device__ void vertex_track(float *T, const float *z) {
    using namespace phys;
    const float x0 = T[OR_TRK_X0], y0 = T[OR_TRK_Y0], tx = T[OR_TRK_TX], ty = T[OR_TRK_TY];
    const float invP = T[OR_TRK_INVP], charge = T[OR_TRK_CHARGE];
    const short detid_first = first_hit_detid(T, z);
    float x0_st1, tx_st1;
    x0_tx_st1(x0, tx, invP, (short)charge, x0_st1, tx_st1);
    const double z_0 = z[detid_first];
    const double s0 = charge * invP * sqrtf((1.f + tx_st1 * tx_st1) / (1.f + tx_st1 * tx_st1 + ty * ty));
    const double s1 = tx_st1, s2 = ty;
    const double s3 = (float)z_0 * tx_st1 + x0_st1, s4 = (float)z_0 * ty + y0;
    double px = s3 + s1 * (FMAG_LENGTH - z_0), py = s4 + s2 * (FMAG_LENGTH - z_0), pz = FMAG_LENGTH;
    const double pz_0 = 1.f / (fabs(s0) * sqrtf(1.f + s1 * s1 + s2 * s2));
    double mx = pz_0 * s1, my = pz_0 * s2, mz = pz_0;
    double dca2_min = 1.e18;
    bool found = false;
    double v[6];
    auto visit = [&]() {
        if (!(FMAGSTR * charge * mx < 0.)) {
            const double dca2 = (px - X_BEAM) * (px - X_BEAM) + (py - Y_BEAM) * (py - Y_BEAM);
            if (dca2 < dca2_min) {
                dca2_min = dca2;
                found = true;
                v[0] = px; v[1] = py; v[2] = pz;
                v[3] = mx; v[4] = my; v[5] = mz;
            }
        }
    };
    visit();
    for (int step = 1; step <= NSTEPS_FMAG; ++step) {
        const double tx_i = mx / mz;
        const double tx_f = tx_i + 2.f * charge * PTKICK_UNIT * STEP_FMAG / sqrt(mx * mx + mz * mz);
        const double t10 = tx_i * STEP_FMAG, t11 = ty * STEP_FMAG, t12 = STEP_FMAG;
        const double b0 = px - t10, b1 = py - t11, b2 = pz - t12;
        const double ptot_i = sqrt(mx * mx + my * my + mz * mz);
        double ptot_b = ptot_i;
        if (b2 > FMAG_HOLE_LENGTH || b0 * b0 + b1 * b1 > FMAG_HOLE_RADIUS)
            ptot_b += dedx_poly(ptot_i) * sqrtf(t10 * t10 + t11 * t11 + t12 * t12);
        const double t20 = tx_f * STEP_FMAG, t21 = ty * STEP_FMAG, t22 = STEP_FMAG;
        px = b0 - t20;
        py = b1 - t21;
        pz = b2 - t22;
        double ptot_f = ptot_b;
        if (pz > FMAG_HOLE_LENGTH || px * px + py * py > FMAG_HOLE_RADIUS)
            ptot_f += dedx_poly(ptot_b) * sqrtf(t20 * t20 + t21 * t21 + t22 * t22);
        const double pz_f = ptot_f / sqrt(1.f + tx_f * tx_f + ty * ty);
        mx = pz_f * tx_f;
        my = pz_f * ty;
        mz = pz_f;
        visit();
    }
    for (int step = NSTEPS_FMAG + 1; step <= NSTEPS_FMAG + NSTEPS_TARGET; ++step) {
        const double tx_i = mx / mz;
        px = px - tx_i * STEP_TARGET;
        py = py - ty * STEP_TARGET;
        pz = pz - STEP_TARGET;
        visit();
    }
    if (!found) {  // the last point (K:2752)
        v[0] = px; v[1] = py; v[2] = pz;
        v[3] = mx; v[4] = my; v[5] = mz;
    }
    T[OR_TRK_STID] = 7.f;  // K:2796
    T[OR_TRK_VX] = (float)v[0];
    T[OR_TRK_VX + 1] = (float)v[1];
    T[OR_TRK_VX + 2] = (float)v[2];
    T[OR_TRK_PX] = (float)v[3];
    T[OR_TRK_PX + 1] = (float)v[4];
    T[OR_TRK_PX + 2] = (float)v[5];
}

// candidates of one event: stationID >= 6, in (slot, position) order
__device__ __forceinline__ int vertex_candidates(const or_tracks_view_t &tv, long e, uint32_t *out, int r0, int lo,
                                                 int hi, uint32_t tag) {
    int r = r0;
    for (int s = 0; s < OR_NSLOTS; ++s) {
        const int n = min((int)tv.ntracks[e * OR_NSLOTS + s], OR_SLOTCAP);
        for (int k = 0; k < n; ++k) {
            if (trk_rec(tv, e, s, k)[OR_TRK_STID] < 6) continue;  // K:2594
            if (out && r >= lo && r < hi) out[r - lo] = tag | (uint32_t)(s * OR_SLOTCAP + k);
            ++r;
        }
    }
    return r - r0;
}

template <int W>
__global__ void __launch_bounds__(W * 32)
    vertex_kernel(const or_plane_t *__restrict__ gplane, or_tracks_view_t tv, const uint8_t *__restrict__ toomany,
                  int n_events) {
    __shared__ float zs[OR_NDET];
    __shared__ uint32_t list[W][phys::VTX_LIST];
    for (int i = threadIdx.x; i < OR_NDET; i += blockDim.x) zs[i] = gplane->z[i];
    __syncthreads();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (long e0 = ((long)blockIdx.x * W + w) * 32; e0 < n_events; e0 += (long)gridDim.x * W * 32) {
        const long e = e0 + lane;
        const bool live = e < n_events && !toomany[e];
        const int cnt = live ? vertex_candidates(tv, e, nullptr, 0, 0, 0, 0) : 0;
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        const int excl = incl - cnt;
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        for (int w0 = 0; w0 < total; w0 += phys::VTX_LIST) {
            if (live && cnt > 0 && excl + cnt > w0 && excl < w0 + phys::VTX_LIST)
                vertex_candidates(tv, e, list[w], excl, w0, w0 + phys::VTX_LIST, (uint32_t)lane << 9);
            __syncwarp();
            const int m = min(phys::VTX_LIST, total - w0);
            for (int i = lane; i < m; i += 32) {
                const uint32_t c = list[w][i];
                const int sk = (int)(c & 511u);
                vertex_track(trk_rec(tv, e0 + (c >> 9), sk / OR_SLOTCAP, sk % OR_SLOTCAP), zs);
            }
            __syncwarp();
        }
    }
}

// ---------------------------------------------------------------------------
// dimuons (K:2820-3090, H:1269-1477), in float as there

struct SwimPt {
    float x, y, z, mx, my, mz;
};

__device__ __forceinline__ float E4(float m, const float *p) { return sqrtf(m * m + p[0] * p[0] + p[1] * p[1] + p[2] * p[2]); }
__device__ __forceinline__ float mult4(const float *a, const float *b) {
    return a[3] * b[3] - (a[0] * b[0] + a[1] * b[1] + a[2] * b[2]);
}

// start of a track's swim (K:2927-2947)
__device__ __forceinline__ SwimPt dim_start(const float *T, const float *z, float &ty, float &charge) {
    using namespace phys;
    const float x0 = T[OR_TRK_X0], y0 = T[OR_TRK_Y0], tx = T[OR_TRK_TX];
    ty = T[OR_TRK_TY];
    const float invP = T[OR_TRK_INVP];
    charge = T[OR_TRK_CHARGE];
    const short detid_first = first_hit_detid(T, z);
    float x0_st1, tx_st1;
    x0_tx_st1(x0, tx, invP, (short)charge, x0_st1, tx_st1);
    const float z_0 = z[detid_first];
    const float s0 = charge * invP * sqrtf((1.f + tx_st1 * tx_st1) / (1.f + tx_st1 * tx_st1 + ty * ty));
    const float s1 = tx_st1, s2 = ty;
    const float s3 = z_0 * tx_st1 + x0_st1, s4 = z_0 * ty + y0;
    SwimPt p;
    p.x = (float)(s3 + s1 * (FMAG_LENGTH - z_0));
    p.y = (float)(s4 + s2 * (FMAG_LENGTH - z_0));
    p.z = (float)FMAG_LENGTH;
    const float pz_0 = 1.f / (fabsf(s0) * sqrtf(1.f + s1 * s1 + s2 * s2));
    p.mx = pz_0 * s1;
    p.my = pz_0 * s2;
    p.mz = pz_0;
    return p;
}

// one FMag step (H:1290-1333); d1 = the linear energy-loss coefficient of the
// first update, DEDX_UNIT_2 for the reference's second track (H:1354)
__device__ __forceinline__ void dim_fmag_step(SwimPt &s, float charge, float ty, double d1) {
    using namespace phys;
    const float tx_i = s.mx / s.mz;
    const float tx_f = (float)(tx_i + 2.f * charge * PTKICK_UNIT * STEP_FMAG / sqrtf(s.mx * s.mx + s.mz * s.mz));
    const float t10 = (float)(tx_i * STEP_FMAG), t11 = (float)(ty * STEP_FMAG), t12 = (float)STEP_FMAG;
    const float b0 = s.x - t10, b1 = s.y - t11, b2 = s.z - t12;
    const float ptot_i = sqrtf(s.mx * s.mx + s.my * s.my + s.mz * s.mz);
    float ptot_b = ptot_i;
    if (b2 > FMAG_HOLE_LENGTH || b0 * b0 + b1 * b1 > FMAG_HOLE_RADIUS)
        ptot_b = (float)(ptot_b + (DEDX_UNIT_0 + d1 * ptot_i + DEDX_UNIT_2 * ptot_i * ptot_i +
                                   DEDX_UNIT_3 * ptot_i * ptot_i * ptot_i + DEDX_UNIT_4 * ptot_i * ptot_i * ptot_i * ptot_i) *
                                      sqrtf(t10 * t10 + t11 * t11 + t12 * t12));
    const float t20 = (float)(tx_f * STEP_FMAG), t21 = (float)(ty * STEP_FMAG), t22 = (float)STEP_FMAG;
    s.x = b0 - t20;
    s.y = b1 - t21;
    s.z = b2 - t22;
    float ptot_f = ptot_b;
    if (s.z > FMAG_HOLE_LENGTH || s.x * s.x + s.y * s.y > FMAG_HOLE_RADIUS)
        ptot_f = (float)(ptot_f + dedx_poly(ptot_b) * sqrtf(t20 * t20 + t21 * t21 + t22 * t22));
    const float pz_f = ptot_f / sqrtf(1.f + tx_f * tx_f + ty * ty);
    s.mx = pz_f * tx_f;
    s.my = pz_f * ty;
    s.mz = pz_f;
}

__device__ __forceinline__ void dim_target_step(SwimPt &s, float ty) {  // H:1395-1408
    using namespace phys;
    const float tx_i = s.mx / s.mz;
    const float t0 = (float)(tx_i * STEP_TARGET), t1 = (float)(ty * STEP_TARGET), t2 = (float)STEP_TARGET;
    s.x = s.x - t0;
    s.y = s.y - t1;
    s.z = s.z - t2;
}

// FindDimuonClosestApproach (H:1269-1477)
__device__ float closest_approach(float *v, float *p_pos, float *p_neg, float c1, float c2, float ty1, float ty2,
                                  SwimPt s1, SwimPt s2) {
    using namespace phys;
    float dca2_min = 1.e18f;
    int best = -1;
    SwimPt b1 = s1, b2 = s2;
    float z66_1 = 0.f, z66_2 = 0.f;  // element 200 of the reference's flat arrays (H:1447-1449)
    for (int j = 0; j <= NSTEPS_FMAG + NSTEPS_TARGET; ++j) {
        if (j >= 1 && j <= NSTEPS_FMAG) {
            dim_fmag_step(s1, c1, ty1, DEDX_UNIT_1);
            dim_fmag_step(s2, c2, ty2, DEDX_UNIT_2);
        } else if (j > NSTEPS_FMAG) {
            dim_target_step(s1, ty1);
            dim_target_step(s2, ty2);
        }
        if (j == 66) {
            z66_1 = s1.z;
            z66_2 = s2.z;
        }
        if (FMAGSTR * c1 * s1.mx < 0. && FMAGSTR * c2 * s2.mx < 0.) continue;
        const float dx = s1.x - s2.x, dy = s1.y - s2.y;
        const float dca2 = dx * dx + dy * dy;
        if (dca2 < dca2_min) {
            dca2_min = dca2;
            best = j;
            b1 = s1;
            b2 = s2;
        }
    }
    if (best < 0) {
        const float m = (float)((z66_1 + z66_2) * 0.5);
        v[0] = v[1] = v[2] = m;
        return Z_DUMP;
    }
    const SwimPt &sp = c1 > 0 ? b1 : b2, &sn = c1 > 0 ? b2 : b1;
    p_pos[0] = sp.mx; p_pos[1] = sp.my; p_pos[2] = sp.mz;
    p_neg[0] = sn.mx; p_neg[1] = sn.my; p_neg[2] = sn.mz;
    v[0] = (float)((b1.x + b2.x) * 0.5);
    v[1] = (float)((b1.y + b2.y) * 0.5);
    v[2] = (float)((b1.z + b2.z) * 0.5);
    return b1.z;
}

__global__ void __launch_bounds__(128)
    dimuon_kernel(const or_plane_t *__restrict__ gplane, or_tracks_view_t tv, or_dimuons_view_t dv,
                  const uint8_t *__restrict__ toomany, int n_events) {
    using namespace phys;
    __shared__ float zs[OR_NDET];
    for (int i = threadIdx.x; i < OR_NDET; i += blockDim.x) zs[i] = gplane->z[i];
    __syncthreads();
    const float p_beam[4] = {0, 0, PBEAM, EBEAM};
    const float p_target[4] = {0, 0, 0, MP};
    const float p_cms[4] = {0, 0, PBEAM, EBEAM + MP};
    const float s = p_cms[3] * p_cms[3] - (p_cms[0] * p_cms[0] + p_cms[1] * p_cms[1] + p_cms[2] * p_cms[2]);
    const float sqrt_s = sqrtf(s);
    const float cms_bz = p_cms[2] / p_cms[3];
    for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < n_events; e += (long)gridDim.x * blockDim.x) {
        if (toomany[e]) continue;
        // slots holding a vertexed track
        unsigned smask = 0;
        for (int sl = 0; sl < OR_NSLOTS; ++sl) {
            const int n = min((int)tv.ntracks[e * OR_NSLOTS + sl], OR_SLOTCAP);
            for (int k = 0; k < n; ++k)
                if (trk_rec(tv, e, sl, k)[OR_TRK_STID] >= 7) {
                    smask |= 1u << sl;
                    break;
                }
        }
        float p_pos[4] = {0, 0, 0, 0}, p_neg[4] = {0, 0, 0, 0}, pos_v[3] = {0, 0, 0}, neg_v[3] = {0, 0, 0};
        float *out = dv.dimuons + (size_t)e * OR_EVT_DIM_FLOATS;
        int ndim = 0;
        for (unsigned mi = smask; mi; mi &= mi - 1) {
            const int it = __ffs(mi) - 1;
            const int ni = min((int)tv.ntracks[e * OR_NSLOTS + it], OR_SLOTCAP);
            for (unsigned mj = smask & ~((1u << it) - 1u); mj; mj &= mj - 1) {
                const int jt = __ffs(mj) - 1;
                const int nj = min((int)tv.ntracks[e * OR_NSLOTS + jt], OR_SLOTCAP);
                for (int i = 0; i < ni; ++i) {
                    const float *Ti = trk_rec(tv, e, it, i);
                    if (Ti[OR_TRK_STID] < 7) continue;
                    const float qi = Ti[OR_TRK_CHARGE];
                    {
                        float *pv = qi > 0 ? p_pos : p_neg, *vv = qi > 0 ? pos_v : neg_v;
                        for (int k = 0; k < 3; ++k) {
                            pv[k] = Ti[OR_TRK_PX + k];
                            vv[k] = Ti[OR_TRK_VX + k];
                        }
                        pv[3] = E4(MMU, pv);
                    }
                    for (int j = 0; j < nj; ++j) {
                        const float *Tj = trk_rec(tv, e, jt, j);
                        if (Tj[OR_TRK_STID] < 7) continue;
                        const float qj = Tj[OR_TRK_CHARGE];
                        if (qj * qi > 0) continue;
                        {
                            float *qv = qj > 0 ? p_pos : p_neg, *wv = qj > 0 ? pos_v : neg_v;
                            for (int k = 0; k < 3; ++k) {
                                qv[k] = Tj[OR_TRK_PX + k];
                                wv[k] = Tj[OR_TRK_VX + k];
                            }
                            qv[3] = E4(MMU, qv);
                        }
                        float p_pos_single[4], p_neg_single[4], v_1[3], v_2[3], dim_v[3], p_sum[4];
                        for (int k = 0; k < 4; ++k) {
                            p_pos_single[k] = p_pos[k];
                            p_neg_single[k] = p_neg[k];
                        }
                        for (int k = 0; k < 3; ++k) v_1[k] = (pos_v[k] + neg_v[k]) * 0.5f;
                        float ty1, ty2, c1, c2;
                        const SwimPt s1 = dim_start(Ti, zs, ty1, c1);
                        const SwimPt s2 = dim_start(Tj, zs, ty2, c2);
                        const float vz_2 = closest_approach(v_2, p_pos, p_neg, c1, c2, ty1, ty2, s1, s2);
                        p_pos[3] = E4(MMU, p_pos);
                        p_neg[3] = E4(MMU, p_neg);
                        if (fabsf(vz_2 - v_2[2]) < STEP_FMAG) {
                            for (int k = 0; k < 4; ++k) p_sum[k] = p_pos[k] + p_neg[k];
                            for (int k = 0; k < 3; ++k) dim_v[k] = v_2[k];
                        } else {
                            for (int k = 0; k < 4; ++k) p_sum[k] = p_pos_single[k] + p_neg_single[k];
                            for (int k = 0; k < 3; ++k) dim_v[k] = v_1[k];
                        }
                        const float m =
                            sqrtf(p_sum[3] * p_sum[3] - (p_sum[0] * p_sum[0] + p_sum[1] * p_sum[1] + p_sum[2] * p_sum[2]));
                        const float pT = sqrtf(p_sum[0] * p_sum[0] + p_sum[1] * p_sum[1]);
                        const float x1 = mult4(p_target, p_sum) / mult4(p_target, p_cms);
                        const float x2 = mult4(p_beam, p_sum) / mult4(p_beam, p_cms);
                        {  // Boost(p_sum, cms_bv, -1), H:1245-1267
                            const float bx = 0.0f * -1, by = 0.0f * -1, bz = cms_bz * -1;
                            const float b2 = bx * bx + by * by + bz * bz;
                            const float gamma = 1.0f / sqrtf(1.0f - b2);
                            const float bp = p_sum[0] * bx + p_sum[1] * by + p_sum[2] * bz;
                            const float gamma2 = b2 > 0.0f ? (gamma - 1.0f) / b2 : 0.0f;
                            p_sum[0] = p_sum[0] + gamma2 * bp * bx + gamma * bx * p_sum[3];
                            p_sum[1] = p_sum[1] + gamma2 * bp * by + gamma * by * p_sum[3];
                            p_sum[2] = p_sum[2] + gamma2 * bp * bz + gamma * bz * p_sum[3];
                            p_sum[3] = gamma * (p_sum[3] + bp);
                        }
                        const float xF = 2.0f * p_sum[2] / (sqrt_s * (1.f - m * m / s));
                        const float costheta =
                            2 * (p_neg[3] * p_pos[2] - p_neg[2] * p_pos[3]) / (m * sqrtf(m * m + pT * pT));
                        const float phi = atan2f(2 * sqrtf(m * m + pT * pT) * (p_neg[0] * p_pos[1] - p_neg[1] * p_pos[0]),
                                                 m * (p_pos[0] * p_pos[0] - p_neg[0] * p_neg[0] + p_pos[1] * p_pos[1] -
                                                      p_neg[1] * p_neg[1]));
                        // K:3028-3042
                        if (FMAGSTR * (p_pos[0] - p_neg[0]) < 0.) continue;
                        if (m < 0 || m > 10.f) continue;
                        if (fabsf(xF) > 1.f) continue;
                        if (x1 < 0.f || x1 > 1.f) continue;
                        if (x2 < 0.f || x2 > 1.f) continue;
                        if (fabsf(costheta) > 1.f) continue;
                        if (p_pos[2] + p_neg[2] > 120.f || p_pos[2] + p_neg[2] < 30.f) continue;
                        if (fabsf(p_pos[0] + p_neg[0]) > 3.f) continue;
                        if (dim_v[0] * dim_v[0] + dim_v[1] * dim_v[1] > 225.f) continue;
                        // the reference writes a 17th record past its event's
                        // 16 (K:3059); the event's 16 records are the limit here
                        if (ndim >= OR_DIMUON_MAX) continue;
                        float *D = out + (size_t)ndim * OR_NDIMUONPARAM;
                        D[OR_DIM_MASS] = m;
                        D[OR_DIM_PT] = pT;
                        D[OR_DIM_XF] = xF;
                        D[OR_DIM_X1] = x1;
                        D[OR_DIM_X2] = x2;
                        D[OR_DIM_COSTHETA] = costheta;
                        D[OR_DIM_PHI] = phi;
                        D[OR_DIM_MASS_SINGLE] = 0.f;
                        D[OR_DIM_CHI2_SINGLE] = 0.f;
                        for (int k = 0; k < 3; ++k) {
                            D[OR_DIM_VTX + k] = dim_v[k];
                            D[OR_DIM_POS_VTX + k] = pos_v[k];
                            D[OR_DIM_NEG_VTX + k] = neg_v[k];
                        }
                        for (int k = 0; k < 4; ++k) {
                            D[OR_DIM_POS_P + k] = p_pos[k];
                            D[OR_DIM_NEG_P + k] = p_neg[k];
                            D[OR_DIM_POS_P_SINGLE + k] = p_pos_single[k];
                            D[OR_DIM_NEG_P_SINGLE + k] = p_neg_single[k];
                        }
                        D[OR_DIM_CHI2_VTX] = 0.f;
                        D[OR_DIM_CHI2_KF] = 0.f;
                        ++ndim;
                    }
                }
            }
        }
        dv.ndimuons[e] = (uint16_t)ndim;
    }
}

// ---------------------------------------------------------------------------
// histograms (K:3100-3195)

__device__ __forceinline__ void hist_fill(or_hists_t *H, const int16_t *nbins, const float *hw, unsigned tmask, int k,
                                          float v, int lane) {
    for (unsigned m = tmask; m; m &= m - 1) {
        const int t = __ffs(m) - 1;
        const int i = t * OR_HIST_NVARS + k;
        const float h = hw[i];
        const float *xp = H->xpts + (size_t)i * OR_HIST_NBINS_MAX;
        float *val = H->values + (size_t)i * OR_HIST_NBINS_MAX;
        for (int j = lane; j < nbins[i]; j += 32) {
            const float x = xp[j];
            if (x - h <= v && v < x + h) atomicAdd(val + j, 1.f);
        }
    }
}

template <int W>
__global__ void __launch_bounds__(W * 32)
    hist_kernel(or_tracks_view_t tv, or_dimuons_view_t dv, const int32_t *__restrict__ trigger_bits,
                const uint8_t *__restrict__ toomany, or_hists_t *H, int n_events) {
    __shared__ int16_t nbins[OR_HIST_NTRIGGERS * OR_HIST_NVARS];
    __shared__ float hw[OR_HIST_NTRIGGERS * OR_HIST_NVARS];
    for (int i = threadIdx.x; i < OR_HIST_NTRIGGERS * OR_HIST_NVARS; i += blockDim.x) {
        nbins[i] = min((int)H->nbins[i], OR_HIST_NBINS_MAX);
        hw[i] = H->pts_hw[i];
    }
    __syncthreads();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (long e = (long)blockIdx.x * W + w; e < n_events; e += (long)gridDim.x * W) {
        if (toomany[e]) continue;
        const int tb = trigger_bits ? trigger_bits[e] : 0;
        unsigned tmask = 1u << (OR_HIST_NTRIGGERS - 1);  // "all triggers" (K:3110)
        for (int t = 0; t < OR_HIST_NTRIGGERS - 1; ++t)
            if (tb & t) tmask |= 1u << t;  // K:3108: the bit test the reference makes
        const int nslot = min((int)tv.ntracks[e * OR_NSLOTS + lane], OR_SLOTCAP);
        for (unsigned have = __ballot_sync(0xffffffffu, nslot > 0); have; have &= have - 1) {
            const int sl = __ffs(have) - 1;
            const int n = __shfl_sync(0xffffffffu, nslot, sl);
            for (int k = 0; k < n; ++k) {
                const float *T = trk_rec(tv, e, sl, k);
                if (T[OR_TRK_STID] < 7 || T[OR_TRK_CHI2] / (T[OR_TRK_NHITS] - 5) > phys::CHI2DOF_MAX) continue;
                const float vars[6] = {T[OR_TRK_PX], T[OR_TRK_PX + 1], T[OR_TRK_PX + 2],
                                       T[OR_TRK_VX], T[OR_TRK_VX + 1], T[OR_TRK_VX + 2]};
#pragma unroll
                for (int kv = 0; kv < OR_HIST_NVARS_TRACKS; ++kv) hist_fill(H, nbins, hw, tmask, kv, vars[kv], lane);
            }
        }
        const int nd = min((int)dv.ndimuons[e], OR_DIMUON_MAX);
        for (int i = 0; i < nd; ++i) {
            const float *D = dv.dimuons + (size_t)e * OR_EVT_DIM_FLOATS + (size_t)i * OR_NDIMUONPARAM;
            const float vars[12] = {D[OR_DIM_MASS], D[OR_DIM_XF], D[OR_DIM_X1], D[OR_DIM_X2],
                                    D[OR_DIM_PT], D[OR_DIM_PHI], D[OR_DIM_POS_P] + D[OR_DIM_NEG_P],
                                    D[OR_DIM_POS_P + 1] + D[OR_DIM_NEG_P + 1], D[OR_DIM_POS_P + 2] + D[OR_DIM_NEG_P + 2],
                                    D[OR_DIM_VTX], D[OR_DIM_VTX + 1], D[OR_DIM_VTX + 2]};
#pragma unroll
            for (int kv = 0; kv < 12; ++kv)
                hist_fill(H, nbins, hw, tmask, OR_HIST_NVARS_TRACKS + kv, vars[kv], lane);
        }
    }
}

// ---------------------------------------------------------------------------

cudaError_t launch_vertexing(const or_plane_t *d_plane, or_tracks_view_t tv, const uint8_t *toomany, int n_events,
                             cudaStream_t stream, int sm_count) {
    if (n_events <= 0) return cudaSuccess;
    constexpr int W = 4;
    long blocks = ((long)n_events + 32 * W - 1) / (32 * W);
    blocks = min(blocks, (long)sm_count * 16);
    vertex_kernel<W><<<(unsigned)blocks, W * 32, 0, stream>>>(d_plane, tv, toomany, n_events);
    return cudaGetLastError();
}

cudaError_t launch_dimuons(const or_plane_t *d_plane, or_tracks_view_t tv, or_dimuons_view_t dv,
                           const uint8_t *toomany, int n_events, cudaStream_t stream, int sm_count) {
    if (n_events <= 0) return cudaSuccess;
    long blocks = ((long)n_events + 127) / 128;
    blocks = min(blocks, (long)sm_count * 16);
    dimuon_kernel<<<(unsigned)blocks, 128, 0, stream>>>(d_plane, tv, dv, toomany, n_events);
    return cudaGetLastError();
}

cudaError_t launch_histograms(or_tracks_view_t tv, or_dimuons_view_t dv, const int32_t *trigger_bits,
                              const uint8_t *toomany, or_hists_t *d_hists, int n_events, cudaStream_t stream,
                              int sm_count) {
    if (n_events <= 0) return cudaSuccess;
    constexpr int W = 8;
    long blocks = ((long)n_events + W - 1) / W;
    blocks = min(blocks, (long)sm_count * 8);
    hist_kernel<W><<<(unsigned)blocks, W * 32, 0, stream>>>(tv, dv, trigger_bits, toomany, d_hists, n_events);
    return cudaGetLastError();
}

}  // namespace orgpu
