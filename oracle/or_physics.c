/*
 * or_physics.c -- CPU oracle for the stages after global tracking:
 * vertexing (FMag swim), dimuon building and the monitoring histograms.
 *
 * TEST INFRASTRUCTURE ONLY, like or_oracle.c: a plain-C restatement of the
 * reference kernels used by the tests as the checker.  The CUDA library never
 * links or calls it.
 *
 *   orc_vertexing       gKernel_Vertexing          reconstruction_kernels.cuh:2542-2810
 *   orc_dimuons         gKernel_DimuonBuilding     reconstruction_kernels.cuh:2820-3090
 *                       FindDimuonClosestApproach  reconstruction_helper.cuh:1269-1477
 *   orc_hist_table      the host's table setup     online_reconstruction.cu:670-723
 *   orc_fill_histograms gKernel_fill_display_histograms reconstruction_kernels.cuh:3100-3195
 *
 * The reference mixes float and double in these kernels (its step and
 * energy-loss constants are double, its track parameters float, and it calls
 * sqrtf on double expressions); every expression below keeps the operand
 * types of the reference expression it restates, so the promotions and
 * roundings are the same.  Built with -ffp-contract=off: one rounding per
 * operation, as a reference build with -fmad=false.
 *
 * The reference stores each swim in arrays of 201 points and then scans them
 * for the closest approach; the scan visits the points in step order with a
 * strict "smaller than" test, so it is evaluated here as the points are made,
 * which gives the same step.
 */
#include <math.h>
#include <string.h>

#include "or_oracle.h"

/* reconstruction_constants.h, E1039 build (K0:75-121, K0:209-214) */
static const float X_BEAM = 0.f, Y_BEAM = 0.f; /* K0:75-76 */
static const float Z_DUMP = 42.f;             /* K0:77 */
static const float PT_KICK_KMAG = -0.3819216f; /* K0:85 */
static const float FMAGSTR = -1.054f;          /* K0:91 */
static const double PTKICK_UNIT = -0.006096568; /* K0:93 */
static const float Z_KMAG_BEND = 1064.26f;      /* K0:94 */
static const double FMAG_LENGTH = 502.92;       /* K0:110 */
static const double FMAG_HOLE_LENGTH = 27.94;   /* K0:111 */
static const double FMAG_HOLE_RADIUS = 1.27;    /* K0:112 */
#define NSTEPS_FMAG 100                         /* K0:113 */
static const double STEP_FMAG = 2.514600;       /* K0:114 */
static const double DEDX_UNIT_0 = 0.014282073;  /* K0:115-119 */
static const double DEDX_UNIT_1 = 7.1869681e-05;
static const double DEDX_UNIT_2 = -1.4279150e-06;
static const double DEDX_UNIT_3 = 1.5853655e-08;
static const double DEDX_UNIT_4 = -6.0741470e-11;
#define NSTEPS_TARGET 100                       /* K0:120 */
static const double STEP_TARGET = 5.0;          /* K0:121 */
static const float Ebeam = 120.f, Mp = 0.938272f, Pbeam = 119.996331801f, Mmu = 0.105658f; /* K0:210-213 */
static const float CHI2DOF_MAX = 250.f;         /* K0:194 */

static inline float *trk(or_tracks_view_t tv, long e, int slot, int k) {
    return tv.tracks + (size_t)e * OR_EVT_TRK_FLOATS + (size_t)(slot * OR_SLOTCAP + k) * OR_NTRKPARAM;
}

/* gTracks::get_firsthitdetid, reconstruction_classes.cuh:517-532 */
static short first_hit_detid(const float *T, const float *z) {
    const int nhits = (int)T[OR_TRK_NHITS];
    short detid_min = 30;
    float z_min = 10000.f;
    for (short i = 0; i < nhits && i < OR_MAXHITS_PER_TRACK; i++) {
        const short d = (short)T[OR_TRK_HIT_DETID + i];
        if (d > 0 && z[d] < z_min) {
            detid_min = d;
            z_min = z[d];
        }
    }
    return detid_min;
}

/* calculate_x0_tx_st1, reconstruction_helper.cuh:622-626 */
static void x0_tx_st1(float x0, float tx, float invP, short charge, float *x0_st1, float *tx_st1) {
    *tx_st1 = tx + PT_KICK_KMAG * invP * charge;
    *x0_st1 = tx * Z_KMAG_BEND + x0 - *tx_st1 * Z_KMAG_BEND;
}

static inline float x_trk(float x0, float tx, float z) { return z * tx + x0; } /* H:50-53 */

static inline double dedx_poly(double p) {
    return DEDX_UNIT_0 + DEDX_UNIT_1 * p + DEDX_UNIT_2 * p * p + DEDX_UNIT_3 * p * p * p + DEDX_UNIT_4 * p * p * p * p;
}

/* ------------------------------------------------------------------------ */
/* vertexing: one track swum back through FMag in double (K:2594-2803)      */

static void vertex_track(float *T, const float *z) {
    const float x0 = T[OR_TRK_X0], y0 = T[OR_TRK_Y0], tx = T[OR_TRK_TX], ty = T[OR_TRK_TY];
    const float invP = T[OR_TRK_INVP], charge = T[OR_TRK_CHARGE];
    const short detid_first = first_hit_detid(T, z);
    float x0_st1, tx_st1;
    x0_tx_st1(x0, tx, invP, (short)charge, &x0_st1, &tx_st1);
    const double z_0 = z[detid_first];
    double s0[5];
    s0[0] = charge * invP * sqrtf((1.f + tx_st1 * tx_st1) / (1.f + tx_st1 * tx_st1 + ty * ty));
    s0[1] = tx_st1;
    s0[2] = ty;
    s0[3] = x_trk(x0_st1, tx_st1, (float)z_0);
    s0[4] = x_trk(y0, ty, (float)z_0);
    double pos[3], mom[3];
    pos[0] = s0[3] + s0[1] * (FMAG_LENGTH - z_0);
    pos[1] = s0[4] + s0[2] * (FMAG_LENGTH - z_0);
    pos[2] = FMAG_LENGTH;
    const double pz_0 = 1.f / (fabs(s0[0]) * sqrtf(1.f + s0[1] * s0[1] + s0[2] * s0[2]));
    mom[0] = pz_0 * s0[1];
    mom[1] = pz_0 * s0[2];
    mom[2] = pz_0;
    /* closest approach to the beam line over the points 0..200 (K:2746-2781) */
    double dca2_min = 1.e18;
    int found = 0;
    double vpos[3], vmom[3];
#define VTX_VISIT()                                                                                     \
    do {                                                                                                \
        if (!(FMAGSTR * charge * mom[0] < 0.)) {                                                        \
            const double dca2 = (pos[0] - X_BEAM) * (pos[0] - X_BEAM) + (pos[1] - Y_BEAM) * (pos[1] - Y_BEAM); \
            if (dca2 < dca2_min) {                                                                      \
                dca2_min = dca2;                                                                        \
                found = 1;                                                                              \
                memcpy(vpos, pos, sizeof(pos));                                                         \
                memcpy(vmom, mom, sizeof(mom));                                                         \
            }                                                                                           \
        }                                                                                               \
    } while (0)
    VTX_VISIT();
    for (int step = 1; step <= NSTEPS_FMAG; ++step) { /* K:2646-2716 */
        const double tx_i = mom[0] / mom[2];
        const double tx_f = tx_i + 2.f * charge * PTKICK_UNIT * STEP_FMAG / sqrt(mom[0] * mom[0] + mom[2] * mom[2]);
        const double t1[3] = {tx_i * STEP_FMAG, ty * STEP_FMAG, STEP_FMAG};
        const double pb[3] = {pos[0] - t1[0], pos[1] - t1[1], pos[2] - t1[2]};
        const double ptot_i = sqrt(mom[0] * mom[0] + mom[1] * mom[1] + mom[2] * mom[2]);
        double ptot_b = ptot_i;
        if (pb[2] > FMAG_HOLE_LENGTH || pb[0] * pb[0] + pb[1] * pb[1] > FMAG_HOLE_RADIUS)
            ptot_b += dedx_poly(ptot_i) * sqrtf(t1[0] * t1[0] + t1[1] * t1[1] + t1[2] * t1[2]);
        const double t2[3] = {tx_f * STEP_FMAG, ty * STEP_FMAG, STEP_FMAG};
        pos[0] = pb[0] - t2[0];
        pos[1] = pb[1] - t2[1];
        pos[2] = pb[2] - t2[2];
        double ptot_f = ptot_b;
        if (pos[2] > FMAG_HOLE_LENGTH || pos[0] * pos[0] + pos[1] * pos[1] > FMAG_HOLE_RADIUS)
            ptot_f += dedx_poly(ptot_b) * sqrtf(t2[0] * t2[0] + t2[1] * t2[1] + t2[2] * t2[2]);
        const double pz_f = ptot_f / sqrt(1.f + tx_f * tx_f + ty * ty);
        mom[0] = pz_f * tx_f;
        mom[1] = pz_f * ty;
        mom[2] = pz_f;
        VTX_VISIT();
    }
    for (int step = NSTEPS_FMAG + 1; step <= NSTEPS_FMAG + NSTEPS_TARGET; ++step) { /* K:2718-2740 */
        const double tx_i = mom[0] / mom[2];
        pos[0] = pos[0] - tx_i * STEP_TARGET;
        pos[1] = pos[1] - ty * STEP_TARGET;
        pos[2] = pos[2] - STEP_TARGET;
        VTX_VISIT();
    }
#undef VTX_VISIT
    if (!found) { /* no point passes: the last one (step = 200, K:2752) */
        memcpy(vpos, pos, sizeof(pos));
        memcpy(vmom, mom, sizeof(mom));
    }
    T[OR_TRK_STID] = 7.f; /* K:2796 */
    for (int k = 0; k < 3; k++) {
        T[OR_TRK_VX + k] = (float)vpos[k];
        T[OR_TRK_PX + k] = (float)vmom[k];
    }
}

static void vertex_event(const or_plane_t *P, or_tracks_view_t tv, long e) {
    for (int s = 0; s < OR_NSLOTS; s++) {
        const int n = tv.ntracks[e * OR_NSLOTS + s] < OR_SLOTCAP ? tv.ntracks[e * OR_NSLOTS + s] : OR_SLOTCAP;
        for (int i = 0; i < n; i++) {
            float *T = trk(tv, e, s, i);
            if (T[OR_TRK_STID] < 6) continue; /* K:2594 */
            vertex_track(T, P->z);
        }
    }
}

void orc_vertexing(const or_plane_t *p, or_tracks_view_t t, const uint8_t *toomany, int n_events, int n_threads) {
    (void)n_threads;
    for (long e = 0; e < n_events; e++)
        if (!toomany[e]) vertex_event(p, t, e);
}

/* ------------------------------------------------------------------------ */
/* dimuons (K:2820-3090), everything in float as there                      */

static inline float E4(float m, const float *p) { return sqrtf(m * m + p[0] * p[0] + p[1] * p[1] + p[2] * p[2]); }
static inline float mult4(const float *a, const float *b) { return a[3] * b[3] - (a[0] * b[0] + a[1] * b[1] + a[2] * b[2]); }

/* H:1245-1263 */
static void boost(float *p, float bx, float by, float bz) {
    const float b2 = bx * bx + by * by + bz * bz;
    const float gamma = 1.0f / sqrtf(1.0f - b2);
    const float bp = p[0] * bx + p[1] * by + p[2] * bz;
    const float gamma2 = b2 > 0.0f ? (gamma - 1.0f) / b2 : 0.0f;
    p[0] = p[0] + gamma2 * bp * bx + gamma * bx * p[3];
    p[1] = p[1] + gamma2 * bp * by + gamma * by * p[3];
    p[2] = p[2] + gamma2 * bp * bz + gamma * bz * p[3];
    p[3] = gamma * (p[3] + bp);
}

typedef struct {
    float pos[3], mom[3];
} swim_pt_t;

/* the start point of a track's swim (K:2927-2947 / K:2949-2970) */
static void dim_start(const float *T, const float *z, float *ty_out, float *charge_out, swim_pt_t *s) {
    const float x0 = T[OR_TRK_X0], y0 = T[OR_TRK_Y0], tx = T[OR_TRK_TX], ty = T[OR_TRK_TY];
    const float invP = T[OR_TRK_INVP], charge = T[OR_TRK_CHARGE];
    const short detid_first = first_hit_detid(T, z);
    float x0_st1, tx_st1;
    x0_tx_st1(x0, tx, invP, (short)charge, &x0_st1, &tx_st1);
    const float z_0 = z[detid_first];
    float s0[5];
    s0[0] = charge * invP * sqrtf((1.f + tx_st1 * tx_st1) / (1.f + tx_st1 * tx_st1 + ty * ty));
    s0[1] = tx_st1;
    s0[2] = ty;
    s0[3] = x_trk(x0_st1, tx_st1, z_0);
    s0[4] = x_trk(y0, ty, z_0);
    s->pos[0] = (float)(s0[3] + s0[1] * (FMAG_LENGTH - z_0));
    s->pos[1] = (float)(s0[4] + s0[2] * (FMAG_LENGTH - z_0));
    s->pos[2] = (float)FMAG_LENGTH;
    const float pz_0 = 1.f / (fabsf(s0[0]) * sqrtf(1.f + s0[1] * s0[1] + s0[2] * s0[2]));
    s->mom[0] = pz_0 * s0[1];
    s->mom[1] = pz_0 * s0[2];
    s->mom[2] = pz_0;
    *ty_out = ty;
    *charge_out = charge;
}

/* one FMag step of FindDimuonClosestApproach for one track (H:1290-1333);
 * `d1` is the linear energy-loss coefficient of the first update: the
 * reference uses DEDX_UNIT_2 there for its second track (H:1354) */
static void dim_fmag_step(swim_pt_t *s, float charge, float ty, double d1) {
    const float tx_i = s->mom[0] / s->mom[2];
    const float tx_f = (float)(tx_i + 2.f * charge * PTKICK_UNIT * STEP_FMAG /
                                           sqrtf(s->mom[0] * s->mom[0] + s->mom[2] * s->mom[2]));
    float t1[3], pb[3], t2[3];
    t1[0] = (float)(tx_i * STEP_FMAG);
    t1[1] = (float)(ty * STEP_FMAG);
    t1[2] = (float)STEP_FMAG;
    pb[0] = s->pos[0] - t1[0];
    pb[1] = s->pos[1] - t1[1];
    pb[2] = s->pos[2] - t1[2];
    const float ptot_i = sqrtf(s->mom[0] * s->mom[0] + s->mom[1] * s->mom[1] + s->mom[2] * s->mom[2]);
    float ptot_b = ptot_i;
    if (pb[2] > FMAG_HOLE_LENGTH || pb[0] * pb[0] + pb[1] * pb[1] > FMAG_HOLE_RADIUS)
        ptot_b = (float)(ptot_b + (DEDX_UNIT_0 + d1 * ptot_i + DEDX_UNIT_2 * ptot_i * ptot_i +
                                   DEDX_UNIT_3 * ptot_i * ptot_i * ptot_i + DEDX_UNIT_4 * ptot_i * ptot_i * ptot_i * ptot_i) *
                                      sqrtf(t1[0] * t1[0] + t1[1] * t1[1] + t1[2] * t1[2]));
    t2[0] = (float)(tx_f * STEP_FMAG);
    t2[1] = (float)(ty * STEP_FMAG);
    t2[2] = (float)STEP_FMAG;
    s->pos[0] = pb[0] - t2[0];
    s->pos[1] = pb[1] - t2[1];
    s->pos[2] = pb[2] - t2[2];
    float ptot_f = ptot_b;
    if (s->pos[2] > FMAG_HOLE_LENGTH || s->pos[0] * s->pos[0] + s->pos[1] * s->pos[1] > FMAG_HOLE_RADIUS)
        ptot_f = (float)(ptot_f + dedx_poly(ptot_b) * sqrtf(t2[0] * t2[0] + t2[1] * t2[1] + t2[2] * t2[2]));
    const float pz_f = ptot_f / sqrtf(1.f + tx_f * tx_f + ty * ty);
    s->mom[0] = pz_f * tx_f;
    s->mom[1] = pz_f * ty;
    s->mom[2] = pz_f;
}

static void dim_target_step(swim_pt_t *s, float ty) { /* H:1395-1408 */
    const float tx_i = s->mom[0] / s->mom[2];
    float t1[3];
    t1[0] = (float)(tx_i * STEP_TARGET);
    t1[1] = (float)(ty * STEP_TARGET);
    t1[2] = (float)STEP_TARGET;
    s->pos[0] = s->pos[0] - t1[0];
    s->pos[1] = s->pos[1] - t1[1];
    s->pos[2] = s->pos[2] - t1[2];
}

/* FindDimuonClosestApproach (H:1269-1477): both tracks swum together; the
 * closest point in x-y where at least one track still bends the FMag way.
 * Returns the z it reports and updates p_pos / p_neg (momenta at that
 * point) and v (the midpoint). */
static float closest_approach(float *v, float *p_pos, float *p_neg, float charge_1, float charge_2, float ty_1,
                              float ty_2, swim_pt_t *s1, swim_pt_t *s2) {
    float dca2_min = 1.e18f;
    int best = -1;
    swim_pt_t b1, b2;
    /* the fallback reads element 200 of the reference's flat position arrays:
     * the z of point 66 (H:1447-1449) */
    float z66_1 = 0.f, z66_2 = 0.f;
    for (int j = 0; j <= NSTEPS_FMAG + NSTEPS_TARGET; j++) {
        if (j >= 1 && j <= NSTEPS_FMAG) {
            dim_fmag_step(s1, charge_1, ty_1, DEDX_UNIT_1);
            dim_fmag_step(s2, charge_2, ty_2, DEDX_UNIT_2);
        } else if (j > NSTEPS_FMAG) {
            dim_target_step(s1, ty_1);
            dim_target_step(s2, ty_2);
        }
        if (j == 66) {
            z66_1 = s1->pos[2];
            z66_2 = s2->pos[2];
        }
        if (FMAGSTR * charge_1 * s1->mom[0] < 0. && FMAGSTR * charge_2 * s2->mom[0] < 0.) continue;
        const float dx = s1->pos[0] - s2->pos[0], dy = s1->pos[1] - s2->pos[1];
        const float dca2 = dx * dx + dy * dy;
        if (dca2 < dca2_min) {
            dca2_min = dca2;
            best = j;
            b1 = *s1;
            b2 = *s2;
        }
    }
    if (best < 0) {
        const float m = (float)((z66_1 + z66_2) * 0.5);
        v[0] = v[1] = v[2] = m;
        return Z_DUMP;
    }
    const swim_pt_t *sp = charge_1 > 0 ? &b1 : &b2, *sn = charge_1 > 0 ? &b2 : &b1;
    for (int k = 0; k < 3; k++) {
        p_pos[k] = sp->mom[k];
        p_neg[k] = sn->mom[k];
        v[k] = (float)((b1.pos[k] + b2.pos[k]) * 0.5);
    }
    return b1.pos[2];
}

static void dimuon_event(const or_plane_t *P, or_tracks_view_t tv, or_dimuons_view_t dv, long e) {
    const float p_beam[4] = {0, 0, Pbeam, Ebeam};
    const float p_target[4] = {0, 0, 0, Mp};
    const float p_cms[4] = {0, 0, Pbeam, Ebeam + Mp};
    const float s = p_cms[3] * p_cms[3] - (p_cms[0] * p_cms[0] + p_cms[1] * p_cms[1] + p_cms[2] * p_cms[2]);
    const float sqrt_s = sqrtf(s);
    const float cms_bz = p_cms[2] / p_cms[3];
    float p_pos[4] = {0, 0, 0, 0}, p_neg[4] = {0, 0, 0, 0}, pos_v[3] = {0, 0, 0}, neg_v[3] = {0, 0, 0};
    float *out = dv.dimuons + (size_t)e * OR_EVT_DIM_FLOATS;
    int ndim = 0;
    for (int it = 0; it < OR_NSLOTS; it++) {
        const int ni = tv.ntracks[e * OR_NSLOTS + it] < OR_SLOTCAP ? tv.ntracks[e * OR_NSLOTS + it] : OR_SLOTCAP;
        for (int jt = it; jt < OR_NSLOTS; jt++) {
            const int nj = tv.ntracks[e * OR_NSLOTS + jt] < OR_SLOTCAP ? tv.ntracks[e * OR_NSLOTS + jt] : OR_SLOTCAP;
            for (int i = 0; i < ni; i++) {
                const float *Ti = trk(tv, e, it, i);
                if (Ti[OR_TRK_STID] < 7) continue;
                float *pv = Ti[OR_TRK_CHARGE] > 0 ? p_pos : p_neg, *vv = Ti[OR_TRK_CHARGE] > 0 ? pos_v : neg_v;
                for (int k = 0; k < 3; k++) {
                    pv[k] = Ti[OR_TRK_PX + k];
                    vv[k] = Ti[OR_TRK_VX + k];
                }
                pv[3] = E4(Mmu, pv);
                for (int j = 0; j < nj; j++) {
                    const float *Tj = trk(tv, e, jt, j);
                    if (Tj[OR_TRK_STID] < 7) continue;
                    if (Tj[OR_TRK_CHARGE] * Ti[OR_TRK_CHARGE] > 0) continue;
                    float *qv = Tj[OR_TRK_CHARGE] > 0 ? p_pos : p_neg, *wv = Tj[OR_TRK_CHARGE] > 0 ? pos_v : neg_v;
                    for (int k = 0; k < 3; k++) {
                        qv[k] = Tj[OR_TRK_PX + k];
                        wv[k] = Tj[OR_TRK_VX + k];
                    }
                    qv[3] = E4(Mmu, qv);
                    float p_pos_single[4], p_neg_single[4], v_1[3], v_2[3], dim_v[3], p_sum[4];
                    memcpy(p_pos_single, p_pos, sizeof(p_pos_single));
                    memcpy(p_neg_single, p_neg, sizeof(p_neg_single));
                    for (int k = 0; k < 3; k++) v_1[k] = (pos_v[k] + neg_v[k]) * 0.5f;
                    swim_pt_t s1, s2;
                    float ty_1, ty_2, charge_1, charge_2;
                    dim_start(Ti, P->z, &ty_1, &charge_1, &s1);
                    dim_start(Tj, P->z, &ty_2, &charge_2, &s2);
                    const float vz_2 = closest_approach(v_2, p_pos, p_neg, charge_1, charge_2, ty_1, ty_2, &s1, &s2);
                    p_pos[3] = E4(Mmu, p_pos);
                    p_neg[3] = E4(Mmu, p_neg);
                    if (fabsf(vz_2 - v_2[2]) < STEP_FMAG) {
                        for (int k = 0; k < 4; k++) p_sum[k] = p_pos[k] + p_neg[k];
                        memcpy(dim_v, v_2, sizeof(dim_v));
                    } else {
                        for (int k = 0; k < 4; k++) p_sum[k] = p_pos_single[k] + p_neg_single[k];
                        memcpy(dim_v, v_1, sizeof(dim_v));
                    }
                    const float m = sqrtf(p_sum[3] * p_sum[3] - (p_sum[0] * p_sum[0] + p_sum[1] * p_sum[1] + p_sum[2] * p_sum[2]));
                    const float pT = sqrtf(p_sum[0] * p_sum[0] + p_sum[1] * p_sum[1]);
                    const float x1 = mult4(p_target, p_sum) / mult4(p_target, p_cms);
                    const float x2 = mult4(p_beam, p_sum) / mult4(p_beam, p_cms);
                    boost(p_sum, 0.0f * -1, 0.0f * -1, cms_bz * -1);
                    const float xF = 2.0f * p_sum[2] / (sqrt_s * (1.f - m * m / s));
                    const float costheta = 2 * (p_neg[3] * p_pos[2] - p_neg[2] * p_pos[3]) / (m * sqrtf(m * m + pT * pT));
                    const float phi = atan2f(2 * sqrtf(m * m + pT * pT) * (p_neg[0] * p_pos[1] - p_neg[1] * p_pos[0]),
                                             m * (p_pos[0] * p_pos[0] - p_neg[0] * p_neg[0] + p_pos[1] * p_pos[1] -
                                                  p_neg[1] * p_neg[1]));
                    /* K:3028-3042 */
                    if (FMAGSTR * (p_pos[0] - p_neg[0]) < 0.) continue;
                    if (m < 0 || m > 10.f) continue;
                    if (fabsf(xF) > 1.f) continue;
                    if (x1 < 0.f || x1 > 1.f) continue;
                    if (x2 < 0.f || x2 > 1.f) continue;
                    if (fabsf(costheta) > 1.f) continue;
                    if (p_pos[2] + p_neg[2] > 120.f || p_pos[2] + p_neg[2] < 30.f) continue;
                    if (fabsf(p_pos[0] + p_neg[0]) > 3.f) continue;
                    if (dim_v[0] * dim_v[0] + dim_v[1] * dim_v[1] > 225.f) continue;
                    /* the reference stores a 17th record past its event's 16
                     * (K:3059, "ndim > DimuonSizeMax"); here the 16 records
                     * of the event are the limit */
                    if (ndim >= OR_DIMUON_MAX) continue;
                    float *D = out + (size_t)ndim * OR_NDIMUONPARAM;
                    memset(D, 0, OR_NDIMUONPARAM * sizeof(float));
                    D[OR_DIM_MASS] = m;
                    D[OR_DIM_PT] = pT;
                    D[OR_DIM_XF] = xF;
                    D[OR_DIM_X1] = x1;
                    D[OR_DIM_X2] = x2;
                    D[OR_DIM_COSTHETA] = costheta;
                    D[OR_DIM_PHI] = phi;
                    for (int k = 0; k < 3; k++) {
                        D[OR_DIM_VTX + k] = dim_v[k];
                        D[OR_DIM_POS_VTX + k] = pos_v[k];
                        D[OR_DIM_NEG_VTX + k] = neg_v[k];
                    }
                    for (int k = 0; k < 4; k++) {
                        D[OR_DIM_POS_P + k] = p_pos[k];
                        D[OR_DIM_NEG_P + k] = p_neg[k];
                        D[OR_DIM_POS_P_SINGLE + k] = p_pos_single[k];
                        D[OR_DIM_NEG_P_SINGLE + k] = p_neg_single[k];
                    }
                    ndim++;
                }
            }
        }
    }
    dv.ndimuons[e] = (uint16_t)ndim;
}

void orc_dimuons(const or_plane_t *p, or_tracks_view_t t, or_dimuons_view_t d, const uint8_t *toomany, int n_events,
                 int n_threads) {
    (void)n_threads;
    for (long e = 0; e < n_events; e++)
        if (!toomany[e]) dimuon_event(p, t, d, e);
}

/* ------------------------------------------------------------------------ */
/* histograms                                                               */

void orc_hist_table(or_hists_t *h) {
    /* histotools binning, reconstruction_constants.h:225-266, in the order of
     * online_reconstruction.cu:670-694 */
    static const short nb[OR_HIST_NVARS] = {100, 100, 100, 100, 100, 200, 50, 50, 50, 50, 50, 50,
                                            100, 100, 100, 100, 100, 200};
    static const float lo[OR_HIST_NVARS] = {-20.f, -20.f, 0.f, -20.f, -20.f, -500.f, 0.f, 0.f, 0.f, 0.f, 0.f,
                                            -3.141592654f, -20.f, -20.f, 0.f, -20.f, -20.f, -500.f};
    static const float hi[OR_HIST_NVARS] = {20.f, 20.f, 120.f, 20.f, 20.f, 500.f, 10.f, 1.f, 1.f, 0.5f, 5.f,
                                            3.141592654f, 20.f, 20.f, 120.f, 20.f, 20.f, 500.f};
    memset(h, 0, sizeof(*h));
    for (int t = 0; t < OR_HIST_NTRIGGERS; t++)
        for (int k = 0; k < OR_HIST_NVARS; k++) {
            const int i = t * OR_HIST_NVARS + k;
            h->nbins[i] = nb[k];
            h->pts_hw[i] = (hi[k] - lo[k]) * 0.5f / nb[k];
            for (int l = 0; l < nb[k]; l++)
                h->xpts[i * OR_HIST_NBINS_MAX + l] = lo[k] + h->pts_hw[k] * (2.f * l + 1.f); /* M:718 */
        }
}

static void hist_fill(or_hists_t *h, const int *trig, int k, float v) {
    for (int t = 0; t < OR_HIST_NTRIGGERS; t++) {
        if (!trig[t]) continue;
        const int i = t * OR_HIST_NVARS + k;
        const float hw = h->pts_hw[i];
        for (int j = 0; j < h->nbins[i]; j++) {
            const float x = h->xpts[i * OR_HIST_NBINS_MAX + j];
            if (x - hw <= v && v < x + hw) h->values[i * OR_HIST_NBINS_MAX + j] += 1.f;
        }
    }
}

void orc_fill_histograms(or_tracks_view_t tv, or_dimuons_view_t dv, or_hists_t *h, const int32_t *trigger_bits,
                         const uint8_t *toomany, int n_events) {
    for (long e = 0; e < n_events; e++) {
        if (toomany[e]) continue;
        int trig[OR_HIST_NTRIGGERS];
        for (int t = 0; t < OR_HIST_NTRIGGERS; t++) trig[t] = (trigger_bits ? trigger_bits[e] : 0) & t; /* K:3108 */
        trig[OR_HIST_NTRIGGERS - 1] = 1;
        for (int s = 0; s < OR_NSLOTS; s++) {
            const int n = tv.ntracks[e * OR_NSLOTS + s] < OR_SLOTCAP ? tv.ntracks[e * OR_NSLOTS + s] : OR_SLOTCAP;
            for (int i = 0; i < n; i++) {
                const float *T = trk(tv, e, s, i);
                if (T[OR_TRK_STID] < 7 || T[OR_TRK_CHI2] / (T[OR_TRK_NHITS] - 5) > CHI2DOF_MAX) continue;
                const float vars[6] = {T[OR_TRK_PX], T[OR_TRK_PX + 1], T[OR_TRK_PX + 2],
                                       T[OR_TRK_VX], T[OR_TRK_VX + 1], T[OR_TRK_VX + 2]};
                for (int k = 0; k < OR_HIST_NVARS_TRACKS; k++) hist_fill(h, trig, k, vars[k]);
            }
        }
        const int nd = dv.ndimuons[e] < OR_DIMUON_MAX ? dv.ndimuons[e] : OR_DIMUON_MAX;
        for (int i = 0; i < nd; i++) {
            const float *D = dv.dimuons + (size_t)e * OR_EVT_DIM_FLOATS + (size_t)i * OR_NDIMUONPARAM;
            const float vars[12] = {D[OR_DIM_MASS], D[OR_DIM_XF], D[OR_DIM_X1], D[OR_DIM_X2], D[OR_DIM_PT],
                                    D[OR_DIM_PHI], D[OR_DIM_POS_P] + D[OR_DIM_NEG_P],
                                    D[OR_DIM_POS_P + 1] + D[OR_DIM_NEG_P + 1], D[OR_DIM_POS_P + 2] + D[OR_DIM_NEG_P + 2],
                                    D[OR_DIM_VTX], D[OR_DIM_VTX + 1], D[OR_DIM_VTX + 2]};
            for (int k = 0; k < 12; k++) hist_fill(h, trig, OR_HIST_NVARS_TRACKS + k, vars[k]);
        }
    }
}
