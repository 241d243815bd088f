/*
 * or_oracle.c -- CPU oracle for the e1039 online-reconstruction hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see or_oracle.h).  A line-by-line restatement of
 * the reference algorithm in plain C; citations are file:line inside the
 * reference project:
 *   K  = OnlineReconstruction/reconstruction_kernels.cuh
 *   H  = OnlineReconstruction/reconstruction_helper.cuh
 *   AM = OnlineReconstruction/trackanalyticalminimizer.cuh
 *   FT = OnlineReconstruction/trackfittingtools.cuh
 *   K0 = OnlineReconstruction/reconstruction_constants.h
 *   M  = OnlineReconstruction/online_reconstruction.cu
 *
 * Build with -ffp-contract=off: every float operation rounds once, in the
 * order the reference source writes it.  Literals keep their C types
 * (0.9*0.5 is double, 5.08f is float, ...), exactly as in the reference.
 *
 * Per-thread scratch arrays of the reference kernels (XZ: K:378-396,
 * YZ: K:1142-1196, Global: K:1993-2035) live for the whole kernel, so values
 * written for one candidate are still there for the next.  The left/right
 * resolution walk (H:725-735, H:820-828) reads the entry just past the hit
 * count when the walk lands on the last hit; the oracle keeps the same
 * persistent arrays so those reads see the same data the reference sees.
 */
#define _GNU_SOURCE
#include "or_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

/* ------------------------------------------------------------------------ */
/* constants, K0:20-207                                                     */
/* ------------------------------------------------------------------------ */
static const float TX_MAX = 0.15f, TY_MAX = 0.1f, X0_MAX = 150.f, Y0_MAX = 50.f;
static const float INVP_MAX = 0.2f, INVP_MIN = 0.01f;

static const short eff_detid_chambers[24] = {1, 2, 3, 4, 5, 6, 13, 14, 15, 16, 17, 18,
                                             19, 20, 21, 22, 23, 24, 25, 26, 27, 28, 29, 30}; /* K0:60 (E1039) */
static const float spacingplane[28] = {0.f,  0.40f, 0.40f, 0.40f, 0.40f, 0.40f, 0.40f, 1.3f,  1.3f, 1.3f,
                                       1.2f, 1.2f,  1.2f,  1.2f,  1.2f,  1.2f,  4.0f,  4.0f,  7.0f, 7.0f,
                                       8.0f, 12.0f, 12.0f, 10.0f, 3.0f,  3.0f,  3.0f,  3.0f}; /* K0:64 */
static const short detsuperid[7][3] = {{2, 1, 3},   {5, 6, 4},   {8, 9, 7}, {11, 12, 10},
                                       {14, 15, 13}, {25, 24, -1}, {26, 27, -1}}; /* K0:65 */
static const short planetype[15] = {1, 0, 2, 1, 0, 2, 2, 0, 1, 2, 0, 1, 2, 0, 1}; /* K0:66 */
static const short hodoplanesx[4][2] = {{31, 32}, {37, 38}, {39, 40}, {45, 46}};  /* K0:71 */
static const float hodofudgefac[4] = {0.25f, 0.2f, 0.15f, 0.0f};                /* K0:73 */
static const float hodoXcellwidth[4] = {7.32f, 13.0f, 14.5875f, 19.6475f};       /* K0:74 */
static const float Z_DUMP = 42.f;                                                /* K0:77 */
static const float SAGITTA_TARGET_CENTER = 1.85f, SAGITTA_TARGET_WIDTH = 0.25f;  /* K0:78-79 */
static const float SAGITTA_DUMP_CENTER = 1.5f, SAGITTA_DUMP_WIDTH = 0.3f;        /* K0:80-81 */
static const float PT_KICK_KMAG = -0.3819216f;                                   /* K0:85 */
static const float FMAGSTR = -1.054f;                                            /* K0:91 */
static const float Z_KMAG_BEND = 1064.26f;                                       /* K0:94 */
static const float Z_TARGET = -300.f;                                            /* K0:96 */
static const short lrpossibility[4][2] = {{1, 1}, {1, -1}, {-1, 1}, {-1, -1}};   /* K0:122 */
#define MaxHitsProj_X 20                                                         /* K0:154 */
static const short WCHitsBins_X[3][2][28] = {                                    /* K0:155-162 */
    {{1, 5, 9, 13, 17, 21, 25, 29, 33, 37, 41, 45, 49, 53, 57, 61, 65, 69, 73, 77, 81, 85, 89, 93, 97, 101, 105, 109},
     {4, 8, 12, 16, 20, 24, 28, 32, 36, 40, 44, 48, 52, 56, 60, 64, 68, 72, 76, 80, 84, 88, 92, 96, 100, 104, 108, 112}},
    {{1, 5, 9, 13, 17, 21, 25, 29, 33, 37, 41, 45, 49, 53, 57, 61, 65, 69, 73, 77, 81, 85, 89, 93, 97, 101, 105, 109},
     {4, 8, 12, 16, 20, 24, 28, 32, 36, 40, 44, 48, 52, 56, 60, 64, 68, 72, 76, 80, 84, 88, 92, 96, 100, 104, 108, 116}},
    {{1, 5, 9, 13, 17, 21, 25, 29, 33, 37, 41, 45, 49, 53, 57, 61, 65, 69, 73, 77, 81, 85, 89, 93, 97, 101, 105, 109},
     {4, 8, 12, 16, 20, 24, 28, 32, 36, 40, 44, 48, 52, 56, 60, 64, 68, 72, 76, 80, 84, 88, 92, 96, 100, 104, 108, 116}},
};
#define MaxD0Multiplicity 210 /* K0:188 */
#define MaxD2Multiplicity 120 /* K0:189 */
#define MaxD3Multiplicity 90  /* K0:190 */
#define NpropXYhitsMin 2      /* K0:195 */
#define ClusterSizeMax 192    /* K0:27 */

/* a detector id that is never adjacent to a real plane: marks scratch-array
 * entries the reference leaves uninitialised */
#define DET_SENTINEL ((short)-100)

/* ------------------------------------------------------------------------ */
/* hit-collection access                                                   */
/* ------------------------------------------------------------------------ */
typedef struct {
    const float *d; /* slot base */
    int n;          /* hit count = SoA stride */
} hitcoll_t;

static inline float hc_chan(hitcoll_t h, int i) { return h.d[i]; }
static inline float hc_pos(hitcoll_t h, int i) { return h.d[h.n + i]; }
static inline float hc_tdc(hitcoll_t h, int i) { return h.d[2 * h.n + i]; }
static inline float hc_flag(hitcoll_t h, int i) { return h.d[3 * h.n + i]; }
static inline float hc_drift(hitcoll_t h, int i) { return h.d[4 * h.n + i]; }

/* reconstruction_classes.cuh:89-102 */
static hitcoll_t hits_chamber(or_hits_view_t hv, long e, int detid) {
    hitcoll_t h;
    h.n = (int)hv.nhits_cham[e * OR_NCHAM + detid - 1];
    h.d = hv.hits_cham + e * OR_EVT_CHAM_FLOATS + (long)OR_NHITSPARAM * OR_MAXHITS_CHAM * (detid - 1);
    return h;
}
static hitcoll_t hits_hodo(or_hits_view_t hv, long e, int detid) {
    hitcoll_t h;
    h.n = (int)hv.nhits_hodo[e * OR_NHODO + detid - OR_NCHAM - 1];
    h.d = hv.hits_hodo + e * OR_EVT_HODO_FLOATS + (long)OR_NHITSPARAM * OR_MAXHITS_HODO * (detid - OR_NCHAM - 1);
    return h;
}
static hitcoll_t hits_prop(or_hits_view_t hv, long e, int detid) {
    hitcoll_t h;
    h.n = (int)hv.nhits_prop[e * OR_NPROP + detid - OR_NCHAM - OR_NHODO - 1];
    h.d = hv.hits_prop + e * OR_EVT_PROP_FLOATS +
          (long)OR_NHITSPARAM * OR_MAXHITS_PROP * (detid - OR_NCHAM - OR_NHODO - 1);
    return h;
}

/* ------------------------------------------------------------------------ */
/* geometry, M:123-218                                                     */
/* ------------------------------------------------------------------------ */
/* Read the next whitespace-separated number the way `istream >> T` does:
 * strtof/strtol on the longest valid prefix, so glued fields such as
 * "2.749630657183.4666022" split into 2.749630657183 and .4666022 (the
 * reference file has those, basic_geometry_e906.txt:48,51,52).  A missing
 * token leaves the target unchanged. */
static int next_float(const char **s, float *out) {
    char *end;
    while (**s == ' ' || **s == '\t' || **s == '\r' || **s == '\n') (*s)++;
    if (!**s) return 0;
    float v = strtof(*s, &end);
    if (end == *s) return 0;
    *out = v;
    *s = end;
    return 1;
}
static int next_int(const char **s, int *out) {
    char *end;
    while (**s == ' ' || **s == '\t' || **s == '\r' || **s == '\n') (*s)++;
    if (!**s) return 0;
    long v = strtol(*s, &end, 10);
    if (end == *s) return 0;
    *out = (int)v;
    *s = end;
    return 1;
}

int orc_parse_geometry(const char *path, or_plane_t *plane, double *wire_pos) {
    FILE *f = fopen(path, "r");
    if (!f) return -1;
    memset(plane, 0, sizeof(*plane));
    static const float TXM = 0.15f, TYM = 0.1f, X0M = 150.f, Y0M = 50.f;
    float deltaW_det[OR_NDET][9];
    memset(deltaW_det, 0, sizeof(deltaW_det));
    char buf[4096];
    int ipl = 0, nelem = 0;
    float z = 0, cellwidth = 0, spacing = 0, xoffset = 0, scalex = 0, x0 = 0, x1 = 0, x2 = 0, costheta = 0, scaley = 0,
          y0 = 0, y1 = 0, y2 = 0, sintheta = 0, resolution = 0, deltaW_ = 0;
    float p1x = 0, p1y = 0, p1z = 0, deltapx = 0, deltapy = 0, deltapz = 0, dp1x = 0, dp1y = 0, dp1z = 0;
    while (fgets(buf, sizeof(buf), f)) {
        if (buf[0] == '#') continue; /* M:129 */
        const char *s = buf;
        /* M:133, field order of the geometry file */
        next_int(&s, &ipl);
        next_float(&s, &z);
        next_int(&s, &nelem);
        next_float(&s, &cellwidth);
        next_float(&s, &spacing);
        next_float(&s, &xoffset);
        next_float(&s, &scalex);
        next_float(&s, &x0);
        next_float(&s, &x1);
        next_float(&s, &x2);
        next_float(&s, &costheta);
        next_float(&s, &scaley);
        next_float(&s, &y0);
        next_float(&s, &y1);
        next_float(&s, &y2);
        next_float(&s, &sintheta);
        next_float(&s, &resolution);
        next_float(&s, &p1x);
        next_float(&s, &p1y);
        next_float(&s, &p1z);
        next_float(&s, &deltapx);
        next_float(&s, &deltapy);
        next_float(&s, &deltapz);
        next_float(&s, &dp1x);
        next_float(&s, &dp1y);
        next_float(&s, &dp1z);
        if (ipl < 0 || ipl >= OR_NDET) continue;
        plane->z[ipl] = z;
        plane->nelem[ipl] = nelem;
        plane->cellwidth[ipl] = cellwidth;
        plane->spacing[ipl] = spacing;
        plane->xoffset[ipl] = xoffset;
        plane->scalex[ipl] = scalex;
        plane->x0[ipl] = x0;
        plane->x1[ipl] = x1;
        plane->x2[ipl] = x2;
        plane->costheta[ipl] = costheta;
        plane->scaley[ipl] = scaley;
        plane->y0[ipl] = y0;
        plane->y1[ipl] = y1;
        plane->y2[ipl] = y2;
        plane->sintheta[ipl] = sintheta;
        plane->resolution[ipl] = resolution; /* USE_DET_RESOL, M:150-151 */
        plane->p1x_w1[ipl] = p1x;
        plane->p1y_w1[ipl] = p1y;
        plane->p1z_w1[ipl] = p1z;
        plane->deltapx[ipl] = deltapx;
        plane->deltapy[ipl] = deltapy;
        plane->deltapz[ipl] = deltapz;
        plane->dp1x[ipl] = dp1x;
        plane->dp1y[ipl] = dp1y;
        plane->dp1z[ipl] = dp1z;
        if (ipl > OR_NCHAM + OR_NHODO) { /* M:164-176 */
            for (int k = 0; k < 9; k++) {
                next_float(&s, &deltaW_);
                deltaW_det[ipl][k] = deltaW_;
            }
        } else {
            next_float(&s, &deltaW_);
            deltaW_det[ipl][0] = deltaW_;
        }
        plane->slope_max[ipl] = costheta * TXM + sintheta * TYM; /* M:177-178 */
        plane->inter_max[ipl] = costheta * X0M + sintheta * Y0M;
        if (ipl % 2 == 0 && ipl > 1) { /* M:179-186 */
            double dslope = (double)((plane->resolution[ipl] + plane->resolution[ipl - 1]) /
                                     (plane->z[ipl] - plane->z[ipl - 1]));
            double dinter = dslope * (double)plane->z[ipl];
            plane->slope_max[ipl] = (float)((double)plane->slope_max[ipl] + dslope);
            plane->inter_max[ipl] = (float)((double)plane->inter_max[ipl] + dinter);
            plane->slope_max[ipl - 1] = (float)((double)plane->slope_max[ipl - 1] + dslope);
            plane->inter_max[ipl - 1] = (float)((double)plane->inter_max[ipl - 1] + dinter);
        }
    }
    fclose(f);
    if (wire_pos) { /* M:191-218 */
        for (int i = 0; i < OR_NDET * 400; i++) wire_pos[i] = 0.0;
        for (int i = 1; i <= OR_NCHAM; ++i) {
            for (int j = 1; j <= plane->nelem[i] && j < 400; ++j) {
                double pos = ((double)j - ((double)plane->nelem[i] + 1.) / 2.) * (double)plane->spacing[i];
                pos = pos + (double)plane->xoffset[i];
                pos = pos + (double)(float)(plane->x0[i] * plane->costheta[i]);
                pos = pos + (double)(float)(plane->y0[i] * plane->sintheta[i]);
                pos = pos + (double)deltaW_det[i][0];
                wire_pos[i * 400 + j] = pos;
            }
        }
        for (int i = OR_NCHAM + 1; i <= OR_NCHAM + OR_NHODO + OR_NPROP; ++i) {
            for (int j = 1; j <= plane->nelem[i] && j < 400; ++j) {
                float f = plane->x0[i] * plane->costheta[i];
                f = f + plane->y0[i] * plane->sintheta[i];
                f = f + plane->xoffset[i];
                double pos = (double)f + ((double)j - (double)(plane->nelem[i] + 1) / 2.) * (double)plane->spacing[i];
                int module = (i > OR_NCHAM + OR_NHODO) ? 8 - (j - 1) / 8 : 0;
                pos = pos + (double)deltaW_det[i][module];
                wire_pos[i * 400 + j] = pos;
            }
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* device helpers restated, H:8-158                                         */
/* ------------------------------------------------------------------------ */
static inline float x_bep(int d, int elid, const or_plane_t *p) { return p->p1x_w1[d] + p->dp1x[d] * (float)(elid - 1); }
static inline float y_bep(int d, int elid, const or_plane_t *p) { return p->p1y_w1[d] + p->dp1y[d] * (float)(elid - 1); }
static inline float z_bep(int d, int elid, const or_plane_t *p) { return p->p1z_w1[d] + p->dp1z[d] * (float)(elid - 1); }
static inline float x_tep(int d, int elid, const or_plane_t *p) { return x_bep(d, elid, p) + p->deltapx[d]; }

/* H:75-100 */
static int calculate_y_uvhit(int d, int elid, float drift, short hitsign, float x0, float tx, const or_plane_t *p,
                             float *y, float *err_y) {
    float p1x = x_bep(d, elid, p);
    float p2x = p1x + p->deltapx[d];
    float x_trk = x0 + p->z[d] * tx;
    if (x_trk - drift > p1x && x_trk - drift > p2x) return 0;
    if (x_trk + drift < p1x && x_trk + drift < p2x) return 0;
    float p1y = y_bep(d, elid, p);
    float yy = p1y + (x_trk - p1x) * p->deltapy[d] / p->deltapx[d];
    if (hitsign != 0) yy += copysignf(1.f, p->sintheta[d]) * 2.f * (drift - 0.5f * (float)hitsign);
    yy = fmaxf(yy, p1y);
    yy = fminf(yy, p1y + p->deltapy[d]);
    *y = yy;
    *err_y = p->resolution[d] * fabsf(p->deltapy[d] / p->deltapx[d]);
    return 1;
}

/* H:140-158 */
static void calculate_xz_fy(int d, int elid, float drift, short hitsign, float y0, float ty, const or_plane_t *p,
                            float *x, float *z) {
    float p1x = x_bep(d, elid, p);
    float p1y = y_bep(d, elid, p);
    float p1z = z_bep(d, elid, p);
    float dpy = p->deltapy[d];
    float dpz = p->deltapz[d];
    float zz = p1z - p1y * dpz / dpy;
    float y_trk = y0 + zz * ty;
    float xx = p1x + (y_trk - p1y) * p->deltapx[d] / dpy;
    zz = p1z + (y_trk - p1y) * dpz / dpy;
    if (hitsign != 0) xx += (float)hitsign * drift;
    *x = xx;
    *z = zz;
}

/* Arithmetic type of the fits, residuals and chi2 sums.  float restates the
 * reference; building with -DORC_FIT_T=double gives the FP64 oracle the
 * FP32 fit errors are measured against (inputs and stored results stay
 * float, as the reference's records are). */
#ifndef ORC_FIT_T
#define ORC_FIT_T float
#endif
typedef ORC_FIT_T fit_t;

/* FT:3-82 (Gauss-Jordan with partial pivoting; operations.h:39-62) */
static void matinv_2x2_t(const fit_t *A, fit_t *Ainv) {
    int perm0 = 0, perm1 = 1, icol0, icol1, i;
    fit_t AA00 = A[0], AA10 = A[1], AA01 = A[2], AA11 = A[3], tmp, t, pp;
    int pvt;
    pp = (fit_t)fabs(AA00);
    pvt = 0;
    t = (fit_t)fabs(AA10);
    if (t > pp) {
        pp = t;
        pvt = 1;
    }
    if (pvt == 1) {
        tmp = AA00; AA00 = AA10; AA10 = tmp;
        tmp = AA01; AA01 = AA11; AA11 = tmp;
        i = perm0; perm0 = perm1; perm1 = i;
    }
    tmp = (fit_t)1.0f / AA00;
    icol0 = perm0;
    AA00 = tmp;
    AA01 = tmp * AA01;
    tmp = AA10;
    AA10 = (-tmp) * AA00;
    AA11 = -(tmp * AA01) + AA11;
    tmp = (fit_t)1.0f / AA11;
    icol1 = perm1;
    AA10 = tmp * AA10;
    AA11 = tmp;
    tmp = AA01;
    AA00 = -(tmp * AA10) + AA00;
    AA01 = (-tmp) * AA11;
    Ainv[0 * 2 + icol0] = AA00;
    Ainv[1 * 2 + icol0] = AA10;
    Ainv[0 * 2 + icol1] = AA01;
    Ainv[1 * 2 + icol1] = AA11;
}

void orc_matinv_2x2(const float *A, float *Ainv) {
    fit_t a[4] = {A[0], A[1], A[2], A[3]}, r[4];
    matinv_2x2_t(a, r);
    for (int k = 0; k < 4; k++) Ainv[k] = (float)r[k];
}

/* AM:32-74; the returned "chi2" of the reference is never read by the hot
 * path (each caller overwrites it), so it is not computed */
void orc_fit_2d(int n, const float *x, const float *z, const float *w, float *par, float *err) {
    fit_t A[4] = {0, 0, 0, 0}, Ainv[4] = {0, 0, 0, 0}, B[2] = {0, 0};
    for (int i = 0; i < n; i++) {
        const fit_t wi = w[i], xi = x[i], zi = z[i];
        B[0] += wi * xi;
        B[1] += wi * xi * zi;
        A[0] += wi;
        A[1] += wi * zi;
        A[2] += wi * zi;
        A[3] += wi * zi * zi;
    }
    matinv_2x2_t(A, Ainv);
    for (int j = 0; j < 2; j++) {
        fit_t pj = 0;
        err[j] = (float)sqrt((double)(fit_t)fabs(Ainv[j * 2 + j]));
        for (int k = 0; k < 2; k++) pj += Ainv[j * 2 + k] * B[k];
        par[j] = (float)pj;
    }
}

/* AM:78-119 */
void orc_fit_2d_drift(int n, const float *x, const float *drift, const short *sign, const float *z, const float *w,
                      float *par, float *err) {
    fit_t A[4] = {0, 0, 0, 0}, Ainv[4] = {0, 0, 0, 0}, B[2] = {0, 0};
    for (int i = 0; i < n; i++) {
        const fit_t wi = w[i], zi = z[i], xd = (fit_t)x[i] + (fit_t)drift[i] * (fit_t)sign[i];
        B[0] += wi * xd;
        B[1] += wi * xd * zi;
        A[0] += wi;
        A[1] += wi * zi;
        A[2] += wi * zi;
        A[3] += wi * zi * zi;
    }
    matinv_2x2_t(A, Ainv);
    for (int j = 0; j < 2; j++) {
        fit_t pj = 0;
        err[j] = (float)sqrt((double)(fit_t)fabs(Ainv[j * 2 + j]));
        for (int k = 0; k < 2; k++) pj += Ainv[j * 2 + k] * B[k];
        par[j] = (float)pj;
    }
}

static inline float position(float pos, float drift, short sign) { return pos + (float)sign * drift; } /* H:40-43 */

/* H:714-780 */
static void resolve_leftright_newhits(float x0, float tx, float y0, float ty, float err_x0, float err_tx, float err_y0,
                                      float err_ty, short nhits, const short *hits_detid, const float *hits_pos,
                                      const float *hits_drift, short *hits_sign, const or_plane_t *p, float thr) {
    for (short n = 0; n < nhits; n += 2) {
        short i = n, j = (short)(i + 1);
        short di = hits_detid[i], dj = hits_detid[j];
        if (abs(di - dj) != 1) {
            n--;
            continue;
        }
        float slope_exp = p->costheta[di] * tx + p->sintheta[di] * ty;
        float err_slope = fabsf(p->costheta[di] * err_tx) + fabsf(p->sintheta[di] * err_ty);
        float inter_exp = p->costheta[di] * x0 + p->sintheta[di] * y0;
        float err_inter = fabsf(p->costheta[di] * err_x0) + fabsf(p->sintheta[di] * err_y0);
        if (hits_sign[i] * hits_sign[j] == 0) {
            int indexmin = -1;
            float pull_min = 1.e6f;
            for (short k = 0; k < 4; k++) {
                float pi = position(hits_pos[i], hits_drift[i], lrpossibility[k][0]);
                float pj = position(hits_pos[j], hits_drift[j], lrpossibility[k][1]);
                float slope_local = (pi - pj) / (p->z[di] - p->z[dj]);
                float inter_local = pi - slope_local * p->z[di];
                if (fabsf(slope_local) > p->slope_max[di] || fabsf(inter_local) > p->inter_max[di]) continue;
                float pull = sqrtf((slope_exp - slope_local) * (slope_exp - slope_local) / err_slope / err_slope +
                                   (inter_exp - inter_local) * (inter_exp - inter_local) / err_inter / err_inter);
                if (pull < pull_min) {
                    indexmin = k;
                    pull_min = pull;
                }
            }
            if (indexmin > 0 && pull_min < thr) {
                hits_sign[i] = lrpossibility[indexmin][0];
                hits_sign[j] = lrpossibility[indexmin][1];
            }
        }
    }
}

/* H:785-804 */
static void resolve_single_leftright_newhits(float x0, float tx, float y0, float ty, short nhits,
                                             const short *hits_detid, const float *hits_pos, short *hits_sign,
                                             const or_plane_t *p) {
    for (short n = 0; n < nhits; n++) {
        if (hits_sign[n]) continue;
        short d = hits_detid[n];
        if (d < 0) continue;
        float pos_exp = (p->z[d] * tx + x0) * p->costheta[d] + (p->z[d] * ty + y0) * p->sintheta[d];
        hits_sign[n] = pos_exp > hits_pos[n] ? 1 : -1;
    }
}

/* H:808-872 */
static void resolve_leftright_xhits(float x0, float tx, float err_x0, float err_tx, short nhits, const short *hits_detid,
                                    const float *hits_pos, const float *hits_drift, short *hits_sign,
                                    const float *zarray, float thr) {
    for (short n = 0; n < nhits; n += 2) {
        short i = n, j = (short)(i + 1);
        short di = hits_detid[i], dj = hits_detid[j];
        if (abs(di - dj) != 1) {
            n--;
            continue;
        }
        float slope_exp = tx, err_slope = err_tx, inter_exp = x0, err_inter = err_x0;
        if (hits_sign[i] * hits_sign[j] == 0) {
            int indexmin = -1;
            float pull_min = 1.e6f;
            for (int k = 0; k < 4; k++) {
                float pi = position(hits_pos[i], hits_drift[i], lrpossibility[k][0]);
                float pj = position(hits_pos[j], hits_drift[j], lrpossibility[k][1]);
                float slope_local = (pi - pj) / (zarray[di] - zarray[dj]);
                float inter_local = pi - slope_local * zarray[di];
                float pull = sqrtf((slope_exp - slope_local) * (slope_exp - slope_local) / err_slope / err_slope +
                                   (inter_exp - inter_local) * (inter_exp - inter_local) / err_inter / err_inter);
                if (pull < pull_min) {
                    indexmin = k;
                    pull_min = pull;
                }
            }
            if (indexmin > 0 && pull_min < thr) {
                hits_sign[i] = lrpossibility[indexmin][0];
                hits_sign[j] = lrpossibility[indexmin][1];
            }
        }
    }
}

/* H:875-892 */
static void resolve_single_leftright_xhits(float x0, float tx, short nhits, const short *hits_detid,
                                           const float *hits_pos, short *hits_sign, const float *z_array) {
    for (short n = 0; n < nhits; n++) {
        if (hits_sign[n]) continue;
        short d = hits_detid[n];
        float pos_exp = z_array[d] * tx + x0;
        hits_sign[n] = pos_exp > hits_pos[n] ? 1 : -1;
    }
}

/* H:1002-1087 (MATCH_Y_HODO undefined) */
static int match_tracklet_to_hodo(int stid, int detid, int nhits, hitcoll_t hits, float x0, float y0, float tx,
                                  float ty, float err_x0, float err_y0, float err_tx, float err_ty,
                                  const or_plane_t *p) {
    if (nhits == 0) return 0;
    if (detid > 40) stid = 3;
    const float fudgefac = hodofudgefac[stid];
    const float cellwidth = p->cellwidth[detid];
    const float xhodo = p->z[detid] * tx + x0;
    const float yhodo = p->z[detid] * ty + y0;
    float err_x = 3.f * (fabsf(p->z[detid] * err_tx) + err_x0);
    float err_y = 3.f * (fabsf(p->z[detid] * err_ty) + err_y0);
    for (int i = 0; i < nhits; i++) {
        float xmin = hc_pos(hits, i) - cellwidth * 0.5f;
        float xmax = hc_pos(hits, i) + cellwidth * 0.5f;
        float ymin = p->y1[detid];
        float ymax = p->y2[detid];
        xmin -= (xmax - xmin) * fudgefac;
        xmax += (xmax - xmin) * fudgefac;
        ymin -= (ymax - ymin) * fudgefac;
        ymax += (ymax - ymin) * fudgefac;
        err_x += (xmax - xmin) * 0.15f;
        xmin -= err_x;
        xmax += err_x;
        ymin -= err_y;
        ymax += err_y;
        if (xmin <= xhodo && xhodo <= xmax && ymin <= yhodo && yhodo <= ymax) return 1;
    }
    return 0;
}

/* H:1090-1144 */
static int match_track_XZ_to_hodo(int stid, int detid, int nhits, hitcoll_t hits, float x0, float tx, float err_x0,
                                  float err_tx, const float *z_array) {
    if (nhits == 0) return 0;
    if (detid > 40) stid = 3;
    const float xhodo = z_array[detid] * tx + x0;
    const float fudgefac = hodofudgefac[stid];
    const float cellwidth = hodoXcellwidth[stid];
    float err_x = 3.f * (fabsf(z_array[detid] * err_tx) + err_x0);
    for (int i = 0; i < nhits; i++) {
        float xmin = hc_pos(hits, i) - cellwidth * 0.5f;
        float xmax = hc_pos(hits, i) + cellwidth * 0.5f;
        xmin -= (xmax - xmin) * fudgefac;
        xmax += (xmax - xmin) * fudgefac;
        err_x += (xmax - xmin) * 0.15f;
        xmin -= err_x;
        xmax += err_x;
        if (xmin <= xhodo && xhodo <= xmax) return 1;
    }
    return 0;
}

/* H:1149-1165 */
static float residual(short d, short elid, float drift, short sign, const or_plane_t *p, float x0_, float y0_,
                      float tx_, float ty_) {
    const fit_t x0 = x0_, y0 = y0_, tx = tx_, ty = ty_;
    const fit_t p1x = x_bep(d, elid, p), p1y = y_bep(d, elid, p), p1z = z_bep(d, elid, p);
    const fit_t deltapx = p->deltapx[d], deltapy = p->deltapy[d], deltapz = p->deltapz[d];
    const fit_t den2 = deltapy * deltapy * (1 + tx * tx) + deltapx * deltapx * (1 + ty * ty) -
                       2 * (ty * deltapx * deltapz + ty * deltapy * deltapz + tx * ty * deltapx * deltapy);
    const fit_t dca = ((ty * deltapz - deltapy) * (p1x - x0) + (deltapx - tx * deltapz) * (p1y - y0) +
                       p1z * (tx * deltapy - ty * deltapx)) /
                      (fit_t)sqrt((double)den2);
    return (float)((fit_t)drift * (fit_t)sign - dca);
}

/* H:1182-1204 */
static float chi2_track(int n, float *residuals, const float *driftdist, const short *sign, const float *resol,
                        const float *p1x, const float *p1y, const float *p1z, const float *dpx, const float *dpy,
                        const float *dpz, float x0, float y0, float tx, float ty) {
    fit_t chi2 = 0;
    const fit_t X0 = x0, Y0 = y0, TX = tx, TY = ty;
    for (int i = 0; i < n; i++) {
        const fit_t px = dpx[i], py = dpy[i], pz = dpz[i];
        const fit_t den2 = py * py * (1 + TX * TX) + px * px * (1 + TY * TY) -
                           2 * (TY * px * pz + TY * py * pz + TX * TY * px * py);
        const fit_t dca = ((TY * pz - py) * ((fit_t)p1x[i] - X0) + (px - TX * pz) * ((fit_t)p1y[i] - Y0) +
                           (fit_t)p1z[i] * (TX * py - TY * px)) /
                          (fit_t)sqrt((double)den2);
        const fit_t r = (fit_t)driftdist[i] * (fit_t)sign[i] - dca;
        residuals[i] = (float)r;
        chi2 += r * r / (fit_t)resol[i] / (fit_t)resol[i];
    }
    return (float)chi2;
}

/* H:556-613 */
static void sagitta_ratio_st1(float x0, float tx, float y0, float ty, int detid_lasthit, float *pos_exp,
                              float *window, const or_plane_t *p) {
    float z_st3 = p->z[detid_lasthit];
    float x_st3 = x0 + tx * z_st3;
    float y_st3 = y0 + ty * z_st3;
    for (int i = 0; i < 3; i++) {
        short detid = (short)(2 * i + 2);
        short idx = planetype[detid / 2 - 1];
        short detid_2 = (short)(detsuperid[2][idx] * 2);
        float pos_st3 = x_st3 * p->costheta[detid_2] + y_st3 * p->sintheta[detid_2];
        float z_st1 = p->z[detid];
        float z_st2 = p->z[detid_2];
        float x_st2 = x0 + tx * z_st2;
        float y_st2 = y0 + ty * z_st2;
        float pos_st2 = x_st2 * p->costheta[detid_2] + y_st2 * p->sintheta[detid_2];
        float s2_target = pos_st2 - pos_st3 * (z_st2 - Z_TARGET) / (z_st3 - Z_TARGET);
        float s2_dump = pos_st2 - pos_st3 * (z_st2 - Z_DUMP) / (z_st3 - Z_DUMP);
        float pos_exp_target = SAGITTA_TARGET_CENTER * s2_target + pos_st3 * (z_st1 - Z_TARGET) / (z_st3 - Z_TARGET);
        float pos_exp_dump = SAGITTA_DUMP_CENTER * s2_dump + pos_st3 * (z_st1 - Z_DUMP) / (z_st3 - Z_DUMP);
        float win_target = fabsf(s2_target * SAGITTA_TARGET_WIDTH);
        float win_dump = fabsf(s2_dump * SAGITTA_DUMP_WIDTH);
        float p_min = fminf(pos_exp_target - win_target, pos_exp_dump - win_dump);
        float p_max = fmaxf(pos_exp_target + win_target, pos_exp_dump + win_dump);
        pos_exp[idx] = (float)(0.5 * (double)(p_max + p_min));
        window[idx] = (float)(0.5 * (double)(p_max - p_min));
    }
}

/* H:684-691 (E1039 branch): the product is formed in double */
static short calculate_charge(float tx, float x0) {
    return (-0.0033f * copysign(1.0, (double)FMAGSTR) * (double)x0 < (double)tx) ? 1 : -1;
}
/* H:652-655 */
static float calculate_invP(float tx, float tx_st1, short charge) {
    return (tx_st1 - tx) * (float)charge / PT_KICK_KMAG;
}
/* H:670-673: err_tx - err_tx, as written */
static float calculate_invP_error(float err_tx, float err_tx_st1) {
    (void)err_tx_st1;
    return (err_tx - err_tx) / PT_KICK_KMAG;
}

/* ------------------------------------------------------------------------ */
/* pairing, H:368-549                                                       */
/* ------------------------------------------------------------------------ */
typedef struct {
    int first, second;
} pair_t;

/* H:464-549.  `pairs` must hold n1*n2+n1+n2 entries. */
static int make_hitpairs_in_station(hitcoll_t h1, int n1, hitcoll_t h2, int n2, pair_t *pairs, int stID, int projID,
                                    const or_plane_t *p, float xmin, float xmax, short *idx1buf, short *idx2buf,
                                    short *flag1, short *flag2, int64_t *dommax) {
    int npairs = 0;
    const int detid1 = detsuperid[stID][projID] * 2;
    const int detid2 = detsuperid[stID][projID] * 2 - 1;
    const int superdetid = detsuperid[stID][projID];
    int c1 = 0, c2 = 0;
    float p1x, p2x;
    for (int i = 0; i < n1; i++) {
        int el = (int)hc_chan(h1, i);
        if (p->deltapx[detid1] > 0) {
            p1x = x_bep(detid1, el, p);
            p2x = x_tep(detid1, el, p);
        } else {
            p1x = x_tep(detid1, el, p);
            p2x = x_bep(detid1, el, p);
        }
        if ((p1x <= xmax) && (p2x >= xmin)) idx1buf[c1++] = (short)i;
    }
    for (int i = 0; i < n2; i++) {
        int el = (int)hc_chan(h2, i);
        if (p->deltapx[detid2] > 0) {
            p1x = x_bep(detid2, el, p);
            p2x = x_tep(detid2, el, p);
        } else {
            p1x = x_tep(detid2, el, p);
            p2x = x_bep(detid2, el, p);
        }
        if ((p1x <= xmax) && (p2x >= xmin)) idx2buf[c2++] = (short)i;
    }
    for (int i = 0; i < c1; i++) flag1[i] = 0;
    for (int i = 0; i < c2; i++) flag2[i] = 0;
    for (int a = 0; a < c1; a++) {
        for (int b = 0; b < c2; b++) {
            if (fabsf(hc_pos(h1, idx1buf[a]) - hc_pos(h2, idx2buf[b])) > spacingplane[superdetid]) continue;
            pairs[npairs].first = idx1buf[a];
            pairs[npairs].second = idx2buf[b];
            npairs++;
            flag1[a] = 1;
            flag2[b] = 1;
        }
    }
    for (int a = 0; a < c1; a++)
        if (flag1[a] < 1) {
            pairs[npairs].first = idx1buf[a];
            pairs[npairs].second = -1;
            npairs++;
        }
    for (int b = 0; b < c2; b++)
        if (flag2[b] < 1) {
            pairs[npairs].first = -1;
            pairs[npairs].second = idx2buf[b];
            npairs++;
        }
    /* the reference's hitidx/hitpairs arrays hold 100 entries (K:890-903, K:1857-1867) */
    if (dommax) {
        int m = c1 > c2 ? c1 : c2;
        if (npairs > m) m = npairs;
        if (m > *dommax) *dommax = m;
    }
    return npairs;
}

/* H:368-460 over all 28 bins at once: pairs[bin][k] for k <= MaxHitsProj_X.
 * Returns 1 when some bin holds more than MaxHitsProj_X entries. */
static int make_hitpairs_in_station_bins(hitcoll_t h1, int n1, hitcoll_t h2, int n2, pair_t pairs[28][MaxHitsProj_X + 1],
                                         int npairs[28], int stID, short *flag1, short *flag2) {
    const int superdetid = detsuperid[stID][0];
    for (int b = 0; b < 28; b++) npairs[b] = 0;
    for (int i = 0; i < n1; i++) flag1[i] = 0;
    for (int i = 0; i < n2; i++) flag2[i] = 0;
    const short *lo = WCHitsBins_X[stID - 2][0], *hi = WCHitsBins_X[stID - 2][1];
    for (int i = 0; i < n1; i++) {
        for (int j = 0; j < n2; j++) {
            if (fabsf(hc_pos(h1, i) - hc_pos(h2, j)) > spacingplane[superdetid]) continue;
            float c = hc_chan(h1, i);
            for (int b = 0; b < 28; b++) {
                if ((float)lo[b] <= c && c <= (float)hi[b]) {
                    if (npairs[b] <= MaxHitsProj_X) {
                        pairs[b][npairs[b]].first = i;
                        pairs[b][npairs[b]].second = j;
                    }
                    npairs[b]++;
                }
            }
            flag1[i] = 1;
            flag2[j] = 1;
        }
    }
    for (int i = 0; i < n1; i++) {
        if (flag1[i] < 1) {
            float c = hc_chan(h1, i);
            for (int b = 0; b < 28; b++)
                if ((float)lo[b] <= c && c <= (float)hi[b]) {
                    if (npairs[b] <= MaxHitsProj_X) {
                        pairs[b][npairs[b]].first = i;
                        pairs[b][npairs[b]].second = -1;
                    }
                    npairs[b]++;
                }
        }
    }
    for (int j = 0; j < n2; j++) {
        if (flag2[j] < 1) {
            float c = hc_chan(h2, j);
            for (int b = 0; b < 28; b++)
                if ((float)lo[b] <= c && c <= (float)hi[b]) {
                    if (npairs[b] <= MaxHitsProj_X) {
                        pairs[b][npairs[b]].first = -1;
                        pairs[b][npairs[b]].second = j;
                    }
                    npairs[b]++;
                }
        }
    }
    int over = 0;
    for (int b = 0; b < 28; b++)
        if (npairs[b] > MaxHitsProj_X) over = 1;
    return over;
}

/* ------------------------------------------------------------------------ */
/* event reducer, H:168-361 and K:8-140                                     */
/* ------------------------------------------------------------------------ */
int orc_reduce_plane(const float *slot, int nhits, int detid, short *hitflag) {
    hitcoll_t h = {slot, nhits};
    int cl[ClusterSizeMax + 8];
    int cls = 0, nred = 0;
    for (int iAH = 0; iAH < nhits; ++iAH) {
        hitflag[iAH] = 1;
        if ((((int)hc_flag(h, iAH)) & 2) == 0) { /* H:198 */
            hitflag[iAH] = -1;
            continue;
        }
        /* H:204-230: uniqueID_curr is reset to -1 for every hit, so the
         * after-pulse branch never runs; nothing to restate. */
        if (detid <= OR_NCHAM) { /* H:234-328 */
            if (cls == 0) {
                cl[0] = iAH;
                ++cls;
            } else {
                if (fabsf(hc_chan(h, iAH) - hc_chan(h, cl[cls - 1])) > 1 || iAH == nhits - 1) {
                    if (iAH == nhits - 1 && fabsf(hc_chan(h, iAH) - hc_chan(h, cl[cls - 1])) <= 1) {
                        cl[cls] = iAH;
                        ++cls;
                    }
                    if (cls == 2) {
                        float w_max = (float)(0.9 * 0.5 * (double)(hc_pos(h, cl[cls - 1]) - hc_pos(h, cl[0])));
                        float w_min = (float)(4.0 / 9.0 * (double)w_max);
                        if ((hc_drift(h, cl[0]) > w_max && hc_drift(h, cl[cls - 1]) > w_min) ||
                            (hc_drift(h, cl[0]) > w_min && hc_drift(h, cl[cls - 1]) > w_max)) {
                            if (hc_drift(h, cl[0]) > hc_drift(h, cl[cls - 1]))
                                hitflag[cl[0]] = -1;
                            else
                                hitflag[cl[cls - 1]] = -1;
                        } else {
                            float dt = hc_tdc(h, cl[0]) - hc_tdc(h, cl[cls - 1]);
                            if ((((double)dt >= 0.0 && (double)dt < 8.0) || ((double)dt <= 0.0 && (double)dt > -8.0)) &&
                                (detid >= 19 && detid <= 24)) {
                                hitflag[cl[0]] = -1;
                                hitflag[cl[cls - 1]] = -1;
                            }
                        }
                    }
                    if (cls >= 3) {
                        float dt_mean = 0.0f;
                        for (int c = 1; c < cls; ++c) {
                            float d = hc_tdc(h, cl[c]) - hc_tdc(h, cl[c - 1]);
                            dt_mean += ((double)d > 0.0 ? d : (hc_tdc(h, cl[c - 1]) - hc_tdc(h, cl[c])));
                        }
                        dt_mean = dt_mean / (float)(cls - 1);
                        if ((double)dt_mean < 10.0) {
                            for (int c = 0; c < cls; ++c) hitflag[cl[c]] = -1;
                        } else {
                            for (int c = 1; c < cls; ++c) hitflag[cl[c]] = -1;
                        }
                    }
                    cls = 0;
                } else {
                    if (cls < ClusterSizeMax + 7) cl[cls] = iAH;
                    ++cls;
                }
            }
        }
    }
    unsigned char chanhashit[202]; /* H:334-349 */
    memset(chanhashit, 0, sizeof(chanhashit));
    for (int iAH = 0; iAH < nhits; ++iAH) {
        if (hitflag[iAH] > 0) {
            short c = (short)hc_chan(h, iAH);
            if (c < 0 || c >= 202) { /* outside the reference's array: keep it, unique */
                ++nred;
                continue;
            }
            if (chanhashit[c]) {
                hitflag[iAH] = -1;
            } else {
                chanhashit[c] = 1;
                ++nred;
            }
        }
    }
    return nred;
}

/* K:59-75: compact the survivors of one plane in place, new stride */
static int reduce_and_compact(float *slot, uint32_t *count, int detid, int cap) {
    int n = (int)*count;
    if (n > cap) n = cap; /* outside the reference's domain; keeps the oracle in bounds */
    short hitflag[OR_MAXHITS_CHAM + 8];
    float copy[OR_NHITSPARAM * OR_MAXHITS_CHAM];
    int nk = orc_reduce_plane(slot, n, detid, hitflag);
    int idx = 0;
    for (int k = 0; k < n; k++) {
        if (hitflag[k] > 0) {
            for (int f = 0; f < OR_NHITSPARAM; f++) copy[idx + nk * f] = slot[n * f + k];
            idx++;
        }
    }
    for (int k = 0; k < OR_NHITSPARAM * nk; k++) slot[k] = copy[k];
    *count = (uint32_t)nk;
    return nk;
}

static void er_event(or_hits_view_t hv, long e, uint8_t *toomany, uint32_t *status) {
    unsigned short mult[5] = {0, 0, 0, 0, 0};
    for (int t = 0; t < 8; t++) {
        int dp = 47 + t; /* K:55-77 */
        float *slot = hv.hits_prop + e * OR_EVT_PROP_FLOATS + (long)OR_NHITSPARAM * OR_MAXHITS_PROP * t;
        int nk = reduce_and_compact(slot, &hv.nhits_prop[e * OR_NPROP + t], dp, OR_MAXHITS_PROP);
        mult[4] = (unsigned short)(mult[4] + nk);
        for (int c = 0; c < 3; c++) { /* K:80-106 */
            int d = eff_detid_chambers[t + 8 * c];
            int stid = d <= 12 ? 0 : (d - 7) / 6;
            float *cs = hv.hits_cham + e * OR_EVT_CHAM_FLOATS + (long)OR_NHITSPARAM * OR_MAXHITS_CHAM * (d - 1);
            nk = reduce_and_compact(cs, &hv.nhits_cham[e * OR_NCHAM + d - 1], d, OR_MAXHITS_CHAM);
            mult[stid] = (unsigned short)(mult[stid] + nk);
        }
        for (int c = 0; c < 2; c++) { /* K:107-125 */
            int hi = t + 8 * c;
            float *hs = hv.hits_hodo + e * OR_EVT_HODO_FLOATS + (long)OR_NHITSPARAM * OR_MAXHITS_HODO * hi;
            reduce_and_compact(hs, &hv.nhits_hodo[e * OR_NHODO + hi], 31 + hi, OR_MAXHITS_HODO);
        }
    }
    /* K:128-139, summing the eight threads' rows only */
    int bad = mult[0] > MaxD0Multiplicity || mult[1] > MaxD2Multiplicity || mult[2] > MaxD3Multiplicity ||
              mult[3] > MaxD3Multiplicity;
    toomany[e] = (uint8_t)bad;
    if (status) status[e] = bad ? ORC_ST_TOOMANY_ER : 0u;
}

/* ------------------------------------------------------------------------ */
/* track-record access                                                      */
/* ------------------------------------------------------------------------ */
static inline float *trk_rec(or_tracks_view_t tv, long e, int slot, int k) {
    return tv.tracks + e * OR_EVT_TRK_FLOATS + (long)slot * OR_SLOTCAP * OR_NTRKPARAM + (long)k * OR_NTRKPARAM;
}

/* ------------------------------------------------------------------------ */
/* XZ tracking, K:182-855                                                   */
/* ------------------------------------------------------------------------ */
typedef struct {
    float rec[OR_NTRKPARAM];
} tkl_t;

typedef struct {
    pair_t bins[3][28][MaxHitsProj_X + 1]; /* st2, st3p, st3m */
    int np[3][28];
    short flag1[OR_MAXHITS_CHAM], flag2[OR_MAXHITS_CHAM];
    tkl_t *tkl[2];
    int ntkl[2], cap[2];
    pair_t *pairbuf;
    short idx1[OR_MAXHITS_CHAM], idx2[OR_MAXHITS_CHAM];
} xz_scratch_t;

static void push_tkl(xz_scratch_t *s, int parity, const float *rec) {
    if (s->ntkl[parity] == s->cap[parity]) {
        s->cap[parity] = s->cap[parity] ? 2 * s->cap[parity] : 64;
        s->tkl[parity] = (tkl_t *)realloc(s->tkl[parity], sizeof(tkl_t) * (size_t)s->cap[parity]);
    }
    memcpy(s->tkl[parity][s->ntkl[parity]].rec, rec, sizeof(float) * OR_NTRKPARAM);
    s->ntkl[parity]++;
}

static void xz_event(const or_plane_t *P, or_hits_view_t hv, or_tracks_view_t tv, long e, int32_t *ntracklets,
                     uint8_t *toomany, uint32_t *status, xz_scratch_t *s, int64_t *cnt) {
    for (int k = 0; k < OR_NSLOTS; k++) tv.ntracks[e * OR_NSLOTS + k] = 0;
    if (toomany[e]) return; /* K:195-200 */
    /* pairs per station over all bins (K:247-288) */
    const int st_of[3] = {2, 3, 4};
    int over = 0;
    hitcoll_t hx[3], hxp[3];
    for (int q = 0; q < 3; q++) {
        int d = detsuperid[st_of[q]][0] * 2;
        hx[q] = hits_chamber(hv, e, d);
        hxp[q] = hits_chamber(hv, e, d - 1);
        over |= make_hitpairs_in_station_bins(hx[q], hx[q].n, hxp[q], hxp[q].n, s->bins[q], s->np[q], st_of[q],
                                              s->flag1, s->flag2);
    }
    if (over) { /* K:359-375 */
        toomany[e] = 1;
        if (status) status[e] |= ORC_ST_TOOMANY_XZBIN;
        ntracklets[e] = 0;
        return;
    }
    /* prop-tube and hodoscope planes (K:306-354) */
    hitcoll_t p1x1 = hits_prop(hv, e, detsuperid[5][0] * 2), p1x2 = hits_prop(hv, e, detsuperid[5][0] * 2 - 1);
    hitcoll_t p2x1 = hits_prop(hv, e, detsuperid[6][0] * 2), p2x2 = hits_prop(hv, e, detsuperid[6][0] * 2 - 1);
    const float z_p1x1 = P->z[detsuperid[5][0] * 2], z_p1x2 = P->z[detsuperid[5][0] * 2 - 1];
    const float z_p2x1 = P->z[detsuperid[6][0] * 2], z_p2x2 = P->z[detsuperid[6][0] * 2 - 1];
    hitcoll_t hod[4][2];
    for (int q = 1; q < 4; q++)
        for (int c = 0; c < 2; c++) hod[q][c] = hits_hodo(hv, e, hodoplanesx[q][c]);

    s->ntkl[0] = s->ntkl[1] = 0;
    float rec[OR_NTRKPARAM];
    for (int t = 0; t < OR_NSLOTS; t++) {
        const int st3 = 3 + t % 2;        /* K:219 */
        const int g2 = (t / 8) * 7;       /* K:217 */
        const int g3 = (t % 8 / 2) * 7;   /* K:218 */
        const int q3 = st3 - 2;
        short detid_list[4];
        detid_list[0] = (short)(detsuperid[2][0] * 2);
        detid_list[1] = (short)(detid_list[0] - 1);
        detid_list[2] = (short)(detsuperid[st3][0] * 2);
        detid_list[3] = (short)(detid_list[2] - 1);
        const float res_l[4] = {P->resolution[detid_list[0]], P->resolution[detid_list[1]],
                                P->resolution[detid_list[2]], P->resolution[detid_list[3]]};
        /* thread-lifetime scratch, K:378-396 (index 4 is never written) */
        short detID[5], elID[5], sign[5];
        float X[5], errX[5], Z[5], drift[5], tdc[5];
        for (int k = 0; k < 5; k++) {
            detID[k] = DET_SENTINEL;
            elID[k] = 0;
            sign[k] = 0;
            X[k] = errX[k] = Z[k] = drift[k] = tdc[k] = 0.f;
        }
        for (short i = 0; i < 49; i++) { /* K:440 */
            short bin2 = (short)(i % 7), bin3 = (short)((i - bin2) / 7);
            int binId = t + OR_NSLOTS * i;
            int nx2 = s->np[0][g2 + bin2], nx3 = s->np[q3][g3 + bin3];
            if (nx2 == 0 || nx3 == 0) continue;
            int ncomb = nx2 * nx3;
            for (short i_x = 0; i_x < ncomb; i_x++) {
                short i_x2 = (short)(i_x % nx2), i_x3 = (short)((i_x - i_x2) / nx2);
                if (cnt) cnt[0]++;
                pair_t p2 = s->bins[0][g2 + bin2][i_x2], p3 = s->bins[q3][g3 + bin3][i_x3];
                short nh = 0;
                const pair_t pp[2] = {p2, p3};
                const hitcoll_t *hc1[2] = {&hx[0], &hx[q3]}, *hc2[2] = {&hxp[0], &hxp[q3]};
                short nhx2 = 0;
                for (int st = 0; st < 2; st++) {
                    for (int w = 0; w < 2; w++) {
                        int hidx = w == 0 ? pp[st].first : pp[st].second;
                        if (hidx < 0) continue;
                        hitcoll_t hh = w == 0 ? *hc1[st] : *hc2[st];
                        detID[nh] = detid_list[2 * st + w];
                        errX[nh] = res_l[2 * st + w];
                        elID[nh] = (short)hc_chan(hh, hidx);
                        tdc[nh] = hc_tdc(hh, hidx);
                        drift[nh] = hc_drift(hh, hidx);
                        sign[nh] = 0;
                        calculate_xz_fy(detID[nh], elID[nh], drift[nh], sign[nh], 0, 0, P, &X[nh], &Z[nh]);
                        nh++;
                    }
                    if (st == 0) {
                        nhx2 = nh;
                        if (nhx2 == 0) break;
                    }
                }
                if (nhx2 == 0 || nh - nhx2 == 0) continue; /* K:510, K:544 */
                float par[2], perr[2];
                orc_fit_2d(nh, X, Z, errX, par, perr); /* K:547-553 */
                float x0 = par[0], tx = par[1], errx0 = perr[0], errtx = perr[1];
                if (fabsf(x0) > X0_MAX + 2 * errx0 || fabsf(tx) > TX_MAX + 2 * errtx) continue;
                resolve_leftright_xhits(x0, tx, errx0, errtx, nh, detID, X, drift, sign, P->z, 150.f);
                resolve_single_leftright_xhits(x0, tx, nh, detID, X, sign, P->z);
                orc_fit_2d_drift(nh, X, drift, sign, Z, errX, par, perr); /* K:558-564 */
                x0 = par[0];
                tx = par[1];
                errx0 = perr[0];
                errtx = perr[1];
                if (fabsf(x0) > X0_MAX || fabsf(tx) > TX_MAX) continue;
                /* prop matching K:577-640 */
                short nprop = 0;
                int checknext = 1;
                for (int n = 0; n < p1x1.n; n++) {
                    float ipos = hc_pos(p1x1, n), xExp = tx * z_p1x1 + x0;
                    if (fabsf(ipos - xExp) < 5.08f) {
                        nprop++;
                        checknext = 0;
                        break;
                    }
                }
                if (checknext) {
                    for (int n = 0; n < p1x2.n; n++) {
                        float ipos = hc_pos(p1x2, n), xExp = tx * z_p1x2 + x0;
                        if (fabsf(ipos - xExp) < 5.08f) {
                            nprop++;
                            break;
                        }
                    }
                }
                checknext = 1;
                for (int n = 0; n < p2x1.n; n++) {
                    float ipos = hc_pos(p2x1, n), xExp = tx * z_p2x1 + x0;
                    if (fabsf(ipos - xExp) < 7.62f) {
                        nprop++;
                        checknext = 0;
                        break;
                    }
                }
                if (checknext) {
                    for (int n = 0; n < p2x2.n; n++) {
                        float ipos = hc_pos(p2x2, n), xExp = tx * z_p2x2 + x0;
                        if (fabsf(ipos - xExp) < 7.62f) {
                            nprop++;
                            break;
                        }
                    }
                }
                if (nprop < NpropXYhitsMin) continue;
                /* hodoscopes K:643-672 */
                int ok = 1;
                for (int q = 1; q < 4 && ok; q++) {
                    int m = match_track_XZ_to_hodo(q, hodoplanesx[q][0], hod[q][0].n, hod[q][0], x0, tx, errx0, errtx,
                                                   P->z);
                    if (!m)
                        m = match_track_XZ_to_hodo(q, hodoplanesx[q][1], hod[q][1].n, hod[q][1], x0, tx, errx0, errtx,
                                                   P->z);
                    ok = m;
                }
                if (!ok) continue;
                /* store, K:788-806 (fields the reference does not write stay zero) */
                memset(rec, 0, sizeof(rec));
                rec[OR_TRK_STID] = (float)binId;
                rec[OR_TRK_THREAD] = (float)t;
                rec[OR_TRK_NHITS] = (float)nh;
                rec[OR_TRK_TX] = tx;
                rec[OR_TRK_X0] = x0;
                rec[OR_TRK_ERR_TX] = errtx;
                rec[OR_TRK_ERR_X0] = errx0;
                for (int n = 0; n < nh; n++) {
                    rec[OR_TRK_HIT_DETID + n] = (float)detID[n];
                    rec[OR_TRK_HIT_CHAN + n] = (float)elID[n];
                    rec[OR_TRK_HIT_POS + n] = X[n];
                    rec[OR_TRK_HIT_DRIFT + n] = drift[n];
                    rec[OR_TRK_HIT_SIGN + n] = (float)sign[n];
                    rec[OR_TRK_HIT_TDC + n] = tdc[n];
                    rec[OR_TRK_HIT_RESID + n] = 0.0f;
                }
                push_tkl(s, t % 2, rec);
            }
        }
    }
    int total = s->ntkl[0] + s->ntkl[1];
    ntracklets[e] = total; /* K:830 */
    if (total >= OR_TRKMAX || s->ntkl[0] > OR_NSLOTS / 2 * OR_SLOTCAP || s->ntkl[1] > OR_NSLOTS / 2 * OR_SLOTCAP) {
        toomany[e] = 1; /* K:719-723, K:824-839 */
        if (status) status[e] |= ORC_ST_TOOMANY_TKL;
        return;
    }
    for (int par = 0; par < 2; par++) {
        for (int k = 0; k < s->ntkl[par]; k++) {
            int slot = 2 * (k % (OR_NSLOTS / 2)) + par;
            int pos = k / (OR_NSLOTS / 2);
            memcpy(trk_rec(tv, e, slot, pos), s->tkl[par][k].rec, sizeof(float) * OR_NTRKPARAM);
            tv.ntracks[e * OR_NSLOTS + slot] = (uint16_t)(pos + 1);
        }
    }
}

/* ------------------------------------------------------------------------ */
/* YZ tracking, K:864-1832                                                  */
/* ------------------------------------------------------------------------ */
typedef struct {
    pair_t *pairs[4];
    short idx1[OR_MAXHITS_CHAM], idx2[OR_MAXHITS_CHAM], flag1[OR_MAXHITS_CHAM], flag2[OR_MAXHITS_CHAM];
} pair_scratch_t;

static pair_t *alloc_pairs(void) {
    return (pair_t *)malloc(sizeof(pair_t) * (size_t)(OR_MAXHITS_CHAM * OR_MAXHITS_CHAM + 2 * OR_MAXHITS_CHAM));
}

/* Analysis hook (orc_yz_outer_dump): one record per (u3, v3) outer iteration
 * that loads a u3 and a v3 hit, with its station-3 hits and whether it held
 * the tracklet's best combination.  Single-threaded use only. */
#define ORC_OUTER_FIELDS 24
static struct {
    float *buf;
    int64_t cap, n;
} g_outer;

static void outer_record(long e, int slot, int i, int i_uv3, int nu3h, int nv3h, const float *Y, const float *eY,
                         const float *Z, int ncomb_uv2, float x0, float tx, int nhits_x) {
    if (!g_outer.buf || g_outer.n >= g_outer.cap) return;
    float *r = g_outer.buf + g_outer.n * ORC_OUTER_FIELDS;
    memset(r, 0, ORC_OUTER_FIELDS * sizeof(float));
    r[0] = (float)e;
    r[1] = (float)slot;
    r[2] = (float)i;
    r[3] = (float)i_uv3;
    r[4] = (float)nu3h;
    r[5] = (float)nv3h;
    for (int k = 0; k < nu3h + nv3h && k < 4; k++) {
        r[6 + k] = Y[k];
        r[10 + k] = eY[k];
        r[14 + k] = Z[k];
    }
    r[18] = (float)ncomb_uv2;
    r[19] = x0;
    r[20] = tx;
    r[22] = (float)nhits_x;
    g_outer.n++;
}

static void yz_event(const or_plane_t *P, or_hits_view_t hv, or_tracks_view_t tv, long e, const uint8_t *toomany,
                     pair_scratch_t *ps, int64_t *cnt) {
    if (toomany[e]) return; /* K:873-878 */
    for (int slot = 0; slot < OR_NSLOTS; slot++) {
        const int st3 = 3 + slot % 2; /* K:884 */
        short detid_list[8];
        float det_spacing[8];
        hitcoll_t hc[8];
        float zl[8];
        /* K:910-984: u2 u2' v2 v2' u3 u3' v3 v3' */
        const int stids[4] = {2, 2, st3, st3}, projs[4] = {1, 2, 1, 2};
        for (int q = 0; q < 4; q++) {
            int d = detsuperid[stids[q]][projs[q]] * 2;
            detid_list[2 * q] = (short)d;
            detid_list[2 * q + 1] = (short)(d - 1);
        }
        for (int k = 0; k < 8; k++) {
            det_spacing[k] = P->spacing[detid_list[k]];
            hc[k] = hits_chamber(hv, e, detid_list[k]);
            zl[k] = P->z[detid_list[k]];
        }
        /* K:986-1013 */
        hitcoll_t p1y1 = hits_prop(hv, e, detsuperid[5][1] * 2), p1y2 = hits_prop(hv, e, detsuperid[5][1] * 2 - 1);
        hitcoll_t p2y1 = hits_prop(hv, e, detsuperid[6][1] * 2), p2y2 = hits_prop(hv, e, detsuperid[6][1] * 2 - 1);
        const float z_p1y1 = P->z[detsuperid[5][1] * 2], z_p1y2 = P->z[detsuperid[5][1] * 2 - 1];
        const float z_p2y1 = P->z[detsuperid[6][1] * 2], z_p2y2 = P->z[detsuperid[6][1] * 2 - 1];
        hitcoll_t hod[4][2];
        for (int q = 1; q < 4; q++)
            for (int c = 0; c < 2; c++) hod[q][c] = hits_hodo(hv, e, hodoplanesx[q][c]);

        /* slot-lifetime scratch, K:1142-1196 (index 8 stands for the memory
         * just past the arrays and is never written) */
        short detID[9], elID[9], sign[9];
        float Y[9], errY[9], Z[9], pos[9], drift[9], tdc[9];
        float dd[12], res[12], p1x[12], p1y[12], p1z[12], dpx[12], dpy[12], dpz[12], residuals[12];
        short hs[12];
        float best[OR_NTRKPARAM];
        for (int k = 0; k < 9; k++) {
            detID[k] = DET_SENTINEL;
            elID[k] = sign[k] = 0;
            Y[k] = errY[k] = Z[k] = pos[k] = drift[k] = tdc[k] = 0.f;
        }
        memset(dd, 0, sizeof(dd));
        memset(res, 0, sizeof(res));
        memset(p1x, 0, sizeof(p1x));
        memset(p1y, 0, sizeof(p1y));
        memset(p1z, 0, sizeof(p1z));
        memset(dpx, 0, sizeof(dpx));
        memset(dpy, 0, sizeof(dpy));
        memset(dpz, 0, sizeof(dpz));
        memset(residuals, 0, sizeof(residuals));
        memset(hs, 0, sizeof(hs));
        memset(best, 0, sizeof(best));

        int ntr = tv.ntracks[e * OR_NSLOTS + slot];
        for (int i = 0; i < ntr; i++) {
            float *T = trk_rec(tv, e, slot, i);
            float x0 = T[OR_TRK_X0], tx = T[OR_TRK_TX], err_x0 = T[OR_TRK_ERR_X0], err_tx = T[OR_TRK_ERR_TX];
            int nhits_x = (int)T[OR_TRK_NHITS];
            int update_track = 0;
            float chi2min = 10000.1f;
            int npair[4];
            for (int q = 0; q < 4; q++) { /* K:1252-1283 */
                int a = 2 * q;
                float xmin = fminf((tx - err_tx) * zl[a], (tx - err_tx) * zl[a + 1]) + x0 - err_x0 - det_spacing[a];
                float xmax = fmaxf((tx + err_tx) * zl[a], (tx + err_tx) * zl[a + 1]) + x0 + err_x0 + det_spacing[a];
                npair[q] = make_hitpairs_in_station(hc[a], hc[a].n, hc[a + 1], hc[a + 1].n, ps->pairs[q], stids[q],
                                                    projs[q], P, xmin, xmax, ps->idx1, ps->idx2, ps->flag1, ps->flag2,
                                                    cnt ? cnt + 6 : NULL);
            }
            const int nu2 = npair[0], nv2 = npair[1], nu3 = npair[2], nv3 = npair[3];
            T[OR_TRK_STID] = 3.f; /* K:1285 */
            if (nu2 == 0 || nu3 == 0) continue;
            if (nv2 == 0 || nv3 == 0) continue;
            for (int m = 0; m < nhits_x; m++) { /* K:1300-1316 */
                short detid = (short)T[OR_TRK_HIT_DETID + m];
                short chan = (short)T[OR_TRK_HIT_CHAN + m];
                dd[m] = T[OR_TRK_HIT_DRIFT + m];
                hs[m] = (short)T[OR_TRK_HIT_SIGN + m];
                res[m] = P->resolution[detid];
                p1x[m] = x_bep(detid, chan, P);
                p1y[m] = y_bep(detid, chan, P);
                p1z[m] = z_bep(detid, chan, P);
                dpx[m] = P->deltapx[detid];
                dpy[m] = P->deltapy[detid];
                dpz[m] = P->deltapz[detid];
            }
            const int ncomb_uv3 = nu3 * nv3, ncomb_uv2 = nu2 * nv2;
            int best_uv3 = -1;
            const int64_t outer0 = g_outer.n;
            /* one uv hit load, K:1326-1355 */
#define YZ_LOAD(LISTK, HIDX)                                                                                     \
    do {                                                                                                         \
        int hidx_ = (HIDX);                                                                                      \
        hitcoll_t hh_ = hc[LISTK];                                                                               \
        detID[nuv] = detid_list[LISTK];                                                                          \
        Z[nuv] = zl[LISTK];                                                                                      \
        elID[nuv] = (short)hc_chan(hh_, hidx_);                                                                  \
        tdc[nuv] = hc_tdc(hh_, hidx_);                                                                           \
        sign[nuv] = 0;                                                                                           \
        drift[nuv] = hc_drift(hh_, hidx_);                                                                       \
        pos[nuv] = hc_pos(hh_, hidx_);                                                                           \
        float y_, err_y_;                                                                                        \
        if (calculate_y_uvhit(detID[nuv], elID[nuv], drift[nuv], 0, x0, tx, P, &y_, &err_y_)) {                 \
            res[nhits_x + nuv] = P->resolution[detID[nuv]];                                                      \
            dd[nhits_x + nuv] = drift[nuv];                                                                      \
            hs[nhits_x + nuv] = sign[nuv];                                                                       \
            p1x[nhits_x + nuv] = x_bep(detID[nuv], elID[nuv], P);                                                \
            p1y[nhits_x + nuv] = y_bep(detID[nuv], elID[nuv], P);                                                \
            p1z[nhits_x + nuv] = z_bep(detID[nuv], elID[nuv], P);                                                \
            dpx[nhits_x + nuv] = P->deltapx[detID[nuv]];                                                         \
            dpy[nhits_x + nuv] = P->deltapy[detID[nuv]];                                                         \
            dpz[nhits_x + nuv] = P->deltapz[detID[nuv]];                                                         \
            Y[nuv] = y_;                                                                                         \
            errY[nuv] = err_y_;                                                                                  \
            nuv++;                                                                                               \
        }                                                                                                        \
    } while (0)
            for (int i_uv3 = 0; i_uv3 < ncomb_uv3; i_uv3++) {
                short i_u3 = (short)(i_uv3 % nu3), i_v3 = (short)((i_uv3 - i_u3) / nu3);
                short nuv = 0;
                pair_t pu3 = ps->pairs[2][i_u3], pv3 = ps->pairs[3][i_v3];
                if (pu3.first >= 0) YZ_LOAD(4, pu3.first);
                if (pu3.second >= 0) YZ_LOAD(5, pu3.second);
                short nhits_u3 = nuv;
                if (nhits_u3 == 0) continue;
                if (pv3.first >= 0) YZ_LOAD(6, pv3.first);
                if (pv3.second >= 0) YZ_LOAD(7, pv3.second);
                short nhits_v3 = (short)(nuv - nhits_u3);
                if (nhits_v3 == 0) continue;
                outer_record(e, slot, i, i_uv3, nhits_u3, nhits_v3, Y, errY, Z, ncomb_uv2, x0, tx, nhits_x);
                for (int i_uv2 = 0; i_uv2 < ncomb_uv2; i_uv2++) {
                    short i_u2 = (short)(i_uv2 % nu2), i_v2 = (short)((i_uv2 - i_u2) / nu2);
                    if (cnt) cnt[1]++;
                    nuv = (short)(nhits_u3 + nhits_v3);
                    pair_t pu2 = ps->pairs[0][i_u2], pv2 = ps->pairs[1][i_v2];
                    if (pu2.first >= 0) YZ_LOAD(0, pu2.first);
                    if (pu2.second >= 0) YZ_LOAD(1, pu2.second);
                    short nhits_u2 = (short)(nuv - nhits_u3 - nhits_v3);
                    if (nhits_u2 == 0) continue;
                    if (pv2.first >= 0) YZ_LOAD(2, pv2.first);
                    if (pv2.second >= 0) YZ_LOAD(3, pv2.second);
                    short nhits_v2 = (short)(nuv - nhits_u3 - nhits_v3 - nhits_u2);
                    if (nhits_v2 == 0) continue;
                    float par[2], perr[2];
                    orc_fit_2d(nuv, Y, Z, errY, par, perr); /* K:1602-1611 */
                    float y0 = par[0], ty = par[1], err_y0 = perr[0], err_ty = perr[1];
                    if (cnt) cnt[3]++;
                    if (fabsf(y0) > Y0_MAX + 2 * err_y0 || fabsf(ty) > TY_MAX + 2 * err_ty) continue;
                    if (cnt) cnt[4]++;
                    resolve_leftright_newhits(x0, tx, y0, ty, err_x0, err_tx, err_y0, err_ty, nuv, detID, pos, drift,
                                              sign, P, 150.f);
                    resolve_single_leftright_newhits(x0, tx, y0, ty, nuv, detID, pos, sign, P);
                    for (int ll = 0; ll < nuv; ll++) hs[nhits_x + ll] = sign[ll];
                    orc_fit_2d(nuv, Y, Z, errY, par, perr); /* K:1628-1638 */
                    y0 = par[0];
                    ty = par[1];
                    err_y0 = perr[0];
                    err_ty = perr[1];
                    if (fabsf(y0) > Y0_MAX || fabsf(ty) > TY_MAX) continue;
                    /* PROP_Y_MATCH, K:1640-1701 */
                    short nprop = 0;
                    int checknext = 1;
                    for (int n = 0; n < p1y1.n; n++) {
                        float ipos = hc_pos(p1y1, n), yExp = ty * z_p1y1 + y0;
                        if (fabsf(ipos - yExp) < 5.08f) {
                            nprop++;
                            checknext = 0;
                            break;
                        }
                    }
                    if (checknext) {
                        for (int n = 0; n < p1y2.n; n++) {
                            float ipos = hc_pos(p1y2, n), yExp = ty * z_p1y2 + y0;
                            if (fabsf(ipos - yExp) < 5.08f) {
                                nprop++;
                                break;
                            }
                        }
                    }
                    checknext = 1;
                    for (int n = 0; n < p2y1.n; n++) {
                        float ipos = hc_pos(p2y1, n), yExp = ty * z_p2y1 + y0;
                        if (fabsf(ipos - yExp) < 10.16f) {
                            nprop++;
                            checknext = 0;
                            break;
                        }
                    }
                    if (checknext) {
                        for (int n = 0; n < p2y2.n; n++) {
                            float ipos = hc_pos(p2y2, n), yExp = ty * z_p2y2 + y0;
                            if (fabsf(ipos - yExp) < 10.16f) {
                                nprop++;
                                break;
                            }
                        }
                    }
                    if (nprop < NpropXYhitsMin) continue;
                    /* hodoscopes, K:1708-1769 */
                    int ok = 1;
                    for (int q = 1; q < 4 && ok; q++) {
                        int m = match_tracklet_to_hodo(q, hodoplanesx[q][0], hod[q][0].n, hod[q][0], x0, y0, tx, ty,
                                                       err_x0, err_y0, err_tx, err_ty, P);
                        if (!m)
                            m = match_tracklet_to_hodo(q, hodoplanesx[q][1], hod[q][1].n, hod[q][1], x0, y0, tx, ty,
                                                       err_x0, err_y0, err_tx, err_ty, P);
                        ok = m;
                    }
                    if (!ok) continue;
                    if (cnt) cnt[5]++;
                    float chi2 = chi2_track(nhits_x + nuv, residuals, dd, hs, res, p1x, p1y, p1z, dpx, dpy, dpz, x0,
                                            y0, tx, ty); /* K:1773 */
                    if (chi2 < chi2min) {              /* K:1778-1799 */
                        chi2min = chi2;
                        update_track = 1;
                        best_uv3 = i_uv3;
                        best[2] = nuv;
                        best[3] = chi2;
                        best[6] = ty;
                        best[8] = y0;
                        best[11] = err_ty;
                        best[13] = err_y0;
                        for (int n = 0; n < nuv; n++) {
                            best[16 + n] = detID[n];
                            best[34 + n] = elID[n];
                            best[52 + n] = pos[n];
                            best[70 + n] = drift[n];
                            best[88 + n] = sign[n];
                            best[106 + n] = tdc[n];
                            if (n < nhits_x) best[124 + n] = residuals[n];
                            best[128 + n] = residuals[nhits_x + n];
                        }
                    }
                }
            }
#undef YZ_LOAD
            if (g_outer.buf && update_track)
                for (int64_t q = outer0; q < g_outer.n; q++)
                    if ((int)g_outer.buf[q * ORC_OUTER_FIELDS + 3] == best_uv3) g_outer.buf[q * ORC_OUTER_FIELDS + 21] = 1.f;
            if (update_track) { /* K:1804-1825 */
                T[OR_TRK_STID] = 5.f;
                nhits_x = (int)T[OR_TRK_NHITS];
                int nuv = (int)best[2];
                T[OR_TRK_NHITS] = (float)nhits_x + best[2];
                T[OR_TRK_CHI2] = best[3];
                T[OR_TRK_TY] = best[6];
                T[OR_TRK_Y0] = best[8];
                T[OR_TRK_ERR_TY] = best[11];
                T[OR_TRK_ERR_Y0] = best[13];
                for (int n = 0; n < nuv; n++) {
                    T[OR_TRK_HIT_DETID + nhits_x + n] = best[16 + n];
                    T[OR_TRK_HIT_CHAN + nhits_x + n] = best[34 + n];
                    T[OR_TRK_HIT_POS + nhits_x + n] = best[52 + n];
                    T[OR_TRK_HIT_DRIFT + nhits_x + n] = best[70 + n];
                    T[OR_TRK_HIT_SIGN + nhits_x + n] = best[88 + n];
                    T[OR_TRK_HIT_TDC + nhits_x + n] = best[106 + n];
                    if (n < nhits_x) T[OR_TRK_HIT_RESID + n] = best[124 + n];
                    T[OR_TRK_HIT_RESID + nhits_x + n] = best[128 + n];
                }
            }
        }
    }
}

/* ------------------------------------------------------------------------ */
/* back-track cleaning, H:1789-1909                                         */
/* ------------------------------------------------------------------------ */
static int common_hits(const float *A, short na, const float *B, short nb, int acc) {
    for (short ih = 0; ih < na; ih++) {
        for (short jh = 0; jh < nb; jh++) {
            if (B[OR_TRK_HIT_DETID + jh] == A[OR_TRK_HIT_DETID + ih] &&
                B[OR_TRK_HIT_CHAN + jh] == A[OR_TRK_HIT_CHAN + ih]) {
                acc++;
                break;
            }
        }
    }
    return acc;
}

static void clean_event(or_tracks_view_t tv, long e, const uint8_t *toomany) {
    if (toomany[e]) return;
    /* H:1789-1843, each slot on its own */
    for (int s = 0; s < OR_NSLOTS; s++) {
        int n = tv.ntracks[e * OR_NSLOTS + s];
        for (int i = 0; i < n; i++) {
            float *Ti = trk_rec(tv, e, s, i);
            if (Ti[OR_TRK_STID] < 5) continue;
            short ni = (short)Ti[OR_TRK_NHITS];
            int nc = 0;
            for (int j = i + 1; j < n; j++) {
                float *Tj = trk_rec(tv, e, s, j);
                if (Tj[OR_TRK_STID] < 5) continue;
                short nj = (short)Tj[OR_TRK_NHITS];
                nc = common_hits(Ti, ni, Tj, nj, nc);
                if (Ti[OR_TRK_CHI2] / (float)(ni - 4) < Tj[OR_TRK_CHI2] / (float)(nj - 4)) {
                    if ((float)nc > (float)ni * 0.3333f) Tj[OR_TRK_STID] = 3.f;
                } else {
                    if ((float)nc > (float)nj * 0.3333f) Ti[OR_TRK_STID] = 3.f;
                }
            }
        }
    }
}

static void clean_cross_event(or_tracks_view_t tv, long e, const uint8_t *toomany) {
    if (toomany[e]) return;
    /* H:1846-1909.  The reference block's 32 threads (one slot each) run this
     * loop together: at each step (i_trd, i, j) every thread whose slot is
     * not i_trd compares its track i with track j of slot i_trd, reading the
     * stationIDs left by the steps before, and the demotions of the step
     * (stationID = 3, H:1895-1903) land together after it.  The threads are
     * emulated in that lockstep order. */
    int nt[OR_NSLOTS], maxn = 0;
    for (int t = 0; t < OR_NSLOTS; t++) {
        nt[t] = tv.ntracks[e * OR_NSLOTS + t];
        if (nt[t] > maxn) maxn = nt[t];
    }
    for (int u = 0; u < OR_NSLOTS; u++) { /* i_trd */
        const int m = nt[u];
        for (int i = 0; i < maxn; i++) {
            int act[OR_NSLOTS], nc[OR_NSLOTS];
            short ni[OR_NSLOTS];
            for (int t = 0; t < OR_NSLOTS; t++) {
                act[t] = t != u && i < nt[t] && trk_rec(tv, e, t, i)[OR_TRK_STID] >= 5;
                ni[t] = act[t] ? (short)trk_rec(tv, e, t, i)[OR_TRK_NHITS] : 0;
                nc[t] = 0;
            }
            for (int j = 0; j < m; j++) {
                float *Tj = trk_rec(tv, e, u, j);
                if (Tj[OR_TRK_STID] < 5) continue;
                const short nj = (short)Tj[OR_TRK_NHITS];
                int demote_j = 0, demote_i[OR_NSLOTS];
                for (int t = 0; t < OR_NSLOTS; t++) {
                    demote_i[t] = 0;
                    if (!act[t]) continue;
                    const float *Ti = trk_rec(tv, e, t, i);
                    nc[t] = common_hits(Ti, ni[t], Tj, nj, nc[t]);
                    if (Ti[OR_TRK_CHI2] / (float)(ni[t] - 4) < Tj[OR_TRK_CHI2] / (float)(nj - 4)) {
                        if ((float)nc[t] > (float)ni[t] * 0.3333f) demote_j = 1;
                    } else {
                        if ((float)nc[t] > (float)nj * 0.3333f) demote_i[t] = 1;
                    }
                }
                if (demote_j) Tj[OR_TRK_STID] = 3.f;
                for (int t = 0; t < OR_NSLOTS; t++)
                    if (demote_i[t]) trk_rec(tv, e, t, i)[OR_TRK_STID] = 3.f;
            }
        }
    }
}

/* ------------------------------------------------------------------------ */
/* global tracking across KMag, K:1841-2534                                 */
/* ------------------------------------------------------------------------ */
static void global_event(const or_plane_t *P, or_hits_view_t hv, or_tracks_view_t tv, long e, const uint8_t *toomany,
                         pair_scratch_t *ps, int64_t *cnt) {
    if (toomany[e]) return;
    /* station-1 planes, K:1880-1923 */
    short detid_list[6];
    hitcoll_t hc[6];
    float zl[6], resl[6];
    for (int q = 0; q < 3; q++) {
        int d = detsuperid[0][q] * 2;
        detid_list[2 * q] = eff_detid_chambers[d - 1];
        detid_list[2 * q + 1] = eff_detid_chambers[d - 2];
        hc[2 * q] = hits_chamber(hv, e, eff_detid_chambers[d - 1]);
        hc[2 * q + 1] = hits_chamber(hv, e, eff_detid_chambers[d - 2]);
        zl[2 * q] = P->z[d];
        zl[2 * q + 1] = P->z[d - 1];
        resl[2 * q] = P->resolution[d];
        resl[2 * q + 1] = P->resolution[d - 1];
    }
    for (int slot = 0; slot < OR_NSLOTS; slot++) {
        /* slot-lifetime scratch, K:1993-2035 (index 18 is never written) */
        short detID[19], elID[19], sign[19];
        float pos[19], drift[19], tdc[19], Y[19], errY[19], Z_[19];
        float X[3], errX[3], Z[3];
        float res[19], p1x[19], p1y[19], p1z[19], dpx[19], dpy[19], dpz[19], residuals[19];
        short detid_st23[12], chan_st23[12], sign_st23[12];
        float drift_st23[12], residuals_st23[12], resolution_st23[12];
        float best[OR_NTRKPARAM];
        for (int k = 0; k < 19; k++) {
            detID[k] = DET_SENTINEL;
            elID[k] = sign[k] = 0;
            pos[k] = drift[k] = tdc[k] = Y[k] = errY[k] = Z_[k] = 0.f;
            res[k] = p1x[k] = p1y[k] = p1z[k] = dpx[k] = dpy[k] = dpz[k] = residuals[k] = 0.f;
        }
        for (int k = 0; k < 3; k++) X[k] = errX[k] = Z[k] = 0.f;
        memset(best, 0, sizeof(best));
        memset(detid_st23, 0, sizeof(detid_st23));
        memset(chan_st23, 0, sizeof(chan_st23));
        memset(sign_st23, 0, sizeof(sign_st23));
        memset(drift_st23, 0, sizeof(drift_st23));
        memset(residuals_st23, 0, sizeof(residuals_st23));
        memset(resolution_st23, 0, sizeof(resolution_st23));

        int ntr = tv.ntracks[e * OR_NSLOTS + slot];
        for (int i = 0; i < ntr; i++) {
            float *T = trk_rec(tv, e, slot, i);
            int update_track = 0;
            short nhits_st23 = (short)T[OR_TRK_NHITS];
            if (T[OR_TRK_STID] < 5) continue; /* K:2053 */
            float chi2min = 10000.1f;
            float x0 = T[OR_TRK_X0], tx = T[OR_TRK_TX], errx0 = T[OR_TRK_ERR_X0], errtx = T[OR_TRK_ERR_TX];
            float y0 = T[OR_TRK_Y0], ty = T[OR_TRK_TY], erry0 = T[OR_TRK_ERR_Y0], errty = T[OR_TRK_ERR_TY];
            /* get_lasthitdetid, reconstruction_classes.cuh:500-515 */
            short detid_max = 1;
            float z_max = -10000.f;
            for (short h = 0; h < nhits_st23; h++) {
                short d = (short)T[OR_TRK_HIT_DETID + h];
                if (d > 0 && P->z[d] > z_max) {
                    detid_max = d;
                    z_max = P->z[d];
                }
            }
            float pos_exp[3], window[3];
            sagitta_ratio_st1(x0, tx, y0, ty, detid_max, pos_exp, window, P); /* K:2066 */
            int np[3];
            for (int q = 0; q < 3; q++) /* K:2068-2075 */
                np[q] = make_hitpairs_in_station(hc[2 * q], hc[2 * q].n, hc[2 * q + 1], hc[2 * q + 1].n, ps->pairs[q],
                                                 0, q, P, pos_exp[q] - window[q] * 1.0f,
                                                 pos_exp[q] + window[q] * 1.0f, ps->idx1, ps->idx2, ps->flag1,
                                                 ps->flag2, cnt ? cnt + 7 : NULL);
            const int nx1 = np[0], nu1 = np[1], nv1 = np[2];
            if (nx1 == 0 || nu1 == 0 || nv1 == 0) continue;
            short nyhits = 0; /* K:2086-2102 */
            for (int k = 0; k < nhits_st23; k++) {
                detid_st23[k] = (short)T[OR_TRK_HIT_DETID + k];
                chan_st23[k] = (short)T[OR_TRK_HIT_CHAN + k];
                drift_st23[k] = T[OR_TRK_HIT_DRIFT + k];
                sign_st23[k] = (short)T[OR_TRK_HIT_SIGN + k];
                resolution_st23[k] = P->resolution[(short)T[OR_TRK_HIT_DETID + k]];
                if ((double)P->costheta[(short)T[OR_TRK_HIT_DETID + k]] > 0.99) continue;
                float y, err_y;
                if (calculate_y_uvhit((int)T[OR_TRK_HIT_DETID + k], (int)T[OR_TRK_HIT_CHAN + k],
                                      T[OR_TRK_HIT_DRIFT + k], (short)T[OR_TRK_HIT_SIGN + k], x0, tx, P, &y,
                                      &err_y)) {
                    Y[nyhits] = y;
                    errY[nyhits] = err_y;
                    Z_[nyhits] = P->z[(short)T[OR_TRK_HIT_DETID + k]];
                    nyhits++;
                }
            }
            const int ncomb_uv = nu1 * nv1;
            for (int i_x = 0; i_x < nx1; i_x++) { /* K:2107 */
                int nhits_x = 0;
                pair_t px = ps->pairs[0][i_x];
                for (int w = 0; w < 2; w++) {
                    int hidx = w == 0 ? px.first : px.second;
                    if (hidx < 0) continue;
                    hitcoll_t hh = hc[w];
                    detID[nhits_x] = detid_list[w];
                    pos[nhits_x] = hc_pos(hh, hidx);
                    errX[nhits_x] = resl[w];
                    elID[nhits_x] = (short)hc_chan(hh, hidx);
                    tdc[nhits_x] = hc_tdc(hh, hidx);
                    sign[nhits_x] = 0;
                    drift[nhits_x] = hc_drift(hh, hidx);
                    calculate_xz_fy(detID[nhits_x], elID[nhits_x], drift[nhits_x], sign[nhits_x], y0, ty, P,
                                    &X[nhits_x], &Z[nhits_x]);
                    res[nhits_x] = P->resolution[detID[nhits_x]];
                    p1x[nhits_x] = x_bep(detID[nhits_x], elID[nhits_x], P);
                    p1y[nhits_x] = y_bep(detID[nhits_x], elID[nhits_x], P);
                    p1z[nhits_x] = z_bep(detID[nhits_x], elID[nhits_x], P);
                    dpx[nhits_x] = P->deltapx[detID[nhits_x]];
                    dpy[nhits_x] = P->deltapy[detID[nhits_x]];
                    dpz[nhits_x] = P->deltapz[detID[nhits_x]];
                    nhits_x++;
                }
                if (nhits_x == 0) continue;
                X[nhits_x] = x0 + tx * Z_KMAG_BEND; /* K:2163-2165 */
                errX[nhits_x] = errx0 + errtx * Z_KMAG_BEND;
                Z[nhits_x] = Z_KMAG_BEND;
                float par[2], perr[2];
                orc_fit_2d(nhits_x + 1, X, Z, errX, par, perr);
                float x0_st1 = par[0], tx_st1 = par[1];
                float errx0_st1 = par[0], errtx_st1 = par[1]; /* K:2175-2176 as written */
                resolve_leftright_xhits(x0_st1, tx_st1, errx0_st1, errtx_st1, (short)nhits_x, detID, X, drift, sign,
                                        P->z, 150.f);
                resolve_single_leftright_xhits(x0_st1, tx_st1, (short)nhits_x, detID, X, sign, P->z);
                for (short l = 0; l < nhits_x; l++) X[l] += (float)sign[l] * drift[l];
                orc_fit_2d(nhits_x + 1, X, Z, errX, par, perr);
                x0_st1 = par[0];
                tx_st1 = par[1];
                errx0_st1 = par[0];
                errtx_st1 = par[1];
                short charge = calculate_charge(tx, x0); /* K:2198-2203 */
                float invP = calculate_invP(tx, tx_st1, charge);
                float errinvP = calculate_invP_error(errtx, errtx_st1);
                if (invP > INVP_MAX + errinvP || invP < INVP_MIN - errinvP) continue;
                for (int i_uv = 0; i_uv < ncomb_uv; i_uv++) { /* K:2216 */
                    int i_u = i_uv % nu1, i_v = (i_uv - i_u) / nu1;
                    if (cnt) cnt[2]++;
                    int nuv = 0;
                    pair_t pu = ps->pairs[1][i_u], pv = ps->pairs[2][i_v];
                    int nhits_u = 0;
                    for (int w = 0; w < 4; w++) {
                        pair_t pp = w < 2 ? pu : pv;
                        int hidx = (w % 2 == 0) ? pp.first : pp.second;
                        if (w == 2) {
                            nhits_u = nuv;
                            if (nhits_u == 0) break;
                        }
                        if (hidx < 0) continue;
                        int lk = 2 + w;
                        hitcoll_t hh = hc[lk];
                        int a = nhits_x + nuv;
                        detID[a] = detid_list[lk];
                        elID[a] = (short)hc_chan(hh, hidx);
                        tdc[a] = hc_tdc(hh, hidx);
                        sign[a] = 0;
                        drift[a] = hc_drift(hh, hidx);
                        pos[a] = hc_pos(hh, hidx);
                        float y, err_y;
                        if (calculate_y_uvhit(detID[a], elID[a], drift[a], 0, x0_st1, tx_st1, P, &y, &err_y)) {
                            res[a] = P->resolution[detID[a]];
                            p1x[a] = x_bep(detID[a], elID[a], P);
                            p1y[a] = y_bep(detID[a], elID[a], P);
                            p1z[a] = z_bep(detID[a], elID[a], P);
                            dpx[a] = P->deltapx[detID[a]];
                            dpy[a] = P->deltapy[detID[a]];
                            dpz[a] = P->deltapz[detID[a]];
                            Y[nyhits + nuv] = y;
                            errY[nyhits + nuv] = err_y;
                            Z_[nyhits + nuv] = zl[lk];
                            nuv++;
                        }
                    }
                    if (nhits_u == 0) continue; /* K:2292 */
                    int nhits_v = nuv - nhits_u;
                    if (nhits_v == 0) continue; /* K:2366 */
                    orc_fit_2d(nyhits + nuv, Y, Z_, errY, par, perr); /* K:2368-2379 */
                    y0 = par[0];
                    ty = par[1];
                    erry0 = perr[0];
                    errty = perr[1];
                    if (fabsf(y0) > Y0_MAX + 2 * erry0 || fabsf(ty) > TY_MAX + 2 * errty) continue;
                    resolve_leftright_newhits(x0_st1, tx_st1, y0, ty, errx0_st1, errtx_st1, erry0, errty,
                                              (short)(nhits_x + nuv), detID, pos, drift, sign, P, 150.f);
                    resolve_single_leftright_newhits(x0_st1, tx_st1, y0, ty, (short)(nhits_x + nuv), detID, pos, sign,
                                                     P);
                    orc_fit_2d(nyhits + nuv, Y, Z_, errY, par, perr); /* K:2398-2410 */
                    y0 = par[0];
                    ty = par[1];
                    erry0 = perr[0];
                    errty = perr[1];
                    if (fabsf(y0) > Y0_MAX || fabsf(ty) > TY_MAX) continue;
                    /* the H1 match (K:2416-2428) is not enforced without HODO_Y_MATCH */
                    float chi2 = 0; /* K:2449-2461 */
                    for (short mm = 0; mm < nhits_st23; mm++) {
                        residuals_st23[mm] = residual(detid_st23[mm], chan_st23[mm], drift_st23[mm], sign_st23[mm], P,
                                                      x0, y0, tx, ty);
                        chi2 += residuals_st23[mm] * residuals_st23[mm] /
                                (resolution_st23[mm] * resolution_st23[mm]);
                    }
                    chi2 += chi2_track(nhits_x + nuv, residuals, drift, sign, res, p1x, p1y, p1z, dpx, dpy, dpz,
                                       x0_st1, y0, tx_st1, ty);
                    if (chi2 > 10000.f) continue;
                    if (chi2 < chi2min) { /* K:2470-2496 */
                        chi2min = chi2;
                        update_track = 1;
                        best[2] = (float)(nhits_x + nuv);
                        best[3] = chi2;
                        best[6] = ty;
                        best[8] = y0;
                        best[9] = invP;
                        best[11] = errty;
                        best[13] = erry0;
                        best[14] = errinvP;
                        best[15] = charge;
                        for (short m = 0; m < nhits_st23; m++) best[124 + m] = residuals_st23[m];
                        for (short m = 0; m < nhits_x + nuv; m++) {
                            best[16 + m] = detID[m];
                            best[34 + m] = elID[m];
                            best[52 + m] = pos[m];
                            best[70 + m] = drift[m];
                            best[88 + m] = sign[m];
                            best[106 + m] = tdc[m];
                            best[124 + nhits_st23 + m] = residuals[m];
                        }
                    }
                }
            }
            if (update_track) { /* K:2504-2528 */
                T[OR_TRK_STID] = 6.f;
                int nhits_st1 = (int)best[2];
                T[OR_TRK_NHITS] = (float)nhits_st23 + best[2];
                T[OR_TRK_CHI2] = best[3];
                T[OR_TRK_TY] = best[6];
                T[OR_TRK_Y0] = best[8];
                T[OR_TRK_INVP] = best[9];
                T[OR_TRK_ERR_TY] = best[11];
                T[OR_TRK_ERR_Y0] = best[13];
                T[OR_TRK_ERR_INVP] = best[14];
                T[OR_TRK_CHARGE] = best[15];
                for (int n = 0; n < nhits_st23; n++) T[OR_TRK_HIT_RESID + n] = best[124 + n];
                for (int n = 0; n < nhits_st1; n++) {
                    T[OR_TRK_HIT_DETID + nhits_st23 + n] = best[16 + n];
                    T[OR_TRK_HIT_CHAN + nhits_st23 + n] = best[34 + n];
                    T[OR_TRK_HIT_POS + nhits_st23 + n] = best[52 + n];
                    T[OR_TRK_HIT_DRIFT + nhits_st23 + n] = best[70 + n];
                    T[OR_TRK_HIT_SIGN + nhits_st23 + n] = best[88 + n];
                    T[OR_TRK_HIT_TDC + nhits_st23 + n] = best[106 + n];
                    T[OR_TRK_HIT_RESID + nhits_st23 + n] = best[124 + nhits_st23 + n];
                }
            }
        }
    }
}

/* ------------------------------------------------------------------------ */
/* threaded drivers                                                         */
/* ------------------------------------------------------------------------ */
/* ------------------------------------------------------------------------ */
/* post-global selection, H:1916-2380                                        */
/* ------------------------------------------------------------------------ */
#define SEL_CHI2DOF_MAX 250.f  /* K0:194 */
#define SEL_MERGE_THRES 0.015f /* K0:196 */

/* H:1995-2131 (x) and H:2137-2273 (y): is there a prop-tube segment (a hit
 * of the first station within win1 of the track, one of the second within
 * win2) whose line agrees with the track?  The reference's loops only set a
 * flag, so the answer is an existence test over (p1a then p1b) x (p2a then
 * p2b). */
static int prop_segment(float x0, float tx, hitcoll_t p1a, float z1a, hitcoll_t p1b, float z1b, hitcoll_t p2a,
                        float z2a, hitcoll_t p2b, float z2b, float win1, float win2, float slope_max,
                        float inter_max) {
    const float cut = 0.03f; /* H:1992, H:2000 */
    for (int s1 = 0; s1 < 2; s1++) {
        hitcoll_t h1 = s1 ? p1b : p1a;
        const float z1 = s1 ? z1b : z1a;
        for (int n = 0; n < h1.n; n++) {
            const float ipos1 = hc_pos(h1, n);
            if (!(fabsf(ipos1 - (tx * z1 + x0)) < win1)) continue;
            for (int s2 = 0; s2 < 2; s2++) {
                hitcoll_t h2 = s2 ? p2b : p2a;
                const float z2 = s2 ? z2b : z2a;
                for (int m = 0; m < h2.n; m++) {
                    const float ipos2 = hc_pos(h2, m);
                    if (fabsf(ipos2 - (tx * z2 + x0)) > win2) continue;
                    const float a = (ipos2 - ipos1) / (z2 - z1);
                    if (fabsf(a) > slope_max) continue;
                    if (fabsf(a - tx) > cut) continue;
                    const float b = ipos1 - a * z1;
                    if (fabsf(b) > inter_max) continue;
                    if (fabsf((tx * 2028.19f + x0) - (a * 2028.19f + b)) > 3.0f) continue;
                    return 1;
                }
            }
        }
    }
    return 0;
}

/* gKernel_PropSegmentMatching, H:1916-2277: every track of the slot (any
 * stationID) without an x and a y prop-tube segment gets stationID 5 */
static void prop_match_event(const or_plane_t *P, or_hits_view_t hv, or_tracks_view_t tv, long e,
                             const uint8_t *toomany) {
    if (toomany[e]) return;
    const int px1 = detsuperid[5][0] * 2, px2 = detsuperid[6][0] * 2; /* 50/49, 52/51 */
    const int py1 = detsuperid[5][1] * 2, py2 = detsuperid[6][1] * 2; /* 48/47, 54/53 */
    hitcoll_t p1x1 = hits_prop(hv, e, px1), p1x2 = hits_prop(hv, e, px1 - 1);
    hitcoll_t p2x1 = hits_prop(hv, e, px2), p2x2 = hits_prop(hv, e, px2 - 1);
    hitcoll_t p1y1 = hits_prop(hv, e, py1), p1y2 = hits_prop(hv, e, py1 - 1);
    hitcoll_t p2y1 = hits_prop(hv, e, py2), p2y2 = hits_prop(hv, e, py2 - 1);
    for (int slot = 0; slot < OR_NSLOTS; slot++) {
        const int n = tv.ntracks[e * OR_NSLOTS + slot];
        for (int i = 0; i < n; i++) {
            float *T = trk_rec(tv, e, slot, i);
            const float x0 = T[OR_TRK_X0], y0 = T[OR_TRK_Y0], tx = T[OR_TRK_TX], ty = T[OR_TRK_TY];
            if (!prop_segment(x0, tx, p1x1, P->z[px1], p1x2, P->z[px1 - 1], p2x1, P->z[px2], p2x2, P->z[px2 - 1],
                              5.08f, 7.62f, TX_MAX, X0_MAX)) {
                T[OR_TRK_STID] = 5.f;
                continue;
            }
            if (!prop_segment(y0, ty, p1y1, P->z[py1], p1y2, P->z[py1 - 1], p2y1, P->z[py2], p2y2, P->z[py2 - 1],
                              5.08f, 10.16f, TY_MAX, Y0_MAX))
                T[OR_TRK_STID] = 5.f;
        }
    }
}

/* gKernel_GlobalTrackCleaning, H:2289-2331, each slot on its own.  The else
 * branch compares invP(i) with itself (H:2323), so it demotes i whenever the
 * charges agree. */
static void gclean_event(or_tracks_view_t tv, long e, const uint8_t *toomany) {
    if (toomany[e]) return;
    for (int s = 0; s < OR_NSLOTS; s++) {
        const int n = tv.ntracks[e * OR_NSLOTS + s];
        for (int i = 0; i < n; i++) {
            float *Ti = trk_rec(tv, e, s, i);
            if (Ti[OR_TRK_STID] < 6) continue;
            if (Ti[OR_TRK_CHI2] / (Ti[OR_TRK_NHITS] - 5) > SEL_CHI2DOF_MAX) {
                Ti[OR_TRK_STID] = 5.f;
                continue;
            }
            for (int j = i + 1; j < n; j++) {
                float *Tj = trk_rec(tv, e, s, j);
                if (Tj[OR_TRK_STID] < 6) continue;
                if (Ti[OR_TRK_CHI2] / (Ti[OR_TRK_NHITS] - 5) < Tj[OR_TRK_CHI2] / (Tj[OR_TRK_NHITS] - 5)) {
                    if ((Ti[OR_TRK_INVP] - Tj[OR_TRK_INVP]) / Ti[OR_TRK_INVP] < SEL_MERGE_THRES &&
                        Ti[OR_TRK_CHARGE] * Tj[OR_TRK_CHARGE] > 0)
                        Tj[OR_TRK_STID] = 5.f;
                } else {
                    if ((Ti[OR_TRK_INVP] - Ti[OR_TRK_INVP]) / Tj[OR_TRK_INVP] < SEL_MERGE_THRES &&
                        Ti[OR_TRK_CHARGE] * Tj[OR_TRK_CHARGE] > 0)
                        Ti[OR_TRK_STID] = 5.f;
                }
            }
        }
    }
}

/* gKernel_GlobalTrackCleaning_crossthreads, H:2333-2380, the block's 32
 * threads in lockstep as in clean_cross_event: at each step (i_trd, i, j)
 * the demotions (stationID = 5) land after every thread has decided. */
static void gclean_cross_event(or_tracks_view_t tv, long e, const uint8_t *toomany) {
    if (toomany[e]) return;
    int nt[OR_NSLOTS], maxn = 0;
    for (int t = 0; t < OR_NSLOTS; t++) {
        nt[t] = tv.ntracks[e * OR_NSLOTS + t];
        if (nt[t] > maxn) maxn = nt[t];
    }
    for (int u = 0; u < OR_NSLOTS; u++) {
        const int m = nt[u];
        for (int i = 0; i < maxn; i++) {
            int act[OR_NSLOTS];
            for (int t = 0; t < OR_NSLOTS; t++)
                act[t] = t != u && i < nt[t] && trk_rec(tv, e, t, i)[OR_TRK_STID] >= 6;
            for (int j = 0; j < m; j++) {
                float *Tj = trk_rec(tv, e, u, j);
                if (Tj[OR_TRK_STID] < 6) continue;
                int demote_j = 0, demote_i[OR_NSLOTS];
                for (int t = 0; t < OR_NSLOTS; t++) {
                    demote_i[t] = 0;
                    if (!act[t]) continue;
                    const float *Ti = trk_rec(tv, e, t, i);
                    if (Ti[OR_TRK_CHI2] / (Ti[OR_TRK_NHITS] - 5) < Tj[OR_TRK_CHI2] / (Tj[OR_TRK_NHITS] - 5)) {
                        if ((Ti[OR_TRK_INVP] - Tj[OR_TRK_INVP]) / Ti[OR_TRK_INVP] < SEL_MERGE_THRES &&
                            Ti[OR_TRK_CHARGE] * Tj[OR_TRK_CHARGE] > 0)
                            demote_j = 1;
                    } else {
                        if ((Ti[OR_TRK_INVP] - Tj[OR_TRK_INVP]) / Tj[OR_TRK_INVP] < SEL_MERGE_THRES &&
                            Ti[OR_TRK_CHARGE] * Tj[OR_TRK_CHARGE] > 0)
                            demote_i[t] = 1;
                    }
                }
                if (demote_j) Tj[OR_TRK_STID] = 5.f;
                for (int t = 0; t < OR_NSLOTS; t++)
                    if (demote_i[t]) trk_rec(tv, e, t, i)[OR_TRK_STID] = 5.f;
            }
        }
    }
}

/* ------------------------------------------------------------------------ */
/* learned-scorer inputs: the 16 features of every XZ tracklet               */
/* ------------------------------------------------------------------------ */
/* Rows: tracklets of the accepted events in event, slot, position order.
 * Windows as YZ builds them (K:1252-1283, H:480-511); accepted = the
 * calculate_y_uvhit test (H:75-100) with no sign. */
int64_t orc_tracklet_features(const or_plane_t *P, or_hits_view_t hv, or_tracks_view_t tv, const uint8_t *toomany,
                              int n_events, int32_t *row_off, float *feat, int64_t max_rows) {
    int64_t row = 0;
    for (long e = 0; e < n_events; e++) {
        row_off[e] = (int32_t)row;
        if (toomany[e]) continue;
        for (int slot = 0; slot < OR_NSLOTS; slot++) {
            const int st3 = 3 + slot % 2;
            short dl[8];
            const int stids[4] = {2, 2, st3, st3}, projs[4] = {1, 2, 1, 2};
            for (int q = 0; q < 4; q++) {
                int d = detsuperid[stids[q]][projs[q]] * 2;
                dl[2 * q] = (short)d;
                dl[2 * q + 1] = (short)(d - 1);
            }
            int ntr = tv.ntracks[e * OR_NSLOTS + slot];
            if (ntr > OR_SLOTCAP) ntr = OR_SLOTCAP;
            for (int it = 0; it < ntr; it++, row++) {
                const float *T = trk_rec(tv, e, slot, it);
                const float x0 = T[OR_TRK_X0], tx = T[OR_TRK_TX], ex0 = T[OR_TRK_ERR_X0], etx = T[OR_TRK_ERR_TX];
                int nwin[4], nacc[4], nall = 0;
                for (int q = 0; q < 4; q++) {
                    const int a = 2 * q;
                    const float za = P->z[dl[a]], zb = P->z[dl[a + 1]];
                    const float sp = P->spacing[dl[a]];
                    const float xmin = fminf((tx - etx) * za, (tx - etx) * zb) + x0 - ex0 - sp;
                    const float xmax = fmaxf((tx + etx) * za, (tx + etx) * zb) + x0 + ex0 + sp;
                    int cw = 0, ca = 0;
                    for (int side = 0; side < 2; side++) {
                        const int det = dl[a + side];
                        hitcoll_t h = hits_chamber(hv, e, det);
                        nall += h.n;
                        for (int i = 0; i < h.n; i++) {
                            const int el = (int)hc_chan(h, i);
                            float p1x, p2x;
                            if (P->deltapx[det] > 0) {
                                p1x = x_bep(det, el, P);
                                p2x = x_tep(det, el, P);
                            } else {
                                p1x = x_tep(det, el, P);
                                p2x = x_bep(det, el, P);
                            }
                            if (!((p1x <= xmax) && (p2x >= xmin))) continue;
                            cw++;
                            float yy, ey;
                            if (calculate_y_uvhit(det, el, hc_drift(h, i), 0, x0, tx, P, &yy, &ey)) ca++;
                        }
                    }
                    nwin[q] = cw;
                    nacc[q] = ca;
                }
                if (row < max_rows) {
                    float *f = feat + row * OR_NFEAT;
                    f[0] = x0 * 0.01f;
                    f[1] = tx * 10.f;
                    f[2] = ex0;
                    f[3] = etx * 100.f;
                    f[4] = log1pf((float)nall);
                    f[5] = T[OR_TRK_NHITS];
                    f[6] = (float)(slot & 1);
                    for (int q = 0; q < 4; q++) {
                        f[7 + q] = log1pf((float)nwin[q]);
                        f[11 + q] = log1pf((float)nacc[q]);
                    }
                    f[15] = log1pf((float)nacc[0]) + log1pf((float)nacc[1]) + log1pf((float)nacc[2]) +
                            log1pf((float)nacc[3]);
                }
            }
        }
    }
    row_off[n_events] = (int32_t)row;
    return row;
}

int orc_hardware_threads(void) {
    long n = sysconf(_SC_NPROCESSORS_ONLN);
    return n > 0 ? (int)n : 1;
}

enum { ST_ER, ST_XZ, ST_YZ, ST_CLEAN, ST_CLEANX, ST_GLOBAL, ST_ALL, ST_PROP, ST_GCLEAN, ST_GCLEANX };

typedef struct {
    int stage;
    const or_plane_t *P;
    or_hits_view_t h;
    or_tracks_view_t t;
    int32_t *ntkl;
    uint8_t *toomany;
    uint32_t *status;
    int64_t *counts;
    long e0, e1;
} job_t;

static void *worker(void *arg) {
    job_t *j = (job_t *)arg;
    xz_scratch_t *xs = NULL;
    pair_scratch_t *ps = NULL;
    if (j->stage == ST_XZ || j->stage == ST_ALL) {
        xs = (xz_scratch_t *)calloc(1, sizeof(xz_scratch_t));
    }
    if (j->stage == ST_YZ || j->stage == ST_GLOBAL || j->stage == ST_ALL) {
        ps = (pair_scratch_t *)calloc(1, sizeof(pair_scratch_t));
        for (int q = 0; q < 4; q++) ps->pairs[q] = alloc_pairs();
    }
    for (long e = j->e0; e < j->e1; e++) {
        int64_t *c = j->counts ? j->counts + ORC_NCOUNTS * e : NULL;
        switch (j->stage) {
        case ST_ER: er_event(j->h, e, j->toomany, j->status); break;
        case ST_XZ: xz_event(j->P, j->h, j->t, e, j->ntkl, j->toomany, j->status, xs, c); break;
        case ST_YZ: yz_event(j->P, j->h, j->t, e, j->toomany, ps, c); break;
        case ST_CLEAN: clean_event(j->t, e, j->toomany); break;
        case ST_CLEANX: clean_cross_event(j->t, e, j->toomany); break;
        case ST_GLOBAL: global_event(j->P, j->h, j->t, e, j->toomany, ps, c); break;
        case ST_PROP: prop_match_event(j->P, j->h, j->t, e, j->toomany); break;
        case ST_GCLEAN: gclean_event(j->t, e, j->toomany); break;
        case ST_GCLEANX: gclean_cross_event(j->t, e, j->toomany); break;
        case ST_ALL:
            er_event(j->h, e, j->toomany, j->status);
            xz_event(j->P, j->h, j->t, e, j->ntkl, j->toomany, j->status, xs, c);
            yz_event(j->P, j->h, j->t, e, j->toomany, ps, c);
            clean_event(j->t, e, j->toomany);
            clean_cross_event(j->t, e, j->toomany);
            global_event(j->P, j->h, j->t, e, j->toomany, ps, c);
            break;
        }
    }
    if (xs) {
        free(xs->tkl[0]);
        free(xs->tkl[1]);
        free(xs);
    }
    if (ps) {
        for (int q = 0; q < 4; q++) free(ps->pairs[q]);
        free(ps);
    }
    return NULL;
}

static void run_stage(int stage, const or_plane_t *P, or_hits_view_t h, or_tracks_view_t t, int32_t *ntkl,
                      uint8_t *toomany, uint32_t *status, int64_t *counts, int n_events, int n_threads) {
    if (n_threads <= 0) n_threads = orc_hardware_threads();
    if (n_threads > n_events) n_threads = n_events > 0 ? n_events : 1;
    pthread_t th[256];
    job_t jobs[256];
    if (n_threads > 256) n_threads = 256;
    for (int k = 0; k < n_threads; k++) {
        jobs[k].stage = stage;
        jobs[k].P = P;
        jobs[k].h = h;
        jobs[k].t = t;
        jobs[k].ntkl = ntkl;
        jobs[k].toomany = toomany;
        jobs[k].status = status;
        jobs[k].counts = counts;
        jobs[k].e0 = (long)n_events * k / n_threads;
        jobs[k].e1 = (long)n_events * (k + 1) / n_threads;
    }
    if (n_threads == 1) {
        worker(&jobs[0]);
        return;
    }
    for (int k = 0; k < n_threads; k++) pthread_create(&th[k], NULL, worker, &jobs[k]);
    for (int k = 0; k < n_threads; k++) pthread_join(th[k], NULL);
}

void orc_event_reduce(or_hits_view_t h, uint8_t *toomany, uint32_t *status, int n_events, int n_threads) {
    or_tracks_view_t t = {0, 0};
    run_stage(ST_ER, NULL, h, t, NULL, toomany, status, NULL, n_events, n_threads);
}
void orc_xz(const or_plane_t *p, or_hits_view_t h, or_tracks_view_t t, int32_t *ntracklets, uint8_t *toomany,
            uint32_t *status, int n_events, int n_threads) {
    run_stage(ST_XZ, p, h, t, ntracklets, toomany, status, NULL, n_events, n_threads);
}
void orc_yz(const or_plane_t *p, or_hits_view_t h, or_tracks_view_t t, const uint8_t *toomany, int n_events,
            int n_threads) {
    run_stage(ST_YZ, p, h, t, NULL, (uint8_t *)toomany, NULL, NULL, n_events, n_threads);
}
void orc_back_clean(or_tracks_view_t t, const uint8_t *toomany, int n_events, int n_threads) {
    or_hits_view_t h = {0, 0, 0, 0, 0, 0};
    run_stage(ST_CLEAN, NULL, h, t, NULL, (uint8_t *)toomany, NULL, NULL, n_events, n_threads);
    run_stage(ST_CLEANX, NULL, h, t, NULL, (uint8_t *)toomany, NULL, NULL, n_events, n_threads);
}
void orc_global(const or_plane_t *p, or_hits_view_t h, or_tracks_view_t t, const uint8_t *toomany, int n_events,
                int n_threads) {
    run_stage(ST_GLOBAL, p, h, t, NULL, (uint8_t *)toomany, NULL, NULL, n_events, n_threads);
}
void orc_prop_matching(const or_plane_t *p, or_hits_view_t h, or_tracks_view_t t, const uint8_t *toomany,
                       int n_events, int n_threads) {
    run_stage(ST_PROP, p, h, t, NULL, (uint8_t *)toomany, NULL, NULL, n_events, n_threads);
}

void orc_global_clean(or_tracks_view_t t, const uint8_t *toomany, int n_events, int n_threads) {
    or_hits_view_t h;
    memset(&h, 0, sizeof(h));
    run_stage(ST_GCLEAN, NULL, h, t, NULL, (uint8_t *)toomany, NULL, NULL, n_events, n_threads);
    run_stage(ST_GCLEANX, NULL, h, t, NULL, (uint8_t *)toomany, NULL, NULL, n_events, n_threads);
}

void orc_run_all(const or_plane_t *p, or_hits_view_t h, or_tracks_view_t t, int32_t *ntracklets, uint8_t *toomany,
                 uint32_t *status, int n_events, int n_threads) {
    run_stage(ST_ALL, p, h, t, ntracklets, toomany, status, NULL, n_events, n_threads);
}
void orc_run_all_counted(const or_plane_t *p, or_hits_view_t h, or_tracks_view_t t, int32_t *ntracklets,
                         uint8_t *toomany, uint32_t *status, int64_t *counts, int n_events, int n_threads) {
    for (long e = 0; e < (long)ORC_NCOUNTS * n_events; e++) counts[e] = 0;
    run_stage(ST_ALL, p, h, t, ntracklets, toomany, status, counts, n_events, n_threads);
}

int64_t orc_yz_outer_dump(const or_plane_t *p, or_hits_view_t h, or_tracks_view_t t, const uint8_t *toomany,
                          int n_events, float *buf, int64_t cap) {
    g_outer.buf = buf;
    g_outer.cap = cap;
    g_outer.n = 0;
    run_stage(ST_YZ, p, h, t, NULL, (uint8_t *)toomany, NULL, NULL, n_events, 1);
    const int64_t n = g_outer.n;
    g_outer.buf = NULL;
    return n;
}
