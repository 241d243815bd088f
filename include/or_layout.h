/*
 * or_layout.h -- in-memory layout of the e1039 online-reconstruction event,
 * hit, track and geometry records.  Plain C, shared by the CUDA library, its
 * C-ABI callers and the CPU oracle.
 *
 * The layout is the reference's own, kept bit-for-bit so that buffers filled
 * by a reference-style host (OnlineReconstruction/online_reconstruction.cu
 * :589-636) can be handed to this library unchanged:
 *
 *  - hit slot of plane d in event e starts at
 *        e*OR_EVT_FLOATS[type] + 5*OR_MAXHITS[type]*(d - d0[type])  floats
 *    (reconstruction_classes.cuh:89-102, reconstruction_constants.h:166-180);
 *  - inside a slot the five hit fields are SoA with stride = the plane's
 *    current hit count n:  [chan | pos | tdc | flag | drift], n floats each
 *    (reconstruction_classes.cuh:9, :18-46);
 *  - a track record is 148 floats (reconstruction_classes.cuh:558-635);
 *  - an event owns 512 track records in 32 slots of 16
 *    (reconstruction_classes.cuh:542-556); the slot count of slot s in
 *    event e is ntracks[e*32+s] (unsigned short).
 *
 * The fixed-capacity reference structs (gEventHitCollections,
 * gEventTrackCollection, gEvent) are sized for EstnEvtMax = 10000 events;
 * the views below carry plain pointers so any number of events can be used,
 * and or_hits_view_from_collection()/or_tracks_view_from_collection() in
 * or_gb300.h map a reference struct onto them.
 */
#ifndef OR_LAYOUT_H
#define OR_LAYOUT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* detector planes: 1..30 drift chambers, 31..46 hodoscopes, 47..54 prop tubes
 * (reconstruction_constants.h:10-13) */
#define OR_NCHAM 30
#define OR_NHODO 16
#define OR_NPROP 8
#define OR_NDET 55 /* index 0 unused */

#define OR_NHITSPARAM 5
#define OR_MAXHITS_CHAM 200 /* reconstruction_constants.h:173 */
#define OR_MAXHITS_HODO 60  /* :174 */
#define OR_MAXHITS_PROP 120 /* :175 */

#define OR_EVT_CHAM_FLOATS (OR_NCHAM * OR_NHITSPARAM * OR_MAXHITS_CHAM) /* 30000 */
#define OR_EVT_HODO_FLOATS (OR_NHODO * OR_NHITSPARAM * OR_MAXHITS_HODO) /* 4800 */
#define OR_EVT_PROP_FLOATS (OR_NPROP * OR_NHITSPARAM * OR_MAXHITS_PROP) /* 4800 */

#define OR_NTRKPARAM 148 /* reconstruction_constants.h:171 */
#define OR_TRKMAX 512    /* :181 */
#define OR_NSLOTS 32     /* THREADS_PER_BLOCK, :21 */
#define OR_SLOTCAP (OR_TRKMAX / OR_NSLOTS) /* 16 */
#define OR_EVT_TRK_FLOATS (OR_TRKMAX * OR_NTRKPARAM) /* 75776 */
#define OR_MAXHITS_PER_TRACK 18

/* learned tracklet scorer: 16 features per XZ tracklet, MLP 16-64-64-1
 * (BF16 weights and activations, FP32 accumulation, sigmoid output) */
#define OR_NFEAT 16
#define OR_MLP_H 64
typedef struct or_mlp {
    float mean[OR_NFEAT];               /* input normalisation: (x - mean) * inv_std */
    float inv_std[OR_NFEAT];
    uint16_t w1[OR_MLP_H * OR_NFEAT];   /* bf16 bits, [out][in] */
    float b1[OR_MLP_H];
    uint16_t w2[OR_MLP_H * OR_MLP_H];   /* bf16 bits, [out][in] */
    float b2[OR_MLP_H];
    float w3[OR_MLP_H];
    float b3;
    float pad[3];
} or_mlp_t;
/* trainable parameters in FP32, in this order: w1, b1, w2, b2, w3, b3 */
#define OR_MLP_NPARAM (OR_MLP_H * OR_NFEAT + OR_MLP_H + OR_MLP_H * OR_MLP_H + OR_MLP_H + OR_MLP_H + 1)

/* wire-position table row stride: wire_pos[det*400 + element]
 * (online_reconstruction.cu:191) */
#define OR_WIREPOS_STRIDE 400

/* row of the track-collection output: [event, slot*16+position, record] */
#define OR_COLLECT_STRIDE (OR_NTRKPARAM + 2)

/* capacity of the reference's fixed structs (reconstruction_constants.h:20) */
#define OR_REF_EVTMAX 10000

/* track-record field offsets: the setter offsets the kernels write
 * (reconstruction_classes.cuh:558-635) */
enum or_trk_field {
    OR_TRK_STID = 0,
    OR_TRK_THREAD = 1,
    OR_TRK_NHITS = 2,
    OR_TRK_CHI2 = 3,
    OR_TRK_CHI2VTX = 4,
    OR_TRK_TX = 5,
    OR_TRK_TY = 6,
    OR_TRK_X0 = 7,
    OR_TRK_Y0 = 8,
    OR_TRK_INVP = 9,
    OR_TRK_ERR_TX = 10,
    OR_TRK_ERR_TY = 11,
    OR_TRK_ERR_X0 = 12,
    OR_TRK_ERR_Y0 = 13,
    OR_TRK_ERR_INVP = 14,
    OR_TRK_CHARGE = 15,
    OR_TRK_VX = 16,
    OR_TRK_PX = 19,
    OR_TRK_HIT_DETID = 22,
    OR_TRK_HIT_CHAN = 40,
    OR_TRK_HIT_POS = 58,
    OR_TRK_HIT_DRIFT = 76,
    OR_TRK_HIT_SIGN = 94,
    OR_TRK_HIT_TDC = 112,
    OR_TRK_HIT_RESID = 130
};

/* Geometry carrier: field-for-field the reference's gPlane
 * (reconstruction_classes.cuh:947-977), 55 entries per field. */
typedef struct or_plane {
    float z[OR_NDET];
    int nelem[OR_NDET];
    float cellwidth[OR_NDET];
    float spacing[OR_NDET];
    float xoffset[OR_NDET];
    float scalex[OR_NDET];
    float x0[OR_NDET];
    float x1[OR_NDET];
    float x2[OR_NDET];
    float costheta[OR_NDET];
    float scaley[OR_NDET];
    float y0[OR_NDET];
    float y1[OR_NDET];
    float y2[OR_NDET];
    float sintheta[OR_NDET];
    float resolution[OR_NDET];
    float p1x_w1[OR_NDET];
    float p1y_w1[OR_NDET];
    float p1z_w1[OR_NDET];
    float deltapx[OR_NDET];
    float deltapy[OR_NDET];
    float deltapz[OR_NDET];
    float dp1x[OR_NDET];
    float dp1y[OR_NDET];
    float dp1z[OR_NDET];
    float slope_max[OR_NDET];
    float inter_max[OR_NDET];
} or_plane_t;

/* Hit collections of n_events events in the reference layout.  Either host
 * or device pointers, depending on the call. */
typedef struct or_hits_view {
    uint32_t *nhits_cham; /* [n_events*30] */
    float *hits_cham;     /* [n_events*30000] */
    uint32_t *nhits_hodo; /* [n_events*16] */
    float *hits_hodo;     /* [n_events*4800] */
    uint32_t *nhits_prop; /* [n_events*8] */
    float *hits_prop;     /* [n_events*4800] */
} or_hits_view_t;

/* Track collections of n_events events in the reference layout. */
typedef struct or_tracks_view {
    uint16_t *ntracks; /* [n_events*32] */
    float *tracks;     /* [n_events*512*148] */
} or_tracks_view_t;

/* Dimuon collections (gEventDimuonCollection, reconstruction_classes.cuh:
 * 870-936): per event a count and 16 records of 36 floats, written by
 * or_dimuons (gKernel_DimuonBuilding, reconstruction_kernels.cuh:2820-3090). */
#define OR_DIMUON_MAX 16     /* datasizes::DimuonSizeMax, reconstruction_constants.h:184 */
#define OR_NDIMUONPARAM 36   /* datasizes::NDimuonParam, :183 */
#define OR_EVT_DIM_FLOATS (OR_DIMUON_MAX * OR_NDIMUONPARAM)
enum {
    OR_DIM_MASS = 0,
    OR_DIM_PT = 1,
    OR_DIM_XF = 2,
    OR_DIM_X1 = 3,
    OR_DIM_X2 = 4,
    OR_DIM_COSTHETA = 5,
    OR_DIM_PHI = 6,
    OR_DIM_MASS_SINGLE = 7, /* never computed by the reference: 0 here */
    OR_DIM_CHI2_SINGLE = 8, /* never computed by the reference: 0 here */
    OR_DIM_VTX = 9,         /* 3 floats */
    OR_DIM_POS_VTX = 12,    /* 3 */
    OR_DIM_NEG_VTX = 15,    /* 3 */
    OR_DIM_POS_P = 18,      /* px, py, pz, E */
    OR_DIM_NEG_P = 22,
    OR_DIM_POS_P_SINGLE = 26,
    OR_DIM_NEG_P_SINGLE = 30,
    OR_DIM_CHI2_VTX = 34, /* never computed by the reference: 0 here */
    OR_DIM_CHI2_KF = 35   /* never computed by the reference: 0 here */
};

typedef struct or_dimuons_view {
    uint16_t *ndimuons; /* [n_events] */
    float *dimuons;     /* [n_events*16*36] */
} or_dimuons_view_t;

/* Monitoring histograms (gHistsArrays, reconstruction_classes.cuh:938-944):
 * 11 trigger classes x 18 variables (6 per track, 12 per dimuon), each a
 * table of at most 256 bins given by centre and half width.  Same byte
 * layout as the reference struct. */
#define OR_HIST_NTRIGGERS 11   /* histotools::ntriggers, reconstruction_constants.h:217 */
#define OR_HIST_NVARS 18       /* histotools::nvars_total, :223 */
#define OR_HIST_NVARS_TRACKS 6 /* :220 */
#define OR_HIST_NBINS_MAX 256  /* :218 */
typedef struct or_hists {
    int16_t nbins[OR_HIST_NTRIGGERS * OR_HIST_NVARS];
    float pts_hw[OR_HIST_NTRIGGERS * OR_HIST_NVARS];
    float xpts[OR_HIST_NTRIGGERS * OR_HIST_NVARS * OR_HIST_NBINS_MAX];
    float values[OR_HIST_NTRIGGERS * OR_HIST_NVARS * OR_HIST_NBINS_MAX];
} or_hists_t;

/* Event output rows: the fields of the reference's output tree
 * (ORoutput_tree, OnlineReconstruction/OROutput.h:25-102) in its order, filled
 * as online_reconstruction.cu:1063-1222 fills it: events with raw hits and no
 * reject flag, every reduced hit, the tracks with stationID >= a threshold (7
 * in the reference build) with their hits, every dimuon. */
enum { /* int64 per event */
    OR_OUT_EV_INDEX = 0,     /* index in the batch */
    OR_OUT_EV_ID = 1,        /* fEventID */
    OR_OUT_EV_NHITS = 2,     /* fNHits */
    OR_OUT_EV_NTRACKS = 3,   /* fNTracks */
    OR_OUT_EV_NDIMUONS = 4,  /* fNDimuons */
    OR_OUT_EV_HIT0 = 5,      /* first row of each table */
    OR_OUT_EV_TRACK0 = 6,
    OR_OUT_EV_TRACKHIT0 = 7,
    OR_OUT_EV_DIMUON0 = 8,
    OR_OUT_EV_FIELDS = 9
};
#define OR_OUT_HIT_FIELDS 5       /* DetID, Chan, Pos, TDC, Drift */
#define OR_OUT_TRACK_FIELDS 20    /* StID, NHits, Chi2, X0, Y0, TX, TY, InvP, ErrX0, ErrY0, ErrTX, ErrTY,
                                     ErrInvP, Charge, Vx, Vy, Vz, Px, Py, Pz */
#define OR_OUT_TRACKHIT_FIELDS 7  /* DetID, Chan, Pos, Drift, Sign, TDC, Residual */
#define OR_OUT_DIMUON_FIELDS 39   /* Mass, PT, XF, X1, X2, Costheta, Phi, MassSingle, Chi2Single, Vx, Vy,
                                     Vz, Px, Py, Pz, PosVx, PosVy, PosVz, NegVx, NegVy, NegVz, PosE,
                                     PosPx, PosPy, PosPz, NegE, NegPx, NegPy, NegPz, PosSingleE,
                                     PosSinglePx, PosSinglePy, PosSinglePz, NegSingleE, NegSinglePx,
                                     NegSinglePy, NegSinglePz, Chi2Vtx, Chi2KF */
typedef struct or_output_view {
    int64_t *events;     /* [cap_events * OR_OUT_EV_FIELDS] */
    float *hits;         /* [cap_hits * 5] */
    float *tracks;       /* [cap_tracks * 20] */
    float *track_hits;   /* [cap_track_hits * 7] */
    float *dimuons;      /* [cap_dimuons * 39] */
    int64_t cap_events, cap_hits, cap_tracks, cap_track_hits, cap_dimuons;
    int64_t *counts;     /* [5] (device): rows of each table the batch needs */
} or_output_view_t;

/* Compact hit record, the raw-event format of the reference's input
 * (OnlineReconstruction/LoadInput.h:10-20: detectorID, elementID, tdcTime,
 * driftDistance, plus the in-time flag bit the host packer turns into
 * flag = 1<<in_time, online_reconstruction.cu:599). */
typedef struct or_hit_record {
    int16_t det;
    int16_t elem;
    float tdc;
    float drift;
    int32_t flag; /* the packed float flag value: 2 = in time, 1 = out of time */
} or_hit_record_t;

/* R-T (drift time -> drift distance) calibration: per plane a cubic spline
 * through the calibration points (T_k, R_k), clamped with zero slope at both
 * ends (the reference builds ROOT TSpline3(name, T, R, n, "b1e1") per plane,
 * online_reconstruction.cu:220-242), plus the plane's time window.  Spline
 * piece k covers (t[k], t[k+1]]:  R(x) = r[k] + dx*(b[k] + dx*(c[k] + dx*d[k])),
 * dx = x - t[k], all in double.  nknots[d] = 0: plane d has no profile and
 * its hits keep the record's drift distance. */
#define OR_RT_MAXKNOTS 500 /* the reference's T[500], R[500] (online_reconstruction.cu:226) */
typedef struct or_rt_table {
    int32_t nknots[OR_NDET];
    float tmin[OR_NDET];      /* tdc < tmin: drift = cellwidth/2 (online_reconstruction.cu:390-391) */
    float tmax[OR_NDET];      /* tdc > tmax: drift = 0 (:392-393) */
    float cellwidth[OR_NDET]; /* gPlane::cellwidth */
    double t[OR_NDET][OR_RT_MAXKNOTS];
    double r[OR_NDET][OR_RT_MAXKNOTS];
    double b[OR_NDET][OR_RT_MAXKNOTS];
    double c[OR_NDET][OR_RT_MAXKNOTS];
    double d[OR_NDET][OR_RT_MAXKNOTS];
} or_rt_table_t;

#ifdef __cplusplus
}
#endif

#endif /* OR_LAYOUT_H */
