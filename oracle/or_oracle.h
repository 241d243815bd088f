/*
 * or_oracle.h -- CPU oracle for the e1039 online-reconstruction hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm (OnlineReconstruction/reconstruction_kernels.cuh and
 * reconstruction_helper.cuh), used by the tests, by __graft_entry__.smoke()
 * and by bench.py's CPU baseline as the checker.  The CUDA library never links
 * or calls it.
 *
 * Every stage works on the reference memory layout (or_layout.h) and mutates
 * the buffers in place exactly like the reference kernels do.  Arithmetic is
 * IEEE single precision, one rounding per operation (built with
 * -ffp-contract=off), matching a reference build with -fmad=false.
 *
 * Where the reference is not deterministic the oracle fixes one canonical
 * behaviour, shared with the CUDA kernels:
 *  - XZ tracklets go to slots round-robin per station-3 half (the k-th
 *    tracklet of parity p lands in slot 2*(k%16)+p, position k/16), in the
 *    order (reference thread t, bin pair, candidate);
 *  - per-thread/per-slot scratch arrays start from a sentinel that never
 *    pairs (the reference leaves them uninitialised);
 *  - the cross-slot cleaning pass visits slots 0..31 in order.
 */
#ifndef OR_ORACLE_H
#define OR_ORACLE_H

#include "../include/or_layout.h"

#ifdef __cplusplus
extern "C" {
#endif

/* geometry: OnlineReconstruction/online_reconstruction.cu:123-218 */
int orc_parse_geometry(const char *path, or_plane_t *plane, double *wire_pos /* [55*400] */);

/* per-event status bits (the reference's HasTooManyHits plus the reason) */
#define ORC_ST_TOOMANY_ER 1u      /* station multiplicity over limit, K:135-139 */
#define ORC_ST_TOOMANY_XZBIN 2u   /* >20 pairs in an element bin, K:359-375 */
#define ORC_ST_TOOMANY_TKL 4u     /* tracklet storage exhausted, K:719-839 */

/* Stage entry points; n_threads <= 0 uses all hardware threads. */
void orc_event_reduce(or_hits_view_t h, uint8_t *toomany, uint32_t *status, int n_events, int n_threads);
void orc_xz(const or_plane_t *p, or_hits_view_t h, or_tracks_view_t t, int32_t *ntracklets,
            uint8_t *toomany, uint32_t *status, int n_events, int n_threads);
void orc_yz(const or_plane_t *p, or_hits_view_t h, or_tracks_view_t t, const uint8_t *toomany,
            int n_events, int n_threads);
void orc_back_clean(or_tracks_view_t t, const uint8_t *toomany, int n_events, int n_threads);
void orc_global(const or_plane_t *p, or_hits_view_t h, or_tracks_view_t t, const uint8_t *toomany,
                int n_events, int n_threads);
/* all five stages in the reference launch order (online_reconstruction.cu:776-894) */
void orc_run_all(const or_plane_t *p, or_hits_view_t h, or_tracks_view_t t, int32_t *ntracklets,
                 uint8_t *toomany, uint32_t *status, int n_events, int n_threads);

/* orc_run_all plus work counters per event (ORC_NCOUNTS each), in the
 * reference's enumeration: [0] XZ (pair2, pair3) candidates, [1] YZ
 * (u3,v3,u2,v2) combinations, [2] Global (x1,u1,v1) combinations, [3] YZ
 * combinations reaching the first y fit, [4] passing its 2-sigma cut,
 * [5] passing every gate up to the chi2, [6] the largest windowed hit list
 * or pair list of any YZ tracklet, [7] the same for global tracking (the
 * reference's arrays hold 100, K:890-903, K:1857-1867). */
#define ORC_NCOUNTS 8
void orc_run_all_counted(const or_plane_t *p, or_hits_view_t h, or_tracks_view_t t, int32_t *ntracklets,
                         uint8_t *toomany, uint32_t *status, int64_t *counts, int n_events, int n_threads);

/* Single-primitive entry points used by the known-answer tests. */
void orc_fit_2d(int n, const float *x, const float *z, const float *w, float *par, float *err);
void orc_fit_2d_drift(int n, const float *x, const float *drift, const short *sign, const float *z,
                      const float *w, float *par, float *err);
void orc_matinv_2x2(const float *a, float *ainv);
int orc_reduce_plane(const float *slot, int n, int detid, short *hitflag);

/* post-global selection (online_reconstruction.cu:914-933):
 * gKernel_PropSegmentMatching (reconstruction_helper.cuh:1916-2277), then
 * gKernel_GlobalTrackCleaning and ..._crossthreads (:2289-2380) */
void orc_prop_matching(const or_plane_t *p, or_hits_view_t h, or_tracks_view_t t, const uint8_t *toomany,
                       int n_events, int n_threads);
void orc_global_clean(or_tracks_view_t t, const uint8_t *toomany, int n_events, int n_threads);

/* the learned scorer's 16 features per XZ tracklet (row order of
 * or_tracklet_rows); returns the row count */
int64_t orc_tracklet_features(const or_plane_t *p, or_hits_view_t h, or_tracks_view_t t, const uint8_t *toomany,
                              int n_events, int32_t *row_off, float *feat, int64_t max_rows);

/* after global tracking (or_physics.c): vertexing (gKernel_Vertexing,
 * reconstruction_kernels.cuh:2542-2810), dimuons (gKernel_DimuonBuilding,
 * :2820-3090), the histogram table (online_reconstruction.cu:670-723) and the
 * histogram fill (gKernel_fill_display_histograms, :3100-3195); trigger_bits
 * may be NULL (all zero) */
void orc_vertexing(const or_plane_t *p, or_tracks_view_t t, const uint8_t *toomany, int n_events, int n_threads);
void orc_dimuons(const or_plane_t *p, or_tracks_view_t t, or_dimuons_view_t d, const uint8_t *toomany, int n_events,
                 int n_threads);
void orc_hist_table(or_hists_t *h);
void orc_fill_histograms(or_tracks_view_t t, or_dimuons_view_t d, or_hists_t *h, const int32_t *trigger_bits,
                         const uint8_t *toomany, int n_events);

/* analysis hook: the YZ stage run single-threaded, recording every (u3, v3)
 * outer iteration that loads a u3 and a v3 hit (24 floats: event, slot,
 * tracklet, outer index, u3/v3 hit counts, their y, y errors and z, u2 x v2
 * combinations, x0, tx, 1 if it held the tracklet's best combination, x-hit
 * count); returns the records written (at most cap) */
int64_t orc_yz_outer_dump(const or_plane_t *p, or_hits_view_t h, or_tracks_view_t t, const uint8_t *toomany,
                          int n_events, float *buf, int64_t cap);

int orc_hardware_threads(void);

#ifdef __cplusplus
}
#endif

#endif
