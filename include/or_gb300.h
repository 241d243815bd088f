/*
 * or_gb300.h -- C ABI of the GB300 (sm_103a) online-reconstruction library.
 *
 * This is the drop-in boundary for the reference's hot path.  Each stage
 * entry point replaces one reference kernel launch of the host driver
 * (OnlineReconstruction/online_reconstruction.cu:776-894) and takes the same
 * buffers, in the same memory layout (or_layout.h), mutating them in place
 * the way the reference kernels do:
 *
 *   or_event_reduce    <- gkernel_eR<<<N,8>>>                 reconstruction_kernels.cuh:8
 *   or_xz              <- gKernel_XZ_tracking<<<N,32>>>        reconstruction_kernels.cuh:182
 *   or_yz              <- gKernel_YZ_tracking<<<N,32>>>        reconstruction_kernels.cuh:864
 *   or_back_clean      <- gKernel_BackTrackCleaning<<<N,32>>> and
 *                         gKernel_BackTrackCleaning_crossthreads<<<N,32>>>
 *                                                              reconstruction_helper.cuh:1789, :1846
 *   or_global          <- gKernel_Global_tracking<<<N,32>>>    reconstruction_kernels.cuh:1841
 *   or_run_batch       <- the whole launch chain above
 *
 * All pointers inside the views are DEVICE pointers unless the name of the
 * call says _host.  `stream` is a cudaStream_t passed as void* (NULL = the
 * legacy default stream).  Calls are asynchronous on that stream, like the
 * kernel launches they replace, except where noted.
 *
 * Per-event outcome: `toomany` (uint8, one per event) is the reference's
 * gEvent::HasTooManyHits, set by the event reducer on station multiplicity,
 * by XZ on bin overflow or tracklet-storage exhaustion.  Events with it set
 * are skipped by the later stages, as in the reference.
 *
 * Every call returns an or_status_t.  Argument errors are detected on the
 * host before any launch; CUDA errors are reported as OR_ERR_CUDA with the
 * message available from or_last_error().
 */
#ifndef OR_GB300_H
#define OR_GB300_H

#include "or_layout.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef enum or_status {
    OR_OK = 0,
    OR_ERR_ARG = 1,      /* bad pointer, count or size */
    OR_ERR_CUDA = 2,     /* a CUDA call failed; see or_last_error() */
    OR_ERR_IO = 3,       /* geometry file missing or unreadable */
    OR_ERR_NOMEM = 4,    /* device allocation failed */
    OR_ERR_CAPACITY = 5, /* an input exceeds a fixed capacity */
    OR_ERR_TIMEOUT = 6,  /* a bounded device wait gave up */
    OR_ERR_NOGEOM = 7    /* no geometry set on the context */
} or_status_t;

typedef struct or_ctx or_ctx_t;

/* Tunable launch shapes (or_set_launch): events -- or, for the dynamically
 * scheduled YZ and global kernels, work units -- per CTA, one warp each,
 * so CTAs of 32 to 512 threads.  Results do not depend on them. */
typedef enum or_kernel_id {
    OR_K_EVENT_REDUCE = 0,
    OR_K_XZ = 1, /* at most 8 */
    OR_K_YZ = 2,
    OR_K_BACK_CLEAN = 3,
    OR_K_GLOBAL = 4,
    OR_K_SELECT = 5,
    OR_K_FEATURES = 6,
    OR_K_COUNT = 7
} or_kernel_id_t;

/* Library version string and the CUDA arch it was built for. */
const char *or_version(void);
/* Text of the most recent error on this thread. */
const char *or_last_error(void);
const char *or_status_string(int status);

/* Geometry: parse the plain-text geometry table (online_reconstruction.cu
 * :123-188) and compute wire positions (:191-218).  wire_pos may be NULL;
 * otherwise it must hold OR_NDET*OR_WIREPOS_STRIDE doubles.  Host only. */
int or_geometry_load(const char *path, or_plane_t *plane, double *wire_pos);

/* Context: one per device.  or_create() selects `device` and allocates the
 * context's device state: the geometry, error words, and the YZ scratch
 * (work queue, per-warp arenas and survivor queues, the 6 GB survivor pool of
 * the split YZ path and the 2.25 GiB of window images: about 10.8 GB in all,
 * sized for 100,000-event batches of the uneven workload). */
int or_create(int device, or_ctx_t **out);
/* or_create() with the YZ queue, survivor pool and window images sized for
 * batches of at most `max_events` events (0, or 100,000 and above: the
 * or_create() sizes): about 1.4 GB at 10,000 events.  Larger batches stay
 * correct -- work that does not fit the queue is evaluated in the planning
 * pass, survivors that do not fit the pool on the combined path -- and only
 * lose speed.  OR_ERR_ARG for max_events < 0. */
int or_create_sized(int device, int max_events, or_ctx_t **out);
/* Device bytes or_create_sized(max_events) allocates on a GPU with
 * `sm_count` SMs (0 for max_events < 0 or sm_count <= 0).  Host only. */
size_t or_context_bytes(int max_events, int sm_count);
int or_destroy(or_ctx_t *ctx);
/* Events per CTA of `kernel` (1, 2, 4, 8 or 16; default 4), e.g. as chosen by
 * the autotuner (orgpu/autotune.py); or_get_launch returns the current one. */
int or_set_launch(or_ctx_t *ctx, int kernel, int events_per_cta);
int or_get_launch(or_ctx_t *ctx, int kernel);
/* The YZ stage runs as a first-cut kernel that keeps each work unit's
 * surviving combinations, in order, in a survivor pool of the context, and a
 * second kernel that evaluates them; a unit whose survivors do not fit runs
 * whole in the second kernel, with the same results.  Limit the pool to
 * `entries` survivors (< 0: the whole pool, 192 Mi).  A tuning and test
 * knob: results do not depend on it. */
int or_set_yz_pool_limit(or_ctx_t *ctx, int64_t entries);
/* Copy a host or_plane_t to the device (online_reconstruction.cu:754). */
int or_set_geometry(or_ctx_t *ctx, const or_plane_t *plane);
/* Wait for `stream` and report the device-side error words raised since the
 * last call: OR_ERR_TIMEOUT when a bounded bulk-copy wait gave up,
 * OR_ERR_CAPACITY when a hit window overflowed its fixed list (100 windowed
 * hits or pairs per projection in YZ, 128 pairs in global tracking; that
 * tracklet or track is left unextended), OR_ERR_ARG when the packer met an
 * event whose hit records are not sorted by (det, elem, tdc).  The error
 * words are cleared by the call.  The reference has no such report; its
 * kernels write past their arrays instead, and its host aborts on CUDA
 * errors (online_reconstruction.cu:50-64). */
int or_stream_sync(or_ctx_t *ctx, void *stream);
/* The combination scorer (no counterpart in the reference): or_yz() on the
 * same buffers, where a learned model prunes the station-3 (u3, v3) outer
 * iterations of the u3 x v3 x u2 x v2 loop (reconstruction_kernels.cuh
 * :1320-1461) before their combinations are evaluated.  For every live outer
 * iteration (both pairs give a hit in the acceptance) of every tracklet the
 * stage queues (those with more than 32 live combinations), one row of
 * OR_NFEAT features goes to `features` (16-byte aligned) and the row's
 * outer index (u3 pair + v3 pair * u3 pairs) to `outer_index`; *rows (device
 * uint32) gets the row count.  With `model`, the rows are scored on the
 * tensor cores into `scores` and an outer iteration scoring below t_keep is
 * skipped -- none of its combinations can win, and the scratch entries its
 * load attempts would leave are still set, so every kept combination is
 * evaluated exactly as in or_yz().  An event where some tracklet's rows all
 * score below t_keep but the best at or above t_unc is uncertain
 * (uncertain[e] = 1) and runs plain.  model == NULL: the rows are written
 * and nothing is pruned (the plain result, plus training rows).  Tracklets
 * whose rows do not fit in max_rows are not pruned. */
int or_yz_scored(or_ctx_t *ctx, or_hits_view_t hits, or_tracks_view_t tracks, const uint8_t *toomany, int n_events,
                 const or_mlp_t *model, float t_keep, float t_unc, float *features, int32_t *outer_index,
                 float *scores, uint32_t *rows, uint8_t *uncertain, int64_t max_rows, void *stream);
/* Labels of the rows of the last or_yz_scored() call on this context, after
 * back-track cleaning and global tracking of the same batch: 1 for the row
 * of the outer iteration holding its tracklet's best combination when that
 * tracklet ended as a global track (stationID 6), else 0. */
int or_outer_labels(or_ctx_t *ctx, or_tracks_view_t tracks, const uint8_t *toomany, const int32_t *outer_index,
                    const uint32_t *rows, int64_t max_rows, uint8_t *labels, void *stream);
/* or_run_batch() with or_yz_scored() as its YZ stage. */
int or_run_batch_scored(or_ctx_t *ctx, or_hits_view_t hits, or_tracks_view_t tracks, int32_t *ntracklets,
                        uint8_t *toomany, int n_events, const or_mlp_t *model, float t_keep, float t_unc,
                        float *features, int32_t *outer_index, float *scores, uint32_t *rows, uint8_t *uncertain,
                        int64_t max_rows, void *stream);
/* Work counters of the YZ stage, for throughput accounting.  With counting
 * enabled (or_set_yz_work_counting(ctx, 1); off by default, as it costs
 * about 2 % of the stage), each or_yz() / or_yz_pruned() call on this
 * context counts, and or_yz_work_counts() returns the last call's:
 * counts[0] = combinations that reached the first y fit (fit_2D_track,
 * reconstruction_kernels.cuh:1602), counts[1] = the sum of their hit
 * counts, counts[2] = combinations that passed its 2-sigma cut (:1611) and
 * went on to the left/right resolution and gates.  or_yz_work_counts() is
 * synchronous: call it after or_stream_sync() on the stream that ran the
 * stage.  No counterpart in the reference. */
int or_set_yz_work_counting(or_ctx_t *ctx, int enabled);
int or_yz_work_counts(or_ctx_t *ctx, int64_t counts[3]);
/* Self-test of the bounded device waits: launches one warp that waits on a
 * shared-memory mbarrier nothing arrives at (no bulk copy targets it) for at
 * most `polls` polls (1..1000000).  The wait runs out and raises the same
 * error word as a bulk-copy wait of the event reducer that gave up, so the
 * next or_stream_sync() returns OR_ERR_TIMEOUT; the context stays usable.
 * No counterpart in the reference, which has no bounded waits. */
int or_selftest_bounded_wait(or_ctx_t *ctx, int polls, void *stream);

/* Stage entry points on device buffers (see the table above). */
int or_event_reduce(or_ctx_t *ctx, or_hits_view_t hits, uint8_t *toomany, int n_events, void *stream);
int or_xz(or_ctx_t *ctx, or_hits_view_t hits, or_tracks_view_t tracks, int32_t *ntracklets, uint8_t *toomany,
          int n_events, void *stream);
int or_yz(or_ctx_t *ctx, or_hits_view_t hits, or_tracks_view_t tracks, const uint8_t *toomany, int n_events,
          void *stream);
int or_back_clean(or_ctx_t *ctx, or_tracks_view_t tracks, const uint8_t *toomany, int n_events, void *stream);
int or_global(or_ctx_t *ctx, or_hits_view_t hits, or_tracks_view_t tracks, const uint8_t *toomany, int n_events,
              void *stream);
/* The five stages in the reference order, one call. */
int or_run_batch(or_ctx_t *ctx, or_hits_view_t hits, or_tracks_view_t tracks, int32_t *ntracklets,
                 uint8_t *toomany, int n_events, void *stream);

/* Post-global selection (online_reconstruction.cu:914-933), after or_global:
 *   or_prop_matching  <- gKernel_PropSegmentMatching     reconstruction_helper.cuh:1916
 *                        (every track without an x and a y prop-tube segment
 *                        agreeing with it gets stationID 5)
 *   or_global_clean   <- gKernel_GlobalTrackCleaning and ..._crossthreads  :2289, :2333
 *                        (chi2/ndf and same-charge momentum duplicates)
 *   or_run_selection  <- both, one launch. */
int or_prop_matching(or_ctx_t *ctx, or_hits_view_t hits, or_tracks_view_t tracks, const uint8_t *toomany,
                     int n_events, void *stream);
int or_global_clean(or_ctx_t *ctx, or_tracks_view_t tracks, const uint8_t *toomany, int n_events, void *stream);
int or_run_selection(or_ctx_t *ctx, or_hits_view_t hits, or_tracks_view_t tracks, const uint8_t *toomany,
                     int n_events, void *stream);

/* After the selection (online_reconstruction.cu:939-983), reconstruction_kernels.cuh:
 *   or_vertexing        <- gKernel_Vertexing (tracks, z, flags)                     :2542
 *                          stationID >= 6 tracks swum back through FMag in double:
 *                          stationID 7, vertex position and momentum
 *   or_dimuons          <- gKernel_DimuonBuilding (tracks, dimuons, z, flags)       :2820
 *                          opposite-charge pairs of vertexed tracks, closest
 *                          approach, kinematics, cuts; ndimuons written for every
 *                          accepted event
 *   or_fill_histograms  <- gKernel_fill_display_histograms (tracks, dimuons,
 *                          hists, trigger bits, flags)                             :3100
 *                          adds exact counts into d_hists->values (device
 *                          memory); trigger_bits may be NULL (all zero)
 *   or_hist_table_init     the host's table setup (online_reconstruction.cu:670-723)
 *                          into host memory, values zeroed
 *   or_run_physics         the three kernels in order; d_hists may be NULL. */
int or_vertexing(or_ctx_t *ctx, or_tracks_view_t tracks, const uint8_t *toomany, int n_events, void *stream);
int or_dimuons(or_ctx_t *ctx, or_tracks_view_t tracks, or_dimuons_view_t dimuons, const uint8_t *toomany,
               int n_events, void *stream);
int or_fill_histograms(or_ctx_t *ctx, or_tracks_view_t tracks, or_dimuons_view_t dimuons,
                       const int32_t *trigger_bits, const uint8_t *toomany, or_hists_t *d_hists, int n_events,
                       void *stream);
void or_hist_table_init(or_hists_t *host_table);
int or_run_physics(or_ctx_t *ctx, or_tracks_view_t tracks, or_dimuons_view_t dimuons, const int32_t *trigger_bits,
                   const uint8_t *toomany, or_hists_t *d_hists, int n_events, void *stream);

/* The reference's per-event output (the host loop online_reconstruction.cu:
 * 1063-1222 that fills ORoutput_tree, OROutput.h:25-102) as row tables in
 * device memory (or_output_view_t), events in batch order: events with raw
 * hits (raw_hits[e] > 0; NULL: every event) and no reject flag; every reduced
 * hit; the tracks with stationID >= min_stid (7 in the reference build) and
 * their hits; the dimuons.  event_ids may be NULL (the batch index is used).
 * out.counts[0..4] receives the rows each table needs (events, hits, tracks,
 * track hits, dimuons); rows beyond a table's capacity are not written, so a
 * caller compares counts with capacities after the stream completes. */
int or_output_rows(or_ctx_t *ctx, or_hits_view_t hits, or_tracks_view_t tracks, or_dimuons_view_t dimuons,
                   const uint8_t *toomany, const int32_t *raw_hits, const int32_t *event_ids, float min_stid,
                   or_output_view_t out, int n_events, void *stream);

/* Map the reference's fixed-capacity structs (EstnEvtMax = 10000 events)
 * onto views.  `coll` points at a gEventHitCollections / gEventTrackCollection
 * laid out exactly as reconstruction_classes.cuh:76-87 / :542-544. */
or_hits_view_t or_hits_view_from_collection(void *coll);
or_tracks_view_t or_tracks_view_from_collection(void *coll);
/* Bytes of the views for n_events events. */
size_t or_hits_view_bytes(int n_events);
size_t or_tracks_view_bytes(int n_events);

/* Device-side packer: compact hit records (det, elem, tdc, drift, flag),
 * sorted by (det, elem, tdc) inside each event, into the reference hit
 * layout, with pos = (float)wire_pos[det][elem] (online_reconstruction.cu
 * :589-636).  rec_offsets[e]..rec_offsets[e+1] are event e's records.
 * wire_pos_f is a device float table [OR_NDET*OR_WIREPOS_STRIDE].  Records
 * with det outside 1..54 (they sort first or last) are skipped, an elem
 * outside the wire table gives pos 0, and hits past a plane's slot capacity
 * are dropped.  An event whose records are out of order is reported by the
 * next or_stream_sync() as OR_ERR_ARG; its slots are then undefined, but no
 * write leaves them. */
int or_pack_hits(or_ctx_t *ctx, const or_hit_record_t *records, const int64_t *rec_offsets, int n_events,
                 const float *wire_pos_f, or_hits_view_t hits, void *stream);

/* R-T calibration (online_reconstruction.cu:220-242): parse the calibration
 * file and build every listed chamber / prop-tube plane's clamped cubic
 * spline into *rt (host memory, or_rt_table_bytes() bytes); cellwidth comes
 * from `plane`.  *nplanes_out (may be NULL) receives the number of planes
 * that got a profile.  Host only. */
int or_rt_load(const char *path, const or_plane_t *plane, or_rt_table_t *rt, int *nplanes_out);
/* Build one plane's profile from n points (t strictly increasing, n <=
 * OR_RT_MAXKNOTS); det must be a chamber (1..30) or prop-tube (47..54) plane. */
int or_rt_set_plane(or_rt_table_t *rt, int det, int n, const double *t, const double *r, float tmin, float tmax,
                    float cellwidth);
size_t or_rt_table_bytes(void);

/* or_pack_hits with the drift distance taken from the R-T calibration
 * instead of the record (online_reconstruction.cu:387-396): on a chamber or
 * prop-tube plane with a profile, tdc < tmin gives cellwidth/2, tdc > tmax
 * gives 0, otherwise (float)R(tdc).  rt_dev: an or_rt_table_t in device
 * memory.  Hodoscope hits and planes without a profile keep the record's. */
int or_pack_hits_rt(or_ctx_t *ctx, const or_hit_record_t *records, const int64_t *rec_offsets, int n_events,
                    const float *wire_pos_f, const or_rt_table_t *rt_dev, or_hits_view_t hits, void *stream);
/* The same conversion in place on hits already in the reference layout
 * (packed by a reference-style host, online_reconstruction.cu:406-417):
 * every chamber and prop-tube hit's drift field from its tdc field. */
int or_rt_apply(or_ctx_t *ctx, const or_rt_table_t *rt_dev, or_hits_view_t hits, int n_events, void *stream);

/* Gather the tracks whose stationID equals `stid` (6 = global tracks) into
 * `out`, OR_COLLECT_STRIDE floats per row: [event, slot*16 + position,
 * 148-float record].  *d_count (device, uint64) receives the number of
 * matching tracks; rows past `capacity` are counted but not written.  Rows of
 * different thread blocks come in no fixed order.  Replaces the host walk of
 * the copied-back collections (online_reconstruction.cu:1023-1224). */
int or_collect_tracks(or_ctx_t *ctx, or_tracks_view_t tracks, const uint8_t *toomany, int n_events, float stid,
                      float *out, int64_t capacity, uint64_t *d_count, void *stream);

/* ---- learned tracklet scorer (no counterpart in the reference) ----------
 *
 * A 16-64-64-1 MLP (or_mlp_t, BF16 weights and activations, FP32 sums)
 * scores every XZ tracklet; the YZ combinatorics of low-scoring tracklets
 * are skipped.  Rows: tracklet r of event e is row row_off[e] + its rank in
 * the event (slots in order, tracklets in slot order); flagged events own no
 * rows; row_off has n_events+1 entries, row_off[n_events] = total rows.
 * Buffers of max_rows rows: rows past max_rows get no features or scores
 * and are always kept. */
int or_tracklet_rows(or_ctx_t *ctx, or_tracks_view_t tracks, const uint8_t *toomany, int n_events, int32_t *row_off,
                     void *stream);
/* OR_NFEAT floats per row (16-byte aligned): x0/100, 10 tx, err_x0,
 * 100 err_tx, log1p(hits in the eight u/v planes), x-hit count, station-3
 * half, log1p of the windowed and of the accepted u2, v2, u3, v3 hits, and
 * the sum of the last four logs. */
int or_tracklet_features(or_ctx_t *ctx, or_hits_view_t hits, or_tracks_view_t tracks, const uint8_t *toomany,
                         int n_events, const int32_t *row_off, float *features, int64_t max_rows, void *stream);
/* Scores (sigmoid outputs) of n_rows feature rows on the tensor cores
 * (tcgen05, 128 rows per tile). */
int or_mlp_score(or_ctx_t *ctx, const or_mlp_t *model, const float *features, int64_t n_rows, float *scores,
                 void *stream);
/* keep[r] = score >= t_keep, except that an event with any score in
 * [t_unc, t_keep) keeps all of its rows (it is re-run plain). */
int or_keep_mask(or_ctx_t *ctx, const float *scores, const int32_t *row_off, int n_events, float t_keep, float t_unc,
                 uint8_t *keep, int64_t max_rows, void *stream);
/* or_yz with the keep flags: a pruned tracklet is left as one no
 * combination extends (stationID 3); kept tracklets get or_yz's result. */
int or_yz_pruned(or_ctx_t *ctx, or_hits_view_t hits, or_tracks_view_t tracks, const uint8_t *toomany, int n_events,
                 const int32_t *row_off, const uint8_t *keep, int64_t max_rows, void *stream);
/* or_run_batch with the scorer between XZ and YZ; the row count stays on the
 * device. */
int or_run_batch_learned(or_ctx_t *ctx, or_hits_view_t hits, or_tracks_view_t tracks, int32_t *ntracklets,
                         uint8_t *toomany, int n_events, const or_mlp_t *model, float t_keep, float t_unc,
                         int32_t *row_off, float *features, float *scores, uint8_t *keep, int64_t max_rows,
                         void *stream);
/* Training labels: 1 for the rows whose tracklet ended as a global track
 * (stationID 6) in the run that left `tracks`. */
int or_tracklet_labels(or_ctx_t *ctx, or_tracks_view_t tracks, const uint8_t *toomany, int n_events,
                       const int32_t *row_off, uint8_t *labels, int64_t max_rows, void *stream);
/* Recall of run b against run a on the same events: counts[0] = global
 * tracks of a, counts[1] = those with the identical record in b, counts[2] =
 * global tracks of b (device uint64[3]). */
int or_track_agreement(or_ctx_t *ctx, or_tracks_view_t tracks_a, or_tracks_view_t tracks_b, const uint8_t *toomany,
                       int n_events, uint64_t *counts, void *stream);
/* Training (CUDA cores, same rounding points as or_mlp_score): forward of the
 * rows idx[0..n); per-block partial gradients of the mean weighted binary
 * cross-entropy over a batch (or_mlp_grad_blocks(batch) blocks of
 * OR_MLP_NPARAM floats, parameter order w1, b1, w2, b2, w3, b3) and per-block
 * loss sums; an Adam step on the FP32 parameters that also refreshes the
 * model's BF16 copies. */
int or_mlp_grad_blocks(int batch);
int or_mlp_forward(or_ctx_t *ctx, const or_mlp_t *model, const float *features, const int64_t *idx, int n,
                   float *prob, void *stream);
int or_mlp_gradient(or_ctx_t *ctx, const or_mlp_t *model, const float *features, const uint8_t *labels,
                    const int64_t *idx, int batch, float pos_weight, float *grad_part, float *loss_part, void *stream);
int or_mlp_adam(or_ctx_t *ctx, float *param, float *m1, float *m2, const float *grad_part, int nblocks, int step,
                float lr, float beta1, float beta2, float eps, or_mlp_t *model, void *stream);

/* YZ tracklet stage that allocates nothing and needs no context.  This entry
 * point has no counterpart in the reference, whose host code allocates all of
 * its device memory up front (online_reconstruction.cu:738-744).
 *
 * It is for callers that cannot allocate device memory when they call: a
 * trigger or serving process that gives all free HBM to its own pool at
 * start-up (or_create() would need about 10.8 GB for its YZ scratch), or
 * a latency-critical loop that must not call cudaMalloc/cudaFree because they
 * synchronise the device.  Results are those of or_yz() on the same buffers.
 *
 *   d_plane  device copy of the geometry (sizeof(or_plane_t) bytes, owned by
 *            the caller);
 *   d_errw   device uint32 owned by the caller; OR_ERRW_CAPACITY is OR'ed
 *            into it when a hit window overflowed (the tracklet is left
 *            unextended; or_stream_sync() reports the same event for or_yz()
 *            as OR_ERR_CAPACITY);
 *   other arguments as or_yz().
 *
 * Scratch: a static device array of OR_YZ_NOALLOC_SCRATCH_BYTES per device,
 * reserved by the CUDA runtime when the library's module is loaded.  The
 * first call on a device, with that device current, looks its address up
 * (cudaGetSymbolAddress) and caches it: make that first call before any
 * stream capture.  The cached address belongs to the device's context of
 * that moment: after cudaDeviceReset() the module is loaded again and the
 * array may move, so a process that resets a device must not call
 * or_yz_noalloc() on it again.  Each call clears the queue counters on
 * `stream`.
 * Calls that overlap on one device (several streams or host threads) share
 * the array and race: serialise them.
 *
 * n_events above OR_YZ_NOALLOC_MAX_EVENTS (the reference's batch, EstnEvtMax
 * in reconstruction_constants.h:20) returns OR_ERR_CAPACITY before any launch;
 * a current device whose index is above the library's per-device table
 * (64 devices) returns OR_ERR_ARG.
 *
 * Its work queue is smaller than a context's (65,536 units and 16,384 heavy
 * tracklets, against 4 Mi and 2 Mi): on large, busy batches a tracklet that
 * finds the queue full is evaluated by its planning warp, which gives the
 * same result more slowly. */
#define OR_YZ_NOALLOC_MAX_EVENTS 10000
#define OR_ERRW_CAPACITY 2u
#define OR_YZ_NOALLOC_SCRATCH_BYTES (56u << 20)
int or_yz_noalloc(const or_plane_t *d_plane, or_hits_view_t hits, or_tracks_view_t tracks, const uint8_t *toomany,
                  int n_events, uint32_t *d_errw, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* OR_GB300_H */
