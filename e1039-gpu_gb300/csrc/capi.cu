// capi.cu -- the C ABI of the library (include/or_gb300.h): context,
// argument checks, stage launches, error reporting.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>

#include <mutex>

#include "../../include/or_dropin.h"
#include "../../include/or_gb300.h"
#include "or_device.cuh"

namespace orgpu {
cudaError_t launch_event_reduce(or_hits_view_t, uint8_t *, int, uint32_t *, cudaStream_t, int, int);
cudaError_t launch_xz(const or_plane_t *, or_hits_view_t, or_tracks_view_t, int32_t *, uint8_t *, int, cudaStream_t,
                      int, int);
cudaError_t launch_yz_tuned(const or_plane_t *, or_hits_view_t, or_tracks_view_t, const uint8_t *, int, uint32_t *,
                            void *, int, int, int, cudaStream_t, int, int, long long, int);
cudaError_t launch_yz(const or_plane_t *, or_hits_view_t, or_tracks_view_t, const uint8_t *, int, uint32_t *, void *,
                      int, int, int, cudaStream_t, int);
size_t yz_scratch_bytes_ctx(int, int, int);
size_t output_scratch_bytes(int);
cudaError_t launch_output_rows(or_hits_view_t, or_tracks_view_t, or_dimuons_view_t, const uint8_t *, const int32_t *,
                               const int32_t *, float, or_output_view_t, int, void *, cudaStream_t, int);
cudaError_t launch_vertexing(const or_plane_t *, or_tracks_view_t, const uint8_t *, int, cudaStream_t, int);
cudaError_t launch_dimuons(const or_plane_t *, or_tracks_view_t, or_dimuons_view_t, const uint8_t *, int,
                           cudaStream_t, int);
cudaError_t launch_histograms(or_tracks_view_t, or_dimuons_view_t, const int32_t *, const uint8_t *, or_hists_t *,
                              int, cudaStream_t, int);
cudaError_t launch_back_clean(or_tracks_view_t, const uint8_t *, int, cudaStream_t, int, int);
cudaError_t launch_global(const or_plane_t *, or_hits_view_t, or_tracks_view_t, const uint8_t *, int, uint32_t *,
                          unsigned long long *, cudaStream_t, int, int);
cudaError_t launch_pack(const or_hit_record_t *, const int64_t *, int, const float *, const or_rt_table_t *,
                        or_hits_view_t, uint32_t *, cudaStream_t, int);
cudaError_t launch_wait_selftest(uint32_t *, uint32_t, cudaStream_t);
cudaError_t yz_read_counts(const void *, long long[3]);
cudaError_t launch_yz_scored(const or_plane_t *, or_hits_view_t, or_tracks_view_t, const uint8_t *, int, uint32_t *,
                             void *, int, int, int, cudaStream_t, int, const or_mlp_t *, float, float, float *,
                             int32_t *, float *, uint32_t *, uint8_t *, long, int, long long, int);
cudaError_t launch_yz_outer_labels(void *, int, int, int, or_tracks_view_t, const uint8_t *, const int32_t *,
                                   const uint32_t *, long, uint8_t *, cudaStream_t, int);
cudaError_t launch_rt_apply(const or_rt_table_t *, or_hits_view_t, int, cudaStream_t, int);
cudaError_t launch_collect(or_tracks_view_t, const uint8_t *, int, float, float *, long long, unsigned long long *,
                           cudaStream_t);
cudaError_t launch_yz_pruned(const or_plane_t *, or_hits_view_t, or_tracks_view_t, const uint8_t *, int, uint32_t *,
                             void *, int, int, int, cudaStream_t, int, const int32_t *, const uint8_t *, long, int,
                             long long, int);
cudaError_t launch_rows(const uint16_t *, const uint8_t *, int, int32_t *, cudaStream_t);
cudaError_t launch_features(const or_plane_t *, or_hits_view_t, or_tracks_view_t, const uint8_t *, int,
                            const int32_t *, float *, long, cudaStream_t, int, int);
cudaError_t launch_keep(const float *, const int32_t *, int, float, float, uint8_t *, long, cudaStream_t, int);
cudaError_t launch_mlp_score(const or_mlp_t *, const float *, long, const int32_t *, float *, uint32_t *, cudaStream_t,
                             int);
int mlp_train_blocks(int);
cudaError_t launch_select(const or_plane_t *, or_hits_view_t, or_tracks_view_t, const uint8_t *, int, int, int,
                          cudaStream_t, int, int);
cudaError_t launch_labels(or_tracks_view_t, const uint8_t *, int, const int32_t *, uint8_t *, long, cudaStream_t, int);
cudaError_t launch_agreement(or_tracks_view_t, or_tracks_view_t, const uint8_t *, int, unsigned long long *,
                             cudaStream_t, int);
cudaError_t launch_mlp_train(const or_mlp_t *, const float *, const uint8_t *, const int64_t *, int, float, float *,
                             float *, float *, cudaStream_t);
cudaError_t launch_mlp_adam(float *, float *, float *, const float *, int, int, float, float, float, float, or_mlp_t *,
                            cudaStream_t);
cudaError_t launch_yz_noalloc(const or_plane_t *, or_hits_view_t, or_tracks_view_t, const uint8_t *, int, uint32_t *,
                              cudaStream_t, const char **);
}  // namespace orgpu

struct or_ctx {
    int device;
    int sm_count;
    or_plane_t *d_plane;
    bool has_geom;
    uint32_t *d_errw;
    unsigned long long *d_sched;  // work-unit counters of the dynamically scheduled kernels
    // YZ work queue: units of heavy tracklets, their best records, overflow arenas
    void *yz_scratch;
    int yz_cap_units, yz_cap_heavy, yz_garena_warps;
    long long yz_pool_limit;  // survivor-pool entries the split YZ path may use (-1: all)
    int yz_count_work = 0;    // YZ calls add up their work counters (or_set_yz_work_counting)
    int warps[OR_K_COUNT];  // events (work units) per CTA of each tunable kernel
    // per-event row counts and offsets of or_output_rows, grown on demand
    void *out_scratch = nullptr;
    size_t out_scratch_bytes = 0;
};

namespace {
thread_local std::string g_last_error;

int fail(int status, const std::string &msg) {
    g_last_error = msg;
    return status;
}
int cuda_fail(cudaError_t e, const char *where) {
    return fail(OR_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}
inline cudaStream_t S(void *s) { return reinterpret_cast<cudaStream_t>(s); }
inline bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

int check_ctx(or_ctx_t *ctx, bool need_geom) {
    if (!ctx) return fail(OR_ERR_ARG, "null context");
    if (need_geom && !ctx->has_geom) return fail(OR_ERR_NOGEOM, "no geometry set (or_set_geometry)");
    int cur = -1;
    if (cudaGetDevice(&cur) != cudaSuccess) return fail(OR_ERR_CUDA, "cudaGetDevice failed");
    if (cur != ctx->device && cudaSetDevice(ctx->device) != cudaSuccess)
        return fail(OR_ERR_CUDA, "cudaSetDevice failed");
    return OR_OK;
}
int check_hits(const or_hits_view_t &h) {
    if (!h.nhits_cham || !h.hits_cham || !h.nhits_hodo || !h.hits_hodo || !h.nhits_prop || !h.hits_prop)
        return fail(OR_ERR_ARG, "null pointer in hits view");
    // slot images are fetched with 16-byte bulk copies
    if (!aligned16(h.hits_cham) || !aligned16(h.hits_hodo) || !aligned16(h.hits_prop))
        return fail(OR_ERR_ARG, "hit arrays must be 16-byte aligned");
    return OR_OK;
}
int check_tracks(const or_tracks_view_t &t) {
    if (!t.ntracks || !t.tracks) return fail(OR_ERR_ARG, "null pointer in tracks view");
    return OR_OK;
}
}  // namespace

extern "C" {

const char *or_version(void) { return "e1039-gb300 0.1 (sm_103a)"; }
const char *or_last_error(void) { return g_last_error.c_str(); }
const char *or_status_string(int s) {
    switch (s) {
    case OR_OK: return "ok";
    case OR_ERR_ARG: return "invalid argument";
    case OR_ERR_CUDA: return "CUDA error";
    case OR_ERR_IO: return "I/O error";
    case OR_ERR_NOMEM: return "out of device memory";
    case OR_ERR_CAPACITY: return "capacity exceeded";
    case OR_ERR_TIMEOUT: return "device wait timed out";
    case OR_ERR_NOGEOM: return "no geometry";
    default: return "unknown status";
    }
}

#ifndef OR_YZ_WARPS_SM
#define OR_YZ_WARPS_SM 16
#endif
#ifndef OR_YZ_SPLIT
#define OR_YZ_SPLIT 1
#endif
#ifndef OR_YZ_FIRST_WARPS_SM
#define OR_YZ_FIRST_WARPS_SM 28
#endif

// Room for every heavy tracklet of a 100,000-event batch of the uneven
// workload (about 0.7 M heavy tracklets, 0.75 M units), and in proportion
// for a context sized to a smaller largest batch (42 units and 21 heavy
// tracklets per event, at least 64 Ki and 32 Ki); a batch beyond it
// evaluates the excess in the planning pass, correct but without the queue's
// balance.  The survivor pool and the window images scale with the units.
static void yz_caps(int max_events, int &units, int &heavy) {
    if (max_events <= 0 || max_events >= 100000) {
        units = 1 << 22;
        heavy = 1 << 21;
    } else {
        units = std::max(1 << 16, 42 * max_events);
        heavy = std::max(1 << 15, 21 * max_events);
    }
}

// per-warp arenas and queues for the most warps a YZ kernel launches
static int yz_arena_warps(int sm_count) { return sm_count * (OR_YZ_SPLIT ? OR_YZ_FIRST_WARPS_SM : OR_YZ_WARPS_SM); }

size_t or_context_bytes(int max_events, int sm_count) {
    if (max_events < 0 || sm_count <= 0) return 0;
    int units, heavy;
    yz_caps(max_events, units, heavy);
    return sizeof(or_plane_t) + sizeof(uint32_t) + 256 +
           orgpu::yz_scratch_bytes_ctx(units, heavy, yz_arena_warps(sm_count));
}

int or_create(int device, or_ctx_t **out) { return or_create_sized(device, 0, out); }

int or_create_sized(int device, int max_events, or_ctx_t **out) {
    if (!out) return fail(OR_ERR_ARG, "null output pointer");
    if (max_events < 0) return fail(OR_ERR_ARG, "max_events must be >= 0 (0: the 100,000-event default)");
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceCount");
    if (device < 0 || device >= ndev) return fail(OR_ERR_ARG, "device index out of range");
    if ((e = cudaSetDevice(device)) != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    or_ctx_t *c = new or_ctx_t();
    c->device = device;
    c->has_geom = false;
    for (int k = 0; k < OR_K_COUNT; ++k) c->warps[k] = 4;
    if ((e = cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess) {
        delete c;
        return cuda_fail(e, "cudaDeviceGetAttribute");
    }
    if ((e = cudaMalloc(&c->d_plane, sizeof(or_plane_t))) != cudaSuccess) {
        delete c;
        return fail(OR_ERR_NOMEM, "cudaMalloc geometry");
    }
    if ((e = cudaMalloc(&c->d_errw, sizeof(uint32_t))) != cudaSuccess ||
        (e = cudaMemset(c->d_errw, 0, sizeof(uint32_t))) != cudaSuccess) {
        cudaFree(c->d_plane);
        delete c;
        return fail(OR_ERR_NOMEM, "cudaMalloc error word");
    }
    if ((e = cudaMalloc(&c->d_sched, 256)) != cudaSuccess) {
        cudaFree(c->d_plane);
        cudaFree(c->d_errw);
        delete c;
        return fail(OR_ERR_NOMEM, "cudaMalloc work counters");
    }
    yz_caps(max_events, c->yz_cap_units, c->yz_cap_heavy);
    c->yz_garena_warps = yz_arena_warps(c->sm_count);
    c->yz_pool_limit = -1;
    if ((e = cudaMalloc(&c->yz_scratch,
                        orgpu::yz_scratch_bytes_ctx(c->yz_cap_units, c->yz_cap_heavy, c->yz_garena_warps))) !=
        cudaSuccess) {
        cudaFree(c->d_plane);
        cudaFree(c->d_errw);
        cudaFree(c->d_sched);
        delete c;
        return fail(OR_ERR_NOMEM, "cudaMalloc YZ work queue");
    }
    *out = c;
    return OR_OK;
}

int or_set_yz_pool_limit(or_ctx_t *ctx, int64_t entries) {
    if (!ctx) return fail(OR_ERR_ARG, "null context");
    ctx->yz_pool_limit = entries < 0 ? -1 : (long long)entries;
    return OR_OK;
}

int or_set_launch(or_ctx_t *ctx, int kernel, int events_per_cta) {
    if (!ctx) return fail(OR_ERR_ARG, "null context");
    if (kernel < 0 || kernel >= OR_K_COUNT) return fail(OR_ERR_ARG, "unknown kernel id");
    const int w = events_per_cta;
    if (w != 1 && w != 2 && w != 4 && w != 8 && w != 16)
        return fail(OR_ERR_ARG, "events per CTA must be 1, 2, 4, 8 or 16");
    if (kernel == OR_K_XZ && w > 8) return fail(OR_ERR_ARG, "XZ takes at most 8 events per CTA (shared memory)");
    ctx->warps[kernel] = w;
    return OR_OK;
}

int or_get_launch(or_ctx_t *ctx, int kernel) {
    if (!ctx || kernel < 0 || kernel >= OR_K_COUNT) return -1;
    return ctx->warps[kernel];
}

int or_destroy(or_ctx_t *ctx) {
    if (!ctx) return OR_OK;
    cudaSetDevice(ctx->device);
    cudaFree(ctx->d_plane);
    cudaFree(ctx->d_errw);
    cudaFree(ctx->d_sched);
    cudaFree(ctx->yz_scratch);
    cudaFree(ctx->out_scratch);
    delete ctx;
    return OR_OK;
}

int or_set_geometry(or_ctx_t *ctx, const or_plane_t *plane) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (!plane) return fail(OR_ERR_ARG, "null geometry");
    cudaError_t e = cudaMemcpy(ctx->d_plane, plane, sizeof(or_plane_t), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "copy geometry");
    ctx->has_geom = true;
    return OR_OK;
}

int or_stream_sync(or_ctx_t *ctx, void *stream) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    cudaError_t e = cudaStreamSynchronize(S(stream));
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
    uint32_t w = 0;
    if ((e = cudaMemcpy(&w, ctx->d_errw, sizeof(w), cudaMemcpyDeviceToHost)) != cudaSuccess)
        return cuda_fail(e, "read error word");
    if (w) {
        cudaMemset(ctx->d_errw, 0, sizeof(uint32_t));
        if (w & orgpu::ERRW_TMA_TIMEOUT) return fail(OR_ERR_TIMEOUT, "a bounded bulk-copy wait gave up");
        if (w & orgpu::ERRW_CAPACITY)
            return fail(OR_ERR_CAPACITY, "a hit-pair window exceeded its capacity (128 pairs); tracklet skipped");
        if (w & orgpu::ERRW_INPUT)
            return fail(OR_ERR_ARG, "hit records of an event are not sorted by (det, elem, tdc); its hits are undefined");
    }
    return OR_OK;
}

int or_selftest_bounded_wait(or_ctx_t *ctx, int polls, void *stream) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (polls < 1 || polls > 1000000) return fail(OR_ERR_ARG, "polls must be in 1..1000000");
    cudaError_t e = orgpu::launch_wait_selftest(ctx->d_errw, (uint32_t)polls, S(stream));
    return e == cudaSuccess ? OR_OK : cuda_fail(e, "wait self-test launch");
}

int or_event_reduce(or_ctx_t *ctx, or_hits_view_t hits, uint8_t *toomany, int n_events, void *stream) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (n_events < 0 || !toomany) return fail(OR_ERR_ARG, "bad event count or flag array");
    if ((rc = check_hits(hits))) return rc;
    cudaError_t e = orgpu::launch_event_reduce(hits, toomany, n_events, ctx->d_errw, S(stream), ctx->sm_count,
                                               ctx->warps[OR_K_EVENT_REDUCE]);
    return e == cudaSuccess ? OR_OK : cuda_fail(e, "event reducer launch");
}

int or_xz(or_ctx_t *ctx, or_hits_view_t hits, or_tracks_view_t tracks, int32_t *ntracklets, uint8_t *toomany,
          int n_events, void *stream) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (n_events < 0 || !toomany || !ntracklets) return fail(OR_ERR_ARG, "bad event count or output arrays");
    if ((rc = check_hits(hits)) || (rc = check_tracks(tracks))) return rc;
    cudaError_t e =
        orgpu::launch_xz(ctx->d_plane, hits, tracks, ntracklets, toomany, n_events, S(stream), ctx->sm_count,
                         ctx->warps[OR_K_XZ]);
    return e == cudaSuccess ? OR_OK : cuda_fail(e, "XZ launch");
}

int or_yz(or_ctx_t *ctx, or_hits_view_t hits, or_tracks_view_t tracks, const uint8_t *toomany, int n_events,
          void *stream) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (n_events < 0 || !toomany) return fail(OR_ERR_ARG, "bad event count or flag array");
    if ((rc = check_hits(hits)) || (rc = check_tracks(tracks))) return rc;
    cudaError_t e = orgpu::launch_yz_tuned(ctx->d_plane, hits, tracks, toomany, n_events, ctx->d_errw,
                                           ctx->yz_scratch, ctx->yz_cap_units, ctx->yz_cap_heavy,
                                           ctx->yz_garena_warps, S(stream), ctx->sm_count, ctx->warps[OR_K_YZ],
                                           ctx->yz_pool_limit, ctx->yz_count_work);
    return e == cudaSuccess ? OR_OK : cuda_fail(e, "YZ launch");
}

int or_yz_scored(or_ctx_t *ctx, or_hits_view_t hits, or_tracks_view_t tracks, const uint8_t *toomany, int n_events,
                 const or_mlp_t *model, float t_keep, float t_unc, float *features, int32_t *outer_index,
                 float *scores, uint32_t *rows, uint8_t *uncertain, int64_t max_rows, void *stream) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (n_events < 0 || !toomany || !features || !outer_index || !scores || !rows || !uncertain || max_rows < 0 ||
        !aligned16(features))
        return fail(OR_ERR_ARG, "bad scored-YZ arguments (features must be 16-byte aligned)");
    if ((rc = check_hits(hits)) || (rc = check_tracks(tracks))) return rc;
    cudaError_t e = orgpu::launch_yz_scored(ctx->d_plane, hits, tracks, toomany, n_events, ctx->d_errw,
                                            ctx->yz_scratch, ctx->yz_cap_units, ctx->yz_cap_heavy,
                                            ctx->yz_garena_warps, S(stream), ctx->sm_count, model, t_keep, t_unc,
                                            features, outer_index, scores, rows, uncertain, (long)max_rows,
                                            ctx->warps[OR_K_YZ], ctx->yz_pool_limit, ctx->yz_count_work);
    return e == cudaSuccess ? OR_OK : cuda_fail(e, "scored YZ launch");
}

int or_outer_labels(or_ctx_t *ctx, or_tracks_view_t tracks, const uint8_t *toomany, const int32_t *outer_index,
                    const uint32_t *rows, int64_t max_rows, uint8_t *labels, void *stream) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (!toomany || !outer_index || !rows || !labels || max_rows < 0) return fail(OR_ERR_ARG, "bad label arguments");
    if ((rc = check_tracks(tracks))) return rc;
    cudaError_t e = cudaMemsetAsync(labels, 0, (size_t)max_rows, S(stream));
    if (e != cudaSuccess) return cuda_fail(e, "clear labels");
    e = orgpu::launch_yz_outer_labels(ctx->yz_scratch, ctx->yz_cap_units, ctx->yz_cap_heavy, ctx->yz_garena_warps,
                                      tracks, toomany, outer_index, rows, (long)max_rows, labels, S(stream),
                                      ctx->sm_count);
    return e == cudaSuccess ? OR_OK : cuda_fail(e, "label launch");
}

int or_run_batch_scored(or_ctx_t *ctx, or_hits_view_t hits, or_tracks_view_t tracks, int32_t *ntracklets,
                        uint8_t *toomany, int n_events, const or_mlp_t *model, float t_keep, float t_unc,
                        float *features, int32_t *outer_index, float *scores, uint32_t *rows, uint8_t *uncertain,
                        int64_t max_rows, void *stream) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (n_events < 0 || !toomany || !ntracklets) return fail(OR_ERR_ARG, "bad event count or output arrays");
    if ((rc = check_hits(hits)) || (rc = check_tracks(tracks))) return rc;
    cudaError_t e = cudaMemsetAsync(ntracklets, 0, sizeof(int32_t) * (size_t)n_events, S(stream));
    if (e != cudaSuccess) return cuda_fail(e, "clear tracklet counts");
    if ((rc = or_event_reduce(ctx, hits, toomany, n_events, stream))) return rc;
    if ((rc = or_xz(ctx, hits, tracks, ntracklets, toomany, n_events, stream))) return rc;
    if ((rc = or_yz_scored(ctx, hits, tracks, toomany, n_events, model, t_keep, t_unc, features, outer_index, scores,
                           rows, uncertain, max_rows, stream)))
        return rc;
    if ((rc = or_back_clean(ctx, tracks, toomany, n_events, stream))) return rc;
    return or_global(ctx, hits, tracks, toomany, n_events, stream);
}

int or_set_yz_work_counting(or_ctx_t *ctx, int enabled) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    ctx->yz_count_work = enabled ? 1 : 0;
    return OR_OK;
}

int or_yz_work_counts(or_ctx_t *ctx, int64_t counts[3]) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (!counts) return fail(OR_ERR_ARG, "null counts");
    long long c[3];
    cudaError_t e = orgpu::yz_read_counts(ctx->yz_scratch, c);
    if (e != cudaSuccess) return cuda_fail(e, "read YZ work counters");
    for (int i = 0; i < 3; ++i) counts[i] = (int64_t)c[i];
    return OR_OK;
}

int or_yz_noalloc(const or_plane_t *d_plane, or_hits_view_t hits, or_tracks_view_t tracks, const uint8_t *toomany,
                  int n_events, uint32_t *d_errw, void *stream) {
    if (n_events < 0) return fail(OR_ERR_ARG, "or_yz_noalloc: negative event count");
    if (n_events > OR_YZ_NOALLOC_MAX_EVENTS)
        return fail(OR_ERR_CAPACITY, "or_yz_noalloc: " + std::to_string(n_events) +
                                         " events exceed its static scratch limit of " +
                                         std::to_string(OR_YZ_NOALLOC_MAX_EVENTS) +
                                         " events per call; split the batch or use or_yz");
    if (!d_plane || !toomany || !d_errw) return fail(OR_ERR_ARG, "or_yz_noalloc: null geometry, flag or error word");
    int rc;
    if ((rc = check_hits(hits)) || (rc = check_tracks(tracks))) return rc;
    const char *why = nullptr;
    cudaError_t e = orgpu::launch_yz_noalloc(d_plane, hits, tracks, toomany, n_events, d_errw, S(stream), &why);
    if (e == cudaSuccess) return OR_OK;
    // a device outside the per-device table is an argument error (splitting
    // the batch would not help); a static area smaller than its queue is one
    // of capacity
    if (why) return fail(e == cudaErrorInvalidDevice ? OR_ERR_ARG : OR_ERR_CAPACITY, std::string("or_yz_noalloc: ") + why);
    return cuda_fail(e, "or_yz_noalloc");
}

int or_back_clean(or_ctx_t *ctx, or_tracks_view_t tracks, const uint8_t *toomany, int n_events, void *stream) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (n_events < 0 || !toomany) return fail(OR_ERR_ARG, "bad event count or flag array");
    if ((rc = check_tracks(tracks))) return rc;
    cudaError_t e =
        orgpu::launch_back_clean(tracks, toomany, n_events, S(stream), ctx->sm_count, ctx->warps[OR_K_BACK_CLEAN]);
    return e == cudaSuccess ? OR_OK : cuda_fail(e, "cleaning launch");
}

int or_global(or_ctx_t *ctx, or_hits_view_t hits, or_tracks_view_t tracks, const uint8_t *toomany, int n_events,
              void *stream) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (n_events < 0 || !toomany) return fail(OR_ERR_ARG, "bad event count or flag array");
    if ((rc = check_hits(hits)) || (rc = check_tracks(tracks))) return rc;
    cudaError_t e =
        orgpu::launch_global(ctx->d_plane, hits, tracks, toomany, n_events, ctx->d_errw, ctx->d_sched, S(stream),
                             ctx->sm_count, ctx->warps[OR_K_GLOBAL]);
    return e == cudaSuccess ? OR_OK : cuda_fail(e, "global tracking launch");
}

int or_run_batch(or_ctx_t *ctx, or_hits_view_t hits, or_tracks_view_t tracks, int32_t *ntracklets,
                 uint8_t *toomany, int n_events, void *stream) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (n_events < 0 || !toomany || !ntracklets) return fail(OR_ERR_ARG, "bad event count or output arrays");
    if ((rc = check_hits(hits)) || (rc = check_tracks(tracks))) return rc;
    cudaError_t e = cudaMemsetAsync(ntracklets, 0, sizeof(int32_t) * (size_t)n_events, S(stream));
    if (e != cudaSuccess) return cuda_fail(e, "clear tracklet counts");
    if ((rc = or_event_reduce(ctx, hits, toomany, n_events, stream))) return rc;
    if ((rc = or_xz(ctx, hits, tracks, ntracklets, toomany, n_events, stream))) return rc;
    if ((rc = or_yz(ctx, hits, tracks, toomany, n_events, stream))) return rc;
    if ((rc = or_back_clean(ctx, tracks, toomany, n_events, stream))) return rc;
    return or_global(ctx, hits, tracks, toomany, n_events, stream);
}

/* ---- post-global selection ---------------------------------------------- */

int or_prop_matching(or_ctx_t *ctx, or_hits_view_t hits, or_tracks_view_t tracks, const uint8_t *toomany,
                     int n_events, void *stream) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (n_events < 0 || !toomany) return fail(OR_ERR_ARG, "bad event count or flag array");
    if ((rc = check_hits(hits)) || (rc = check_tracks(tracks))) return rc;
    cudaError_t e = orgpu::launch_select(ctx->d_plane, hits, tracks, toomany, n_events, 1, 0, S(stream), ctx->sm_count,
                                         ctx->warps[OR_K_SELECT]);
    return e == cudaSuccess ? OR_OK : cuda_fail(e, "prop segment matching");
}

int or_global_clean(or_ctx_t *ctx, or_tracks_view_t tracks, const uint8_t *toomany, int n_events, void *stream) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (n_events < 0 || !toomany) return fail(OR_ERR_ARG, "bad event count or flag array");
    if ((rc = check_tracks(tracks))) return rc;
    or_hits_view_t none;
    std::memset(&none, 0, sizeof(none));
    cudaError_t e = orgpu::launch_select(ctx->d_plane, none, tracks, toomany, n_events, 0, 1, S(stream), ctx->sm_count,
                                         ctx->warps[OR_K_SELECT]);
    return e == cudaSuccess ? OR_OK : cuda_fail(e, "global track cleaning");
}

int or_run_selection(or_ctx_t *ctx, or_hits_view_t hits, or_tracks_view_t tracks, const uint8_t *toomany,
                     int n_events, void *stream) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (n_events < 0 || !toomany) return fail(OR_ERR_ARG, "bad event count or flag array");
    if ((rc = check_hits(hits)) || (rc = check_tracks(tracks))) return rc;
    cudaError_t e = orgpu::launch_select(ctx->d_plane, hits, tracks, toomany, n_events, 1, 1, S(stream), ctx->sm_count,
                                         ctx->warps[OR_K_SELECT]);
    return e == cudaSuccess ? OR_OK : cuda_fail(e, "post-global selection");
}

/* ---- vertexing, dimuons, histograms ------------------------------------ */

static int check_dimuons(or_dimuons_view_t d) {
    if (!d.ndimuons || !d.dimuons) return fail(OR_ERR_ARG, "null dimuon view pointer");
    return OR_OK;
}

int or_vertexing(or_ctx_t *ctx, or_tracks_view_t tracks, const uint8_t *toomany, int n_events, void *stream) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (n_events < 0 || !toomany) return fail(OR_ERR_ARG, "bad event count or flag array");
    if ((rc = check_tracks(tracks))) return rc;
    cudaError_t e = orgpu::launch_vertexing(ctx->d_plane, tracks, toomany, n_events, S(stream), ctx->sm_count);
    return e == cudaSuccess ? OR_OK : cuda_fail(e, "vertexing");
}

int or_dimuons(or_ctx_t *ctx, or_tracks_view_t tracks, or_dimuons_view_t dimuons, const uint8_t *toomany,
               int n_events, void *stream) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (n_events < 0 || !toomany) return fail(OR_ERR_ARG, "bad event count or flag array");
    if ((rc = check_tracks(tracks)) || (rc = check_dimuons(dimuons))) return rc;
    cudaError_t e = orgpu::launch_dimuons(ctx->d_plane, tracks, dimuons, toomany, n_events, S(stream), ctx->sm_count);
    return e == cudaSuccess ? OR_OK : cuda_fail(e, "dimuon building");
}

int or_fill_histograms(or_ctx_t *ctx, or_tracks_view_t tracks, or_dimuons_view_t dimuons,
                       const int32_t *trigger_bits, const uint8_t *toomany, or_hists_t *d_hists, int n_events,
                       void *stream) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (n_events < 0 || !toomany || !d_hists) return fail(OR_ERR_ARG, "bad event count, flags or histogram table");
    if ((rc = check_tracks(tracks)) || (rc = check_dimuons(dimuons))) return rc;
    cudaError_t e = orgpu::launch_histograms(tracks, dimuons, trigger_bits, toomany, d_hists, n_events, S(stream),
                                             ctx->sm_count);
    return e == cudaSuccess ? OR_OK : cuda_fail(e, "histogram fill");
}

void or_hist_table_init(or_hists_t *h) {
    /* histotools binning (reconstruction_constants.h:225-266) in the order of
     * online_reconstruction.cu:670-694; centres as M:718 computes them */
    static const short nb[OR_HIST_NVARS] = {100, 100, 100, 100, 100, 200, 50, 50, 50, 50, 50, 50,
                                            100, 100, 100, 100, 100, 200};
    static const float lo[OR_HIST_NVARS] = {-20.f, -20.f, 0.f, -20.f, -20.f, -500.f, 0.f, 0.f, 0.f, 0.f, 0.f,
                                            -3.141592654f, -20.f, -20.f, 0.f, -20.f, -20.f, -500.f};
    static const float hi[OR_HIST_NVARS] = {20.f, 20.f, 120.f, 20.f, 20.f, 500.f, 10.f, 1.f, 1.f, 0.5f, 5.f,
                                            3.141592654f, 20.f, 20.f, 120.f, 20.f, 20.f, 500.f};
    if (!h) return;
    std::memset(h, 0, sizeof(*h));
    for (int t = 0; t < OR_HIST_NTRIGGERS; ++t)
        for (int k = 0; k < OR_HIST_NVARS; ++k) {
            const int i = t * OR_HIST_NVARS + k;
            h->nbins[i] = nb[k];
            h->pts_hw[i] = (hi[k] - lo[k]) * 0.5f / nb[k];
            for (int l = 0; l < nb[k]; ++l) h->xpts[i * OR_HIST_NBINS_MAX + l] = lo[k] + h->pts_hw[k] * (2.f * l + 1.f);
        }
}

int or_run_physics(or_ctx_t *ctx, or_tracks_view_t tracks, or_dimuons_view_t dimuons, const int32_t *trigger_bits,
                   const uint8_t *toomany, or_hists_t *d_hists, int n_events, void *stream) {
    int rc = or_vertexing(ctx, tracks, toomany, n_events, stream);
    if (rc) return rc;
    if ((rc = or_dimuons(ctx, tracks, dimuons, toomany, n_events, stream))) return rc;
    if (!d_hists) return OR_OK;
    return or_fill_histograms(ctx, tracks, dimuons, trigger_bits, toomany, d_hists, n_events, stream);
}

/* ---- event output rows (the reference's output tree) --------------------- */

int or_output_rows(or_ctx_t *ctx, or_hits_view_t hits, or_tracks_view_t tracks, or_dimuons_view_t dimuons,
                   const uint8_t *toomany, const int32_t *raw_hits, const int32_t *event_ids, float min_stid,
                   or_output_view_t out, int n_events, void *stream) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (n_events < 0 || !toomany) return fail(OR_ERR_ARG, "bad event count or flag array");
    if ((rc = check_hits(hits)) || (rc = check_tracks(tracks)) || (rc = check_dimuons(dimuons))) return rc;
    if (!out.counts || (out.cap_events > 0 && !out.events) || (out.cap_hits > 0 && !out.hits) ||
        (out.cap_tracks > 0 && !out.tracks) || (out.cap_track_hits > 0 && !out.track_hits) ||
        (out.cap_dimuons > 0 && !out.dimuons) || out.cap_events < 0 || out.cap_hits < 0 || out.cap_tracks < 0 ||
        out.cap_track_hits < 0 || out.cap_dimuons < 0)
        return fail(OR_ERR_ARG, "output view: null table with a capacity, or no counts array");
    const size_t need = orgpu::output_scratch_bytes(n_events);
    if (need > ctx->out_scratch_bytes) {
        cudaFree(ctx->out_scratch);
        ctx->out_scratch = nullptr;
        ctx->out_scratch_bytes = 0;
        if (cudaMalloc(&ctx->out_scratch, need) != cudaSuccess) return fail(OR_ERR_NOMEM, "output scratch");
        ctx->out_scratch_bytes = need;
    }
    cudaError_t e = orgpu::launch_output_rows(hits, tracks, dimuons, toomany, raw_hits, event_ids, min_stid, out,
                                              n_events, ctx->out_scratch, S(stream), ctx->sm_count);
    return e == cudaSuccess ? OR_OK : cuda_fail(e, "output rows");
}

/* ---- learned tracklet scorer ------------------------------------------- */

int or_tracklet_rows(or_ctx_t *ctx, or_tracks_view_t tracks, const uint8_t *toomany, int n_events, int32_t *row_off,
                     void *stream) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (n_events < 0 || !toomany || !row_off) return fail(OR_ERR_ARG, "bad event count, flags or row offsets");
    if ((rc = check_tracks(tracks))) return rc;
    cudaError_t e = orgpu::launch_rows(tracks.ntracks, toomany, n_events, row_off, S(stream));
    return e == cudaSuccess ? OR_OK : cuda_fail(e, "tracklet rows");
}

int or_tracklet_features(or_ctx_t *ctx, or_hits_view_t hits, or_tracks_view_t tracks, const uint8_t *toomany,
                         int n_events, const int32_t *row_off, float *features, int64_t max_rows, void *stream) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (n_events < 0 || !toomany || !row_off || !features || max_rows < 0)
        return fail(OR_ERR_ARG, "bad feature arguments");
    if (!aligned16(features)) return fail(OR_ERR_ARG, "feature rows must be 16-byte aligned");
    if ((rc = check_hits(hits)) || (rc = check_tracks(tracks))) return rc;
    cudaError_t e =
        orgpu::launch_features(ctx->d_plane, hits, tracks, toomany, n_events, row_off, features, (long)max_rows,
                               S(stream), ctx->sm_count, ctx->warps[OR_K_FEATURES]);
    return e == cudaSuccess ? OR_OK : cuda_fail(e, "tracklet features");
}

int or_mlp_score(or_ctx_t *ctx, const or_mlp_t *model, const float *features, int64_t n_rows, float *scores,
                 void *stream) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (n_rows < 0 || !model || !features || !scores) return fail(OR_ERR_ARG, "bad scorer arguments");
    if (!aligned16(features)) return fail(OR_ERR_ARG, "feature rows must be 16-byte aligned");
    cudaError_t e =
        orgpu::launch_mlp_score(model, features, (long)n_rows, nullptr, scores, ctx->d_errw, S(stream), ctx->sm_count);
    return e == cudaSuccess ? OR_OK : cuda_fail(e, "scorer inference");
}

int or_keep_mask(or_ctx_t *ctx, const float *scores, const int32_t *row_off, int n_events, float t_keep, float t_unc,
                 uint8_t *keep, int64_t max_rows, void *stream) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (n_events < 0 || !scores || !row_off || !keep || max_rows < 0)
        return fail(OR_ERR_ARG, "bad keep-mask arguments");
    cudaError_t e =
        orgpu::launch_keep(scores, row_off, n_events, t_keep, t_unc, keep, (long)max_rows, S(stream), ctx->sm_count);
    return e == cudaSuccess ? OR_OK : cuda_fail(e, "keep mask");
}

int or_yz_pruned(or_ctx_t *ctx, or_hits_view_t hits, or_tracks_view_t tracks, const uint8_t *toomany, int n_events,
                 const int32_t *row_off, const uint8_t *keep, int64_t max_rows, void *stream) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (n_events < 0 || !toomany || !row_off || !keep || max_rows < 0)
        return fail(OR_ERR_ARG, "bad pruned-YZ arguments");
    if ((rc = check_hits(hits)) || (rc = check_tracks(tracks))) return rc;
    cudaError_t e = orgpu::launch_yz_pruned(ctx->d_plane, hits, tracks, toomany, n_events, ctx->d_errw, ctx->yz_scratch,
                                            ctx->yz_cap_units, ctx->yz_cap_heavy, ctx->yz_garena_warps, S(stream),
                                            ctx->sm_count, row_off, keep, (long)max_rows, ctx->warps[OR_K_YZ],
                                            ctx->yz_pool_limit, ctx->yz_count_work);
    return e == cudaSuccess ? OR_OK : cuda_fail(e, "pruned YZ launch");
}

int or_tracklet_labels(or_ctx_t *ctx, or_tracks_view_t tracks, const uint8_t *toomany, int n_events,
                       const int32_t *row_off, uint8_t *labels, int64_t max_rows, void *stream) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (n_events < 0 || !toomany || !row_off || !labels || max_rows < 0) return fail(OR_ERR_ARG, "bad label arguments");
    if ((rc = check_tracks(tracks))) return rc;
    cudaError_t e =
        orgpu::launch_labels(tracks, toomany, n_events, row_off, labels, (long)max_rows, S(stream), ctx->sm_count);
    return e == cudaSuccess ? OR_OK : cuda_fail(e, "tracklet labels");
}

int or_track_agreement(or_ctx_t *ctx, or_tracks_view_t tracks_a, or_tracks_view_t tracks_b, const uint8_t *toomany,
                       int n_events, uint64_t *counts, void *stream) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (n_events < 0 || !toomany || !counts) return fail(OR_ERR_ARG, "bad agreement arguments");
    if ((rc = check_tracks(tracks_a)) || (rc = check_tracks(tracks_b))) return rc;
    cudaError_t e = orgpu::launch_agreement(tracks_a, tracks_b, toomany, n_events,
                                            reinterpret_cast<unsigned long long *>(counts), S(stream), ctx->sm_count);
    return e == cudaSuccess ? OR_OK : cuda_fail(e, "track agreement");
}

int or_mlp_grad_blocks(int batch) { return batch > 0 ? orgpu::mlp_train_blocks(batch) : 0; }

int or_mlp_forward(or_ctx_t *ctx, const or_mlp_t *model, const float *features, const int64_t *idx, int n,
                   float *prob, void *stream) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (n < 0 || !model || !features || !idx || !prob) return fail(OR_ERR_ARG, "bad forward arguments");
    cudaError_t e = orgpu::launch_mlp_train(model, features, nullptr, idx, n, 1.f, nullptr, nullptr, prob, S(stream));
    return e == cudaSuccess ? OR_OK : cuda_fail(e, "scorer forward");
}

int or_mlp_gradient(or_ctx_t *ctx, const or_mlp_t *model, const float *features, const uint8_t *labels,
                    const int64_t *idx, int batch, float pos_weight, float *grad_part, float *loss_part, void *stream) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (batch < 0 || !model || !features || !labels || !idx || !grad_part || !loss_part)
        return fail(OR_ERR_ARG, "bad gradient arguments");
    cudaError_t e = orgpu::launch_mlp_train(model, features, labels, idx, batch, pos_weight, grad_part, loss_part,
                                            nullptr, S(stream));
    return e == cudaSuccess ? OR_OK : cuda_fail(e, "scorer gradient");
}

int or_mlp_adam(or_ctx_t *ctx, float *param, float *m1, float *m2, const float *grad_part, int nblocks, int step,
                float lr, float beta1, float beta2, float eps, or_mlp_t *model, void *stream) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (!param || !m1 || !m2 || !grad_part || !model || nblocks < 1 || step < 1)
        return fail(OR_ERR_ARG, "bad Adam arguments");
    cudaError_t e =
        orgpu::launch_mlp_adam(param, m1, m2, grad_part, nblocks, step, lr, beta1, beta2, eps, model, S(stream));
    return e == cudaSuccess ? OR_OK : cuda_fail(e, "scorer Adam step");
}

int or_run_batch_learned(or_ctx_t *ctx, or_hits_view_t hits, or_tracks_view_t tracks, int32_t *ntracklets,
                         uint8_t *toomany, int n_events, const or_mlp_t *model, float t_keep, float t_unc,
                         int32_t *row_off, float *features, float *scores, uint8_t *keep, int64_t max_rows,
                         void *stream) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (n_events < 0 || !toomany || !ntracklets || !model || !row_off || !features || !scores || !keep ||
        max_rows < 0)
        return fail(OR_ERR_ARG, "bad learned-batch arguments");
    if ((rc = check_hits(hits)) || (rc = check_tracks(tracks))) return rc;
    cudaError_t e = cudaMemsetAsync(ntracklets, 0, sizeof(int32_t) * (size_t)n_events, S(stream));
    if (e != cudaSuccess) return cuda_fail(e, "clear tracklet counts");
    if ((rc = or_event_reduce(ctx, hits, toomany, n_events, stream))) return rc;
    if ((rc = or_xz(ctx, hits, tracks, ntracklets, toomany, n_events, stream))) return rc;
    if ((rc = or_tracklet_rows(ctx, tracks, toomany, n_events, row_off, stream))) return rc;
    if ((rc = or_tracklet_features(ctx, hits, tracks, toomany, n_events, row_off, features, max_rows, stream)))
        return rc;
    // the row count stays on the device: the scorer reads it from row_off[n]
    cudaError_t e2 = orgpu::launch_mlp_score(model, features, (long)max_rows, row_off + n_events, scores, ctx->d_errw,
                                             S(stream), ctx->sm_count);
    if (e2 != cudaSuccess) return cuda_fail(e2, "scorer inference");
    if ((rc = or_keep_mask(ctx, scores, row_off, n_events, t_keep, t_unc, keep, max_rows, stream))) return rc;
    if ((rc = or_yz_pruned(ctx, hits, tracks, toomany, n_events, row_off, keep, max_rows, stream))) return rc;
    if ((rc = or_back_clean(ctx, tracks, toomany, n_events, stream))) return rc;
    return or_global(ctx, hits, tracks, toomany, n_events, stream);
}

or_hits_view_t or_hits_view_from_collection(void *coll) {
    // gEventHitCollections, reconstruction_classes.cuh:76-87 (4-byte members,
    // no padding)
    or_hits_view_t v;
    char *b = static_cast<char *>(coll);
    const size_t E = OR_REF_EVTMAX;
    v.nhits_cham = reinterpret_cast<uint32_t *>(b);
    b += sizeof(uint32_t) * E * OR_NCHAM;
    v.hits_cham = reinterpret_cast<float *>(b);
    b += sizeof(float) * E * OR_EVT_CHAM_FLOATS;
    v.nhits_hodo = reinterpret_cast<uint32_t *>(b);
    b += sizeof(uint32_t) * E * OR_NHODO;
    v.hits_hodo = reinterpret_cast<float *>(b);
    b += sizeof(float) * E * OR_EVT_HODO_FLOATS;
    v.nhits_prop = reinterpret_cast<uint32_t *>(b);
    b += sizeof(uint32_t) * E * OR_NPROP;
    v.hits_prop = reinterpret_cast<float *>(b);
    return v;
}

or_tracks_view_t or_tracks_view_from_collection(void *coll) {
    // gEventTrackCollection, reconstruction_classes.cuh:542-544
    or_tracks_view_t v;
    char *b = static_cast<char *>(coll);
    v.ntracks = reinterpret_cast<uint16_t *>(b);
    v.tracks = reinterpret_cast<float *>(b + sizeof(uint16_t) * (size_t)OR_REF_EVTMAX * OR_NSLOTS);
    return v;
}

size_t or_hits_view_bytes(int n) {
    return (size_t)n * (sizeof(uint32_t) * (OR_NCHAM + OR_NHODO + OR_NPROP) +
                        sizeof(float) * (OR_EVT_CHAM_FLOATS + OR_EVT_HODO_FLOATS + OR_EVT_PROP_FLOATS));
}
size_t or_tracks_view_bytes(int n) {
    return (size_t)n * (sizeof(uint16_t) * OR_NSLOTS + sizeof(float) * OR_EVT_TRK_FLOATS);
}

int or_pack_hits(or_ctx_t *ctx, const or_hit_record_t *records, const int64_t *rec_offsets, int n_events,
                 const float *wire_pos_f, or_hits_view_t hits, void *stream) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (n_events < 0 || !rec_offsets || !wire_pos_f) return fail(OR_ERR_ARG, "bad packer arguments");
    if ((rc = check_hits(hits))) return rc;
    cudaError_t e =
        orgpu::launch_pack(records, rec_offsets, n_events, wire_pos_f, nullptr, hits, ctx->d_errw, S(stream),
                           ctx->sm_count);
    return e == cudaSuccess ? OR_OK : cuda_fail(e, "packer launch");
}

int or_pack_hits_rt(or_ctx_t *ctx, const or_hit_record_t *records, const int64_t *rec_offsets, int n_events,
                    const float *wire_pos_f, const or_rt_table_t *rt_dev, or_hits_view_t hits, void *stream) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (n_events < 0 || !rec_offsets || !wire_pos_f || !rt_dev) return fail(OR_ERR_ARG, "bad packer arguments");
    if ((rc = check_hits(hits))) return rc;
    cudaError_t e =
        orgpu::launch_pack(records, rec_offsets, n_events, wire_pos_f, rt_dev, hits, ctx->d_errw, S(stream),
                           ctx->sm_count);
    return e == cudaSuccess ? OR_OK : cuda_fail(e, "packer launch");
}

int or_rt_apply(or_ctx_t *ctx, const or_rt_table_t *rt_dev, or_hits_view_t hits, int n_events, void *stream) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (n_events < 0 || !rt_dev) return fail(OR_ERR_ARG, "bad R-T arguments");
    if ((rc = check_hits(hits))) return rc;
    cudaError_t e = orgpu::launch_rt_apply(rt_dev, hits, n_events, S(stream), ctx->sm_count);
    return e == cudaSuccess ? OR_OK : cuda_fail(e, "R-T launch");
}

int or_collect_tracks(or_ctx_t *ctx, or_tracks_view_t tracks, const uint8_t *toomany, int n_events, float stid,
                      float *out, int64_t capacity, uint64_t *d_count, void *stream) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (n_events < 0 || !toomany || !d_count || capacity < 0 || (capacity > 0 && !out))
        return fail(OR_ERR_ARG, "bad collect arguments");
    if ((rc = check_tracks(tracks))) return rc;
    cudaError_t e = orgpu::launch_collect(tracks, toomany, n_events, stid, out, (long long)capacity,
                                          reinterpret_cast<unsigned long long *>(d_count), S(stream));
    return e == cudaSuccess ? OR_OK : cuda_fail(e, "collect launch");
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Drop-in calls on the reference's structs (include/or_dropin.h)
// ---------------------------------------------------------------------------
namespace {
constexpr int DROPIN_MAX_DEVICES = 64;
std::mutex g_dropin_mutex;
or_ctx_t *g_dropin[DROPIN_MAX_DEVICES];

// the current device's drop-in context, created at its first use
int dropin_ctx(or_ctx_t **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= DROPIN_MAX_DEVICES) return fail(OR_ERR_ARG, "device index above the drop-in table (64)");
    std::lock_guard<std::mutex> lock(g_dropin_mutex);
    if (!g_dropin[dev]) {
        // the reference's structs hold OR_REF_EVTMAX events: a context sized for them
        int rc = or_create_sized(dev, OR_REF_EVTMAX, &g_dropin[dev]);
        if (rc) return rc;
    }
    *out = g_dropin[dev];
    return OR_OK;
}
}  // namespace

extern "C" int or_gkernel_eR(gEventHitCollections *hitcolls, bool *hastoomanyhits) {
    or_ctx_t *ctx = nullptr;
    int rc = dropin_ctx(&ctx);
    if (rc) return rc;
    if (!hitcolls || !hastoomanyhits) return fail(OR_ERR_ARG, "or_gkernel_eR: null struct or flag array");
    return or_event_reduce(ctx, or_hits_view_from_collection(hitcolls), reinterpret_cast<uint8_t *>(hastoomanyhits),
                           OR_REF_EVTMAX, nullptr);
}

extern "C" int or_gKernel_XZ_tracking(gEventHitCollections *hitcolls, gEventTrackCollection *tklcoll,
                                      const gPlane *planes, int *nTracklets, bool *hastoomanyhits) {
    or_ctx_t *ctx = nullptr;
    int rc = dropin_ctx(&ctx);
    if (rc) return rc;
    if (!hitcolls || !tklcoll || !planes || !nTracklets || !hastoomanyhits)
        return fail(OR_ERR_ARG, "or_gKernel_XZ_tracking: null argument");
    const cudaError_t e = orgpu::launch_xz(reinterpret_cast<const or_plane_t *>(planes),
                                           or_hits_view_from_collection(hitcolls),
                                           or_tracks_view_from_collection(tklcoll), nTracklets,
                                           reinterpret_cast<uint8_t *>(hastoomanyhits), OR_REF_EVTMAX, nullptr,
                                           ctx->sm_count, ctx->warps[OR_K_XZ]);
    return e == cudaSuccess ? OR_OK : cuda_fail(e, "or_gKernel_XZ_tracking launch");
}

extern "C" int or_gKernel_YZ_tracking(gEventHitCollections *hitcolls, gEventTrackCollection *tklcoll,
                                      const gPlane *planes, bool *hastoomanyhits) {
    or_ctx_t *ctx = nullptr;
    int rc = dropin_ctx(&ctx);
    if (rc) return rc;
    if (!hitcolls || !tklcoll || !planes || !hastoomanyhits)
        return fail(OR_ERR_ARG, "or_gKernel_YZ_tracking: null argument");
    const cudaError_t e = orgpu::launch_yz_tuned(
        reinterpret_cast<const or_plane_t *>(planes), or_hits_view_from_collection(hitcolls),
        or_tracks_view_from_collection(tklcoll), reinterpret_cast<const uint8_t *>(hastoomanyhits), OR_REF_EVTMAX,
        ctx->d_errw, ctx->yz_scratch, ctx->yz_cap_units, ctx->yz_cap_heavy, ctx->yz_garena_warps, nullptr,
        ctx->sm_count, ctx->warps[OR_K_YZ], ctx->yz_pool_limit, 0);
    return e == cudaSuccess ? OR_OK : cuda_fail(e, "or_gKernel_YZ_tracking launch");
}

extern "C" int or_gKernel_BackTrackCleaning(gEventTrackCollection *tklcoll, const bool *hastoomanyhits) {
    or_ctx_t *ctx = nullptr;
    int rc = dropin_ctx(&ctx);
    if (rc) return rc;
    if (!tklcoll || !hastoomanyhits) return fail(OR_ERR_ARG, "or_gKernel_BackTrackCleaning: null argument");
    return or_back_clean(ctx, or_tracks_view_from_collection(tklcoll),
                         reinterpret_cast<const uint8_t *>(hastoomanyhits), OR_REF_EVTMAX, nullptr);
}

extern "C" int or_gKernel_Global_tracking(gEventHitCollections *hitcolls, gEventTrackCollection *tklcoll,
                                          const gPlane *planes, bool *hastoomanyhits) {
    or_ctx_t *ctx = nullptr;
    int rc = dropin_ctx(&ctx);
    if (rc) return rc;
    if (!hitcolls || !tklcoll || !planes || !hastoomanyhits)
        return fail(OR_ERR_ARG, "or_gKernel_Global_tracking: null argument");
    const cudaError_t e = orgpu::launch_global(reinterpret_cast<const or_plane_t *>(planes),
                                               or_hits_view_from_collection(hitcolls),
                                               or_tracks_view_from_collection(tklcoll),
                                               reinterpret_cast<const uint8_t *>(hastoomanyhits), OR_REF_EVTMAX,
                                               ctx->d_errw, ctx->d_sched, nullptr, ctx->sm_count,
                                               ctx->warps[OR_K_GLOBAL]);
    return e == cudaSuccess ? OR_OK : cuda_fail(e, "or_gKernel_Global_tracking launch");
}

extern "C" int or_dropin_sync(void) {
    or_ctx_t *ctx = nullptr;
    int rc = dropin_ctx(&ctx);
    if (rc) return rc;
    return or_stream_sync(ctx, nullptr);
}
