/* or_dropin.h -- the reference's five tracking launches as host calls on the
 * reference's own structs, so that its host code (online_reconstruction.cu
 * :776-894) switches to the GB300 kernels by a one-line edit per call site:
 *
 *   gkernel_eR<<<EstnEvtMax, 8>>>(device_gHits, device_gHasTooManyHits);
 *       becomes
 *   or_gkernel_eR(device_gHits, device_gHasTooManyHits);
 *
 * with the same arguments (device pointers to the reference's
 * fixed-capacity structs, EstnEvtMax = 10000 events each,
 * reconstruction_constants.h:20) and the same meaning: the structs are
 * updated in place, per-event outcome in the bool flag array.  Each call
 * queues its kernels on the legacy default stream and returns, as a kernel
 * launch does; the reference's cudaDeviceSynchronize() after each launch
 * waits for them.  The return value is an or_status_t (the reference
 * ignores launch results; its error checks read cudaGetLastError()).
 *
 * The calls run on a library context per device, created at the first call
 * on that device (sized for OR_REF_EVTMAX events: about 1.4 GB of scratch,
 * or_create_sized()) and kept until the
 * process exits; make that first call outside any stream capture.  The
 * geometry is the caller's device gPlane, read in place.  Device-side
 * error words (bounded-wait timeout, window capacity) of these calls are
 * read by or_dropin_sync().
 *
 * The struct types are the reference's (reconstruction_classes.cuh); this
 * header only names them.  Their layouts are those of include/or_layout.h:
 * gEventHitCollections = six arrays of OR_REF_EVTMAX events, gEventTrack-
 * Collection = OR_REF_EVTMAX*OR_NSLOTS uint16 counts then the track records,
 * gPlane = or_plane_t. */
#ifndef OR_DROPIN_H
#define OR_DROPIN_H

#ifdef __cplusplus
extern "C" {
#else
#include <stdbool.h>
#endif

struct gEventHitCollections;  /* reconstruction_classes.cuh:76-104 */
struct gEventTrackCollection; /* reconstruction_classes.cuh:542-655 */
struct gPlane;                /* reconstruction_classes.cuh:947-977 */

/* gkernel_eR<<<EstnEvtMax, 8>>>(hitcolls, hastoomanyhits)
 * (reconstruction_kernels.cuh:8, online_reconstruction.cu:776) */
int or_gkernel_eR(struct gEventHitCollections *hitcolls, bool *hastoomanyhits);

/* gKernel_XZ_tracking<<<EstnEvtMax, 32>>>(hitcolls, tklcoll, planes,
 * nTracklets, hastoomanyhits) (reconstruction_kernels.cuh:182-193,
 * online_reconstruction.cu:806) */
int or_gKernel_XZ_tracking(struct gEventHitCollections *hitcolls, struct gEventTrackCollection *tklcoll,
                           const struct gPlane *planes, int *nTracklets, bool *hastoomanyhits);

/* gKernel_YZ_tracking<<<EstnEvtMax, 32>>>(hitcolls, tklcoll, planes,
 * hastoomanyhits) (reconstruction_kernels.cuh:864-872,
 * online_reconstruction.cu:832) */
int or_gKernel_YZ_tracking(struct gEventHitCollections *hitcolls, struct gEventTrackCollection *tklcoll,
                           const struct gPlane *planes, bool *hastoomanyhits);

/* gKernel_BackTrackCleaning<<<EstnEvtMax, 32>>>(tklcoll, hastoomanyhits)
 * followed by gKernel_BackTrackCleaning_crossthreads<<<EstnEvtMax, 32>>>
 * (reconstruction_helper.cuh:1789, :1846; online_reconstruction.cu:873-881):
 * both passes in one call, which replaces the two launches. */
int or_gKernel_BackTrackCleaning(struct gEventTrackCollection *tklcoll, const bool *hastoomanyhits);

/* gKernel_Global_tracking<<<EstnEvtMax, 32>>>(hitcolls, tklcoll, planes,
 * hastoomanyhits) (reconstruction_kernels.cuh:1841-1849,
 * online_reconstruction.cu:887) */
int or_gKernel_Global_tracking(struct gEventHitCollections *hitcolls, struct gEventTrackCollection *tklcoll,
                               const struct gPlane *planes, bool *hastoomanyhits);

/* Wait for the legacy default stream and report (and clear) the error words
 * of the current device's drop-in context, as or_stream_sync() does. */
int or_dropin_sync(void);

#ifdef __cplusplus
}
#endif

#endif /* OR_DROPIN_H */
