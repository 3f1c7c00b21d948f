/*
 * vgnav.h -- C ABI of the GB300-native batched navigation library (libvgnav).
 *
 * The library replaces the batched navigation hot path of VecGeom 1.2.0:
 * BVH traversal in BVHNavigator / BVHSafetyEstimator / BVHLevelLocator
 * feeding the per-shape DistanceToIn/DistanceToOut/SafetyToIn/SafetyToOut
 * kernels and the Transformation3D global-to-local transforms, over
 * SOA3D<double> point/direction batches and NavStateIndex states.
 *
 * All entry points are plain C: pointers, sizes and an int status.
 * Array arguments may be device pointers (cudaMalloc / torch CUDA tensors),
 * in which case the call only enqueues work on `stream`, or host pointers,
 * in which case the library stages the data through its own device
 * workspace and the call returns once the results are back in host memory.
 * A NULL stream is the legacy default stream.
 */
#ifndef VGNAV_H
#define VGNAV_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define VGN_OK 0
#define VGN_ERR_ARG 1         /* invalid argument (null pointer, bad size, bad id) */
#define VGN_ERR_UNSUPPORTED 2 /* shape or parameter set not supported */
#define VGN_ERR_CUDA 3        /* CUDA runtime error (message in vgn_last_error) */
#define VGN_ERR_NOMEM 4       /* device or host allocation failed */
#define VGN_ERR_STACK 5       /* BVH traversal stack overflow on the device */
#define VGN_ERR_RELOCATE 6    /* relocation exceeded the geometry depth bound */
#define VGN_ERR_STATE 7       /* an input navigation state index is outside the table */

/* ---- shape types (numbering of vgn_geometry_desc.lv_shape) ---------------- */
enum vgn_shape_type {
  VGN_BOX       = 0, /* params: dx, dy, dz                        (UnplacedBox.h)       */
  VGN_TUBE      = 1, /* params: rmin, rmax, dz, sphi, dphi        (UnplacedTube.h:29)   */
  VGN_CONE      = 2, /* params: rmin1, rmax1, rmin2, rmax2, dz, sphi, dphi (UnplacedCone.h) */
  VGN_TRD       = 3, /* params: x1, x2, y1, y2, z                 (UnplacedTrd.h)       */
  VGN_TRAPEZOID = 4, /* params: dz, theta, phi, dy1, dx1, dx2, alpha1, dy2, dx3, dx4, alpha2 (UnplacedTrapezoid.h) */
  VGN_SPHERE    = 5, /* params: rmin, rmax, sphi, dphi, stheta, dtheta (UnplacedSphere.h) */
  VGN_POLYCONE  = 6, /* params: sphi, dphi, nz, z[nz], rmin[nz], rmax[nz] (UnplacedPolycone.h:79) */
  VGN_ORB       = 7, /* params: r                                 (UnplacedOrb.h)       */
  VGN_CUTTUBE   = 8, /* params: rmin, rmax, dz, sphi, dphi, bottom normal bx, by, bz, top normal
                        tx, ty, tz                                (UnplacedCutTube.h:54-57) */
  VGN_BOOLEAN   = 9, /* params: op (VGN_BOOL_UNION / _INTERSECTION / _SUBTRACTION), left operand,
                        right operand: ids of placed volumes whose mother is VGN_BOOLEAN_OPERAND
                        (UnplacedBooleanVolume.h:59, BooleanStruct.h:23-25)        */
  VGN_POLYHEDRON = 10, /* params: sphi, dphi, sides, nz, z[nz], rmin[nz], rmax[nz]; radii are to
                        the sides' middles (UnplacedPolyhedron.h:97-108).  Refused where the
                        reference reads past its arrays: a zero-length first or last segment,
                        three equal z planes in a row, a zero-length segment with equal radii,
                        a face with fewer than three distinct corners, dphi / sides >= pi */
  VGN_TORUS2    = 11  /* params: rmin, rmax, rtor, sphi, dphi with 0 <= rmin < rmax < rtor
                        (UnplacedTorus2.h:64-65)                                     */
};

/* Boolean solids (VGN_BOOLEAN).  The operands are placements of other logical volumes
 * relative to the boolean's frame, listed in vgn_geometry_desc like any placement but with
 * pv_mother = VGN_BOOLEAN_OPERAND: they belong to no mother and take no part in navigation
 * other than through their boolean.  Rules:
 *  - each operand placement (anywhere in the placed-volume list, so VecGeom's own ids can be
 *    kept) is used by exactly one boolean;
 *  - an operand's logical volume has a smaller index than its boolean, has no daughters, and
 *    is a primitive shape or a boolean of primitive shapes (two levels at most).
 * A geometry holding booleans may hold no phi or theta section, polyhedron or torus
 * (VGN_ERR_UNSUPPORTED).
 * vgn_shape_batch with VGN_OP_INSIDE on a union is VGN_ERR_UNSUPPORTED (its surface case takes
 * the operands' normals, which the library does not compute); every navigation call works. */
#define VGN_BOOLEAN_OPERAND (-2)
enum vgn_boolean_op { VGN_BOOL_UNION = 0, VGN_BOOL_INTERSECTION = 1, VGN_BOOL_SUBTRACTION = 2 };

/* ---- shape operations for vgn_shape_batch ------------------------------- */
enum vgn_shape_op {
  VGN_OP_DISTANCE_TO_IN  = 0, /* VUnplacedVolume::DistanceToIn  */
  VGN_OP_DISTANCE_TO_OUT = 1, /* VUnplacedVolume::DistanceToOut */
  VGN_OP_SAFETY_TO_IN    = 2, /* VUnplacedVolume::SafetyToIn    */
  VGN_OP_SAFETY_TO_OUT   = 3, /* VUnplacedVolume::SafetyToOut   */
  VGN_OP_CONTAINS        = 4, /* VUnplacedVolume::Contains, output 0.0 / 1.0 */
  VGN_OP_INSIDE          = 5  /* VUnplacedVolume::Inside, output 1 kInside, 2 kSurface, 3 kOutside */
};

/* ---- flags --------------------------------------------------------------- */
#define VGN_PRECISION_FP64 0x0  /* all-FP64 kernels, bit-exact with the CPU navigator   */
#define VGN_PRECISION_MIXED 0x1 /* FP32 conservative traversal + FP64 refinement         */
#define VGN_NO_RELOCATE 0x10    /* ComputeStep semantics: out state not relocated        */

/* Navigation state, layout-identical to vecgeom::NavStateIndex
 * (VecGeom/navigation/NavStateIndex.h:39-41): 12 bytes. */
typedef struct vgn_state {
  uint32_t nav_ind;     /* index into the navigation table (0 = outside the world) */
  uint32_t last_exited; /* navigation index of the last exited state              */
  uint8_t on_boundary;  /* 1 if the point sits on the boundary of Top()           */
  uint8_t pad[3];
} vgn_state;

/* Flat geometry description.  Placed-volume ids are array indices, in
 * creation order (VPlacedVolume::id(), source/PlacedVolume.cpp:32); the
 * daughters of a logical volume are its placements in id order
 * (LogicalVolume::PlaceDaughter, source/LogicalVolume.cpp:142-148). */
typedef struct vgn_geometry_desc {
  int32_t n_logical;
  const int32_t *lv_shape;        /* [n_logical] vgn_shape_type                      */
  const int32_t *lv_param_offset; /* [n_logical] offset of the shape's params        */
  const double *params;           /* [n_params]                                      */
  int32_t n_params;
  int32_t n_placed;
  const int32_t *pv_logical;   /* [n_placed] logical volume placed                     */
  const int32_t *pv_mother;    /* [n_placed] mother logical volume, -1 for the world   */
  const double *pv_transform;  /* [12*n_placed] tx,ty,tz,r0..r8 (Transformation3D ctor,
                                  source/Transformation3D.cpp:52-61)                    */
  int32_t world_placed;        /* id of the world placement                            */
} vgn_geometry_desc;

typedef struct vgn_geometry vgn_geometry;

/* Close the geometry and make it resident on `device`: daughter bounding
 * boxes (ABBoxManager::InitABBoxesForCompleteGeometry, source/ABBoxManager.cpp:109-142),
 * one BVH per logical volume with daughters (BVHManager::Init,
 * source/BVHManager.cpp:24-30), the navigation index table
 * (GeoManager::MakeNavIndexTable, source/GeoManager.cpp:381-395) and their
 * upload (replaces CudaManager::Synchronize + BVHManager::DeviceInit,
 * source/CudaManager.cpp:101-222, source/BVHManager.cpp:33-45). */
#define VGN_HOST_ONLY (-1) /* `device` value: close on the host only (tables can be inspected, no kernels) */
int vgn_geometry_create(const vgn_geometry_desc *desc, int device, vgn_geometry **out);
/* The same with a transformation cache depth, GeoManager::SetTransformationCacheDepth before
 * closing (VecGeom/management/GeoManager.h:121, used at source/GeoManager.cpp:220-221):
 * navigation-table nodes deeper than `cache_depth` levels store no global matrix, and a
 * state's matrix is accumulated from the placements up to its nearest cached ancestor
 * (NavStateIndex::TopMatrixImpl, NavStateIndex.h:232-265).  0 caches every level, as
 * vgn_geometry_create does; the table then equals the reference's for the same depth. */
int vgn_geometry_create_with_cache_depth(const vgn_geometry_desc *desc, int device, int32_t cache_depth,
                                         vgn_geometry **out);
int vgn_geometry_free(vgn_geometry *geom);

/* Host copy of the navigation index table (NavIndexTable::GetTable,
 * VecGeom/management/NavIndexTable.h:74-76). */
int vgn_geometry_navindex(const vgn_geometry *geom, const uint32_t **table, size_t *n_words);
/* Host copies of one logical volume's BVH (BVH.h:364-370); any out pointer may be NULL. */
int vgn_geometry_bvh_info(const vgn_geometry *geom, int32_t lv, int32_t *depth, int32_t *n_nodes, int32_t *n_prims);
int vgn_geometry_bvh_arrays(const vgn_geometry *geom, int32_t lv, int32_t *prim_id, int32_t *offset, int32_t *nchild,
                            double *nodes_minmax, double *prims_minmax);
/* Bytes of device memory held by the geometry tables. */
int vgn_geometry_device_bytes(const vgn_geometry *geom, size_t *bytes);

/* Batched navigation step with propagated state.
 * Replaces VNavigatorHelper<BVHNavigator<false>>::ComputeStepsAndSafetiesAndPropagatedStates
 * (VecGeom/navigation/VNavigator.h:913-941) and, per track,
 * ComputeStepAndSafetyAndPropagatedState / ComputeStepAndPropagatedState
 * (VNavigator.h:1014-1064, 436-492); with VGN_NO_RELOCATE, ComputeStep
 * (VNavigator.h:494-540).  Unlike the reference batch call, tracks may sit in
 * different volumes.  `safety` may be NULL (no safety computed); otherwise it
 * receives ComputeSafetyForLocalPoint (BVHSafetyEstimator.h:38-46).
 * out->nav_ind after the call is the next volume ("ComputeStepAndNextVolume"). */
int vgn_compute_step_batch(const vgn_geometry *geom, int64_t n, const double *px, const double *py, const double *pz,
                           const double *dx, const double *dy, const double *dz, const double *step_limit,
                           const vgn_state *in, vgn_state *out, double *step, double *safety, int flags,
                           void *stream);

/* The same operation under the name of its result, the next volume
 * ("ComputeStepAndNextVolume"): out->nav_ind is the volume the track enters. */
int vgn_step_and_next_volume(const vgn_geometry *geom, int64_t n, const double *px, const double *py,
                             const double *pz, const double *dx, const double *dy, const double *dz,
                             const double *step_limit, const vgn_state *in, vgn_state *out, double *step,
                             double *safety, int flags, void *stream);

/* Batched isotropic safety: VSafetyEstimatorHelper<BVHSafetyEstimator>::ComputeSafety
 * (VecGeom/navigation/VSafetyEstimator.h:98-107). */
int vgn_compute_safety_batch(const vgn_geometry *geom, int64_t n, const double *px, const double *py,
                             const double *pz, const vgn_state *in, double *safety, int flags, void *stream);

/* Batched point location from the world: GlobalLocator::LocateGlobalPoint(world, p, state, true)
 * (VecGeom/navigation/GlobalLocator.h:35-82) with BVHLevelLocator (BVH.h:234-244). */
int vgn_locate_batch(const vgn_geometry *geom, int64_t n, const double *px, const double *py, const double *pz,
                     vgn_state *out, int flags, void *stream);

/* Batched unplaced-shape query on logical volume `lv`: the per-shape
 * *Implementation kernels behind VUnplacedVolume (e.g.
 * VecGeom/volumes/kernel/TubeImplementation.h:475-960).  dx/dy/dz and
 * step_max are only read for the distance ops (step_max may be NULL). */
int vgn_shape_batch(const vgn_geometry *geom, int32_t lv, int32_t op, int64_t n, const double *px, const double *py,
                    const double *pz, const double *dx, const double *dy, const double *dz, const double *step_max,
                    double *out, int flags, void *stream);

/* BVH::ApproachNextDaughter per track (VecGeom/base/BVH.h:158, source/BVH.cpp:395-449): over
 * the BVH of logical volume lv[i], with the point and direction in that volume's frame, step[i]
 * (in/out) is lowered to the entry distance into the bounding box of the nearest daughter the
 * ray meets before it (the daughter's VUnplacedVolume::ApproachSolid, UnplacedVolume.h:274-281,
 * in its own frame), skipping last_pv[i] at distance <= 0 (the last exited placed volume, -1 for
 * none; NULL: -1 for every track).  FP64, bit-exact with the reference.  Host buffers: a volume
 * out of range or without daughters, or a last_pv out of range, is VGN_ERR_ARG; device buffers:
 * such a track keeps its step and the call (or vgn_synchronize) returns VGN_ERR_STATE. */
int vgn_approach_next_daughter_batch(const vgn_geometry *geom, int64_t n, const int32_t *lv, const double *px,
                                     const double *py, const double *pz, const double *dx, const double *dy,
                                     const double *dz, const int32_t *last_pv, double *step, void *stream);

/* Launch configuration of the step kernel for one precision form (flags &
 * VGN_PRECISION_MIXED): `variant` picks the threads-per-block / register-cap
 * variant, `sort_kbits` (0..6) bins tracks by direction octant and a
 * 2^k-per-axis cell of the world box before the step, for warp coherence
 * (0 = no binning).  Only performance changes, never a result.  Binning takes
 * its scratch (about 12 bytes per track plus the histogram) from a stream-ordered
 * memory pool the library keeps per device, so calls on different streams or
 * threads may overlap, on one geometry too; the pool keeps its blocks for reuse
 * until the process exits.  No counterpart in the reference, which launches 256
 * threads per block (backend/cuda/Backend.h:50-96). */
int vgn_set_step_config(vgn_geometry *geom, int flags, int32_t variant, int32_t sort_kbits);
int vgn_get_step_config(const vgn_geometry *geom, int flags, int32_t *variant, int32_t *sort_kbits);
/* Number of launch variants of the step for the precision form: 0..5 for both forms; the
 * mixed form adds 6..8, which compute the candidates' FP64 DistanceToIn grouped by shape type
 * across the whole thread block (every warp runs 32 candidates of one shape type at a time).
 * vgn_batch_set_jobs takes variants 0..5.  No counterpart in the reference. */
int vgn_get_step_variant_count(int flags, int32_t *count);
/* Staging of step calls made with host buffers: the batch is split into `chunks`
 * pieces that alternate between two internal streams, so the host<->device copies of
 * one piece overlap the kernels of the other (0 = automatic, currently one piece:
 * copies and kernels in sequence on the caller's stream).  Pieces pay off only where the
 * copies are slow against the kernels; each piece bins its tracks separately.  Only
 * performance changes, never a result.  No counterpart in the reference, whose batched
 * navigator works on host memory. */
int vgn_set_staging_chunks(vgn_geometry *geom, int32_t chunks);
int vgn_get_staging_chunks(const vgn_geometry *geom, int32_t *chunks);
/* The safety pass's own visit order (steps that ask for safeties): tracks binned by
 * position alone into 2^kbits cells per axis of the world box, 1..6 (the safety does
 * not depend on the direction, so the octant split of the step's order only scatters
 * neighbours); 0 = the safety pass follows the step's order.  Only performance
 * changes, never a result; its scratch comes with the step's (one pool allocation per call). */
int vgn_set_safety_binning(vgn_geometry *geom, int flags, int32_t kbits);
int vgn_get_safety_binning(const vgn_geometry *geom, int flags, int32_t *kbits);
/* Autotuner: times every (variant, sort_kbits) pair on the given batch (device
 * pointers; outputs are overwritten), keeps the fastest for this precision
 * form and returns it with its time per batch; when `safety` is given, it then
 * times the safety pass's binning (0, 4, 5, 6) with that configuration and keeps
 * the fastest (vgn_get_safety_binning reads it). */
int vgn_autotune_step(vgn_geometry *geom, int64_t n, const double *px, const double *py, const double *pz,
                      const double *dx, const double *dy, const double *dz, const double *step_limit,
                      const vgn_state *in, vgn_state *out, double *step, double *safety, int flags, void *stream,
                      int32_t *variant, int32_t *sort_kbits, float *best_ms);

/* Transport loop on the device: every track is stepped (ComputeStepAndPropagatedState,
 * VNavigator.h:436-492, no safety) and moved by its step, p += step * d, until it leaves
 * the world (nav_ind 0) or after max_steps steps -- the caller-side loop of the
 * reference's transport examples (persistency/gdml/test/TestVGDMLNavigation/
 * TestVGDMLNavigation.cpp:86-102) with the state kept on the device.  Positions and
 * states are updated in place; nsteps[i] receives the steps taken (-1: invalid state).
 * Tracks are visited in the binned order of the geometry's step configuration for this
 * precision form (vgn_set_step_config / vgn_autotune_step), with stream-ordered scratch;
 * batches of fewer than 32768 tracks are walked unbinned.
 * Device pointers only.  No single counterpart call in the reference. */
int vgn_walk_batch(const vgn_geometry *geom, int64_t n, double *px, double *py, double *pz, const double *dx,
                   const double *dy, const double *dz, const double *step_limit, vgn_state *state,
                   int32_t max_steps, int32_t *nsteps, int flags, void *stream);

/* ---- batched uneven workloads: many (geometry, track batch) jobs per launch ------
 * The reference launches one kernel per batch and geometry (NavigationBenchmarker.cu:43,
 * VNavigator.h:913-941); a vgn_batch runs up to VGN_BATCH_MAX_JOBS jobs, each with its
 * own geometry and SOA3D arrays, in ONE persistent launch whose warps take 32-track
 * chunks from a device work queue, so small and large batches share the GPU evenly.
 * Results equal vgn_compute_step_batch on each job bit for bit.
 *   create -> set_jobs (uploads nothing per step; allocates the per-job binning
 *   scratch) -> step (enqueue only: queue reset, optional per-job binning, one launch;
 *   no allocation or host synchronisation, so it can be recorded into a CUDA graph)
 * All job arrays are device pointers on the batch's device; the jobs' geometries must
 * live on that device.  No counterpart in the reference. */
#define VGN_BATCH_MAX_JOBS 64
typedef struct vgn_step_job {
  const vgn_geometry *geom;
  int64_t n;
  const double *px, *py, *pz, *dx, *dy, *dz, *step_limit;
  const vgn_state *in;
  vgn_state *out;
  double *step;
  double *safety; /* may be NULL: no safety */
} vgn_step_job;
typedef struct vgn_batch vgn_batch;
int vgn_batch_create(int device, vgn_batch **out);
int vgn_batch_free(vgn_batch *batch);
/* flags: VGN_PRECISION_MIXED, VGN_NO_RELOCATE; sort_kbits 0..6 as in vgn_set_step_config */
int vgn_batch_set_jobs(vgn_batch *batch, int n_jobs, const vgn_step_job *jobs, int flags, int32_t variant,
                       int32_t sort_kbits);
int vgn_batch_step(vgn_batch *batch, void *stream);
/* waits for `stream` and returns the first device-side error of any job's geometry */
int vgn_batch_synchronize(vgn_batch *batch, void *stream);
/* times every (variant, sort_kbits) pair on the current jobs, keeps the fastest */
int vgn_batch_autotune(vgn_batch *batch, void *stream, int32_t *variant, int32_t *sort_kbits, float *best_ms);

/* Allocation-free binned step.  Same operation and results as
 * vgn_compute_step_batch with track binning at `sort_kbits` (1..5), but the
 * binning scratch (sort keys, histogram, visit permutation) lives in one fixed
 * device buffer that the library declares statically, so the call allocates
 * no device or host memory.  It is for callers that cannot allocate inside a
 * navigation call: a transport loop that runs under a fixed device-memory
 * budget, or one that must not take the device-wide synchronisation that
 * cudaMalloc/cudaFree imply while other streams are busy.
 *  - all arrays must be device pointers (host buffers would need staging memory);
 *  - n <= VGN_STATIC_SCRATCH_MAX_TRACKS, else VGN_ERR_ARG;
 *  - the buffer's address is looked up on every call, in the current context
 *    (with the geometry's device current); the first call on a device may load
 *    the library's device code, so make it before any stream capture begins;
 *  - there is ONE buffer per device: calls that overlap on that device (other
 *    streams, other threads, other geometries) race on it and must be ordered
 *    by the caller;
 *  - the buffer holds one visit permutation, the step's: the safety pass runs
 *    in that order too, not in the order of vgn_set_safety_binning (same
 *    results; vgn_compute_step_batch may be faster on the safety).
 * Uses the step launch variant set for the precision form (vgn_set_step_config).
 * No counterpart in the reference. */
#define VGN_STATIC_SCRATCH_MAX_TRACKS 1048576 /* 2^20 tracks per call */
#define VGN_STATIC_SCRATCH_MAX_KBITS 5        /* largest sort_kbits accepted */
int vgn_compute_step_batch_static(const vgn_geometry *geom, int64_t n, const double *px, const double *py,
                                  const double *pz, const double *dx, const double *dy, const double *dz,
                                  const double *step_limit, const vgn_state *in, vgn_state *out, double *step,
                                  double *safety, int flags, int32_t sort_kbits, void *stream);

/* Bounds of the device loops, for exercising their error paths: BVH traversal stack
 * entries (2..32; the reference's BVH_MAX_DEPTH, BVH.h:33, is 32) and relocation levels
 * (1..30).  A traversal that needs more stack, or a relocation that descends more levels,
 * stops and records VGN_ERR_STACK / VGN_ERR_RELOCATE, which the call (host buffers) or
 * vgn_synchronize (device buffers) returns; no fault, the context stays usable.  Lower
 * bounds than the defaults change results, so they are for tests only; the defaults
 * (32, 30) never bind on a geometry the library accepts.  Applies to later calls on the
 * geometry (a vgn_batch keeps the bounds its jobs were set with).  No counterpart in the
 * reference, whose loops are unbounded or assert. */
int vgn_set_device_limits(vgn_geometry *geom, int32_t stack_entries, int32_t levels);

/* Wait for the work of the previous calls on `stream`; returns the first
 * device-side error status recorded by a kernel since the last call. */
int vgn_synchronize(const vgn_geometry *geom, void *stream);

/* Message of the last error raised on the calling thread. */
const char *vgn_last_error(void);

/* Library version string. */
const char *vgn_version(void);

#ifdef __cplusplus
}
#endif
#endif /* VGNAV_H */
