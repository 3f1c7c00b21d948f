/*
 * vgoracle.h -- CPU oracle for the batched BVH navigation path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker the parity tests,
 * the smoke check and the CPU-baseline leg of the benchmark compare against.
 * It is never linked into, loaded by or called from the product library
 * (libvgnav); the product fails loudly when its CUDA extension is missing.
 *
 * It is a plain-C restatement of the reference algorithm (VecGeom 1.2.0):
 * every function cites the reference file:line it follows, and keeps the
 * reference's floating-point operation order so that results are bit-exact
 * when compiled with -ffp-contract=off.
 */
#ifndef VGORACLE_H
#define VGORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* shape type ids (same numbering as the product's vgn_shape_type) */
enum { OR_BOX = 0, OR_TUBE = 1, OR_CONE = 2, OR_TRD = 3, OR_TRAP = 4, OR_SPHERE = 5, OR_POLYCONE = 6, OR_ORB = 7,
       OR_CUTTUBE = 8, OR_BOOLEAN = 9, OR_POLYHEDRON = 10, OR_TORUS = 11,
       OR_NSHAPES = 12 };
/* pv_mother of a boolean solid's operand placement (outside the hierarchy) */
#define OR_BOOLEAN_OPERAND (-2)

/* shape operations for or_shape_batch */
enum { OR_OP_DIST_IN = 0, OR_OP_DIST_OUT = 1, OR_OP_SAFE_IN = 2, OR_OP_SAFE_OUT = 3, OR_OP_CONTAINS = 4, OR_OP_INSIDE = 5 };

/* navigation state: the 12-byte layout of vecgeom::NavStateIndex
 * (VecGeom/navigation/NavStateIndex.h:39-41) */
typedef struct {
  uint32_t nav_ind;
  uint32_t last_exited;
  uint8_t on_boundary;
  uint8_t pad[3];
} or_state;

/* per-track work counters (roofline accounting) */
typedef struct {
  uint64_t node_slab;   /* internal-node AABB slab tests */
  uint64_t prim_slab;   /* leaf primitive AABB slab tests */
  uint64_t node_safety; /* internal-node AABB safety evaluations */
  uint64_t prim_safety; /* leaf primitive AABB safety evaluations */
  uint64_t prim_contains;
  uint64_t transforms;  /* point(+direction) transforms into a daughter frame */
  uint64_t kernel[OR_NSHAPES][6];
} or_counters;

typedef struct or_geom or_geom;

/* Build the geometry from a flat description.
 *   lv_shape[n_lv], lv_param_off[n_lv] : shape type and offset into params
 *   pv_lv[n_pv], pv_mother[n_pv]        : placed logical volume, mother logical
 *                                         volume (-1 for the world placement);
 *                                         placed-volume id = index (creation order)
 *   pv_trans[12*n_pv]                   : tx,ty,tz,r0..r8 (Transformation3D)
 * Returns NULL and fills err on failure. */
or_geom *or_geom_create(int n_lv, const int *lv_shape, const int *lv_param_off, const double *params, int n_params,
                        int n_pv, const int *pv_lv, const int *pv_mother, const double *pv_trans, int world_pv,
                        char *err, int errlen);
/* the same with GeoManager::SetTransformationCacheDepth(cache_depth) before closing
 * (GeoManager.h:121): table nodes deeper than cache_depth levels store no matrix */
or_geom *or_geom_create_ex(int n_lv, const int *lv_shape, const int *lv_param_off, const double *params,
                           int n_params, int n_pv, const int *pv_lv, const int *pv_mother, const double *pv_trans,
                           int world_pv, int cache_depth, char *err, int errlen);
void or_geom_free(or_geom *g);

/* exported tables for cross-checks against the product's host builder */
const uint32_t *or_geom_navindex(const or_geom *g, size_t *n_words);
int or_geom_bvh_info(const or_geom *g, int lv, int *depth, int *n_nodes, int *n_prims);
int or_geom_bvh_arrays(const or_geom *g, int lv, int *prim_id, int *offset, int *nchild, double *nodes_minmax,
                       double *prims_minmax);

/* unplaced shape queries for logical volume `lv` over n SoA points */
int or_shape_batch(const or_geom *g, int lv, int op, long n, const double *px, const double *py, const double *pz,
                   const double *dx, const double *dy, const double *dz, const double *stepmax, double *out);

/* ComputeStepAndSafetyAndPropagatedState per track (VNavigator.h:1014-1064).
 *   calcsafety: 0 = no safety (ComputeStepAndPropagatedState semantics), 1 = compute
 *   simple    : 0 = BVH navigator + BVH level locator, 1 = brute-force navigator
 *   nthreads  : host threads (<=0 : all cores) */
void or_nav_step_batch(const or_geom *g, long n, const double *px, const double *py, const double *pz,
                       const double *dx, const double *dy, const double *dz, const double *slimit,
                       const or_state *in, or_state *out, double *step, double *safety, int calcsafety, int simple,
                       int nthreads, or_counters *counters);

/* ComputeStep (no relocation, VNavigator.h:494-540) */
void or_nav_step_norel_batch(const or_geom *g, long n, const double *px, const double *py, const double *pz,
                             const double *dx, const double *dy, const double *dz, const double *slimit,
                             const or_state *in, or_state *out, double *step, int nthreads);

/* VSafetyEstimatorHelper::ComputeSafety (VSafetyEstimator.h:98-107) */
void or_safety_batch(const or_geom *g, long n, const double *px, const double *py, const double *pz,
                     const or_state *in, double *safety, int nthreads);

/* GlobalLocator::LocateGlobalPoint from the world (GlobalLocator.h:35-82), top = true */
void or_locate_batch(const or_geom *g, long n, const double *px, const double *py, const double *pz, or_state *out,
                     int nthreads);

/* BVH::ApproachNextDaughter (BVH.cpp:395-449) per track over logical volume lv[i]'s BVH: local
 * point and direction in that volume, step in/out, last[i] the last exited placed volume or -1.
 * Returns 1 (nothing computed) if a volume has no daughters. */
int or_approach_batch(const or_geom *g, long n, const int *lv, const double *px, const double *py,
                      const double *pz, const double *dx, const double *dy, const double *dz, const int *last,
                      double *step);

/* VUnplacedVolume::Extent of logical volume lv's shape: min then max corner */
int or_shape_extent(const or_geom *g, int lv, double *out6);

/* wall-clock helper for the CPU baseline */
double or_now(void);
int or_ncores(void);

#ifdef __cplusplus
}
#endif
#endif
