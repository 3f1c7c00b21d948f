/*
 * or_nav.c -- oracle (test infrastructure): navigation state decoding,
 * BVH traversal, navigator step assembly, relocation, safety and point
 * location, plus the multi-threaded batch drivers used as the CPU baseline.
 *
 * Configuration restated: every logical volume with daughters carries
 * BVHNavigator<false> + BVHSafetyEstimator + BVHLevelLocator; leaf volumes
 * carry NewSimpleNavigator (no daughters to test, so its step equals the BVH
 * navigator's) -- the set-up of test/globalbenchmarks/XRayBenchmarkFromROOTFile.cpp:206-238.
 * The navigation index table caches every level's global matrix unless a
 * transformation cache depth is given (GeoManager.cpp:218-221); top_matrix then
 * accumulates the uncached levels' placements (NavStateIndex.h:232-265).
 */
#define _GNU_SOURCE
#include <pthread.h>
#include <time.h>
#include <unistd.h>

#include "or_internal.h"

/* ---- NavStateIndex decoding (NavStateIndex.h:136-265) ---- */
static inline uint32_t ni_word(const or_geom *g, uint32_t i) { return g->navind[i]; }
static inline int ni_top(const or_geom *g, uint32_t ni) { return ni > 0 ? (int)ni_word(g, ni + 1) : -1; }
static inline uint32_t ni_pop(const or_geom *g, uint32_t ni) { return ni > 0 ? ni_word(g, ni) : 0; }
static inline uint32_t ni_push(const or_geom *g, uint32_t ni, int pv)
{
  return ni > 0 ? ni_word(g, ni + 3 + (uint32_t)g->pv[pv].child_id) : 1;
}
static inline unsigned char ni_hasm(const or_geom *g, uint32_t ni)
{
  return ((const unsigned char *)&g->navind[ni + 2])[1];
}
static inline unsigned short ni_nd(const or_geom *g, uint32_t ni)
{
  unsigned short nd;
  memcpy(&nd, ((const unsigned char *)&g->navind[ni + 2]) + 2, 2);
  return nd;
}

/* TopMatrixImpl (NavStateIndex.h:232-265) starting from an identity transform */
static void top_matrix(const or_geom *g, uint32_t ni, or_xf *trans)
{
  unsigned char hasm = 0;
  xf_identity(trans);
  for (;;) {
    or_xf t;
    if (ni == 0) return;
    hasm = ni_hasm(g, ni);
    if (hasm & 0x04) break;
    t = g->pv[ni_top(g, ni)].xf;
    xf_multiply_from_right(&t, trans);
    *trans = t;
    ni     = ni_word(g, ni);
  }
  if ((hasm & 0x03) == 0) return;
  {
    int has_trans = (hasm & 0x02) > 0, has_rot = (hasm & 0x01) > 0, i;
    unsigned short nd = ni_nd(g, ni);
    uint32_t idx      = ni + 3 + nd + ((nd + 1) & 1);
    const double *addr;
    or_xf t;
    if ((idx * 4) % 8 != 0) idx += 1;
    addr = (const double *)&g->navind[idx];
    xf_identity(&t);
    /* Transformation3D::Set (Transformation3D.h:301-316) */
    if (has_trans)
      for (i = 0; i < 3; ++i) t.t[i] = addr[i];
    if (has_rot)
      for (i = 0; i < 9; ++i) t.r[i] = addr[3 + i];
    t.has_trans = has_trans;
    t.has_rot   = has_rot;
    t.identity  = !has_trans && !has_rot;
    xf_multiply_from_right(&t, trans);
    *trans = t;
  }
}

/* placed-volume queries (SpecializedPlacedVolImplHelper.h:118-175, PlacedVolImplHelper.h:69-101) */
static inline double pv_dist_in(const or_geom *g, int pv, v3 p, v3 d, double stepmax, or_counters *c)
{
  const or_xf *x = &g->pv[pv].xf;
  if (c) c->transforms++;
  return shape_dist_in(&g->lv[g->pv[pv].lv], xf_transform(x, p), xf_transform_dir(x, d), stepmax, c);
}
static inline double pv_safe_in(const or_geom *g, int pv, v3 p, or_counters *c)
{
  if (c) c->transforms++;
  return shape_safe_in(&g->lv[g->pv[pv].lv], xf_transform(&g->pv[pv].xf, p), c);
}
static inline int pv_contains_local(const or_geom *g, int pv, v3 p, v3 *lp, or_counters *c)
{
  if (c) c->transforms++;
  *lp = xf_transform(&g->pv[pv].xf, p);
  return shape_contains(&g->lv[g->pv[pv].lv], *lp, c);
}
static inline int pv_unplaced_contains(const or_geom *g, int pv, v3 p)
{
  return shape_contains(&g->lv[g->pv[pv].lv], p, NULL);
}

#define STACK_DEPTH 32 /* BVH::BVH_MAX_DEPTH, BVH.h:33 */

/* BVH::CheckDaughterIntersections (BVH.h:96-146) */
static void bvh_check_daughters(const or_geom *g, const or_lv *lv, v3 lp, v3 ld, double *step, int last, int *hit,
                                or_counters *c)
{
  unsigned stack[STACK_DEPTH], *ptr = &stack[1];
  v3 invdir = v3_make(1.0 / NonZero(ld.x), 1.0 / NonZero(ld.y), 1.0 / NonZero(ld.z));
  stack[0]  = 0;
  do {
    const unsigned id = *--ptr;
    if (lv->nchild[id] >= 0) {
      int i;
      for (i = 0; i < lv->nchild[id]; ++i) {
        const int prim = lv->prim_id[lv->offset[id] + i];
        double tmin, tmax;
        if (c) c->prim_slab++;
        aabb_intersect_invdir(&lv->aabbs[prim], lp, invdir, &tmin, &tmax);
        if (tmin <= tmax && tmax >= 0.0 && tmin < *step) {
          const int vol     = lv->daughters[prim];
          const double dist = pv_dist_in(g, vol, lp, ld, *step, c);
          if (dist < *step && !(dist <= 0.0 && vol == last)) *step = dist, *hit = vol;
        }
      }
    } else {
      const unsigned L = 2 * id + 1, R = 2 * id + 2;
      double tminL = kInfLength, tmaxL = -kInfLength, tminR = kInfLength, tmaxR = -kInfLength;
      int trL, trR;
      if (c) c->node_slab += 2;
      aabb_intersect_invdir(&lv->nodes[L], lp, invdir, &tminL, &tmaxL);
      aabb_intersect_invdir(&lv->nodes[R], lp, invdir, &tminR, &tmaxR);
      trL = tminL <= tmaxL && tmaxL >= 0.0 && tminL < *step;
      trR = tminR <= tmaxR && tmaxR >= 0.0 && tminR < *step;
      if (tminR < tminL) {
        if (trR) *ptr++ = R;
        if (trL) *ptr++ = L;
      } else {
        if (trL) *ptr++ = L;
        if (trR) *ptr++ = R;
      }
    }
  } while (ptr > stack);
}

/* VUnplacedVolume::ApproachSolid (UnplacedVolume.h:274-281): the ray's entry into the shape's
 * bounding box (its Extent, cached at construction), BoxImplementation::IntersectCachedKernel2
 * (BoxImplementation.h:326-368) with t0 = 0, t1 = kInfLength */
static double approach_solid(v3 mn, v3 mx, v3 p, v3 inv)
{
  const v3 c[2] = {mn, mx};
  const int sx = inv.x < 0, sy = inv.y < 0, sz = inv.z < 0;
  double tmin, tmax, tymin, tymax, tzmin, tzmax;
  int done;
  tmin  = (c[sx].x - p.x) * inv.x;
  tymax = (c[1 - sy].y - p.y) * inv.y;
  done  = tmin > tymax;
  if (done) return kInfLength;
  tmax  = (c[1 - sx].x - p.x) * inv.x;
  tymin = (c[sy].y - p.y) * inv.y;
  done |= tymin > tmax;
  if (done) return kInfLength;
  tmin  = tmin > tymin ? tmin : tymin; /* Max(tmin, tymin) */
  tmax  = tmax < tymax ? tmax : tymax; /* Min(tmax, tymax) */
  tzmin = (c[sz].z - p.z) * inv.z;
  tzmax = (c[1 - sz].z - p.z) * inv.z;
  done |= (tmin > tzmax) || (tzmin > tmax);
  if (done) return kInfLength;
  tmin = tmin > tzmin ? tmin : tzmin;
  tmax = tmax < tzmax ? tmax : tzmax;
  done |= !((tmin <= kInfLength + kTolerance) && (tmax > 0. - kTolerance));
  return done ? kInfLength : tmin;
}

/* BVH::ApproachNextDaughter (BVH.cpp:395-449): the traversal of CheckDaughterIntersections with
 * each daughter's ApproachSolid in its own frame in place of its DistanceToIn */
static void bvh_approach(const or_geom *g, const or_lv *lv, v3 lp, v3 ld, double *step, int last)
{
  unsigned stack[STACK_DEPTH], *ptr = &stack[1];
  v3 invdir = v3_make(1.0 / NonZero(ld.x), 1.0 / NonZero(ld.y), 1.0 / NonZero(ld.z));
  stack[0]  = 0;
  do {
    const unsigned id = *--ptr;
    if (lv->nchild[id] >= 0) {
      int i;
      for (i = 0; i < lv->nchild[id]; ++i) {
        const int prim = lv->prim_id[lv->offset[id] + i];
        double tmin, tmax;
        aabb_intersect_invdir(&lv->aabbs[prim], lp, invdir, &tmin, &tmax);
        if (tmin <= tmax && tmax >= 0.0 && tmin < *step) {
          const int vol      = lv->daughters[prim];
          const or_pv *pv    = &g->pv[vol];
          const v3 p         = xf_transform(&pv->xf, lp);
          const v3 d         = xf_transform_dir(&pv->xf, ld);
          const v3 inv       = v3_make(1.0 / NonZero(d.x), 1.0 / NonZero(d.y), 1.0 / NonZero(d.z));
          const or_lv *dlv   = &g->lv[pv->lv];
          const double dist  = approach_solid(dlv->bbox_min, dlv->bbox_max, p, inv);
          if (dist < *step && !(dist <= 0.0 && vol == last)) *step = dist;
        }
      }
    } else {
      const unsigned L = 2 * id + 1, R = 2 * id + 2;
      double tminL = kInfLength, tmaxL = -kInfLength, tminR = kInfLength, tmaxR = -kInfLength;
      int trL, trR;
      aabb_intersect_invdir(&lv->nodes[L], lp, invdir, &tminL, &tmaxL);
      aabb_intersect_invdir(&lv->nodes[R], lp, invdir, &tminR, &tmaxR);
      trL = tminL <= tmaxL && tmaxL >= 0.0 && tminL < *step;
      trR = tminR <= tmaxR && tmaxR >= 0.0 && tminR < *step;
      if (tminR < tminL) {
        if (trR) *ptr++ = R;
        if (trL) *ptr++ = L;
      } else {
        if (trL) *ptr++ = L;
        if (trR) *ptr++ = R;
      }
    }
  } while (ptr > stack);
}

/* NewSimpleNavigator::CheckDaughterIntersections (NewSimpleNavigator.h:30-70) */
static void simple_check_daughters(const or_geom *g, const or_lv *lv, v3 lp, v3 ld, double *step, int last, int *hit)
{
  int d;
  for (d = 0; d < lv->nd; ++d) {
    const int dau    = lv->daughters[d];
    const double dd  = pv_dist_in(g, dau, lp, ld, *step, NULL);
    const int valid  = (dd < *step && !isinf(dd)) && !((dd <= 0.) && last == dau);
    *hit             = valid ? dau : *hit;
    *step            = valid ? dd : *step;
  }
}

/* BVH::ComputeSafety (BVH.h:172-209) */
static double bvh_safety(const or_geom *g, const or_lv *lv, v3 lp, double safety, or_counters *c)
{
  unsigned stack[STACK_DEPTH], *ptr = &stack[1];
  stack[0] = 0;
  do {
    const unsigned id = *--ptr;
    if (lv->nchild[id] >= 0) {
      int i;
      for (i = 0; i < lv->nchild[id]; ++i) {
        const int prim = lv->prim_id[lv->offset[id] + i];
        if (c) c->prim_safety++;
        if (aabb_safety(&lv->aabbs[prim], lp) < safety) {
          const double dist = pv_safe_in(g, lv->daughters[prim], lp, c);
          if (dist < safety) safety = dist;
        }
      }
    } else {
      const unsigned L = 2 * id + 1, R = 2 * id + 2;
      const double sL = aabb_safety(&lv->nodes[L], lp);
      const double sR = aabb_safety(&lv->nodes[R], lp);
      const int trL = sL < safety, trR = sR < safety;
      if (c) c->node_safety += 2;
      if (sR < sL) {
        if (trR) *ptr++ = R;
        if (trL) *ptr++ = L;
      } else {
        if (trL) *ptr++ = L;
        if (trR) *ptr++ = R;
      }
    }
  } while (ptr > stack);
  return safety;
}

/* BVH::LevelLocate(exclvol, localpoint, pvol, daughterlocalpoint) (BVH.h:255-285) */
static int bvh_level_locate(const or_geom *g, const or_lv *lv, int excl, v3 lp, int *pvol, v3 *dlp, or_counters *c)
{
  unsigned stack[STACK_DEPTH], *ptr = &stack[1];
  stack[0] = 0;
  do {
    const unsigned id = *--ptr;
    if (lv->nchild[id] >= 0) {
      int i;
      for (i = 0; i < lv->nchild[id]; ++i) {
        const int prim = lv->prim_id[lv->offset[id] + i];
        if (c) c->prim_contains++;
        if (aabb_contains(&lv->aabbs[prim], lp)) {
          const int vol = lv->daughters[prim];
          if (vol != excl && pv_contains_local(g, vol, lp, dlp, c)) {
            *pvol = vol;
            return 1;
          }
        }
      }
    } else {
      const unsigned L = 2 * id + 1, R = 2 * id + 2;
      if (aabb_contains(&lv->nodes[L], lp)) *ptr++ = L;
      if (aabb_contains(&lv->nodes[R], lp)) *ptr++ = R;
    }
  } while (ptr > stack);
  return 0;
}

/* SimpleAssemblyLevelLocator-equivalent linear scan (used by the brute-force variant) */
static int linear_level_locate(const or_geom *g, const or_lv *lv, int excl, v3 lp, int *pvol, v3 *dlp)
{
  int d;
  for (d = 0; d < lv->nd; ++d) {
    const int vol = lv->daughters[d];
    if (vol != excl && pv_contains_local(g, vol, lp, dlp, NULL)) {
      *pvol = vol;
      return 1;
    }
  }
  return 0;
}

static int level_locate(const or_geom *g, const or_lv *lv, int excl, v3 lp, int *pvol, v3 *dlp, int simple,
                        or_counters *c)
{
  return simple ? linear_level_locate(g, lv, excl, lp, pvol, dlp) : bvh_level_locate(g, lv, excl, lp, pvol, dlp, c);
}

/* GlobalLocator::LocateGlobalPoint (GlobalLocator.h:35-82) */
static int locate_global_point(const or_geom *g, int vol, v3 point, uint32_t *path, int top, int simple,
                               or_counters *c)
{
  int cand = vol;
  v3 cur   = point;
  if (top) cand = pv_unplaced_contains(g, vol, point) ? vol : -1;
  if (cand >= 0) {
    const or_lv *lv;
    int godeeper = 1;
    *path = ni_push(g, *path, cand);
    lv    = &g->lv[g->pv[cand].lv];
    while (lv->nd > 0 && godeeper) {
      int pv;
      v3 tp;
      godeeper = level_locate(g, lv, -1, cur, &pv, &tp, simple, c);
      if (godeeper) {
        *path = ni_push(g, *path, pv);
        cand  = pv;
        lv    = &g->lv[g->pv[cand].lv];
        cur   = tp;
      }
    }
  }
  return cand >= 0 ? ni_top(g, *path) : -1;
}

/* GlobalLocator::LocateGlobalPointExclVolume (GlobalLocator.h:88-135) */
static int locate_global_point_excl(const or_geom *g, int vol, int excl, v3 point, uint32_t *path, int simple,
                                    or_counters *c)
{
  int cand = vol;
  v3 cur   = point;
  if (cand >= 0) {
    const or_lv *lv;
    int godeeper = 1;
    *path = ni_push(g, *path, cand);
    lv    = &g->lv[g->pv[cand].lv];
    while (lv->nd > 0 && godeeper) {
      v3 tp;
      godeeper = level_locate(g, lv, excl, cur, &cand, &tp, simple, c);
      if (godeeper) {
        lv    = &g->lv[g->pv[cand].lv];
        cur   = tp;
        *path = ni_push(g, *path, cand);
      }
    }
  }
  return cand;
}

/* GlobalLocator::RelocatePointFromPathForceDifferent (GlobalLocator.h:171-200) */
static void relocate_force_different(const or_geom *g, v3 lp, uint32_t *path, int simple, or_counters *c)
{
  int cm = ni_top(g, *path), entry = cm;
  if (cm >= 0) {
    v3 tmp = lp;
    while (cm >= 0) {
      if (cm == entry || !pv_unplaced_contains(g, cm, tmp)) {
        *path = ni_pop(g, *path);
        tmp   = xf_inverse_transform(&g->pv[cm].xf, tmp);
        cm    = ni_top(g, *path);
      } else
        break;
    }
    if (cm >= 0) {
      *path = ni_pop(g, *path);
      locate_global_point_excl(g, cm, entry, tmp, path, simple, c);
    }
  }
}

/* VNavigatorHelper::Relocate (VNavigator.h:1070-1091) */
static void relocate(const or_geom *g, v3 pab, const or_state *in, or_state *out, int simple, or_counters *c)
{
  if (ni_top(g, out->nav_ind) == ni_top(g, in->nav_ind)) {
    relocate_force_different(g, pab, &out->nav_ind, simple, c);
  } else {
    const int nextvol = ni_top(g, out->nav_ind);
    out->nav_ind      = ni_pop(g, out->nav_ind);
    locate_global_point(g, nextvol, xf_transform(&g->pv[nextvol].xf, pab), &out->nav_ind, 0, simple, c);
  }
}

/* BVHSafetyEstimator::ComputeSafetyForLocalPoint (BVHSafetyEstimator.h:38-46) */
static double safety_local(const or_geom *g, v3 lp, int pv, or_counters *c)
{
  const or_lv *lv = &g->lv[g->pv[pv].lv];
  double safety   = shape_safe_out(lv, lp, c);
  if (safety > 0.0 && lv->nd > 0) safety = bvh_safety(g, lv, lp, safety, c);
  return safety;
}

/* ComputeStepAndSafetyAndPropagatedState (VNavigator.h:1014-1064) with
 * PrepareOutState (VNavigator.h:192-235), TreatDistanceToMother (241-249)
 * and MovePointAfterBoundary (168-173); relocate = 0 gives ComputeStep (494-540) */
static double nav_step(const or_geom *g, v3 gp, v3 gd, double slimit, const or_state *in, or_state *out,
                       int calcsafety, double *safety_out, int simple, int do_reloc, or_counters *c)
{
  or_xf m;
  v3 lp, ld;
  double step;
  int hit = -1, pv, last;
  const or_lv *lv;

  top_matrix(g, in->nav_ind, &m);
  lp = xf_transform(&m, gp);
  ld = xf_transform_dir(&m, gd);
  pv = ni_top(g, in->nav_ind);
  lv = &g->lv[g->pv[pv].lv];
  if (safety_out) {
    *safety_out = 0.;
    if (calcsafety) *safety_out = simple ? 0. : safety_local(g, lp, pv, c);
  }

  step = shape_dist_out(lv, lp, ld, slimit, c);
  if (step < 0.) step = 0.;
  last = ni_top(g, in->last_exited);
  if (lv->nd > 0) {
    if (simple)
      simple_check_daughters(g, lv, lp, ld, &step, last, &hit);
    else
      bvh_check_daughters(g, lv, lp, ld, &step, last, &hit, c);
  }

  *out = *in;
  if (step == kInfLength && slimit > 0.) {
    out->on_boundary = 1;
    out->nav_ind     = ni_pop(g, out->nav_ind);
    return kTolerance;
  }
  if (step > slimit) {
    out->on_boundary = 0;
    return slimit;
  }
  out->on_boundary = 1;
  out->last_exited = out->nav_ind;
  if (hit >= 0) out->nav_ind = ni_push(g, out->nav_ind, hit);
  if (step < 0.) step = 0.;
  if (!do_reloc) return step;
  relocate(g, v3_add(lp, v3_scale(step + 1E-6, ld)), in, out, simple, c);
  return step;
}

/* ---------------------------------------------------------------- */
/* threaded batch drivers                                            */
/* ---------------------------------------------------------------- */

typedef struct {
  const or_geom *g;
  long lo, hi;
  const double *px, *py, *pz, *dx, *dy, *dz, *slimit;
  const or_state *in;
  or_state *out;
  double *step, *safety;
  int calcsafety, simple, mode; /* mode 0 step+reloc, 1 step no reloc, 2 safety, 3 locate */
  or_counters cnt;
  int count;
} job_t;

static void *job_run(void *arg)
{
  job_t *j = (job_t *)arg;
  long i;
  or_counters *c = j->count ? &j->cnt : NULL;
  for (i = j->lo; i < j->hi; ++i) {
    v3 p = v3_make(j->px[i], j->py[i], j->pz[i]);
    if (j->mode == 0 || j->mode == 1) {
      v3 d = v3_make(j->dx[i], j->dy[i], j->dz[i]);
      j->step[i] = nav_step(j->g, p, d, j->slimit[i], &j->in[i], &j->out[i], j->calcsafety,
                            j->safety ? &j->safety[i] : NULL, j->simple, j->mode == 0, c);
    } else if (j->mode == 2) {
      or_xf m;
      int pv = ni_top(j->g, j->in[i].nav_ind);
      top_matrix(j->g, j->in[i].nav_ind, &m);
      j->safety[i] = safety_local(j->g, xf_transform(&m, p), pv, c);
    } else {
      or_state s;
      memset(&s, 0, sizeof(s));
      locate_global_point(j->g, j->g->world_pv, p, &s.nav_ind, 1, 0, c);
      j->out[i] = s;
    }
  }
  return NULL;
}

int or_ncores(void)
{
  long n = sysconf(_SC_NPROCESSORS_ONLN);
  return n > 0 ? (int)n : 1;
}

double or_now(void)
{
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static void run_jobs(job_t *proto, long n, int nthreads, or_counters *counters)
{
  int t, k;
  job_t *jobs;
  pthread_t *th;
  if (nthreads <= 0) nthreads = or_ncores();
  if (nthreads > 256) nthreads = 256;
  if ((long)nthreads > n) nthreads = n > 0 ? (int)n : 1;
  jobs = (job_t *)calloc((size_t)nthreads, sizeof(job_t));
  th   = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
  for (t = 0; t < nthreads; ++t) {
    jobs[t]       = *proto;
    jobs[t].lo    = n * t / nthreads;
    jobs[t].hi    = n * (t + 1) / nthreads;
    jobs[t].count = counters != NULL;
    memset(&jobs[t].cnt, 0, sizeof(or_counters));
  }
  if (nthreads == 1)
    job_run(&jobs[0]);
  else {
    for (t = 0; t < nthreads; ++t) pthread_create(&th[t], NULL, job_run, &jobs[t]);
    for (t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
  }
  if (counters) {
    memset(counters, 0, sizeof(*counters));
    for (t = 0; t < nthreads; ++t) {
      const or_counters *s = &jobs[t].cnt;
      counters->node_slab += s->node_slab;
      counters->prim_slab += s->prim_slab;
      counters->node_safety += s->node_safety;
      counters->prim_safety += s->prim_safety;
      counters->prim_contains += s->prim_contains;
      counters->transforms += s->transforms;
      for (k = 0; k < OR_NSHAPES * 6; ++k) (&counters->kernel[0][0])[k] += (&s->kernel[0][0])[k];
    }
  }
  free(jobs);
  free(th);
}

void or_nav_step_batch(const or_geom *g, long n, const double *px, const double *py, const double *pz,
                       const double *dx, const double *dy, const double *dz, const double *slimit,
                       const or_state *in, or_state *out, double *step, double *safety, int calcsafety, int simple,
                       int nthreads, or_counters *counters)
{
  job_t j;
  memset(&j, 0, sizeof(j));
  j.g = g; j.px = px; j.py = py; j.pz = pz; j.dx = dx; j.dy = dy; j.dz = dz; j.slimit = slimit;
  j.in = in; j.out = out; j.step = step; j.safety = safety; j.calcsafety = calcsafety; j.simple = simple;
  j.mode = 0;
  run_jobs(&j, n, nthreads, counters);
}

void or_nav_step_norel_batch(const or_geom *g, long n, const double *px, const double *py, const double *pz,
                             const double *dx, const double *dy, const double *dz, const double *slimit,
                             const or_state *in, or_state *out, double *step, int nthreads)
{
  job_t j;
  memset(&j, 0, sizeof(j));
  j.g = g; j.px = px; j.py = py; j.pz = pz; j.dx = dx; j.dy = dy; j.dz = dz; j.slimit = slimit;
  j.in = in; j.out = out; j.step = step; j.mode = 1;
  run_jobs(&j, n, nthreads, NULL);
}

void or_safety_batch(const or_geom *g, long n, const double *px, const double *py, const double *pz,
                     const or_state *in, double *safety, int nthreads)
{
  job_t j;
  memset(&j, 0, sizeof(j));
  j.g = g; j.px = px; j.py = py; j.pz = pz; j.in = in; j.safety = safety; j.mode = 2;
  run_jobs(&j, n, nthreads, NULL);
}

void or_locate_batch(const or_geom *g, long n, const double *px, const double *py, const double *pz, or_state *out,
                     int nthreads)
{
  job_t j;
  memset(&j, 0, sizeof(j));
  j.g = g; j.px = px; j.py = py; j.pz = pz; j.out = out; j.mode = 3;
  run_jobs(&j, n, nthreads, NULL);
}

/* BVH::ApproachNextDaughter per track over logical volume lv[i]'s BVH (local point and
 * direction, step in/out, last[i] the last exited placed volume or -1); 1 if a volume has no BVH */
int or_approach_batch(const or_geom *g, long n, const int *lv, const double *px, const double *py,
                      const double *pz, const double *dx, const double *dy, const double *dz, const int *last,
                      double *step)
{
  long i;
  for (i = 0; i < n; ++i)
    if (lv[i] < 0 || lv[i] >= g->n_lv || g->lv[lv[i]].nd == 0) return 1;
  for (i = 0; i < n; ++i)
    bvh_approach(g, &g->lv[lv[i]], v3_make(px[i], py[i], pz[i]), v3_make(dx[i], dy[i], dz[i]), &step[i], last[i]);
  return 0;
}

/* the shape's extent (VUnplacedVolume::Extent): min then max corner */
int or_shape_extent(const or_geom *g, int lvi, double *out6)
{
  v3 mn, mx;
  if (lvi < 0 || lvi >= g->n_lv) return -1;
  shape_extent(&g->lv[lvi], &mn, &mx);
  out6[0] = mn.x, out6[1] = mn.y, out6[2] = mn.z, out6[3] = mx.x, out6[4] = mx.y, out6[5] = mx.z;
  return 0;
}

/* unplaced shape queries */
int or_shape_batch(const or_geom *g, int lvi, int op, long n, const double *px, const double *py, const double *pz,
                   const double *dx, const double *dy, const double *dz, const double *stepmax, double *out)
{
  const or_lv *lv;
  long i;
  if (lvi < 0 || lvi >= g->n_lv || op < 0 || op > 5) return -1;
  lv = &g->lv[lvi];
  for (i = 0; i < n; ++i) {
    v3 p = v3_make(px[i], py[i], pz[i]);
    v3 d = (op <= OR_OP_DIST_OUT) ? v3_make(dx[i], dy[i], dz[i]) : v3_make(0, 0, 0);
    double sm = stepmax ? stepmax[i] : kInfLength;
    switch (op) {
    case OR_OP_DIST_IN: out[i] = shape_dist_in(lv, p, d, sm, NULL); break;
    case OR_OP_DIST_OUT: out[i] = shape_dist_out(lv, p, d, sm, NULL); break;
    case OR_OP_SAFE_IN: out[i] = shape_safe_in(lv, p, NULL); break;
    case OR_OP_SAFE_OUT: out[i] = shape_safe_out(lv, p, NULL); break;
    case OR_OP_CONTAINS: out[i] = (double)shape_contains(lv, p, NULL); break;
    case OR_OP_INSIDE: out[i] = (double)shape_inside(lv, p, NULL); break;
    }
  }
  return 0;
}
