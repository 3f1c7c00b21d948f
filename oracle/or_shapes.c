/*
 * or_shapes.c -- oracle (test infrastructure): unplaced shape kernels.
 * Each function restates the scalar (Real_v = double) instantiation of the
 * reference kernel it cites, with the same operation order.
 */
#include <stdio.h>

#include "or_internal.h"

enum { kInsideE = 1, kSurfaceE = 2, kOutsideE = 3 };

static void set_err(char *err, int errlen, const char *msg)
{
  if (err && errlen > 0) snprintf(err, (size_t)errlen, "%s", msg);
}

/* ================================================================== */
/* Box: VecGeom/volumes/kernel/BoxImplementation.h:73-167             */
/* ================================================================== */

static int box_contains(const or_box *b, v3 p)
{
  v3 h = v3_make(b->d[0], b->d[1], b->d[2]);
  return v3_maxc(v3_sub(v3_abs(p), h)) < 0.0;
}

static int box_inside(const or_box *b, v3 p)
{
  v3 h        = v3_make(b->d[0], b->d[1], b->d[2]);
  double dist = v3_maxc(v3_sub(v3_abs(p), h));
  int inside  = dist < 0.0 ? kInsideE : kOutsideE;
  if (fabs(dist) < kHalfTolerance) inside = kSurfaceE;
  return inside;
}

static double box_dist_in(const or_box *b, v3 p, v3 d)
{
  v3 h      = v3_make(b->d[0], b->d[1], b->d[2]);
  v3 invDir = v3_make(1.0 / NonZero(d.x), 1.0 / NonZero(d.y), 1.0 / NonZero(d.z));
  v3 sgn    = v3_make(or_sign(d.x), or_sign(d.y), or_sign(d.z));
  v3 nsgn   = v3_make(-sgn.x, -sgn.y, -sgn.z);
  v3 tempIn  = v3_sub(v3_mul(nsgn, h), p);
  v3 tempOut = v3_sub(v3_mul(sgn, h), p);
  double absOrthogOut = fabs(v3_minc(v3_mul(sgn, tempOut)));
  double distOut      = v3_minc(v3_mul(tempOut, invDir));
  double distance     = v3_maxc(v3_mul(tempIn, invDir));
  if (distance >= distOut || distOut <= kHalfTolerance || absOrthogOut <= kHalfTolerance) distance = kInfLength;
  return distance;
}

static double box_dist_out(const or_box *b, v3 p, v3 d)
{
  v3 h      = v3_make(b->d[0], b->d[1], b->d[2]);
  v3 invDir = v3_make(1.0 / NonZero(d.x), 1.0 / NonZero(d.y), 1.0 / NonZero(d.z));
  v3 sgn    = v3_make(or_sign(d.x), or_sign(d.y), or_sign(d.z));
  double safetyIn = v3_maxc(v3_sub(v3_abs(p), h));
  v3 tempOut      = v3_sub(v3_mul(sgn, h), p);
  double distance = v3_minc(v3_mul(tempOut, invDir));
  if (safetyIn > kHalfTolerance) distance = -1.0;
  return distance;
}

static double box_safe_in(const or_box *b, v3 p)
{
  v3 h = v3_make(b->d[0], b->d[1], b->d[2]);
  return v3_maxc(v3_sub(v3_abs(p), h));
}

static double box_safe_out(const or_box *b, v3 p)
{
  v3 h = v3_make(b->d[0], b->d[1], b->d[2]);
  return v3_minc(v3_sub(h, v3_abs(p)));
}

/* ================================================================== */
/* Tube (UniversalTube, full phi): kernel/TubeImplementation.h        */
/* ================================================================== */

/* TubeStruct constructor + CalculateCached (TubeStruct.h:43-72, 153-175) */
static int tube_init(or_tube *t, const double *a, char *err, int errlen)
{
  t->rmin = a[0] < 0.0 ? 0.0 : a[0];
  t->rmax = a[1];
  t->z    = a[2];
  t->sphi = a[3];
  t->dphi = a[4];
  if (t->dphi < kTwoPi) {
    set_err(err, errlen, "tube: phi sections are not supported");
    return -1;
  }
  /* UpdatedZ */
  t->tolIz  = t->z - kHalfTolerance;
  t->tolOz  = t->z + kHalfTolerance;
  t->maxval = or_max(t->rmax, t->z);
  /* UpdatedRMin */
  t->rmin2     = t->rmin * t->rmin;
  t->tolOrmin  = (t->rmin - kHalfTolerance);
  t->tolIrmin  = (t->rmin + kHalfTolerance);
  t->tolOrmin2 = t->tolOrmin * t->tolOrmin;
  t->tolIrmin2 = t->tolIrmin * t->tolIrmin;
  /* UpdatedRMax */
  t->rmax2     = t->rmax * t->rmax;
  t->tolOrmax  = (t->rmax + kHalfTolerance);
  t->tolIrmax  = (t->rmax - kHalfTolerance);
  t->tolOrmax2 = t->tolOrmax * t->tolOrmax;
  t->tolIrmax2 = t->tolIrmax * t->tolIrmax;
  t->maxval    = or_max(t->rmax, t->z);
  t->alongphi1x = cos(t->sphi);
  t->alongphi1y = sin(t->sphi);
  t->alongphi2x = cos(t->sphi + t->dphi);
  t->alongphi2y = sin(t->sphi + t->dphi);
  t->maxval     = or_max(t->rmax, t->z);
  return 0;
}

/* TubeUtilities::CircleTrajectoryIntersection (TubeImplementation.h:103-160), full phi */
static void tube_circle(double b, double c, const or_tube *t, v3 pos, v3 dir, int largest, int insector, double *dist,
                        int *ok)
{
  double delta = b * b - c;
  *ok          = delta > 0.;
  if (largest) *ok |= delta == 0.;
  if (!*ok) delta = 0.;
  delta = sqrt(delta);
  if (!largest) delta = -delta;
  *dist = -b + delta;
  *ok &= *dist >= -2 * kTolerance;
  if (!*ok) return;
  if (insector) {
    double hitz = pos.z + *dist * dir.z;
    *ok &= (fabs(hitz) <= t->z);
  }
}

/* DistanceToInKernel (TubeImplementation.h:504-681), rmin treatment at run time */
static double tube_dist_in_kernel(const or_tube *t, v3 p, v3 d)
{
  int done = 0, inside, okz, onsurf, ok_rmax, ok_rmin;
  double distance = kInfLength, distz, rsq, rdotn, hitx, hity, r2, invnsq, b, crmax, dist_rmax, dist_rmin;
  const int hasrmin = t->rmin > 0;

  distz = fabs(p.z) - t->z;
  done |= distz > kHalfTolerance && p.z * d.z >= 0;
  rsq   = p.x * p.x + p.y * p.y;
  rdotn = p.x * d.x + p.y * d.y;
  done |= rsq > t->tolIrmax2 && rdotn >= 0;
  if (done) return distance;

  distance = -1.0;
  inside   = distz < -kHalfTolerance;
  inside &= rsq < t->tolIrmax2;
  if (hasrmin) inside &= rsq > t->tolIrmin2;
  done |= inside;
  if (done) return distance;

  distance = kInfLength;
  distz /= NonZeroAbs(d.z);
  hitx = p.x + distz * d.x;
  hity = p.y + distz * d.y;
  r2   = hitx * hitx + hity * hity;
  okz  = distz > -kHalfTolerance && (p.z * d.z < 0);
  okz &= (r2 <= t->rmax2);
  if (hasrmin) okz &= (t->rmin2 <= r2);
  if (!done && okz) distance = distz;
  done |= okz;

  {
    /* IsMovingInsideTubeSurface (TubeImplementation.h:399-435) */
    const double rho = p.x * p.x + p.y * p.y;
    onsurf = (rho >= t->tolIrmax2) && (rho <= t->tolOrmax2) && (fabs(p.z) < (t->z + kTolerance)) &&
             (d.x * p.x + d.y * p.y + d.z * 0. <= 0.);
    if (hasrmin)
      onsurf |= (rho >= t->tolOrmin2) && (rho <= t->tolIrmin2) && (fabs(p.z) < (t->z + kTolerance)) &&
                (d.x * -p.x + d.y * -p.y + d.z * 0. <= 0.);
  }
  if (!done && onsurf) distance = 0.;
  done |= onsurf;
  if (done) return distance;

  invnsq = 1. / NonZero(1. - d.z * d.z);
  b      = invnsq * rdotn;
  crmax  = invnsq * (rsq - t->rmax2);
  tube_circle(b, crmax, t, p, d, 0, 1, &dist_rmax, &ok_rmax);
  ok_rmax &= dist_rmax < distance;
  if (!done && ok_rmax) distance = dist_rmax;
  done |= ok_rmax;
  if (done) return distance;

  if (hasrmin) {
    double crmin = invnsq * (rsq - t->rmin2);
    tube_circle(b, crmin, t, p, d, 1, 1, &dist_rmin, &ok_rmin);
    ok_rmin &= dist_rmin < distance;
    if (!done && ok_rmin) distance = dist_rmin;
  }
  return distance;
}

/* DistanceToIn with the far-point pre-move (TubeImplementation.h:475-502) */
static double tube_dist_in(const or_tube *t, v3 pt, v3 d)
{
  v3 p          = pt;
  double ptDist = sqrt(v3_mag2(p));
  double distToMove = 0., distance;
  const double order = 100.;
  if (ptDist > order * t->maxval) {
    distToMove = ptDist - order * t->maxval;
    p          = v3_add(p, v3_scale(distToMove, d));
  }
  distance = tube_dist_in_kernel(t, p, d);
  distance += distToMove;
  return distance;
}

/* DistanceToOut (TubeImplementation.h:683-823) */
static double tube_dist_out(const or_tube *t, v3 p, v3 d)
{
  int done = 0, ok_rmin, ok_rmax;
  double distance = -1., distz, rsq, rdotn, crmax, crmin, invdirz, invnsq, b, dist_rmin, dist_rmax;
  const int hasrmin = t->rmin > 0;

  distz = t->z - fabs(p.z);
  done |= distz < -kHalfTolerance;
  if (done) return distance;
  rsq   = p.x * p.x + p.y * p.y;
  rdotn = d.x * p.x + d.y * p.y;
  crmax = rsq - t->rmax2;
  crmin = rsq;
  done |= crmax > 2.0 * kTolerance * t->rmax;
  if (done) return distance;
  if (hasrmin) {
    crmin -= t->rmin2;
    done |= crmin < -2.0 * kTolerance * t->rmin;
    if (done) return distance;
  }
  distance = kInfLength;
  invdirz  = 1. / NonZero(d.z);
  distz    = (t->z - p.z) * invdirz;
  if (d.z < 0) distz = (-t->z - p.z) * invdirz;
  if (d.z != 0. && distz < distance) distance = distz;

  invnsq = 1. / NonZero(1. - d.z * d.z);
  b      = invnsq * rdotn;
  if (hasrmin) {
    crmin *= invnsq;
    tube_circle(b, crmin, t, p, d, 0, 0, &dist_rmin, &ok_rmin);
    if (ok_rmin && dist_rmin < distance) distance = dist_rmin;
  }
  crmax *= invnsq;
  tube_circle(b, crmax, t, p, d, 1, 0, &dist_rmax, &ok_rmax);
  if (ok_rmax && dist_rmax < distance) distance = dist_rmax;
  return distance;
}

/* SafetyToInOld (TubeImplementation.h:912-938) */
static double tube_safe_in(const or_tube *t, v3 p)
{
  double safety = fabs(p.z) - t->z;
  double r      = sqrt(p.x * p.x + p.y * p.y);
  double safermax = r - t->rmax;
  if (safermax > safety) safety = safermax;
  if (t->rmin > 0) {
    double safermin = t->rmin - r;
    if (safermin > safety) safety = safermin;
  }
  return safety;
}

/* SafetyToOutOld (TubeImplementation.h:940-960) */
static double tube_safe_out(const or_tube *t, v3 p)
{
  double safety = t->z - fabs(p.z);
  double r      = sqrt(p.x * p.x + p.y * p.y);
  double safermax = t->rmax - r;
  if (safermax < safety) safety = safermax;
  if (t->rmin > 0) {
    double safermin = r - t->rmin;
    if (safermin < safety) safety = safermin;
  }
  return safety;
}

/* GenericKernelForContainsAndInside (TubeImplementation.h:392-450) with
 * MakePlus/MinusTolerant[Square] (kernel/GenericKernels.h:26-82) */
static void tube_generic_ci(const or_tube *t, v3 p, int forinside, int *cin, int *cout)
{
  double absz = fabs(p.z), r2;
  *cout = absz > (forinside ? t->z + kHalfTolerance : t->z);
  if (forinside) *cin = absz < t->z - kHalfTolerance;
  if (*cout) return;
  r2 = p.x * p.x + p.y * p.y;
  *cout |= r2 > (forinside ? t->rmax * (t->rmax + 2.0 * kTolerance) : t->rmax * t->rmax);
  if (forinside) *cin &= r2 < fabs(t->rmax * (t->rmax - 2.0 * kTolerance));
  if (*cout) return;
  if (t->rmin > 0) {
    *cout |= r2 <= (forinside ? fabs(t->rmin * (t->rmin - 2.0 * kTolerance)) : t->rmin * t->rmin);
    if (forinside) *cin &= r2 > t->rmin * (t->rmin + 2.0 * kTolerance);
  }
}

static int tube_contains(const or_tube *t, v3 p)
{
  int cin = 0, cout = 0;
  tube_generic_ci(t, p, 0, &cin, &cout);
  return !cout;
}

static int tube_inside(const or_tube *t, v3 p)
{
  int cin = 0, cout = 0, r = kSurfaceE;
  tube_generic_ci(t, p, 1, &cin, &cout);
  if (cout) r = kOutsideE;
  if (cin) r = kInsideE;
  return r;
}

/* UnplacedTube::Extent (source/UnplacedTube.cpp:214-220), full phi */
static void tube_extent(const or_tube *t, v3 *mn, v3 *mx)
{
  *mn = v3_make(-t->rmax, -t->rmax, -t->z);
  *mx = v3_make(t->rmax, t->rmax, t->z);
}

/* ================================================================== */
/* dispatch                                                           */
/* ================================================================== */

int shape_init(or_lv *lv, const double *p, int n_avail, char *err, int errlen)
{
  (void)n_avail;
  switch (lv->type) {
  case OR_BOX:
    lv->s.box.d[0] = p[0];
    lv->s.box.d[1] = p[1];
    lv->s.box.d[2] = p[2];
    return 0;
  case OR_TUBE: return tube_init(&lv->s.tube, p, err, errlen);
  default: set_err(err, errlen, "unsupported shape type"); return -1;
  }
}

void shape_extent(const or_lv *lv, v3 *mn, v3 *mx)
{
  switch (lv->type) {
  case OR_BOX:
    *mn = v3_make(-lv->s.box.d[0], -lv->s.box.d[1], -lv->s.box.d[2]);
    *mx = v3_make(lv->s.box.d[0], lv->s.box.d[1], lv->s.box.d[2]);
    return;
  case OR_TUBE: tube_extent(&lv->s.tube, mn, mx); return;
  }
}

#define COUNT(op) \
  if (c) c->kernel[lv->type][op]++

double shape_dist_in(const or_lv *lv, v3 p, v3 d, double stepmax, or_counters *c)
{
  (void)stepmax;
  COUNT(OR_OP_DIST_IN);
  switch (lv->type) {
  case OR_BOX: return box_dist_in(&lv->s.box, p, d);
  case OR_TUBE: return tube_dist_in(&lv->s.tube, p, d);
  }
  return kInfLength;
}

double shape_dist_out(const or_lv *lv, v3 p, v3 d, double stepmax, or_counters *c)
{
  (void)stepmax;
  COUNT(OR_OP_DIST_OUT);
  switch (lv->type) {
  case OR_BOX: return box_dist_out(&lv->s.box, p, d);
  case OR_TUBE: return tube_dist_out(&lv->s.tube, p, d);
  }
  return -1.;
}

double shape_safe_in(const or_lv *lv, v3 p, or_counters *c)
{
  COUNT(OR_OP_SAFE_IN);
  switch (lv->type) {
  case OR_BOX: return box_safe_in(&lv->s.box, p);
  case OR_TUBE: return tube_safe_in(&lv->s.tube, p);
  }
  return kInfLength;
}

double shape_safe_out(const or_lv *lv, v3 p, or_counters *c)
{
  COUNT(OR_OP_SAFE_OUT);
  switch (lv->type) {
  case OR_BOX: return box_safe_out(&lv->s.box, p);
  case OR_TUBE: return tube_safe_out(&lv->s.tube, p);
  }
  return 0.;
}

int shape_contains(const or_lv *lv, v3 p, or_counters *c)
{
  COUNT(OR_OP_CONTAINS);
  switch (lv->type) {
  case OR_BOX: return box_contains(&lv->s.box, p);
  case OR_TUBE: return tube_contains(&lv->s.tube, p);
  }
  return 0;
}

int shape_inside(const or_lv *lv, v3 p, or_counters *c)
{
  COUNT(OR_OP_INSIDE);
  switch (lv->type) {
  case OR_BOX: return box_inside(&lv->s.box, p);
  case OR_TUBE: return tube_inside(&lv->s.tube, p);
  }
  return kOutsideE;
}
